// Fused polynomial multiplies with the centred-lift epilogue for moduli
// 2^62 <= q < 2^63 (Mod63), 2^8 <= n <= 2^14, default shape of each degree.
#include "ntt_core.cuh"

namespace vk {

int poly_cta_wide_lifted(cudaStream_t st, const vkcu_poly_job* jobs, int njobs, const vkcu_poly_job& one, int log_n,
                         int sms, const vkcu_lift& lift) {
#define X(L, E, U) \
  launch_cta<Shape<L, E, U, Mod63>, k_polymul<L, E, U, true, Mod63>>(st, (long)njobs, sms, jobs, njobs, one, lift)
  VK_FOR_LOGN_DEFAULT(X)
#undef X
}

}  // namespace vk
