// Inverse transforms for moduli 2^62 <= q < 2^63 (Mod63): one CTA per
// transform for 2^8 <= n <= 2^14 (default shape of each degree), with or
// without the fused centred-lift epilogue, and the 2^14-word sub-blocks
// before the global passes of larger n.
#include "ntt_core.cuh"

namespace vk {

int inv_cta_wide(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int log_n,
                 int sub_log, int sms, const vkcu_lift* lift) {
  if (lift) {
#define X(L, E, U) \
  launch_cta<Shape<L, E, U, Mod63>, k_ntt_inv<L, E, U, true, Mod63>>(st, (long)njobs, sms, jobs, njobs, one, 0, *lift)
    VK_FOR_LOGN_DEFAULT(X)
#undef X
  }
  const vkcu_lift none{};
#define X(L, E, U)                                                                                                \
  launch_cta<Shape<L, E, U, Mod63>, k_ntt_inv<L, E, U, false, Mod63>>(st, (long)njobs << sub_log, sms, jobs, njobs, \
                                                                       one, sub_log, none)
  VK_FOR_LOGN_DEFAULT(X)
#undef X
}

}  // namespace vk
