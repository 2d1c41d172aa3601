// Launcher of the CTA-resident inverse transforms with a fused epilogue (the
// reference's centred-lift element-wise ops after the last stage) for
// 2^8 <= n <= 2^14, default shape of each degree.
#include "ntt_core.cuh"

namespace vk {

template <int LOGN, int E, int U>
static int launch_lift(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int sms,
                       const vkcu_lift& lift) {
  using S = Shape<LOGN, E, U>;
  auto kern = k_ntt_inv<LOGN, E, U, true>;
  static KernelSetup setup;
  int per_sm = 1;
  if (const int e = setup_cta(kern, S::T, S::SMEM_BYTES, setup, &per_sm)) return e;
  const int grid = grid_from(per_sm, (long)njobs, sms);
  kern<<<grid, S::T, S::SMEM_BYTES, st>>>(jobs, njobs, one, 0, lift);
  vkcu_count_launches(1);
  return (int)cudaGetLastError();
}

int inv_cta_lift(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int log_n, int sms,
                 const vkcu_lift& lift) {
#define X(L, E, U) launch_lift<L, E, U>(st, jobs, njobs, one, sms, lift)
  VK_FOR_LOGN_DEFAULT(X)
#undef X
}

}  // namespace vk
