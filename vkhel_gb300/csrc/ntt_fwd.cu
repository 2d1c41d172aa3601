// Launcher of the CTA-resident forward transforms for 2^8 <= n <= 2^14 (kernel in
// ntt_core.cuh); one translation unit per kernel family so they compile in
// parallel.
#include "ntt_core.cuh"

namespace vk {

template <int LOGN, int E, int U>
static int launch(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int sub_log, int sms) {
  using S = Shape<LOGN, E, U>;
  auto kern = k_ntt_fwd<LOGN, E, U>;
  static KernelSetup setup;
  int per_sm = 1;
  if (const int e = setup_cta(kern, S::T, S::SMEM_BYTES, setup, &per_sm)) return e;
  const int grid = grid_from(per_sm, (long)njobs << sub_log, sms);
  kern<<<grid, S::T, S::SMEM_BYTES, st>>>(jobs, njobs, one, sub_log);
  vkcu_count_launches(1);
  return (int)cudaGetLastError();
}

int fwd_cta(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int log_n, int sub_log, int sms,
            int variant) {
retry:
#define X(L, E, U) launch<L, E, U>(st, jobs, njobs, one, sub_log, sms)
  VK_FOR_LOGN(X)
#undef X
}

}  // namespace vk
