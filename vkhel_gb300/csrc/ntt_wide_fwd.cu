// Forward transforms for moduli 2^62 <= q < 2^63 (the Mod63 instantiations of
// the kernels in ntt_core.cuh and ntt_cluster.cuh): one CTA per transform for
// 2^8 <= n <= 2^14 (default shape of each degree), a cluster of 2 / 4 / 8
// CTAs for 2^15 .. 2^17, and the 2^14-word sub-blocks after the global
// passes of larger n.
#include "ntt_cluster.cuh"

namespace vk {

int fwd_cta_wide(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int log_n,
                 int sub_log, int sms) {
#define X(L, E, U) \
  launch_cta<Shape<L, E, U, Mod63>, k_ntt_fwd<L, E, U, Mod63>>(st, (long)njobs << sub_log, sms, jobs, njobs, one, sub_log)
  VK_FOR_LOGN_DEFAULT(X)
#undef X
}

int fwd_cluster_wide(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int logc) {
  switch (logc) {
#define X(L) \
  case L:    \
    return launch_cluster<L, SubShape63, k_ntt_fwd_cluster<L, SubShape63>>(st, njobs, jobs, njobs, one);
    X(1)
    X(2)
    X(3)
#undef X
    default:
      return (int)cudaErrorInvalidValue;
  }
}

}  // namespace vk
