// Inverse transforms and fused polynomial multiplies on a cluster of 2 / 4 / 8
// CTAs (n = 2^15 .. 2^17) for moduli 2^62 <= q < 2^63 (Mod63), with or
// without the centred-lift epilogue.
#include "ntt_cluster.cuh"

namespace vk {

int inv_cluster_wide(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int logc,
                     const vkcu_lift* lift) {
  const vkcu_lift none{};
  switch (logc * 2 + (lift ? 1 : 0)) {
#define X(L)                                                                                                  \
  case 2 * L:                                                                                                 \
    return launch_cluster<L, SubShape63, k_ntt_inv_cluster<L, SubShape63, false>>(st, njobs, jobs, njobs, one, \
                                                                                  none);                      \
  case 2 * L + 1:                                                                                             \
    return launch_cluster<L, SubShape63, k_ntt_inv_cluster<L, SubShape63, true>>(st, njobs, jobs, njobs, one, *lift);
    X(1)
    X(2)
    X(3)
#undef X
    default:
      return (int)cudaErrorInvalidValue;
  }
}

int poly_cluster_wide(cudaStream_t st, const vkcu_poly_job* jobs, int njobs, const vkcu_poly_job& one, int logc,
                      const vkcu_lift* lift) {
  const vkcu_lift none{};
  switch (logc * 2 + (lift ? 1 : 0)) {
#define X(L)                                                                                                    \
  case 2 * L:                                                                                                   \
    return launch_cluster<L, SubShape63, k_polymul_cluster<L, SubShape63, false>>(st, njobs, jobs, njobs, one,   \
                                                                                  none);                        \
  case 2 * L + 1:                                                                                               \
    return launch_cluster<L, SubShape63, k_polymul_cluster<L, SubShape63, true>>(st, njobs, jobs, njobs, one,    \
                                                                                 *lift);
    X(1)
    X(2)
    X(3)
#undef X
    default:
      return (int)cudaErrorInvalidValue;
  }
}

}  // namespace vk
