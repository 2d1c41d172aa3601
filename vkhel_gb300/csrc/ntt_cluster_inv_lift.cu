// Inverse transform on a thread-block cluster with a fused lift epilogue.
#include "ntt_cluster.cuh"

namespace vk {

int inv_cluster_lifted(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int logc,
                       int logs, const vkcu_lift& l) {
#define X(L, S) launch_cluster<L, S, k_ntt_inv_cluster<L, S, true>>(st, njobs, jobs, njobs, one, l)
  VK_CLUSTER_SHAPES(X)
#undef X
}

}  // namespace vk
