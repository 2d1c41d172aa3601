// Forward transform on a thread-block cluster (the kernels are in ntt_cluster.cuh).
#include "ntt_cluster.cuh"

namespace vk {

int fwd_cluster(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int logc, int logs) {
#define X(L, S) launch_cluster<L, S, k_ntt_fwd_cluster<L, S>>(st, njobs, jobs, njobs, one)
  VK_CLUSTER_SHAPES(X)
#undef X
}

}  // namespace vk
