// One persistent launch for a ragged batch of fused limb products of degrees
// 2^12 .. 2^16 (q < 2^62, no epilogue): clusters of four CTAs of 512 threads,
// each CTA with the 2^14-word shared block of the other kernels.
//
// The work is a table of items in decreasing size, taken in order through
// two device counters (reset by a memset before each launch):
//   cluster items  -- one 2^16 product on the four CTAs (the column passes of
//                     k_polymul_cluster<2>), or two 2^15 products, one on
//                     each CTA pair (k_polymul_cluster<1> with the pair's
//                     rank base); rank 0 takes the next item and hands its
//                     index to the other CTAs through their shared memory;
//   CTA items      -- after the cluster items run out, each CTA on its own:
//                     one 2^14 product (512 threads, 32 words each), one 2^13
//                     product (16 words each) or two 2^12 products (256
//                     threads each, in step on two halves of the shared
//                     block).
// The largest items go first, so the short ones fill the end of the launch
// (longest-processing-time order).  A pair item or a two-product 2^12 item
// with one product only gets a copy of it that writes a dummy buffer, so
// that both halves run the same barriers.  Every product is the same
// arithmetic as the per-degree kernels (k_polymul, k_polymul_cluster), so
// the words are identical.
#include "ntt_cluster.cuh"

namespace vk {

using R16 = Shape<14, 32>;                       // 2^16 / 2^15 sub-blocks and 2^14 products
using R13 = Shape<13, 16>;                       // 2^13 products, 512 threads
using R12 = Shape<12, 16, 1, Mod62, true>;       // two 2^12 products, 256 threads each
constexpr int kRaggedThreads = 512;
static_assert(R16::T == kRaggedThreads && R13::T == kRaggedThreads && 2 * R12::T == kRaggedThreads, "CTA shapes");

// One fused product on the threads of shape S (k_polymul's body).
template <class S>
__device__ __noinline__ void ragged_cta_product(u64* sm, const vkcu_poly_job& job) {
  using M = typename S::M;
  const Tw t = load_tw(job.tw);
  u64* scratch = reinterpret_cast<u64*>(job.scratch);
#pragma unroll 1
  for (int ph = 0; ph < 2; ph++) {
    fwd_first<S>(sm, reinterpret_cast<const u64*>(ph ? job.a : job.b), t, 1u);
    fwd_passes<S>(sm, t, 1u, [&](int g, u64(&v)[16]) {
      if (ph == 0) {
#pragma unroll
        for (int j = 0; j < 16; j++) v[j] = M::canon(v[j], t);
        store16(v, scratch + 16 * g);
      } else {
        u64 bh[16];
        load16(bh, scratch + 16 * g);
#pragma unroll
        for (int j = 0; j < 16; j++) v[j] = M::product(v[j], bh[j], t);
        gs_group<M, 4, 0, M::EXACT_AFTER_PRODUCT, false>(v, t.inv, (1u << S::HEAD) + (u32)g, t);
#pragma unroll
        for (int j = 0; j < 16; j++) sm[pad(16 * g + j)] = v[j];
      }
    });
  }
  inv_passes<S>(sm, t, 1u, S::HEAD - 4);
  inv_last<S>(sm, t, 1u, reinterpret_cast<u64*>(job.c), true);
  __syncthreads();
}

// One product of 2^(14 + LOGC) words on the 2^LOGC CTAs from cluster rank
// rbase (k_polymul_cluster's body); rank = this CTA's rank among them.
template <int LOGC>
__device__ __noinline__ void ragged_cluster_product(u64* sm, const cg::cluster_group& cl, const vkcu_poly_job& job,
                                                       int rank, int rbase) {
  using S = R16;
  using K = Cols<LOGC, S>;
  using M = typename S::M;
  const u32 tw_mult = (u32)(K::C + rank);
  const Tw t = load_tw(job.tw);
  u64* scratch = reinterpret_cast<u64*>(job.scratch) + (size_t)rank * K::SUB;
#pragma unroll 1
  for (int ph = 0; ph < 2; ph++) {
    cluster_arrive();  // done with every shared memory the column pass writes (col_fwd waits)
    col_fwd<LOGC, S, true>(reinterpret_cast<const u64*>(ph ? job.a : job.b), sm, cl, rank, t, rbase);
    cl.sync();
    fwd_first_smem<S>(sm, t, tw_mult);
    fwd_passes<S>(sm, t, tw_mult, [&](int g, u64(&v)[16]) {
      if (ph == 0) {
#pragma unroll
        for (int j = 0; j < 16; j++) v[j] = M::canon(v[j], t);
        store16(v, scratch + 16 * g);
      } else {
        u64 bh[16];
        load16(bh, scratch + 16 * g);
#pragma unroll
        for (int j = 0; j < 16; j++) v[j] = M::product(v[j], bh[j], t);
        gs_group<M, 4, 0, M::EXACT_AFTER_PRODUCT, false>(v, t.inv, tw_mult * (u32)(S::N / 16) + (u32)g, t);
#pragma unroll
        for (int j = 0; j < 16; j++) sm[pad(16 * g + j)] = v[j];
      }
    });
  }
  inv_passes<S>(sm, t, tw_mult, S::HEAD - 4);
  inv_last_smem<S>(sm, t, tw_mult);
  cl.sync();
  col_inv_out<LOGC, S, false>(reinterpret_cast<u64*>(job.c), sm, cl, rank, t, nullptr, rbase);
}

__global__ void __launch_bounds__(kRaggedThreads, 1)
    k_polymul_ragged(const vkcu_ragged_item* __restrict__ items, int n_cluster_items, int n_items,
                     const vkcu_poly_job* __restrict__ jobs, unsigned* __restrict__ counters) {
  extern __shared__ u64 sm[];
  __shared__ int s_item;
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  cl.sync();  // every CTA of the cluster runs before its shared memory is written remotely
  // cluster items: rank 0 takes the next one and writes its index into every
  // CTA's s_item before the barrier; the item's own cluster barriers order the
  // reads of s_item before the next write
#pragma unroll 1
  while (true) {
    if (rank == 0 && threadIdx.x == 0) {
      const int i = (int)atomicAdd(&counters[0], 1u);
#pragma unroll
      for (int r = 0; r < 4; r++) *cl.map_shared_rank(&s_item, r) = i;
    }
    cl.sync();
    const int i = s_item;
    if (i >= n_cluster_items) break;
    const vkcu_ragged_item it = items[i];
    if (it.kind == 16) {
      ragged_cluster_product<2>(sm, cl, jobs[it.job0], rank, 0);
    } else {  // two 2^15 products, one per CTA pair
      ragged_cluster_product<1>(sm, cl, jobs[rank < 2 ? it.job0 : it.job1], rank & 1, rank & 2);
    }
  }
  // CTA items, taken by each CTA on its own
#pragma unroll 1
  while (true) {
    __syncthreads();  // everyone has read the previous s_item
    if (threadIdx.x == 0) s_item = n_cluster_items + (int)atomicAdd(&counters[1], 1u);
    __syncthreads();
    const int i = s_item;
    if (i >= n_items) break;
    const vkcu_ragged_item it = items[i];
    if (it.kind == 14) {
      ragged_cta_product<R16>(sm, jobs[it.job0]);
    } else if (it.kind == 13) {
      ragged_cta_product<R13>(sm, jobs[it.job0]);
    } else {  // two 2^12 products, one per half of the block and of the shared memory
      const int h = (int)threadIdx.x / R12::T;
      ragged_cta_product<R12>(sm + h * (R12::SMEM_BYTES / 8), jobs[h ? it.job1 : it.job0]);
    }
  }
}

}  // namespace vk

using namespace vk;

extern "C" int vkcu_polymul_ragged(void* stream, const vkcu_ragged_item* items, int n_cluster_items, int n_items,
                                   const vkcu_poly_job* jobs, unsigned* counters, int sms) {
  cudaStream_t st = (cudaStream_t)stream;
  if (n_items < 1 || !items || !jobs || !counters) return (int)cudaErrorInvalidValue;
  static KernelSetup setup;  // resident clusters per device
  constexpr int C = 4;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(kRaggedThreads);
  cfg.dynamicSmemBytes = R16::SMEM_BYTES;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cfg.gridDim = dim3(C);
  const int dev = current_device();
  const bool cached = dev >= 0 && dev < 32;
  int max_clusters = cached ? setup.per_dev[dev].load(std::memory_order_acquire) : 0;
  cudaError_t e = cudaSuccess;
  if (max_clusters < 1) {
    e = cudaFuncSetAttribute(k_polymul_ragged, cudaFuncAttributeMaxDynamicSharedMemorySize, R16::SMEM_BYTES);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveClusters(&max_clusters, k_polymul_ragged, &cfg);
    if (e != cudaSuccess) return (int)e;
    if (max_clusters < 1) return (int)cudaErrorInvalidConfiguration;
    if (cached) setup.per_dev[dev].store(max_clusters, std::memory_order_release);
  }
  (void)sms;
  e = cudaMemsetAsync(counters, 0, 2 * sizeof(unsigned), st);
  if (e != cudaSuccess) return (int)e;
  cfg.gridDim = dim3(max_clusters * C);
  e = cudaLaunchKernelEx(&cfg, k_polymul_ragged, items, n_cluster_items, n_items, jobs, counters);
  vkcu_count_launches(1);
  return (int)e;
}
