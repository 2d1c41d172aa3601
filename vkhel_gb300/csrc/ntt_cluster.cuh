#pragma once
// Transforms and fused polynomial multiply for n = 2^15 .. 2^17 on a thread-
// block cluster of C = n / 2^14 CTAs with distributed shared memory (the
// four-step decomposition):
//
//   forward:  column pass  -- the first log2 C stages act on columns
//                             (words i, i + 2^14, ..., i + (C-1) 2^14); CTA r
//                             reads its 2^14 / C columns from global memory,
//                             runs the radix-C network in registers and writes
//                             output j of every column into CTA j's shared
//                             memory (DSMEM);
//             row passes   -- each CTA then runs the remaining 14 stages on its
//                             own 2^14-word sub-block, which is the contiguous
//                             words [r 2^14, (r+1) 2^14) of the bit-reversed
//                             output; the twiddle of local stage m' and local
//                             block b is table[(C + r) m' + b];
//   inverse:  row passes on each sub-block, then the column pass gathers every
//             column from the C CTAs over DSMEM and runs the last log2 C
//             stages with n^-1 folded in, writing global memory coalesced.
//
// The sub-block is 2^14 words (n = 2^15 .. 2^17, one CTA per SM), or 2^9 ..
// 2^13 words for n = 2^12 .. 2^16 split over 8 CTAs when there are too few
// jobs to fill the GPU otherwise (single calls, small server micro-batches).
//
// Cluster barriers separate the phases: before a forward column pass writes
// another CTA's shared memory (its owner has finished reading it; in the
// polymul this one is split: each CTA arrives, loads and transforms its first
// columns, and waits just before its first remote store), after it (the
// sub-blocks are complete), and before the inverse gather.  Every CTA of a
// cluster walks the same job sequence, and a final barrier keeps each CTA's
// shared memory alive until the last remote read.
#include <cooperative_groups.h>

#include "ntt_core.cuh"

namespace cg = cooperative_groups;

namespace vk {

using SubShape = Shape<14, 32>;  // the large-n sub-block
using SubShape63 = Shape<14, 32, 1, Mod63>;  // the same for 2^62 <= q < 2^63

template <int LOGC, class S>
struct Cols {
  static constexpr int C = 1 << LOGC, SUB = S::N;
  static constexpr int COLS = SUB >> LOGC;  // columns per CTA
  static constexpr int PER = COLS / S::T;   // columns per thread
  static_assert(PER * C == S::E, "a column pass moves E words per thread");
  __device__ __forceinline__ static int col(int rank, int k) { return rank * COLS + (int)threadIdx.x + k * S::T; }
};

// The cluster barrier split in two: arrive (release: this thread's accesses
// to shared memory so far, its own CTA's and remote, are ordered before what
// other CTAs do after their wait) and wait (acquire).  Every thread of the
// cluster executes each exactly once per barrier phase.
__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }

// Forward column pass: global stages 0 .. LOGC-1 (exact first-stage rule),
// outputs scattered to the owning CTAs' shared memory, forward-lazy.  A
// thread's PER columns go in two rounds of H = PER / 2 (16 words in flight:
// all 32 at once would spill).  SPLIT: the caller has arrived on the cluster
// barrier that frees the other CTAs' shared memory, and the first round's
// loads and butterflies run before the wait, which comes just before the
// first remote store (the fused polymul: 1-2.4 % faster; the forward
// transform alone was 0.8 % slower this way and synchronizes before).
// rbase: the cluster rank of this transform's CTA 0 (a larger cluster can
// hold several transforms of C CTAs each).
template <int LOGC, class S, bool SPLIT>
__device__ __forceinline__ void col_fwd(const u64* __restrict__ in, u64* sm, const cg::cluster_group& cl, int rank,
                                        const Tw& t, int rbase = 0) {
  using K = Cols<LOGC, S>;
  constexpr int H = K::PER >= 2 ? K::PER / 2 : 1;
  const ulonglong2 w0 = ld_tw(t.fwd + 1);
#pragma unroll 1
  for (int k0 = 0; k0 < K::PER; k0 += H) {
    u64 v[H * K::C];
#pragma unroll
    for (int k = 0; k < H; k++)
#pragma unroll
      for (int j = 0; j < K::C; j++) v[k * K::C + j] = ld_stream(in + K::col(rank, k0 + k) + (size_t)j * K::SUB);
    static_for<0, H>([&](auto kc) {
      constexpr int k = decltype(kc)::value;
#pragma unroll
      for (int jj = 0; jj < K::C / 2; jj++)
        ct_first<typename S::M>(v[k * K::C + jj], v[k * K::C + jj + K::C / 2], w0.x, w0.y, t);
      ct_group<typename S::M, LOGC, 1, k * K::C>(v, t.fwd, 1u, t);
    });
    if (SPLIT && k0 == 0) cluster_wait();
#pragma unroll
    for (int j = 0; j < K::C; j++) {
      u64* rem = cl.map_shared_rank(sm, rbase + j);
#pragma unroll
      for (int k = 0; k < H; k++) rem[pad(K::col(rank, k0 + k))] = v[k * K::C + j];
    }
  }
}

// Inverse column pass: gather, global stages LOGC-1 .. 0 with n^-1 folded in,
// canonical words to global memory; two rounds of H columns as above.
template <int LOGC, class S, class Epi>
__device__ __forceinline__ void col_inv(u64* __restrict__ out, u64* sm, const cg::cluster_group& cl, int rank,
                                        const Tw& t, const Epi& epi, int rbase = 0) {
  using K = Cols<LOGC, S>;
  constexpr int H = K::PER >= 2 ? K::PER / 2 : 1;
#pragma unroll 1
  for (int k0 = 0; k0 < K::PER; k0 += H) {
    u64 v[H * K::C];
#pragma unroll
    for (int j = 0; j < K::C; j++) {
      const u64* rem = cl.map_shared_rank(sm, rbase + j);
#pragma unroll
      for (int k = 0; k < H; k++) v[k * K::C + j] = rem[pad(K::col(rank, k0 + k))];
    }
    static_for<0, H>([&](auto kc) {
      constexpr int k = decltype(kc)::value;
      gs_group<typename S::M, LOGC, k * K::C, false, true>(v, t.inv, 1u, t);
    });
#pragma unroll
    for (int k = 0; k < H; k++)
#pragma unroll
      for (int j = 0; j < K::C; j++) out[K::col(rank, k0 + k) + (size_t)j * K::SUB] = epi(v[k * K::C + j]);
  }
}

template <int LOGC, class S, bool LIFT>
__device__ __forceinline__ void col_inv_out(u64* __restrict__ out, u64* sm, const cg::cluster_group& cl, int rank,
                                            const Tw& t, const vkcu_lift* lift, int rbase = 0) {
  if constexpr (LIFT)
    col_inv<LOGC, S>(out, sm, cl, rank, t, LiftRun(lift, t.q), rbase);
  else
    col_inv<LOGC, S>(out, sm, cl, rank, t, NoLift{}, rbase);
}

template <int LOGC, class S>
__global__ void __launch_bounds__(S::T, 1)
    k_ntt_fwd_cluster(const vkcu_ntt_job* __restrict__ jobs, int njobs, vkcu_ntt_job one) {
  using K = Cols<LOGC, S>;
  extern __shared__ u64 sm[];
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int ncl = (int)gridDim.x / K::C, cid = (int)blockIdx.x / K::C;
  const u32 tw_mult = (u32)(K::C + rank);
#pragma unroll 1
  for (int w = cid; w < njobs; w += ncl) {
    const vkcu_ntt_job job = fetch_job(jobs, one, w);
    const Tw t = load_tw(job.tw);
    u64* out = reinterpret_cast<u64*>(job.out) + (size_t)rank * K::SUB;
    cl.sync();
    col_fwd<LOGC, S, false>(reinterpret_cast<const u64*>(job.in), sm, cl, rank, t);
    cl.sync();
    fwd_first_smem<S>(sm, t, tw_mult);
    fwd_passes<S>(sm, t, tw_mult, [&](int g, u64(&v)[16]) {
#pragma unroll
      for (int j = 0; j < 16; j++) v[j] = S::M::canon(v[j], t);
      store16(v, out + 16 * g);
    });
  }
  cl.sync();
}

template <int LOGC, class S, bool LIFT>
__global__ void __launch_bounds__(S::T, 1)
    k_ntt_inv_cluster(const vkcu_ntt_job* __restrict__ jobs, int njobs, vkcu_ntt_job one,
                      const __grid_constant__ vkcu_lift lift) {
  using K = Cols<LOGC, S>;
  extern __shared__ u64 sm[];
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int ncl = (int)gridDim.x / K::C, cid = (int)blockIdx.x / K::C;
  const u32 tw_mult = (u32)(K::C + rank);
#pragma unroll 1
  for (int w = cid; w < njobs; w += ncl) {
    const vkcu_ntt_job job = fetch_job(jobs, one, w);
    const Tw t = load_tw(job.tw);
    const u64* in = reinterpret_cast<const u64*>(job.in) + (size_t)rank * K::SUB;
    cl.sync();
#pragma unroll 1
    for (int i = 0; i < S::E / 16; i++) {
      const int g = (int)threadIdx.x + i * S::T;
      u64 v[16];
      load16(v, in + 16 * g);
      gs_group<typename S::M, 4, 0, true, false>(v, t.inv, tw_mult * (u32)(S::N / 16) + (u32)g, t);
#pragma unroll
      for (int j = 0; j < 16; j++) sm[pad(16 * g + j)] = v[j];
    }
    __syncthreads();
    inv_passes<S>(sm, t, tw_mult, S::HEAD - 4);
    inv_last_smem<S>(sm, t, tw_mult);
    cl.sync();
    col_inv_out<LOGC, S, LIFT>(reinterpret_cast<u64*>(job.out), sm, cl, rank, t, &lift);
  }
  cl.sync();
}

template <int LOGC, class S, bool LIFT>
__global__ void __launch_bounds__(S::T, 1)
    k_polymul_cluster(const vkcu_poly_job* __restrict__ jobs, int njobs, vkcu_poly_job one,
                      const __grid_constant__ vkcu_lift lift) {
  using K = Cols<LOGC, S>;
  extern __shared__ u64 sm[];
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int ncl = (int)gridDim.x / K::C, cid = (int)blockIdx.x / K::C;
  const u32 tw_mult = (u32)(K::C + rank);
  constexpr unsigned kSlice = (unsigned)(K::COLS * 8);
#pragma unroll 1
  for (int w = cid; w < njobs; w += ncl) {
    const vkcu_poly_job job = fetch_job(jobs, one, w);
    const Tw t = load_tw(job.tw);
    // b holds NTT(b): phase 0 is skipped (read by the epilogue instantiations only)
    const bool b_ntt = LIFT && (job.flags & VKCU_JOB_B_NTT);
    u64* scratch = (b_ntt ? const_cast<u64*>(reinterpret_cast<const u64*>(job.b)) : reinterpret_cast<u64*>(job.scratch)) +
                   (size_t)rank * K::SUB;
    if ((int)threadIdx.x < K::C)  // this CTA's column slices of a, for phase 1
      prefetch_l2(reinterpret_cast<const u64*>(job.a) + (size_t)threadIdx.x * K::SUB + rank * K::COLS, kSlice);
#pragma unroll 1
    for (int ph = b_ntt ? 1 : 0; ph < 2; ph++) {
      cluster_arrive();  // done with every shared memory the column pass writes (col_fwd waits)
      col_fwd<LOGC, S, true>(reinterpret_cast<const u64*>(ph ? job.a : job.b), sm, cl, rank, t);
      cl.sync();
      fwd_first_smem<S>(sm, t, tw_mult);
      fwd_passes<S>(sm, t, tw_mult, [&](int g, u64(&v)[16]) {
        using M = typename S::M;
        if (ph == 0) {
#pragma unroll
          for (int j = 0; j < 16; j++) v[j] = M::canon(v[j], t);
          store16(v, scratch + 16 * g);
        } else {
          u64 bh[16];
          load16(bh, scratch + 16 * g);
          if (b_ntt) reduce_operand16(bh, t);
#pragma unroll
          for (int j = 0; j < 16; j++) v[j] = M::product(v[j], bh[j], t);
          // the sub-block's first inverse pass (stages HEAD + 3 .. HEAD) on the same words
          gs_group<M, 4, 0, M::EXACT_AFTER_PRODUCT, false>(v, t.inv, tw_mult * (u32)(S::N / 16) + (u32)g, t);
#pragma unroll
          for (int j = 0; j < 16; j++) sm[pad(16 * g + j)] = v[j];
        }
      });
    }
    if (w + ncl < njobs && (int)threadIdx.x < K::C) {
      // the next job's b: its column slices, or (NTT(b) given) this CTA's sub-block
      const vkcu_poly_job nx = fetch_job(jobs, one, w + ncl);
      const size_t off = (LIFT && (nx.flags & VKCU_JOB_B_NTT)) ? (size_t)rank * K::SUB + (size_t)threadIdx.x * K::COLS
                                                     : (size_t)threadIdx.x * K::SUB + rank * K::COLS;
      prefetch_l2(reinterpret_cast<const u64*>(nx.b) + off, kSlice);
    }
    inv_passes<S>(sm, t, tw_mult, S::HEAD - 4);
    inv_last_smem<S>(sm, t, tw_mult);
    cl.sync();
    col_inv_out<LOGC, S, LIFT>(reinterpret_cast<u64*>(job.c), sm, cl, rank, t, &lift);
  }
  cl.sync();
}

// The kernel is a template argument so that each kernel gets its own
// one-time attribute set-up (forward and inverse kernels share a signature).
// The clusters are spread over SMs: a cluster of small CTAs would otherwise
// be packed onto few SMs.
template <int LOGC, class S, auto kern, class... Args>
static int launch_cluster(cudaStream_t st, int njobs, Args... args) {
  constexpr int C = 1 << LOGC;
  static KernelSetup setup;  // resident clusters per device
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  attr[1].id = cudaLaunchAttributeClusterSchedulingPolicyPreference;
  attr[1].val.clusterSchedulingPolicyPreference = cudaClusterSchedulingPolicySpread;
  cfg.blockDim = dim3(S::T);
  cfg.dynamicSmemBytes = S::SMEM_BYTES;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 2;
  cfg.gridDim = dim3(C);
  const int dev = current_device();
  const bool cached = dev >= 0 && dev < 32;
  int max_clusters = cached ? setup.per_dev[dev].load(std::memory_order_acquire) : 0;
  if (max_clusters < 0) return (int)cudaErrorInvalidConfiguration;  // no such cluster fits this GPU
  cudaError_t e = cudaSuccess;
  if (max_clusters < 1) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, S::SMEM_BYTES);
    if (e == cudaSuccess && C > 8) e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveClusters(&max_clusters, kern, &cfg);
    if (e != cudaSuccess) return (int)e;
    if (max_clusters < 1) {
      if (cached) setup.per_dev[dev].store(-1, std::memory_order_release);
      return (int)cudaErrorInvalidConfiguration;
    }
    if (cached) setup.per_dev[dev].store(max_clusters, std::memory_order_release);
  }
  const int nclusters = njobs < max_clusters ? njobs : max_clusters;
  cfg.gridDim = dim3(nclusters * C);
  e = cudaLaunchKernelEx(&cfg, kern, args...);
  vkcu_count_launches(1);
  return (int)e;
}

// Sub-blocks of 2^9 .. 2^13 words for n = 2^12 .. 2^16 on 8 CTAs (16 words
// per thread; 32 at 2^13, so that 256 threads fit the register file).
using Small9 = Shape<9, 16>;
using Small10 = Shape<10, 16>;
using Small11 = Shape<11, 16>;
using Small12 = Shape<12, 16>;
using Small13 = Shape<13, 32>;

// logc: cluster size 2^logc; logs: sub-block size 2^logs (14, or 9 .. 13
// with logc = 3, or 10 .. 12 with logc = 4: n = 2^14 .. 2^16 on 16 CTAs, a
// cluster size the GPU allows on request).
#define VK_CLUSTER_SHAPES(X)                                 \
  switch (logc * 32 + logs) {                                \
    case 1 * 32 + 14: return X(1, SubShape);                 \
    case 2 * 32 + 14: return X(2, SubShape);                 \
    case 3 * 32 + 14: return X(3, SubShape);                 \
    case 3 * 32 + 9: return X(3, Small9);                    \
    case 3 * 32 + 10: return X(3, Small10);                  \
    case 3 * 32 + 11: return X(3, Small11);                  \
    case 3 * 32 + 12: return X(3, Small12);                  \
    case 3 * 32 + 13: return X(3, Small13);                  \
    case 4 * 32 + 10: return X(4, Small10);                  \
    case 4 * 32 + 11: return X(4, Small11);                  \
    case 4 * 32 + 12: return X(4, Small12);                  \
    default: return (int)cudaErrorInvalidValue;              \
  }

// The lifted inverse and polymul kernels are instantiated in their own
// translation units (ntt_cluster_inv_lift.cu, ntt_cluster_poly_lift.cu) so
// that the cluster kernels compile in parallel.
int inv_cluster_lifted(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int logc,
                       int logs, const vkcu_lift& lift);
int poly_cluster_lifted(cudaStream_t st, const vkcu_poly_job* jobs, int njobs, const vkcu_poly_job& one, int logc,
                        int logs, const vkcu_lift& lift);

}  // namespace vk
