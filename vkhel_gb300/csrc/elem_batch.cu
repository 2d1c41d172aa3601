// Element-wise batch kernel: many independent element-wise jobs of ragged
// lengths (each one of the reference's element-wise ops with its own
// operands and constants) in one launch.
//
// Work is cut into chunks of VKCU_ELEM_CHUNK words listed in a chunk table
// (job, chunk index) built at commit; a persistent grid (one wave) walks
// the table, fetching the next chunk's descriptor while the current chunk
// streams, with 16-byte accesses where the job's three pointers are 16-byte
// aligned (8-byte otherwise; a full aligned chunk issues all of a thread's
// loads before its stores).  The op is uniform per chunk, so the switch costs
// one branch per chunk.  HBM-bound: 16 (unary) or 24 (binary) bytes per word.
#include <cuda_runtime.h>

#include "elem_ops.cuh"
#include "kernels.h"

namespace vk {

constexpr int kThreads = 256;
constexpr int kPairs = VKCU_ELEM_CHUNK / (2 * kThreads);  // 16-byte pairs per thread in a full chunk

template <class Op>
__device__ __forceinline__ void run_chunk(const vkcu_elem_job& j, u64 lo, u64 hi, const Op& op) {
  const u64* a = reinterpret_cast<const u64*>(j.a);
  const u64* b = reinterpret_cast<const u64*>(j.b);
  u64* res = reinterpret_cast<u64*>(j.res);
  const bool vec = ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b) |
                     reinterpret_cast<uintptr_t>(res)) & 15) == 0;
  if (vec && hi - lo == VKCU_ELEM_CHUNK) {
    // full chunk: every load of the thread in flight before the first store
    ulonglong2 x[kPairs], y[kPairs];
#pragma unroll
    for (int k = 0; k < kPairs; k++) {
      const u64 i = lo + 2 * (threadIdx.x + (u64)k * kThreads);
      x[k] = ld2(a + i);
      y[k] = b ? ld2(b + i) : make_ulonglong2(0, 0);
    }
#pragma unroll
    for (int k = 0; k < kPairs; k++) {
      const u64 i = lo + 2 * (threadIdx.x + (u64)k * kThreads);
      st2(res + i, op(x[k].x, y[k].x), op(x[k].y, y[k].y));
    }
  } else if (vec) {
    // lo is a multiple of the (even) chunk size: pairs start 16-byte aligned
    const u64 pairs_end = lo + ((hi - lo) & ~1ull);
#pragma unroll 4
    for (u64 i = lo + 2 * threadIdx.x; i < pairs_end; i += 2 * kThreads) {
      const ulonglong2 xv = ld2(a + i);
      const ulonglong2 yv = b ? ld2(b + i) : make_ulonglong2(0, 0);
      st2(res + i, op(xv.x, yv.x), op(xv.y, yv.y));
    }
    if (pairs_end < hi && threadIdx.x == 0) res[pairs_end] = op(a[pairs_end], b ? b[pairs_end] : 0ull);
  } else {
#pragma unroll 4
    for (u64 i = lo + threadIdx.x; i < hi; i += kThreads) res[i] = op(a[i], b ? b[i] : 0ull);
  }
}

__device__ __forceinline__ void run_job_chunk(const vkcu_elem_job& j, u32 chunk) {
  const u64 w0 = (u64)chunk * VKCU_ELEM_CHUNK;
  const u64 w1 = w0 + VKCU_ELEM_CHUNK < j.len ? w0 + VKCU_ELEM_CHUNK : j.len;
  switch (j.op) {
    case VKCU_ELEM_MUL: run_chunk(j, w0, w1, OpMul{j.c0, j.c1, j.bits}); break;
    case VKCU_ELEM_MULCONST: run_chunk(j, w0, w1, OpMulConst{j.c0, j.c1, j.c2}); break;
    case VKCU_ELEM_FMA: run_chunk(j, w0, w1, OpFmaRef{j.c0, j.c1, j.c2}); break;
    case VKCU_ELEM_FMA_CANON: run_chunk(j, w0, w1, OpFmaCanon{j.c0, j.c1, j.c2, j.c3, j.bits}); break;
    case VKCU_ELEM_GTSUB: run_chunk(j, w0, w1, OpGtSub{j.c0, j.c1, j.c2, j.c3, j.bits}); break;
    case VKCU_ELEM_GTADD: run_chunk(j, w0, w1, OpGtAdd{j.c0, j.c1}); break;
    default: run_chunk(j, w0, w1, OpModTwo{j.c0}); break;
  }
}

// Persistent loop over the work units; the next unit's descriptor is fetched
// before the current one streams, so its latency hides behind the stream.
__global__ void __launch_bounds__(kThreads) k_elem_batch(const vkcu_elem_job* __restrict__ jobs,
                                                         const vkcu_elem_chunk* __restrict__ chunks, u64 nchunks) {
  u64 c = blockIdx.x;
  if (c >= nchunks) return;
  vkcu_elem_chunk cu = chunks[c];
  vkcu_elem_job j = jobs[cu.job];
  for (;;) {
    const u64 cn = c + gridDim.x;
    vkcu_elem_chunk nu = cu;
    vkcu_elem_job nj = j;
    if (cn < nchunks) {
      nu = chunks[cn];
      nj = jobs[nu.job];
    }
    run_job_chunk(j, cu.chunk);
    if (cn >= nchunks) break;
    c = cn;
    cu = nu;
    j = nj;
  }
}

}  // namespace vk

extern "C" int vkcu_elem_batch(void* stream, const vkcu_elem_job* jobs, const vkcu_elem_chunk* chunks,
                               uint64_t nchunks, int sms) {
  if (nchunks == 0) return 0;
  if (!jobs || !chunks) return (int)cudaErrorInvalidValue;
  // one wave of resident CTAs: the loop is persistent
  static const int per_sm = [] {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, vk::k_elem_batch, vk::kThreads, 0) != cudaSuccess || b < 1)
      b = 1;
    return b;
  }();
  const uint64_t cap = (uint64_t)(sms > 0 ? sms : 1) * per_sm;
  const uint64_t blocks = nchunks < cap ? nchunks : cap;
  vk::k_elem_batch<<<(unsigned)blocks, vk::kThreads, 0, (cudaStream_t)stream>>>(jobs, chunks, nchunks);
  vkcu_count_launches(1);
  return (int)cudaGetLastError();
}
