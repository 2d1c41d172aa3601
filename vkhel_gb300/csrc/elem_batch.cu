// Element-wise batch kernel: many independent element-wise jobs of ragged
// lengths (each one of the reference's element-wise ops with its own
// operands and constants) in one launch.
//
// Work is cut into chunks of VKCU_ELEM_CHUNK words; a persistent grid (8 CTAs
// per SM) walks the chunks in order, finds a chunk's job by binary search in
// the prefix sums of chunk counts, and streams it with 16-byte accesses where
// the job's three pointers are 16-byte aligned (8-byte otherwise).  The op is
// uniform per chunk, so the switch costs one branch per chunk.  HBM-bound:
// 16 (unary) or 24 (binary) bytes per word.
#include <cuda_runtime.h>

#include "elem_ops.cuh"
#include "kernels.h"

namespace vk {

template <class Op>
__device__ __forceinline__ void run_chunk(const vkcu_elem_job& j, u64 lo, u64 hi, const Op& op) {
  const u64* a = reinterpret_cast<const u64*>(j.a);
  const u64* b = reinterpret_cast<const u64*>(j.b);
  u64* res = reinterpret_cast<u64*>(j.res);
  const bool vec = ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b) |
                     reinterpret_cast<uintptr_t>(res)) & 15) == 0;
  if (vec) {
    // lo is a multiple of the (even) chunk size: pairs start 16-byte aligned
    const u64 pairs_end = lo + ((hi - lo) & ~1ull);
#pragma unroll 4
    for (u64 i = lo + 2 * threadIdx.x; i < pairs_end; i += 2 * blockDim.x) {
      const ulonglong2 x = ld2(a + i);
      const ulonglong2 y = b ? ld2(b + i) : make_ulonglong2(0, 0);
      st2(res + i, op(x.x, y.x), op(x.y, y.y));
    }
    if (pairs_end < hi && threadIdx.x == 0) res[pairs_end] = op(a[pairs_end], b ? b[pairs_end] : 0ull);
  } else {
#pragma unroll 4
    for (u64 i = lo + threadIdx.x; i < hi; i += blockDim.x) res[i] = op(a[i], b ? b[i] : 0ull);
  }
}

__global__ void __launch_bounds__(256) k_elem_batch(const vkcu_elem_job* __restrict__ jobs,
                                                    const u64* __restrict__ first, u32 njobs, u64 chunks) {
  for (u64 c = blockIdx.x; c < chunks; c += gridDim.x) {
    // last job whose first chunk is <= c (jobs of zero length have none)
    u32 lo = 0, hi = njobs;
    while (hi - lo > 1) {
      const u32 mid = (lo + hi) >> 1;
      if (first[mid] <= c) lo = mid; else hi = mid;
    }
    const vkcu_elem_job j = jobs[lo];
    const u64 w0 = (c - first[lo]) * VKCU_ELEM_CHUNK;
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
}

}  // namespace vk

extern "C" int vkcu_elem_batch(void* stream, const vkcu_elem_job* jobs, const uint64_t* first, uint32_t njobs,
                               uint64_t chunks, int sms) {
  if (chunks == 0) return 0;
  if (!jobs || !first || njobs == 0) return (int)cudaErrorInvalidValue;
  const uint64_t cap = (uint64_t)(sms > 0 ? sms : 1) * 8;
  const uint64_t blocks = chunks < cap ? chunks : cap;
  vk::k_elem_batch<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(
      jobs, reinterpret_cast<const vk::u64*>(first), njobs, chunks);
  vkcu_count_launches(1);
  return (int)cudaGetLastError();
}
