// Element-wise batch kernel: many independent element-wise jobs of ragged
// lengths (each one of the reference's element-wise ops with its own
// operands and constants) in one launch.
//
// At commit every job is cut into units of at most VKCU_ELEM_CHUNK words
// (VKCU_ELEM_CHUNK_UNARY for unary ops, which move 16 instead of 24 bytes a
// word), each a complete descriptor (pointers offset to the unit); a
// persistent grid (one wave) walks the unit table with 16-byte accesses
// where the unit's three pointers share their offset mod 16 (8-byte
// otherwise), every load of a thread's group issued before its stores.  The
// op is uniform per unit, so the switch costs one branch per unit.
// HBM-bound: 16 (unary) or 24 (binary) bytes per word, plus 72 descriptor
// bytes per unit.
#include <cuda_runtime.h>

#include <cstring>

#include "elem_ops.cuh"
#include "kernels.h"

namespace vk {

constexpr int kThreads = 256;
// 16-byte pairs of each operand per thread and group: one full unit per group
constexpr int kPairsBinary = VKCU_ELEM_CHUNK / (2 * kThreads);
constexpr int kPairsUnary = VKCU_ELEM_CHUNK_UNARY / (2 * kThreads);
static_assert(kPairsBinary * 2 == kPairsUnary, "unary units move the bytes of binary ones");

// One unit of `n` words.  Where a, b and res share their offset mod 16 bytes
// (all aligned, or all 8 bytes off: one word is peeled), the words stream as
// 16-byte pairs, otherwise as single words; either way in groups of
// kThreads x P pairs (or words) with every load of a thread's group issued
// before its first store.  Lanes past the end re-read the last element (no
// conditionally defined registers) and store nothing.
template <int P, bool BIN, class Op>
__device__ __forceinline__ void run_chunk(const vkcu_elem_job& j, const Op& op) {
  const u64* a = reinterpret_cast<const u64*>(j.a);
  const u64* b = reinterpret_cast<const u64*>(j.b);
  u64* res = reinterpret_cast<u64*>(j.res);
  const u64 n = j.len;
  const uintptr_t ma = reinterpret_cast<uintptr_t>(a) & 15, mr = reinterpret_cast<uintptr_t>(res) & 15;
  const bool same = ma == mr && (!BIN || (reinterpret_cast<uintptr_t>(b) & 15) == ma);
  if (same) {
    u64 s = 0;
    if (ma && n) {  // peel one word to reach the 16-byte boundary
      if (threadIdx.x == 0) res[0] = op(a[0], BIN ? b[0] : 0ull);
      s = 1;
    }
    const u64 pairs = (n - s) >> 1;
    for (u64 g0 = 0; g0 < pairs; g0 += (u64)kThreads * P) {
      ulonglong2 x[P], y[BIN ? P : 1];
#pragma unroll
      for (int k = 0; k < P; k++) {
        const u64 p = g0 + threadIdx.x + (u64)k * kThreads;
        const u64 pc = p < pairs ? p : pairs - 1;
        x[k] = ld2(a + s + 2 * pc);
        if constexpr (BIN) y[k] = ld2(b + s + 2 * pc);
      }
#pragma unroll
      for (int k = 0; k < P; k++) {
        const u64 p = g0 + threadIdx.x + (u64)k * kThreads;
        const ulonglong2 yk = BIN ? y[BIN ? k : 0] : make_ulonglong2(0, 0);
        if (p < pairs) st2(res + s + 2 * p, op(x[k].x, yk.x), op(x[k].y, yk.y));
      }
    }
    const u64 last = s + 2 * pairs;
    if (last < n && threadIdx.x == 0) res[last] = op(a[last], BIN ? b[last] : 0ull);
  } else {
    for (u64 g0 = 0; g0 < n; g0 += (u64)kThreads * P) {
      u64 x[P], y[BIN ? P : 1];
#pragma unroll
      for (int k = 0; k < P; k++) {
        const u64 i = g0 + threadIdx.x + (u64)k * kThreads;
        const u64 ic = i < n ? i : n - 1;
        x[k] = a[ic];
        if constexpr (BIN) y[k] = b[ic];
      }
#pragma unroll
      for (int k = 0; k < P; k++) {
        const u64 i = g0 + threadIdx.x + (u64)k * kThreads;
        if (i < n) res[i] = op(x[k], BIN ? y[BIN ? k : 0] : 0ull);
      }
    }
  }
}

template <class Op>
__device__ __forceinline__ void run_binary(const vkcu_elem_job& j, const Op& op) {
  run_chunk<kPairsBinary, true>(j, op);
}

template <class Op>
__device__ __forceinline__ void run_unary(const vkcu_elem_job& j, const Op& op) {
  run_chunk<kPairsUnary, false>(j, op);
}

__device__ __forceinline__ void run_unit(const vkcu_elem_job& j) {
  switch (j.op) {
    case VKCU_ELEM_MUL: run_binary(j, OpMul{j.c0, j.c1, j.bits}); break;
    case VKCU_ELEM_FMA: run_binary(j, OpFmaRef{j.c0, j.c1, j.c2}); break;
    case VKCU_ELEM_FMA_CANON: run_binary(j, OpFmaCanon{j.c0, j.c1, j.c2, j.c3, j.bits}); break;
    case VKCU_ELEM_MULCONST: run_unary(j, OpMulConst{j.c0, j.c1, j.c2}); break;
    case VKCU_ELEM_GTSUB: run_unary(j, OpGtSub{j.c0, j.c1, j.c2, j.c3, j.bits}); break;
    case VKCU_ELEM_GTADD: run_unary(j, OpGtAdd{j.c0, j.c1}); break;
    default: run_unary(j, OpModTwo{j.c0}); break;
  }
}

// Persistent loop over the work units (four CTAs per SM, 64 registers a
// thread).  The next unit's 72-byte descriptor is copied into shared memory
// with cp.async (nine 8-byte pieces, one per thread of the first nine) while
// the current unit streams, so its latency is hidden without holding it in
// registers (a register prefetch cost occupancy and measured slower; this
// one measured 5.68 against 5.44 TB/s on GB300).  A buffer is refilled only
// after the barrier that follows every thread's read of it.
__global__ void __launch_bounds__(kThreads, 4) k_elem_batch(const vkcu_elem_job* __restrict__ units, u64 nunits) {
  __shared__ __align__(16) unsigned long long sdesc[2][sizeof(vkcu_elem_job) / 8];
  static_assert(sizeof(vkcu_elem_job) % 8 == 0 && sizeof(vkcu_elem_job) / 8 <= kThreads, "descriptor copy");
  u64 c = blockIdx.x;
  if (c >= nunits) return;
  auto fetch = [&](u64 idx, int b) {
    if (threadIdx.x < sizeof(vkcu_elem_job) / 8) {
      const unsigned long long* src = reinterpret_cast<const unsigned long long*>(units + idx) + threadIdx.x;
      const unsigned dst = (unsigned)__cvta_generic_to_shared(&sdesc[b][threadIdx.x]);
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst), "l"(src) : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  fetch(c, 0);
  int buf = 0;
  for (;;) {
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncthreads();
    vkcu_elem_job j;
    memcpy(&j, sdesc[buf], sizeof j);
    const u64 cn = c + gridDim.x;
    if (cn < nunits) fetch(cn, buf ^ 1);
    run_unit(j);
    if (cn >= nunits) break;
    c = cn;
    buf ^= 1;
  }
}

}  // namespace vk

extern "C" int vkcu_elem_batch(void* stream, const vkcu_elem_job* units, uint64_t nchunks, int sms) {
  if (nchunks == 0) return 0;
  if (!units) return (int)cudaErrorInvalidValue;
  // one wave of resident CTAs: the loop is persistent
  static const int per_sm = [] {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, vk::k_elem_batch, vk::kThreads, 0) != cudaSuccess || b < 1)
      b = 1;
    return b;
  }();
  const uint64_t cap = (uint64_t)(sms > 0 ? sms : 1) * per_sm;
  const uint64_t blocks = nchunks < cap ? nchunks : cap;
  vk::k_elem_batch<<<(unsigned)blocks, vk::kThreads, 0, (cudaStream_t)stream>>>(units, nchunks);
  vkcu_count_launches(1);
  return (int)cudaGetLastError();
}
