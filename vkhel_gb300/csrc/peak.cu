// Integer-pipe peak of this GPU for the roofline of the transform kernels.
//
// The transforms are bound by 64-bit integer multiplies (a Shoup product is
// one mul.hi.u64 and two mul.lo.u64, each several IMADs), not by HBM, and the
// device peaks recorded for this machine cover only copy bandwidth and dense
// bf16.  These kernels measure, on the running GPU:
//   * butterflies/s: independent lazy Cooley-Tukey butterflies (the exact
//     instruction sequence of the transforms, ct_bfly) with all operands in
//     registers, 16 independent chains per thread, grid = 4 CTAs x 256
//     threads per SM;
//   * IMAD/s: independent 32-bit multiply-adds (mad.lo.u32), same shape.
// Each kernel folds its results into one store so nothing is dead code.
#include <cuda_runtime.h>

#include "arith.cuh"
#include "kernels.h"

namespace vk {

constexpr int kChains = 16;

__global__ void __launch_bounds__(256) k_peak_bfly(const u64* __restrict__ seed, u64* __restrict__ sink, int iters) {
  const u64 q = seed[0], q2 = 2 * q, w = seed[1], wp = seed[2];
  u64 x[kChains], y[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) {
    x[c] = (seed[3] + threadIdx.x * 131 + c * 7) % q;
    y[c] = (seed[4] + blockIdx.x * 17 + c * 3) % q;
  }
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int c = 0; c < kChains; c++) ct_bfly(x[c], y[c], w, wp, q, q2);
  }
  u64 acc = 0;
#pragma unroll
  for (int c = 0; c < kChains; c++) acc ^= x[c] + y[c];
  if (acc == 0x5bd1e995ull) sink[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

__global__ void __launch_bounds__(256) k_peak_imad(const u32* __restrict__ seed, u32* __restrict__ sink, int iters) {
  const u32 m = seed[0] | 1u, a = seed[1];
  u32 x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) x[c] = threadIdx.x * 2654435761u + c;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int c = 0; c < kChains; c++) {
      asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(x[c]) : "r"(m), "r"(a));
      asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(x[c]) : "r"(m), "r"(a));
    }
  }
  u32 acc = 0;
#pragma unroll
  for (int c = 0; c < kChains; c++) acc ^= x[c];
  if (acc == 0x5bd1e995u) sink[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

}  // namespace vk

using namespace vk;

// Returns butterflies/s and IMAD/s measured with CUDA events (best of `reps`).
extern "C" int vkcu_measure_int_peak(void* stream, int sms, double* bfly_per_s, double* imad_per_s) {
  cudaStream_t st = (cudaStream_t)stream;
  const int blocks = sms * 4, threads = 256;
  u64 host_seed[5] = {1152921504606748673ull, 641000223749548346ull, 0, 12345, 67890};
  host_seed[2] = (u64)((((unsigned __int128)host_seed[1]) << 64) / host_seed[0]);
  void *dseed = nullptr, *dsink = nullptr;
  cudaError_t e = cudaMalloc(&dseed, 64);
  if (e == cudaSuccess) e = cudaMalloc(&dsink, (size_t)blocks * threads * 8);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dseed, host_seed, sizeof host_seed, cudaMemcpyHostToDevice, st);
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&t0);
  if (e == cudaSuccess) e = cudaEventCreate(&t1);
  double best_b = 0, best_i = 0;
  const int iters_b = 4096, iters_i = 65536;
  for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {
    float ms = 0;
    cudaEventRecord(t0, st);
    k_peak_bfly<<<blocks, threads, 0, st>>>((const u64*)dseed, (u64*)dsink, iters_b);
    cudaEventRecord(t1, st);
    e = cudaEventSynchronize(t1);
    if (e != cudaSuccess) break;
    cudaEventElapsedTime(&ms, t0, t1);
    const double b = (double)blocks * threads * kChains * iters_b / (ms * 1e-3);
    if (rep > 0 && b > best_b) best_b = b;
    cudaEventRecord(t0, st);
    k_peak_imad<<<blocks, threads, 0, st>>>((const u32*)dseed, (u32*)dsink, iters_i);
    cudaEventRecord(t1, st);
    e = cudaEventSynchronize(t1);
    if (e != cudaSuccess) break;
    cudaEventElapsedTime(&ms, t0, t1);
    const double i = (double)blocks * threads * kChains * 2 * iters_i / (ms * 1e-3);
    if (rep > 0 && i > best_i) best_i = i;
  }
  vkcu_count_launches(8);
  if (t0) cudaEventDestroy(t0);
  if (t1) cudaEventDestroy(t1);
  cudaFree(dseed);
  cudaFree(dsink);
  *bfly_per_s = best_b;
  *imad_per_s = best_i;
  return (int)e;
}
