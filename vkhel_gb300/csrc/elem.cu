// Element-wise modular kernels for sm_103a.
//
// Each operation restates one reference shader with the constants its host
// wrapper pushes, so results equal the reference's for every 64-bit input:
//   elemmul        src/kernels/shaders/elemmul.comp:62-73      (elemmul.c:159-168)
//   elemmulconst   src/kernels/shaders/elemmulconst.comp:35-49 (elemmulconst.c:154-163)
//   elemfma        src/kernels/shaders/elemfma.comp:36-55      (elemfma.c:159-169)
//   elemgtsub      src/kernels/shaders/elemgtsub.comp:49-67    (elemgtsub.c:154-168)
//   elemgtadd      src/kernels/shaders/elemgtadd.comp:20-30
//   elemmodbytwo   src/kernels/shaders/elemmodbytwo.comp:19-27
// plus elemfma_canonical, the exact (a m + b) mod q.
//
// These are HBM-bound streams: each thread moves groups of 16-byte pairs
// (loads first), the grid is at most 8 CTAs per SM and loops grid-stride;
// one scalar tail element is handled by one thread.
#include <cuda_runtime.h>

#include <type_traits>

#include "elem_ops.cuh"
#include "kernels.h"

namespace vk {

// B == nullptr for unary operations.  Each thread moves P 16-byte pairs of
// every operand per iteration, all loads issued before the first store, and
// the next iteration's loads issued before this one's arithmetic (2-3.4 %
// faster for the ops with multiplies); lanes past the end re-read the last
// pair and store nothing.  P per op, measured on 2^27-word vectors (fraction
// of the copy bandwidth per public call): the multiply-free unary ops take 8
// (elemgtadd 0.909 with 4 -> 0.94), the unary ops with a reduction or a
// Shoup product 2 (elemgtsub / elemmod 0.87-0.89 with 4 -> 0.92; 8 made
// them 0.80), elemmul 1 (0.937 with 2 -> 0.954), the fused multiply-adds 2
// (elemfma 0.96; 4 made it 0.925).
template <class Op>
constexpr int pairs_per_thread(bool bin) {
  if (bin) return std::is_same<Op, OpMul>::value ? 1 : 2;
  if (std::is_same<Op, OpGtAdd>::value || std::is_same<Op, OpModTwo>::value) return 8;
  return 2;
}

template <class Op, bool BIN>
__global__ void __launch_bounds__(256) k_elementwise(u64* __restrict__ res, const u64* a, const u64* b, u64 len,
                                                     Op op) {
  constexpr int P = pairs_per_thread<Op>(BIN);
  const u64 pairs = len >> 1;
  const u64 step = (u64)gridDim.x * blockDim.x * P;
  const u64 first = (u64)blockIdx.x * blockDim.x * P;
  ulonglong2 x[P], y[BIN ? P : 1];
  // software pipelined: the next group's loads are in flight while this
  // group is computed and stored
  auto load = [&](u64 g0, ulonglong2(&xs)[P], ulonglong2(&ys)[BIN ? P : 1]) {
#pragma unroll
    for (int k = 0; k < P; k++) {
      const u64 p = g0 + threadIdx.x + (u64)k * blockDim.x;
      const u64 pc = p < pairs ? p : pairs - 1;
      xs[k] = ld2(a + 2 * pc);
      if constexpr (BIN) ys[k] = ld2(b + 2 * pc);
    }
  };
  if (first < pairs) load(first, x, y);
  for (u64 g0 = first; g0 < pairs; g0 += step) {
    ulonglong2 xn[P], yn[BIN ? P : 1];
    if (g0 + step < pairs) load(g0 + step, xn, yn);
#pragma unroll
    for (int k = 0; k < P; k++) {
      const u64 p = g0 + threadIdx.x + (u64)k * blockDim.x;
      const ulonglong2 yk = BIN ? y[BIN ? k : 0] : make_ulonglong2(0, 0);
      if (p < pairs) st2(res + 2 * p, op(x[k].x, yk.x), op(x[k].y, yk.y));
    }
#pragma unroll
    for (int k = 0; k < P; k++) {
      x[k] = xn[k];
      if constexpr (BIN) y[k] = yn[BIN ? k : 0];
    }
  }
  if ((len & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    const u64 i = len - 1;
    res[i] = op(a[i], BIN ? b[i] : 0ull);
  }
}

static int g_sms = 0;

// One wave of resident blocks (the kernel's occupancy, looked up once per
// instantiation), or fewer when there is less work.
template <auto kernel>
static unsigned grid(u64 want) {
  static const int per_sm = [] {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, 256, 0) != cudaSuccess || b < 1) b = 1;
    return b;
  }();
  const u64 cap = (u64)g_sms * per_sm;
  const u64 n = want < cap ? want : cap;
  return (unsigned)(n ? n : 1);
}

template <class Op>
static int launch(void* stream, uint64_t* res, const uint64_t* a, const uint64_t* b, uint64_t len, Op op) {
  if (len == 0) return 0;
  if (((reinterpret_cast<uintptr_t>(res) | reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b)) & 15) != 0)
    return (int)cudaErrorMisalignedAddress;
  if (g_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_sms <= 0) g_sms = 1;
  }
  const u64 per_block = 256 * (u64)(b ? pairs_per_thread<Op>(true) : pairs_per_thread<Op>(false));  // pairs a block moves per iteration
  const u64 want = ((len + 1) / 2 + per_block - 1) / per_block;
  auto* r = reinterpret_cast<u64*>(res);
  auto* x = reinterpret_cast<const u64*>(a);
  auto* y = reinterpret_cast<const u64*>(b);
  if (b)
    k_elementwise<Op, true><<<grid<k_elementwise<Op, true>>(want), 256, 0, (cudaStream_t)stream>>>(r, x, y, len, op);
  else
    k_elementwise<Op, false><<<grid<k_elementwise<Op, false>>(want), 256, 0, (cudaStream_t)stream>>>(r, x, y, len, op);
  vkcu_count_launches(1);
  return (int)cudaGetLastError();
}

}  // namespace vk

using namespace vk;

extern "C" int vkcu_elemmul(void* stream, uint64_t* res, const uint64_t* a, const uint64_t* b, uint64_t len,
                            uint64_t mod, uint64_t mu, uint32_t bits) {
  return launch(stream, res, a, b, len, OpMul{mod, mu, bits});
}

extern "C" int vkcu_elemmulconst(void* stream, uint64_t* res, const uint64_t* a, uint64_t len, uint64_t c,
                                 uint64_t c_shoup, uint64_t mod) {
  return launch(stream, res, a, nullptr, len, OpMulConst{c, c_shoup, mod});
}

extern "C" int vkcu_elemfma(void* stream, uint64_t* res, const uint64_t* a, const uint64_t* b, uint64_t len,
                            uint64_t m, uint64_t m_shoup, uint64_t mod) {
  return launch(stream, res, a, b, len, OpFmaRef{m, m_shoup, mod});
}

extern "C" int vkcu_elemfma_canonical(void* stream, uint64_t* res, const uint64_t* a, const uint64_t* b,
                                      uint64_t len, uint64_t m_red, uint64_t m_shoup, uint64_t mod, uint64_t mu,
                                      uint32_t bits) {
  return launch(stream, res, a, b, len, OpFmaCanon{m_red, m_shoup, mod, mu, bits});
}

extern "C" int vkcu_elemgtsub(void* stream, uint64_t* res, const uint64_t* a, uint64_t len, uint64_t bound,
                              uint64_t diff_red, uint64_t mod, uint64_t mu, uint32_t bits) {
  return launch(stream, res, a, nullptr, len, OpGtSub{bound, diff_red, mod, mu, bits});
}

extern "C" int vkcu_elemgtadd(void* stream, uint64_t* res, const uint64_t* a, uint64_t len, uint64_t bound,
                              uint64_t diff) {
  return launch(stream, res, a, nullptr, len, OpGtAdd{bound, diff});
}

extern "C" int vkcu_elemmodbytwo(void* stream, uint64_t* res, const uint64_t* a, uint64_t len,
                                 uint64_t signed_bound) {
  return launch(stream, res, a, nullptr, len, OpModTwo{signed_bound});
}

// ---------------------------------------------------------------------------
// Twiddle tables generated on the device for one (n, q, w) with q < 2^61 and
// w^n = -1.  Word i of the power sequence is w^i = phi[i >> lb] * plo[i & mask]
// (exact Barrett product of two canonical powers, so equal to the reference's
// sequential products); it goes to slot bitrev(i) of the forward table, and
// q - w^i to slot bitrev(n - i) of the inverse table (w^-(n-i) = -w^i).  Each
// entry is stored with its Shoup factor floor(r 2^64 / q).
namespace vk {

__device__ __forceinline__ u64 shoup_factor(u64 r, u64 q) {
  return (u64)((((unsigned __int128)r) << 64) / q);
}

// Thread s writes slot s of both tables, so the 16-byte pairs of consecutive
// threads are contiguous (whole sectors, no read-modify-write in L2):
// fwd[s] = w^j with j = bitrev(s) (the reference's roots[bitrev(j)] = w^j),
// inv[s] = q - w^(n - j) = w^-j for s > 0 (the index rule for w^n = -1) and
// inv[0] = 1.
__device__ __forceinline__ u64 power_of(const u64* __restrict__ phi, const u64* __restrict__ plo, u64 i, u32 lb, u64 q,
                                        u64 mu, u32 qbits) {
  const u64 x = phi[i >> lb], y = plo[i & ((1ull << lb) - 1)];
  return ref_reduce128(mulhi(x, y), x * y, q, mu, qbits);
}

__global__ void k_twiddles(u64* __restrict__ fwd, u64* __restrict__ inv, const u64* __restrict__ phi,
                           const u64* __restrict__ plo, u32 log_n, u32 lb, u64 q, u64 mu, u32 qbits) {
  const u64 n = 1ull << log_n;
  for (u64 s = (u64)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (u64)gridDim.x * blockDim.x) {
    const u64 j = __brev((u32)s) >> (32 - log_n);
    const u64 p = j == 0 ? 1ull : power_of(phi, plo, j, lb, q, mu, qbits);
    const u64 r = s == 0 ? 1ull : q - power_of(phi, plo, n - j, lb, q, mu, qbits);
    fwd[2 * s] = p;
    fwd[2 * s + 1] = shoup_factor(p, q);
    inv[2 * s] = r;
    inv[2 * s + 1] = shoup_factor(r, q);
  }
}

}  // namespace vk

extern "C" int vkcu_twiddles(void* stream, uint64_t* fwd, uint64_t* inv, const uint64_t* phi, const uint64_t* plo,
                             uint32_t log_n, uint32_t lb, uint64_t q, uint64_t mu, uint32_t qbits) {
  if (log_n < 1 || log_n > 31) return (int)cudaErrorInvalidValue;
  const uint64_t n = 1ull << log_n;
  uint64_t blocks = (n + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  vk::k_twiddles<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<vk::u64*>(fwd), reinterpret_cast<vk::u64*>(inv), reinterpret_cast<const vk::u64*>(phi),
      reinterpret_cast<const vk::u64*>(plo), log_n, lb, q, mu, qbits);
  vkcu_count_launches(1);
  return (int)cudaGetLastError();
}
