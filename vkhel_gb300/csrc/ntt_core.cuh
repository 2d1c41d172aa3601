// Shared device code of the negacyclic NTT / INTT / fused polymul kernels.
//
// Transform convention (identical to the reference):
//   forward  = the Cooley-Tukey stage loop of src/vector.c:536-566 with the
//              butterfly of src/kernels/shaders/nttfwdbutterfly.comp:41-57,
//              natural order in, bit-reversed order out;
//   inverse  = the Gentleman-Sande loop of src/vector.c:599-630 with the
//              butterfly of nttrevbutterfly.comp:41-57, bit-reversed in,
//              natural out, then x n^-1 (src/vector.c:632-638);
//   twiddles = powers of w in bit-reversed order, root index m + block
//              (src/ntt_tables.c:25-43, src/kernels/nttfwdbutterfly.c:154-159).
//
// GB300 design.  One CTA owns one polynomial of n = 2^LOGN <= 2^14 words
// held in shared memory (padded by one word per 16: index a -> a + a/16,
// which makes every access pattern below free of bank conflicts).  The
// log2(n) butterfly stages run as passes of up to 4 stages: in a pass every
// thread loads radix-2^k groups of words into registers, one group at a time,
// runs the k stages on them and writes them back, so at most 16 words (plus
// their twiddles) are live per thread.  Exceptions:
//   * the first forward pass reads all of the thread's words from global
//     memory up front (the loads are coalesced and all in flight at once);
//   * the last forward pass works on groups of 16 consecutive words, whose
//     results leave with 32-byte vector stores, or -- in the fused polymul --
//     are multiplied pointwise by NTT(b) and run through the first inverse
//     pass in the same registers;
//   * the last inverse pass folds n^-1 into its final stage and writes global
//     memory coalesced.
// Butterflies are lazy (Harvey): values stay in [0, 4q) (forward) or [0, 2q)
// (inverse) and are made canonical once at the end.  That needs 4q <= 2^64;
// moduli 2^62 <= q < 2^63 (the top of the reference's range: its inverse-mod
// works below 2^63, src/numbers.c:71-99) run the same kernels instantiated
// with the Mod63 class below, whose values stay in [0, 2q) both ways.
//
// Bit-exactness for unreduced inputs.  The reference's first stage computes
// (X + WY) mod 2^64 mod q and (X - WY) mod q (forward), or (X + Y) mod 2^64
// mod q and W (X - Y mod q) (inverse).  All later stages see canonical values,
// so only the first stage needs the reference's wrap-around behaviour; it is
// taken on a rarely-used branch whenever an input is >= 2q.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <type_traits>

#include "arith.cuh"
#include "kernels.h"

namespace vk {

template <int I, int N, typename F>
__device__ __forceinline__ void static_for(F&& f) {
  if constexpr (I < N) {
    f(std::integral_constant<int, I>{});
    static_for<I + 1, N>(f);
  }
}

__device__ __forceinline__ int pad(int a) { return a + (a >> 4); }

__device__ __forceinline__ ulonglong2 ld_tw(const ulonglong2* p) {
  ulonglong2 r;
  asm("ld.global.nc.v2.u64 {%0,%1}, [%2];" : "=l"(r.x), "=l"(r.y) : "l"(p));
  return r;
}

__device__ __forceinline__ u64 ld_stream(const u64* p) {
  u64 r;
  asm volatile("ld.global.L1::no_allocate.u64 %0, [%1];" : "=l"(r) : "l"(p));
  return r;
}

__device__ __forceinline__ void ld4(const u64* p, u64& a, u64& b, u64& c, u64& d) {
  asm volatile("ld.global.v4.u64 {%0,%1,%2,%3}, [%4];" : "=l"(a), "=l"(b), "=l"(c), "=l"(d) : "l"(p));
}

__device__ __forceinline__ void st4(u64* p, u64 a, u64 b, u64 c, u64 d) {
  asm volatile("st.global.v4.u64 [%0], {%1,%2,%3,%4};" ::"l"(p), "l"(a), "l"(b), "l"(c), "l"(d) : "memory");
}

// Bring `bytes` at p into L2 ahead of use (no registers, no completion wait).
__device__ __forceinline__ void prefetch_l2(const void* p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Per-transform constants, loaded once per job into registers.
struct Tw {
  u64 q, q2, mu, ninv, ninv_s, w1ninv, w1ninv_s;
  u32 qbits;
  const ulonglong2* fwd;
  const ulonglong2* inv;
};

__device__ __forceinline__ Tw load_tw(const vkcu_twset* p) {
  Tw t;
  t.q = __ldg(reinterpret_cast<const u64*>(&p->q));
  t.q2 = __ldg(reinterpret_cast<const u64*>(&p->q2));
  t.mu = __ldg(reinterpret_cast<const u64*>(&p->mu));
  t.ninv = __ldg(reinterpret_cast<const u64*>(&p->ninv));
  t.ninv_s = __ldg(reinterpret_cast<const u64*>(&p->ninv_s));
  t.w1ninv = __ldg(reinterpret_cast<const u64*>(&p->w1ninv));
  t.w1ninv_s = __ldg(reinterpret_cast<const u64*>(&p->w1ninv_s));
  t.qbits = __ldg(&p->qbits);
  t.fwd = reinterpret_cast<const ulonglong2*>(__ldg(reinterpret_cast<const u64*>(&p->fwd)));
  t.inv = reinterpret_cast<const ulonglong2*>(__ldg(reinterpret_cast<const u64*>(&p->inv)));
  return t;
}

// A caller-supplied NTT(b) operand reduced as the reference's elemmul reduces
// its operands (reduce64, elemmul.comp:36-47): canonical words pass through.
__device__ __forceinline__ void reduce_operand16(u64 (&v)[16], const Tw& t) {
#pragma unroll
  for (int j = 0; j < 16; j++) v[j] = ref_reduce64_maybe(v[j], t.q, t.mu, t.qbits);
}

// ---------------------------------------------------------------------------
// First-stage butterflies with the reference's exact semantics.

struct U2 {
  u64 x, y;
};

// The reference's stage-0 butterfly for x >= 2q, exactly: X' = (X + WY) mod
// 2^64 mod q, Y' = (X - WY) mod q.  Kept out of line: it is rarely taken.
// reduce64 is an exact remainder for q < 2^62.
static __device__ __noinline__ U2 ct_first_slow(u64 x, u64 y, u64 w, u64 wp, u64 q, u64 mu, u32 qbits) {
  const u64 wy = shoup(y, w, wp, q);
  const u64 xr = ref_reduce64(x, q, mu, qbits);
  return U2{ref_reduce64(x + wy, q, mu, qbits), xr >= wy ? xr - wy : xr + q - wy};
}

// Inverse, stage m = n/2: the sum s and difference d before the twiddle
// product, exactly as the reference's (X + Y) mod 2^64 mod q and the
// residue of its `while (t < Y) t += q; t -= Y` loop.
static __device__ __noinline__ U2 gs_first_slow(u64 x, u64 y, u64 q, u64 mu, u32 qbits) {
  const u64 xr = ref_reduce64(x, q, mu, qbits);
  const u64 yr = ref_reduce64(y, q, mu, qbits);
  return U2{ref_reduce64(x + y, q, mu, qbits), xr >= yr ? xr - yr : xr + q - yr};
}

// The same two for 2^62 <= q < 2^63, with the exact 64-bit remainder.
static __device__ __noinline__ U2 ct_first_slow63(u64 x, u64 y, u64 w, u64 wp, u64 q) {
  const u64 wy = shoup(y, w, wp, q);
  const u64 xr = x % q;
  return U2{(x + wy) % q, xr >= wy ? xr - wy : xr + q - wy};
}

static __device__ __noinline__ U2 gs_first_slow63(u64 x, u64 y, u64 q) {
  const u64 xr = x % q, yr = y % q;
  return U2{(x + y) % q, xr >= yr ? xr - yr : xr + q - yr};
}

// ---------------------------------------------------------------------------
// Modulus classes: the butterfly arithmetic every kernel is instantiated with.
//
// Mod62 (q < 2^62): forward values in [0, 4q), inverse values in [0, 2q), one
// conditional subtraction per butterfly (Harvey).  The pointwise product is
// a Barrett product whose result is congruent to the reference's elemmul
// (exact for these moduli).
//
// Mod63 (2^62 <= q < 2^63, where 4q overflows): forward and inverse values in
// [0, 2q), two conditional subtractions per butterfly.  The pointwise
// product restates the reference's elemmul formula word for word
// (elemmul.comp:49-73): with a 63-bit modulus its Barrett estimate
// (hi << 3) + (lo >> 61) wraps past 2^64 for large products, so its results
// are not the true residues, and the polymul must reproduce them; the
// inverse stage that follows then takes the exact first-stage rule, since
// such a word need not be below q.
struct Mod62 {
  static constexpr bool EXACT_AFTER_PRODUCT = false;
  __device__ __forceinline__ static void ct(u64& x, u64& y, u64 w, u64 wp, const Tw& t) {
    ct_bfly(x, y, w, wp, t.q, t.q2);
  }
  __device__ __forceinline__ static void gs(u64& x, u64& y, u64 w, u64 wp, const Tw& t) {
    gs_bfly(x, y, w, wp, t.q, t.q2);
  }
  // sum and difference of two inverse-lazy words before the twiddle product
  __device__ __forceinline__ static void sd(u64 x, u64 y, const Tw& t, u64& s, u64& d) {
    s = x + y;
    d = x - y + t.q2;
  }
  // forward-lazy word -> canonical
  __device__ __forceinline__ static u64 canon(u64 x, const Tw& t) { return canon4(x, t.q, t.q2); }
  // forward-lazy word -> below the next kernel's first-stage fast-path bound
  __device__ __forceinline__ static u64 handoff(u64 x, const Tw& t) { return csub(x, t.q2); }
  // first-stage fast paths: the lazy butterfly is congruent to the reference's
  __device__ __forceinline__ static bool fwd_fast(u64 x, const Tw& t) { return x < t.q2; }
  __device__ __forceinline__ static bool inv_fast(u64 x, u64 y, const Tw& t) { return x < t.q2 && y < t.q2; }
  __device__ __forceinline__ static U2 ct_slow(u64 x, u64 y, u64 w, u64 wp, const Tw& t) {
    return ct_first_slow(x, y, w, wp, t.q, t.mu, t.qbits);
  }
  __device__ __forceinline__ static U2 gs_slow(u64 x, u64 y, const Tw& t) {
    return gs_first_slow(x, y, t.q, t.mu, t.qbits);
  }
  // pointwise product of a forward-lazy word and a canonical one: an
  // inverse-lazy word (fused kernels) ...
  __device__ __forceinline__ static u64 product(u64 x, u64 y, const Tw& t) {
    return barrett_mul_lazy(canon4(x, t.q, t.q2), y, t.q, t.q2, t.mu, t.qbits);
  }
  // ... or, from two canonical words, the word the reference's elemmul stores
  __device__ __forceinline__ static u64 product_out(u64 x, u64 y, const Tw& t) {
    return csub(barrett_mul_lazy(x, y, t.q, t.q2, t.mu, t.qbits), t.q);
  }
};

struct Mod63 {
  static constexpr bool EXACT_AFTER_PRODUCT = true;
  __device__ __forceinline__ static void ct(u64& x, u64& y, u64 w, u64 wp, const Tw& t) {
    const u64 xr = csub(x, t.q);
    const u64 wy = csub(shoup_lazy(y, w, wp, t.q), t.q);
    x = xr + wy;
    y = xr - wy + t.q;
  }
  __device__ __forceinline__ static void sd(u64 x, u64 y, const Tw& t, u64& s, u64& d) {
    const u64 xr = csub(x, t.q), yr = csub(y, t.q);
    s = xr + yr;
    d = xr - yr + t.q;
  }
  __device__ __forceinline__ static void gs(u64& x, u64& y, u64 w, u64 wp, const Tw& t) {
    u64 s, d;
    sd(x, y, t, s, d);
    x = s;
    y = shoup_lazy(d, w, wp, t.q);
  }
  __device__ __forceinline__ static u64 canon(u64 x, const Tw& t) { return csub(x, t.q); }
  __device__ __forceinline__ static u64 handoff(u64 x, const Tw& t) { return csub(x, t.q); }
  __device__ __forceinline__ static bool fwd_fast(u64 x, const Tw& t) { return x < t.q; }
  __device__ __forceinline__ static bool inv_fast(u64 x, u64 y, const Tw& t) { return x < t.q && y < t.q; }
  __device__ __forceinline__ static U2 ct_slow(u64 x, u64 y, u64 w, u64 wp, const Tw& t) {
    return ct_first_slow63(x, y, w, wp, t.q);
  }
  __device__ __forceinline__ static U2 gs_slow(u64 x, u64 y, const Tw& t) { return gs_first_slow63(x, y, t.q); }
  // the reference's elemmul on canonical operands (its reduce64 returns them
  // unchanged): the full 128-bit product through reduce128
  __device__ __forceinline__ static u64 product_out(u64 x, u64 y, const Tw& t) {
    return ref_reduce128(mulhi(x, y), x * y, t.q, t.mu, t.qbits);
  }
  __device__ __forceinline__ static u64 product(u64 x, u64 y, const Tw& t) { return product_out(csub(x, t.q), y, t); }
};

// Forward, stage m = 1, with the reference's exact rule for inputs outside
// the fast path (x >= 2q for Mod62: then x + WY < 3q < 2^64 no longer holds).
template <class M>
__device__ __forceinline__ void ct_first(u64& x, u64& y, u64 w, u64 wp, const Tw& t) {
  if (M::fwd_fast(x, t)) {
    M::ct(x, y, w, wp, t);
  } else {
    const U2 r = M::ct_slow(x, y, w, wp, t);
    x = r.x;
    y = r.y;
  }
}

// Inverse, stage m = n/2: s and d with the exact rule outside the fast path.
template <class M>
__device__ __forceinline__ void gs_first_sd(u64 x, u64 y, const Tw& t, u64& s, u64& d) {
  if (M::inv_fast(x, y, t)) {
    M::sd(x, y, t, s, d);
  } else {
    const U2 r = M::gs_slow(x, y, t);
    s = r.x;
    d = r.y;
  }
}

// ---------------------------------------------------------------------------
// Register-resident radix-2^KK groups.  A group holds 2^KK words v[G0 + j]
// at stride t_min of the transform, all inside one block of the first stage
// of the pass; `base` = (tw_mult * m0 + block) so that the root of sub-stage u
// and sub-block r is table[(base << u) + r].

template <class M, int KK, int U0, int G0, int NV>
__device__ __forceinline__ void ct_group(u64 (&v)[NV], const ulonglong2* tw, u32 base, const Tw& t) {
  static_for<U0, KK>([&](auto uc) {
    constexpr int u = decltype(uc)::value;
    constexpr int half = 1 << (KK - 1 - u);
    static_for<0, (1 << u)>([&](auto rc) {
      constexpr int r = decltype(rc)::value;
      const ulonglong2 w = ld_tw(tw + ((base << u) + r));
#pragma unroll
      for (int jj = 0; jj < half; jj++)
        M::ct(v[G0 + r * 2 * half + jj], v[G0 + r * 2 * half + jj + half], w.x, w.y, t);
    });
  });
}

// Inverse group: sub-stages KK-1 .. 0.  EXACT_TOP applies the exact rule to
// sub-stage KK-1 (global stage m = n/2); FOLD folds n^-1 into sub-stage 0
// (global stage m = 1, root index 1) and leaves canonical outputs.
template <class M, int KK, int G0, bool EXACT_TOP, bool FOLD, int NV>
__device__ __forceinline__ void gs_group(u64 (&v)[NV], const ulonglong2* tw, u32 base, const Tw& t) {
  static_for<0, KK>([&](auto uc) {
    constexpr int u = KK - 1 - decltype(uc)::value;
    constexpr int half = 1 << (KK - 1 - u);
    if constexpr (FOLD && u == 0) {
#pragma unroll
      for (int jj = 0; jj < half; jj++) {
        u64& x = v[G0 + jj];
        u64& y = v[G0 + jj + half];
        u64 s, d;
        if constexpr (EXACT_TOP && u == KK - 1) {
          gs_first_sd<M>(x, y, t, s, d);
        } else {
          M::sd(x, y, t, s, d);
        }
        x = shoup(s, t.ninv, t.ninv_s, t.q);
        y = shoup(d, t.w1ninv, t.w1ninv_s, t.q);
      }
    } else {
      static_for<0, (1 << u)>([&](auto rc) {
        constexpr int r = decltype(rc)::value;
        const ulonglong2 w = ld_tw(tw + ((base << u) + r));
#pragma unroll
        for (int jj = 0; jj < half; jj++) {
          u64& x = v[G0 + r * 2 * half + jj];
          u64& y = v[G0 + r * 2 * half + jj + half];
          if constexpr (EXACT_TOP && u == KK - 1) {
            u64 s, d;
            gs_first_sd<M>(x, y, t, s, d);
            x = csub(s, t.q2);
            y = shoup_lazy(d, w.x, w.y, t.q);
          } else {
            M::gs(x, y, w.x, w.y, t);
          }
        }
      });
    }
  });
}

// ---------------------------------------------------------------------------
// Pass schedule for n = 2^LOGN held by T = n/E threads.  The first pass has
// FIRSTK <= 4 stages and reads global memory; every later pass has exactly 4
// stages (radix 16) and runs on shared memory; the last one starts at stage
// HEAD = LOGN - 4 and sees groups of 16 consecutive words.  Every pass but the
// first has t_min >= 16 or is the last pass.
//
// Code size matters as much as instruction count here: all radix-16 passes of
// a direction share one loop body (the stage offset is a runtime value), and
// the fused polymul runs its two forward transforms through the same code.

template <int LOGN_, int E_, int U_ = 1, class M_ = Mod62, bool DUAL_ = false>
struct Shape {
  using M = M_;  // modulus class
  // DUAL: the CTA holds 2 T threads running two transforms of this shape in
  // step, thread t on the one of half t / T (shared barriers, separate words)
  static constexpr bool DUAL = DUAL_;
  static constexpr int LOGN = LOGN_, E = E_;
  static constexpr int U = U_;  // radix-16 groups of a thread in flight at once (1 or 2)
  static constexpr int N = 1 << LOGN, T = N / E;
  static constexpr int HEAD = LOGN - 4;  // first stage of the last pass
  static constexpr int FIRSTK = HEAD % 4 == 0 ? 4 : HEAD % 4;
  static constexpr int SMEM_BYTES = (N + N / 16) * 8;
  static_assert(E >= 16 && (E % 16) == 0 && HEAD >= 1 && T >= 1, "unsupported shape");
  // this thread's index within its transform
  __device__ __forceinline__ static int tid() { return DUAL ? (int)(threadIdx.x & (T - 1)) : (int)threadIdx.x; }
};

// A radix-16 pass starting at stage s0 of an n = 2^logn transform: group g
// has block g >> lt (lt = log2 t_min), first word (g >> lt) << lb | (g & mask)
// with lb = log2(n >> s0), words at stride t_min, twiddle base tw0 + block.
struct Pass16 {
  int lt, lb;
  u32 tw0;
  __device__ __forceinline__ Pass16(int logn, int s0, u32 tw_mult)
      : lt(logn - s0 - 4), lb(logn - s0), tw0(tw_mult << s0) {}
  __device__ __forceinline__ int first(int g) const { return ((g >> lt) << lb) | (g & ((1 << lt) - 1)); }
  __device__ __forceinline__ u32 base(int g) const { return tw0 + (u32)(g >> lt); }
};

// Groups of 2^KK words a thread handles at once in the passes that walk G
// such groups: 16 words per round (fewer leave too little independent work
// between the loads and the stores of a round; more spill).
template <int KK, int G>
constexpr int round_groups() {
  return (16 >> KK) < 1 ? 1 : (G < (16 >> KK) ? G : (16 >> KK));
}

// First forward pass: this thread's words come from global memory (coalesced)
// in rounds of 16 (all of a round's loads in flight at once; 32 words at once
// would spill), then FIRSTK stages per group, results to shared memory.
// The first sub-stage uses the exact first-stage rule; after the global pass
// of a large transform the inputs are < 2q and always take its fast path.
template <class S>
__device__ __forceinline__ void fwd_first(u64* sm, const u64* __restrict__ in, const Tw& t, u32 tw_mult) {
  constexpr int KK = S::FIRSTK, G = S::E >> KK, TMIN = S::N >> KK;
  constexpr int GR = round_groups<KK, G>();
#pragma unroll 1
  for (int i0 = 0; i0 < G; i0 += GR) {
    u64 v[GR << KK];
#pragma unroll
    for (int i = 0; i < GR; i++)
#pragma unroll
      for (int j = 0; j < (1 << KK); j++)
        v[i * (1 << KK) + j] = ld_stream(in + S::tid() + (i0 + i) * S::T + j * TMIN);
    const ulonglong2 w0 = ld_tw(t.fwd + tw_mult);
    static_for<0, GR>([&](auto ic) {
      constexpr int i = decltype(ic)::value;
#pragma unroll
      for (int jj = 0; jj < (1 << (KK - 1)); jj++)
        ct_first<typename S::M>(v[i * (1 << KK) + jj], v[i * (1 << KK) + jj + (1 << (KK - 1))], w0.x, w0.y, t);
      ct_group<typename S::M, KK, 1, i * (1 << KK)>(v, t.fwd, tw_mult, t);
      const int g = S::tid() + (i0 + i) * S::T;
#pragma unroll
      for (int j = 0; j < (1 << KK); j++) sm[pad(g + j * TMIN)] = v[i * (1 << KK) + j];
    });
  }
  __syncthreads();
}

// First forward pass on data already in shared memory (the sub-blocks of a
// cluster transform): groups of 2^FIRSTK words, twiddle base tw_mult.
template <class S>
__device__ __forceinline__ void fwd_first_smem(u64* sm, const Tw& t, u32 tw_mult) {
  constexpr int KK = S::FIRSTK, G = S::E >> KK, TMIN = S::N >> KK, GR = round_groups<KK, G>();
#pragma unroll 1
  for (int i0 = 0; i0 < G; i0 += GR) {
    const int g0 = S::tid() + i0 * S::T;
    u64 v[GR << KK];
#pragma unroll
    for (int i = 0; i < GR; i++)
#pragma unroll
      for (int j = 0; j < (1 << KK); j++) v[i * (1 << KK) + j] = sm[pad(g0 + i * S::T + j * TMIN)];
    static_for<0, GR>(
        [&](auto ic) { ct_group<typename S::M, KK, 0, decltype(ic)::value * (1 << KK)>(v, t.fwd, tw_mult, t); });
#pragma unroll
    for (int i = 0; i < GR; i++)
#pragma unroll
      for (int j = 0; j < (1 << KK); j++) sm[pad(g0 + i * S::T + j * TMIN)] = v[i * (1 << KK) + j];
  }
  __syncthreads();
}

// Radix-16 forward passes s0 = FIRSTK, FIRSTK + 4, ..., HEAD on shared
// memory.  The last pass hands each group (words 16g .. 16g+15) to epi(g, v)
// instead of storing it back.  Ends with a barrier.
template <class S, class Epi>
__device__ __forceinline__ void fwd_passes(u64* sm, const Tw& t, u32 tw_mult, Epi&& epi) {
#pragma unroll 1
  for (int s0 = S::FIRSTK; s0 <= S::HEAD; s0 += 4) {
    const Pass16 ps(S::LOGN, s0, tw_mult);
    const int st = 1 << ps.lt;
#pragma unroll(S::U)
    for (int i = 0; i < S::E / 16; i++) {
      const int g = S::tid() + i * S::T;
      const int a0 = ps.first(g);
      u64 v[16];
#pragma unroll
      for (int j = 0; j < 16; j++) v[j] = sm[pad(a0 + j * st)];
      ct_group<typename S::M, 4, 0, 0>(v, t.fwd, ps.base(g), t);
      if (s0 < S::HEAD) {
#pragma unroll
        for (int j = 0; j < 16; j++) sm[pad(a0 + j * st)] = v[j];
      } else {
        epi(g, v);
      }
    }
    __syncthreads();
  }
}

// Radix-16 inverse passes s0 = s_top, s_top - 4, ..., FIRSTK on shared
// memory, each followed by a barrier.
template <class S>
__device__ __forceinline__ void inv_passes(u64* sm, const Tw& t, u32 tw_mult, int s_top) {
#pragma unroll 1
  for (int s0 = s_top; s0 >= S::FIRSTK; s0 -= 4) {
    const Pass16 ps(S::LOGN, s0, tw_mult);
    const int st = 1 << ps.lt;
#pragma unroll(S::U)
    for (int i = 0; i < S::E / 16; i++) {
      const int g = S::tid() + i * S::T;
      const int a0 = ps.first(g);
      u64 v[16];
#pragma unroll
      for (int j = 0; j < 16; j++) v[j] = sm[pad(a0 + j * st)];
      gs_group<typename S::M, 4, 0, false, false>(v, t.inv, ps.base(g), t);
#pragma unroll
      for (int j = 0; j < 16; j++) sm[pad(a0 + j * st)] = v[j];
    }
    __syncthreads();
  }
}

// Last inverse pass of a cluster sub-block: stages FIRSTK-1 .. 0 in place in
// shared memory, lazy [0, 2q), followed by a barrier.
template <class S>
__device__ __forceinline__ void inv_last_smem(u64* sm, const Tw& t, u32 tw_mult) {
  constexpr int KK = S::FIRSTK, G = S::E >> KK, TMIN = S::N >> KK, GR = round_groups<KK, G>();
#pragma unroll 1
  for (int i0 = 0; i0 < G; i0 += GR) {
    const int g0 = S::tid() + i0 * S::T;
    u64 v[GR << KK];
#pragma unroll
    for (int i = 0; i < GR; i++)
#pragma unroll
      for (int j = 0; j < (1 << KK); j++) v[i * (1 << KK) + j] = sm[pad(g0 + i * S::T + j * TMIN)];
    static_for<0, GR>(
        [&](auto ic) { gs_group<typename S::M, KK, decltype(ic)::value * (1 << KK), false, false>(v, t.inv, tw_mult, t); });
#pragma unroll
    for (int i = 0; i < GR; i++)
#pragma unroll
      for (int j = 0; j < (1 << KK); j++) sm[pad(g0 + i * S::T + j * TMIN)] = v[i * (1 << KK) + j];
  }
  __syncthreads();
}

// Epilogue of the inverse transforms: the reference's centred-lift ops in
// order on each canonical output word (src/vector.c:342-386, 429-511), with
// the job's modulus resolved once per job for VKCU_LIFT_TABLE_Q steps.
struct LiftRun {
  const vkcu_lift* L;
  u64 bound[VKCU_MAX_LIFT], d[VKCU_MAX_LIFT];
  __device__ __forceinline__ LiftRun(const vkcu_lift* l, u64 q) : L(l) {
#pragma unroll
    for (int s = 0; s < VKCU_MAX_LIFT; s++) {
      const vkcu_lift_step& st = L->step[s];
      const bool tq = (st.kind & VKCU_LIFT_TABLE_Q) != 0;
      bound[s] = tq ? q >> 1 : st.bound;
      d[s] = tq && s < (int)L->count && (st.kind & 0xff) == VKCU_LIFT_GTSUB ? ref_reduce64(q, st.mod, st.mu, st.bits)
                                                                              : st.d;
    }
  }
  // From constants resolved earlier (bound[], d[] of a LiftRun built for q).
  __device__ __forceinline__ LiftRun(const vkcu_lift* l, const u64* b, const u64* dd) : L(l) {
#pragma unroll
    for (int s = 0; s < VKCU_MAX_LIFT; s++) {
      bound[s] = b[s];
      d[s] = dd[s];
    }
  }
  __device__ __forceinline__ u64 operator()(u64 x) const {
#pragma unroll
    for (int s = 0; s < VKCU_MAX_LIFT; s++) {
      if (s >= (int)L->count) break;
      const vkcu_lift_step& st = L->step[s];
      const u32 kind = st.kind & 0xff;
      if (kind == VKCU_LIFT_MODTWO)
        x = ref_modtwo(x, bound[s]);
      else if (kind == VKCU_LIFT_GTSUB)
        x = ref_gtsub(x, bound[s], d[s], st.mod, st.mu, st.bits);
      else
        x = ref_gtadd(x, bound[s], d[s]);
    }
    return x;
  }
  // K words through the steps together: one walk of the step list, K
  // independent chains.
  template <int K>
  __device__ __forceinline__ void apply(u64 (&v)[K]) const {
#pragma unroll
    for (int s = 0; s < VKCU_MAX_LIFT; s++) {
      if (s >= (int)L->count) break;
      const vkcu_lift_step& st = L->step[s];
      const u32 kind = st.kind & 0xff;
      if (kind == VKCU_LIFT_MODTWO) {
#pragma unroll
        for (int k = 0; k < K; k++) v[k] = ref_modtwo(v[k], bound[s]);
      } else if (kind == VKCU_LIFT_GTSUB) {
#pragma unroll
        for (int k = 0; k < K; k++) v[k] = ref_gtsub(v[k], bound[s], d[s], st.mod, st.mu, st.bits);
      } else {
#pragma unroll
        for (int k = 0; k < K; k++) v[k] = ref_gtadd(v[k], bound[s], d[s]);
      }
    }
  }
};

struct NoLift {
  __device__ __forceinline__ u64 operator()(u64 x) const { return x; }
};

// Last inverse pass (stages FIRSTK-1 .. 0) from shared memory to `out`,
// coalesced, one group at a time (rounds of 16 words measured slower here).
// fold: whole transform, n^-1 folded into stage 0, canonical output;
// otherwise lazy [0, 2q).
template <class S, class Epi>
__device__ __forceinline__ void inv_last_epi(u64* sm, const Tw& t, u32 tw_mult, u64* __restrict__ out, bool fold,
                                             const Epi& epi) {
  constexpr int KK = S::FIRSTK, G = S::E >> KK, TMIN = S::N >> KK;
#pragma unroll 1
  for (int i = 0; i < G; i++) {
    const int g = S::tid() + i * S::T;
    u64 v[1 << KK];
#pragma unroll
    for (int j = 0; j < (1 << KK); j++) v[j] = sm[pad(g + j * TMIN)];
    if (fold)
      gs_group<typename S::M, KK, 0, false, true>(v, t.inv, tw_mult, t);
    else
      gs_group<typename S::M, KK, 0, false, false>(v, t.inv, tw_mult, t);
#pragma unroll
    for (int j = 0; j < (1 << KK); j++) out[g + j * TMIN] = epi(v[j]);
  }
}

// Last inverse pass to global memory; LIFT applies the epilogue (only where
// fold, i.e. this pass ends the transform).
template <class S, bool LIFT = false>
__device__ __forceinline__ void inv_last(u64* sm, const Tw& t, u32 tw_mult, u64* __restrict__ out, bool fold,
                                         const vkcu_lift* lift = nullptr) {
  if constexpr (LIFT)
    inv_last_epi<S>(sm, t, tw_mult, out, fold, LiftRun(lift, t.q));
  else
    inv_last_epi<S>(sm, t, tw_mult, out, fold, NoLift{});
}

// Register groups of 16 consecutive words <-> global memory (32-byte vectors).
__device__ __forceinline__ void load16(u64 (&v)[16], const u64* p) {
#pragma unroll
  for (int h = 0; h < 4; h++) ld4(p + 4 * h, v[4 * h], v[4 * h + 1], v[4 * h + 2], v[4 * h + 3]);
}

__device__ __forceinline__ void store16(const u64 (&v)[16], u64* p) {
#pragma unroll
  for (int h = 0; h < 4; h++) st4(p + 4 * h, v[4 * h], v[4 * h + 1], v[4 * h + 2], v[4 * h + 3]);
}

// Resident CTAs per SM the register budget is sized for: 512 threads per SM
// (128 registers per thread, 16 warps) for the 32-words-per-thread shapes and
// for the 16-words-per-thread transforms from n = 2^9 and polymuls from
// n = 2^12; 384 threads (about 170 registers) for the other 16-word shapes.
// Left at 384, the 2^12 shapes took 222 registers (one CTA of 256 threads per
// SM): 128 made them 9 % (polymul) and 17 % (transforms) faster; the 2^9 ..
// 2^11 transforms gained 4 %, the polymuls of those sizes lost 2-3 %, and
// n = 2^8 (16-thread CTAs) spills above 384.
template <int LOGN, int E, bool POLY = false>
constexpr int min_blocks() {
  constexpr int budget = E >= 32 || LOGN >= (POLY ? 12 : 9) ? 512 : 384;
  return (budget / ((1 << LOGN) / E)) < 1 ? 1 : (budget / ((1 << LOGN) / E));
}

template <class J>
__device__ __forceinline__ J fetch_job(const J* jobs, const J& one, int jid) {
  return jobs ? jobs[jid] : one;
}

// ---------------------------------------------------------------------------
// Kernels.  Jobs come from a device array (persistent loop over
// blockIdx.x, blockIdx.x + gridDim.x, ...) or, for a single job, by value.
// sub_log > 0: each job is split into 2^sub_log sub-blocks of 2^LOGN words
// (transforms of 2^(LOGN + sub_log) words after / before the global passes),
// sub-block `sub` using twiddle multiplier 2^sub_log + sub.

template <int LOGN, int E, int U, class M = Mod62>
__global__ void __launch_bounds__((1 << LOGN) / E, min_blocks<LOGN, E>())
    k_ntt_fwd(const vkcu_ntt_job* __restrict__ jobs, int njobs, vkcu_ntt_job one, int sub_log) {
  using S = Shape<LOGN, E, U, M>;
  extern __shared__ u64 sm[];
  const int total = njobs << sub_log;
#pragma unroll 1
  for (int w = blockIdx.x; w < total; w += gridDim.x) {
    const vkcu_ntt_job job = fetch_job(jobs, one, w >> sub_log);
    const int sub = w & ((1 << sub_log) - 1);
    const Tw t = load_tw(job.tw);
    u64* out = reinterpret_cast<u64*>(job.out) + ((size_t)sub << LOGN);
    const u64* in = sub_log ? out : reinterpret_cast<const u64*>(job.in);
    const u32 tw_mult = (1u << sub_log) + sub;
    fwd_first<S>(sm, in, t, tw_mult);
    fwd_passes<S>(sm, t, tw_mult, [&](int g, u64(&v)[16]) {
#pragma unroll
      for (int j = 0; j < 16; j++) v[j] = M::canon(v[j], t);
      store16(v, out + 16 * g);
    });
  }
}

// LIFT: the epilogue `lift` follows the last stage (sub_log == 0 only).
template <int LOGN, int E, int U, bool LIFT = false, class M = Mod62>
__global__ void __launch_bounds__((1 << LOGN) / E, min_blocks<LOGN, E>())
    k_ntt_inv(const vkcu_ntt_job* __restrict__ jobs, int njobs, vkcu_ntt_job one, int sub_log,
              const __grid_constant__ vkcu_lift lift) {
  using S = Shape<LOGN, E, U, M>;
  extern __shared__ u64 sm[];
  const int total = njobs << sub_log;
#pragma unroll 1
  for (int w = blockIdx.x; w < total; w += gridDim.x) {
    const vkcu_ntt_job job = fetch_job(jobs, one, w >> sub_log);
    const int sub = w & ((1 << sub_log) - 1);
    const Tw t = load_tw(job.tw);
    const u64* in = reinterpret_cast<const u64*>(job.in) + ((size_t)sub << LOGN);
    u64* out = reinterpret_cast<u64*>(job.out) + ((size_t)sub << LOGN);
    // the next work item's words into L2 while this one runs (2.6-3.4 % on
    // batched inverse transforms; the forward kernel measured no better so)
    if (w + (int)gridDim.x < total && threadIdx.x < 4) {
      const int w2 = w + (int)gridDim.x, sub2 = w2 & ((1 << sub_log) - 1);
      const vkcu_ntt_job nx = fetch_job(jobs, one, w2 >> sub_log);
      prefetch_l2(reinterpret_cast<const char*>(reinterpret_cast<const u64*>(nx.in) + ((size_t)sub2 << LOGN)) +
                      threadIdx.x * (S::N * 2),
                  S::N * 2);
    }
    const u32 tw_mult = (1u << sub_log) + sub;
    // first inverse pass (global stage m = n/2 first, exact rule) from global;
    // U groups in flight, as in the other passes
#pragma unroll(S::U)
    for (int i = 0; i < S::E / 16; i++) {
      const int g = (int)threadIdx.x + i * S::T;
      u64 v[16];
      load16(v, in + 16 * g);
      gs_group<M, 4, 0, true, false>(v, t.inv, tw_mult * (u32)(S::N / 16) + (u32)g, t);
#pragma unroll
      for (int j = 0; j < 16; j++) sm[pad(16 * g + j)] = v[j];
    }
    __syncthreads();
    inv_passes<S>(sm, t, tw_mult, S::HEAD - 4);
    inv_last<S, LIFT>(sm, t, tw_mult, out, sub_log == 0, &lift);
    __syncthreads();
  }
}

// Fused c = INTT(NTT(a) . NTT(b)).  Phase 0 transforms b and parks NTT(b)
// (canonical) in job.scratch; phase 1 transforms a with the same code, and its
// last pass multiplies by NTT(b) (read back at the words this thread wrote)
// and runs the first inverse pass on the products in the same registers; the
// rest of the inverse transform then writes c.  a is prefetched
// into L2 while b is transformed, the next job's b while a is.
template <int LOGN, int E, int U, bool LIFT = false, class M = Mod62>
__global__ void __launch_bounds__((1 << LOGN) / E, min_blocks<LOGN, E, true>())
    k_polymul(const vkcu_poly_job* __restrict__ jobs, int njobs, vkcu_poly_job one,
              const __grid_constant__ vkcu_lift lift) {
  using S = Shape<LOGN, E, U, M>;
  extern __shared__ u64 sm[];
  constexpr unsigned kChunk = (unsigned)(S::N * 8 / 4);
#pragma unroll 1
  for (int w = blockIdx.x; w < njobs; w += gridDim.x) {
    const vkcu_poly_job job = fetch_job(jobs, one, w);
    const Tw t = load_tw(job.tw);
    // b holds NTT(b): phase 0 is skipped (read by the epilogue instantiations only)
    const bool b_ntt = LIFT && (job.flags & VKCU_JOB_B_NTT);
    u64* scratch = b_ntt ? const_cast<u64*>(reinterpret_cast<const u64*>(job.b)) : reinterpret_cast<u64*>(job.scratch);
    if (threadIdx.x < 4) prefetch_l2(reinterpret_cast<const char*>(job.a) + threadIdx.x * kChunk, kChunk);
#pragma unroll 1
    for (int ph = b_ntt ? 1 : 0; ph < 2; ph++) {
      fwd_first<S>(sm, reinterpret_cast<const u64*>(ph ? job.a : job.b), t, 1u);
      if (ph == 1 && w + (int)gridDim.x < njobs && threadIdx.x < 4) {
        const vkcu_poly_job nx = fetch_job(jobs, one, w + (int)gridDim.x);
        prefetch_l2(reinterpret_cast<const char*>(nx.b) + threadIdx.x * kChunk, kChunk);
      }
      fwd_passes<S>(sm, t, 1u, [&](int g, u64(&v)[16]) {
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
          // the first inverse pass (stages HEAD + 3 .. HEAD) on the same 16 words
          gs_group<M, 4, 0, M::EXACT_AFTER_PRODUCT, false>(v, t.inv, (1u << S::HEAD) + (u32)g, t);
#pragma unroll
          for (int j = 0; j < 16; j++) sm[pad(16 * g + j)] = v[j];
        }
      });
    }
    inv_passes<S>(sm, t, 1u, S::HEAD - 4);
    inv_last<S, LIFT>(sm, t, 1u, reinterpret_cast<u64*>(job.c), true, &lift);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Host side: per-family launchers (one translation unit each).

// variant: 0 = default shape, 1 = two radix-16 groups per thread in flight,
// 2 = the other words-per-thread shape (2^10..2^13 only); others -> 0.
int fwd_cta(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int log_n, int sub_log,
            int sms, int variant);
int inv_cta(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int log_n, int sub_log,
            int sms, int variant);
int poly_cta(cudaStream_t st, const vkcu_poly_job* jobs, int njobs, const vkcu_poly_job& one, int log_n, int sms,
             int variant);
// With an epilogue, one CTA per transform: the inverse in the default shape
// of each degree, the polymul in the variant given.
int inv_cta_lift(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int log_n, int sms,
                 const vkcu_lift& lift);
int poly_cta_lift(cudaStream_t st, const vkcu_poly_job* jobs, int njobs, const vkcu_poly_job& one, int log_n, int sms,
                  int variant, const vkcu_lift& lift);
// cluster of 2^logc CTAs with sub-blocks of 2^logs words, n = 2^(logc + logs):
// logs = 14 for n = 2^15 .. 2^17; logc = 3 with logs = 10 / 11 for n = 2^13 / 2^14
int fwd_cluster(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int logc, int logs);
int inv_cluster(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int logc, int logs,
                const vkcu_lift* lift = nullptr);
int poly_cluster(cudaStream_t st, const vkcu_poly_job* jobs, int njobs, const vkcu_poly_job& one, int logc, int logs,
                 const vkcu_lift* lift = nullptr);

// The same families for 2^62 <= q < 2^63 (Mod63), default shape of each
// degree, sub-blocks of 2^14 words for the cluster kernels (translation units
// ntt_wide_*.cu).
int fwd_cta_wide(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int log_n,
                 int sub_log, int sms);
int inv_cta_wide(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int log_n,
                 int sub_log, int sms, const vkcu_lift* lift);
int poly_cta_wide(cudaStream_t st, const vkcu_poly_job* jobs, int njobs, const vkcu_poly_job& one, int log_n, int sms,
                  const vkcu_lift* lift);
int fwd_cluster_wide(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int logc);
int inv_cluster_wide(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int logc,
                     const vkcu_lift* lift);
int poly_cluster_wide(cudaStream_t st, const vkcu_poly_job* jobs, int njobs, const vkcu_poly_job& one, int logc,
                      const vkcu_lift* lift);

// Launch set-up of one kernel, per device: the dynamic shared-memory opt-in
// and the occupancy figure its grid is sized from (resident blocks per SM,
// or resident clusters), both fixed for a kernel on a device, so they are
// computed once per device instead of on every launch (devices beyond 31
// recompute every time).
struct KernelSetup {
  std::atomic<int> per_dev[32];
};

__host__ inline int current_device() {
  int dev = 0;
  return cudaGetDevice(&dev) == cudaSuccess ? dev : -1;
}

// Opts `kernel` into `smem_limit` (default: `smem`) bytes of dynamic shared
// memory -- the attribute belongs to the kernel, so a kernel launched with
// several sizes is opted into the largest -- and returns its resident blocks
// per SM for `threads` threads and `smem` bytes (at least 1) in *per_sm.
template <class K>
static int setup_cta(K kernel, int threads, int smem, KernelSetup& ks, int* per_sm, int smem_limit = 0) {
  const int dev = current_device();
  const bool cached = dev >= 0 && dev < 32;
  if (cached) {
    const int v = ks.per_dev[dev].load(std::memory_order_acquire);
    if (v > 0) {
      *per_sm = v;
      return 0;
    }
  }
  const int e = (int)cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          smem_limit > smem ? smem_limit : smem);
  if (e) return e;
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, threads, smem) != cudaSuccess || b < 1) b = 1;
  if (cached) ks.per_dev[dev].store(b, std::memory_order_release);
  *per_sm = b;
  return 0;
}

// A persistent grid: one wave of resident blocks, or fewer when there is less work.
__host__ inline int grid_from(int per_sm, long work, int sms) {
  const long cap = (long)per_sm * (sms > 0 ? sms : 1);
  return (int)(work < cap ? work : cap);
}

// One launch of the CTA-resident kernel `kern` of shape S over `work` work
// items (one-time set-up per kernel and device; grid = one wave of resident
// blocks, or fewer when there is less work).
template <class S, auto kern, class... Args>
static int launch_cta(cudaStream_t st, long work, int sms, Args... args) {
  static KernelSetup setup;
  int per_sm = 1;
  if (const int e = setup_cta(kern, S::T, S::SMEM_BYTES, setup, &per_sm)) return e;
  kern<<<grid_from(per_sm, work, sms), S::T, S::SMEM_BYTES, st>>>(args...);
  vkcu_count_launches(1);
  return (int)cudaGetLastError();
}

// Shapes per degree and variant: words per thread E and group unroll U.
#define VK_FOR_LOGN(X)                                                        \
  switch (log_n * 4 + (variant == 1 ? 1 : variant == 2 ? 2 : 0)) {            \
    case 8 * 4: return X(8, 16, 1);                                           \
    case 8 * 4 + 1: return X(8, 16, 2);                                       \
    case 9 * 4: return X(9, 16, 1);                                           \
    case 9 * 4 + 1: return X(9, 16, 2);                                       \
    case 10 * 4: return X(10, 16, 1);                                         \
    case 10 * 4 + 1: return X(10, 16, 2);                                     \
    case 10 * 4 + 2: return X(10, 32, 1);                                     \
    case 11 * 4: return X(11, 16, 1);                                         \
    case 11 * 4 + 1: return X(11, 16, 2);                                     \
    case 11 * 4 + 2: return X(11, 32, 1);                                     \
    case 12 * 4: return X(12, 16, 1);                                         \
    case 12 * 4 + 1: return X(12, 16, 2);                                     \
    case 12 * 4 + 2: return X(12, 32, 1);                                     \
    case 13 * 4: return X(13, 32, 1);                                         \
    case 13 * 4 + 1: return X(13, 32, 2);                                     \
    case 13 * 4 + 2: return X(13, 16, 1);                                     \
    case 14 * 4: return X(14, 32, 1);                                         \
    case 14 * 4 + 1: return X(14, 32, 2);                                     \
    default:                                                                  \
      if (variant != 0) { variant = 0; goto retry; }                          \
      return (int)cudaErrorInvalidValue;                                      \
  }

// Default shape of each degree (variant 0 above).
#define VK_FOR_LOGN_DEFAULT(X)                                                \
  switch (log_n) {                                                            \
    case 8: return X(8, 16, 1);                                               \
    case 9: return X(9, 16, 1);                                               \
    case 10: return X(10, 16, 1);                                             \
    case 11: return X(11, 16, 1);                                             \
    case 12: return X(12, 16, 1);                                             \
    case 13: return X(13, 32, 1);                                             \
    case 14: return X(14, 32, 1);                                             \
    default: return (int)cudaErrorInvalidValue;                               \
  }

}  // namespace vk
