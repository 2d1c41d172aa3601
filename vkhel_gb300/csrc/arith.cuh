// Device-side 64-bit modular arithmetic for the vkhel GB300 kernels.
//
// Two families live here:
//
//  * Reference-exact element-wise formulas.  The element-wise operations of the
//    reference are defined by their shader arithmetic, including a Barrett
//    reduction with alpha = 62, beta = -2 (include/priv/numbers.h:7-9,
//    src/kernels/shaders/elemmul.comp:36-60) and a Shoup product with a single
//    conditional subtraction (elemmulconst.comp:42-46).  Those are restated
//    here with the same constants so that every output, canonical or not,
//    equals the reference's for every 64-bit input.
//
//  * Lazy (Harvey) butterflies for the transforms.  Values travel in [0, 4q)
//    (forward) or [0, 2q) (inverse) and are made canonical once at the end, so
//    a butterfly costs one Shoup product and no full reduction.  This needs
//    4q <= 2^64, i.e. q < 2^62, which the table builder enforces.  Canonical
//    outputs equal the reference's stage-by-stage canonical arithmetic
//    (nttfwdbutterfly.comp:44-57, nttrevbutterfly.comp:44-57) because both are
//    the same residues mod q.
#pragma once

#include <cstdint>

namespace vk {

typedef unsigned long long u64;
typedef unsigned int u32;

__device__ __forceinline__ u64 mulhi(u64 a, u64 b) { return __umul64hi(a, b); }

// x * w mod q in [0, 2q) for any 64-bit x, given w < q and wp = floor(w 2^64 / q).
__device__ __forceinline__ u64 shoup_lazy(u64 x, u64 w, u64 wp, u64 q) {
  return x * w - mulhi(x, wp) * q;
}

// Same, with one conditional subtraction: canonical for any 64-bit x.
__device__ __forceinline__ u64 shoup(u64 x, u64 w, u64 wp, u64 q) {
  u64 r = shoup_lazy(x, w, wp, q);
  return r >= q ? r - q : r;
}

__device__ __forceinline__ u64 csub(u64 x, u64 m) { return x >= m ? x - m : x; }

// [0, 4q) -> [0, q)
__device__ __forceinline__ u64 canon4(u64 x, u64 q, u64 q2) { return csub(csub(x, q2), q); }

// Cooley-Tukey butterfly on lazy values: X, Y in [0, 4q) -> [0, 4q).
__device__ __forceinline__ void ct_bfly(u64& x, u64& y, u64 w, u64 wp, u64 q, u64 q2) {
  const u64 xr = csub(x, q2);
  const u64 t = shoup_lazy(y, w, wp, q);
  x = xr + t;
  y = xr - t + q2;
}

// Gentleman-Sande butterfly on lazy values: X, Y in [0, 2q) -> [0, 2q).
__device__ __forceinline__ void gs_bfly(u64& x, u64& y, u64 w, u64 wp, u64 q, u64 q2) {
  const u64 s = x + y;
  const u64 d = x - y + q2;
  x = csub(s, q2);
  y = shoup_lazy(d, w, wp, q);
}

// ---- reference-exact Barrett (alpha = 62, beta = -2) ----------------------
// n = bit length of mod (>= 2), mu = floor(2^(n+62) / mod).

// reduce64 (elemmul.comp:36-47): exact for every 64-bit x.
__device__ __forceinline__ u64 ref_reduce64(u64 x, u64 mod, u64 mu, u32 n) {
  const u64 qh = mulhi(x >> (n - 2), mu);
  const u64 z = x - qh * mod;
  return z >= mod ? z - mod : z;
}

// The same for operands that are usually reduced already.  For x < mod the
// estimate floor(k mu / 2^64), k = x >> (n - 2) <= 3, mu <= 2^63, is 0: it
// needs k mu >= 2^64, i.e. k = 2 with mod = 2^(n-1) (but x < mod gives
// k <= 1 then) or k = 3 with mod <= 3 2^(n-2) (but x < mod gives k <= 2
// then).  So reduce64 returns x there, the shortcut gives the same word for
// every 64-bit x, and canonical operands skip the multiplies (the branch is
// uniform across a warp of them).
__device__ __forceinline__ u64 ref_reduce64_maybe(u64 x, u64 mod, u64 mu, u32 n) {
  if (__builtin_expect(x < mod, 1)) return x;
  return ref_reduce64(x, mod, mu, n);
}

// reduce128 (elemmul.comp:49-60).  A shift by 64 (only for a 2-bit modulus,
// where the high word is zero) yields zero.
__device__ __forceinline__ u64 ref_reduce128(u64 hi, u64 lo, u64 mod, u64 mu, u32 n) {
  const u32 sh = 66u - n;
  const u64 top = sh >= 64u ? 0ull : (hi << sh);
  const u64 qh = mulhi(top + (lo >> (n - 2)), mu);
  const u64 z = lo - qh * mod;
  return z >= mod ? z - mod : z;
}

// Barrett product for the fused pointwise step: x, y in [0, q), q < 2^62,
// result in [0, 2q) (the estimate is at most two short for a 62-bit q, so one
// subtraction of 2q is applied when needed).
__device__ __forceinline__ u64 barrett_mul_lazy(u64 x, u64 y, u64 q, u64 q2, u64 mu, u32 n) {
  const u64 lo = x * y;
  const u64 hi = mulhi(x, y);
  const u64 qh = mulhi((hi << (66u - n)) | (lo >> (n - 2)), mu);
  return csub(lo - qh * q, q2);
}

// The reference's centred-lift element-wise ops on one word, as their
// shaders compute them (64-bit wrap included):
//   elemgtsub    src/kernels/shaders/elemgtsub.comp:49-67 (d = diff reduced mod `mod`)
//   elemgtadd    src/kernels/shaders/elemgtadd.comp:20-30
//   elemmodbytwo src/kernels/shaders/elemmodbytwo.comp:19-27 (sb = q / 2)
__device__ __forceinline__ u64 ref_gtsub(u64 a, u64 bound, u64 d, u64 mod, u64 mu, u32 bits) {
  const u64 r = ref_reduce64_maybe(a, mod, mu, bits);
  if (a > bound) {
    const u64 z = r + mod - d;
    return z >= mod ? z - mod : z;
  }
  return r;
}

__device__ __forceinline__ u64 ref_gtadd(u64 a, u64 bound, u64 diff) { return a > bound ? a + diff : a; }

__device__ __forceinline__ u64 ref_modtwo(u64 a, u64 sb) {
  const u64 bit = a & 1;
  return a > sb ? 1 - bit : bit;
}

}  // namespace vk
