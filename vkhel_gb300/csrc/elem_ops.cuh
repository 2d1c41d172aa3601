// Per-word element-wise operations shared by the single-vector kernels
// (elem.cu) and the element-wise batch kernel (elem_batch.cu).  Each restates
// one reference shader with the constants its host wrapper pushes:
//   OpMul        src/kernels/shaders/elemmul.comp:62-73      (elemmul.c:159-168)
//   OpMulConst   src/kernels/shaders/elemmulconst.comp:35-49 (elemmulconst.c:154-163)
//   OpFmaRef     src/kernels/shaders/elemfma.comp:36-55      (elemfma.c:159-169)
//   OpGtSub      src/kernels/shaders/elemgtsub.comp:49-67    (elemgtsub.c:154-168)
//   OpGtAdd      src/kernels/shaders/elemgtadd.comp:20-30
//   OpModTwo     src/kernels/shaders/elemmodbytwo.comp:19-27
// plus OpFmaCanon, the exact (a m + b) mod q.
#pragma once

#include "arith.cuh"

namespace vk {

struct OpMul {
  u64 mod, mu;
  u32 bits;
  __device__ __forceinline__ u64 operator()(u64 a, u64 b) const {
    const u64 x = ref_reduce64_maybe(a, mod, mu, bits);
    const u64 y = ref_reduce64_maybe(b, mod, mu, bits);
    return ref_reduce128(mulhi(x, y), x * y, mod, mu, bits);
  }
};

struct OpMulConst {
  u64 c, cs, mod;
  __device__ __forceinline__ u64 operator()(u64 a, u64) const { return shoup(a, c, cs, mod); }
};

// elemfma.comp:43-54 as written: both "reductions" compute mod - x.
struct OpFmaRef {
  u64 m, ms, mod;
  __device__ __forceinline__ u64 operator()(u64 a, u64 b) const {
    u64 p = a * m - mulhi(a, ms) * mod;
    if (p >= mod) p = mod - p;
    const u64 s = p + b;
    return s >= mod ? mod - s : s;
  }
};

// (a m + b) mod q for any 64-bit a, b; m is given reduced with its Shoup factor.
// A Shoup product is exact only while 2q fits in 64 bits; moduli of 2^63 and
// above take an exact 128-bit remainder instead.
struct OpFmaCanon {
  u64 m, ms, mod, mu;
  u32 bits;
  __device__ __forceinline__ u64 operator()(u64 a, u64 b) const {
    const u64 x = ref_reduce64_maybe(a, mod, mu, bits);
    const u64 p = bits < 64 ? shoup(x, m, ms, mod)
                            : (u64)(((unsigned __int128)x * m) % mod);
    const u64 y = ref_reduce64_maybe(b, mod, mu, bits);
    const u64 s = p + y;
    return (s < p || s >= mod) ? s - mod : s;
  }
};

struct OpGtSub {
  u64 bound, d, mod, mu;
  u32 bits;
  __device__ __forceinline__ u64 operator()(u64 a, u64) const { return ref_gtsub(a, bound, d, mod, mu, bits); }
};

struct OpGtAdd {
  u64 bound, diff;
  __device__ __forceinline__ u64 operator()(u64 a, u64) const { return ref_gtadd(a, bound, diff); }
};

struct OpModTwo {
  u64 sb;
  __device__ __forceinline__ u64 operator()(u64 a, u64) const { return ref_modtwo(a, sb); }
};

__device__ __forceinline__ ulonglong2 ld2(const u64* p) {
  ulonglong2 r;
  asm volatile("ld.global.L1::no_allocate.v2.u64 {%0,%1}, [%2];" : "=l"(r.x), "=l"(r.y) : "l"(p));
  return r;
}

__device__ __forceinline__ void st2(u64* p, u64 a, u64 b) {
  asm volatile("st.global.v2.u64 [%0], {%1,%2};" ::"l"(p), "l"(a), "l"(b) : "memory");
}

}  // namespace vk
