// Negacyclic NTT / INTT / fused polynomial-multiply kernels for sm_103a.
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
// GB300 design.  One CTA owns one polynomial of n = 2^LOGN <= 2^14 words:
//   * every thread holds E words in registers; a "pass" runs up to log2(E)
//     butterfly stages on register-resident radix-2^k groups;
//   * passes exchange data through shared memory padded by one word per 16
//     (index a -> a + a/16), which makes every access pattern used here free
//     of bank conflicts;
//   * the first pass reads global memory coalesced, the last pass leaves each
//     thread with groups of 16 consecutive outputs (written with 32-byte
//     vector stores, or kept in registers for the pointwise step of a fused
//     polynomial multiply);
//   * butterflies are lazy (Harvey): values stay in [0, 4q) / [0, 2q) and are
//     made canonical once; the inverse folds n^-1 into its last stage.
// Larger n runs one register pass over global memory for the first (forward)
// or last (inverse) log2(n) - 14 stages and the CTA kernel on each 2^14-word
// sub-block.
//
// Bit-exactness for unreduced inputs.  The reference's first stage computes
// (X + WY) mod 2^64 mod q and (X - WY) mod q (forward), or (X + Y) mod 2^64
// mod q and W (X - Y mod q) (inverse).  All later stages see canonical values,
// so only the first stage needs the reference's exact wrap-around behaviour;
// it is taken on a rarely-used branch whenever an input is >= 2q.
#include <cuda_runtime.h>

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
  asm volatile("ld.global.v4.u64 {%0,%1,%2,%3}, [%4];"
               : "=l"(a), "=l"(b), "=l"(c), "=l"(d) : "l"(p));
}

__device__ __forceinline__ void st4(u64* p, u64 a, u64 b, u64 c, u64 d) {
  asm volatile("st.global.v4.u64 [%0], {%1,%2,%3,%4};" ::"l"(p), "l"(a), "l"(b), "l"(c), "l"(d)
               : "memory");
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

// ---------------------------------------------------------------------------
// First-stage butterflies with the reference's exact semantics.

// Forward, stage m = 1.  Fast path whenever x < 2q: then x + WY < 3q < 2^64,
// so the reference does not wrap and the lazy result is congruent.
__device__ __forceinline__ void ct_first(u64& x, u64& y, u64 w, u64 wp, const Tw& t) {
  if (x < t.q2) {
    ct_bfly(x, y, w, wp, t.q, t.q2);
  } else {
    const u64 wy = shoup(y, w, wp, t.q);
    const u64 xr = ref_reduce64(x, t.q, t.mu, t.qbits);
    const u64 s = ref_reduce64(x + wy, t.q, t.mu, t.qbits);
    y = xr >= wy ? xr - wy : xr + t.q - wy;
    x = s;
  }
}

// Inverse, stage m = n/2: returns the sum s and difference d before the
// twiddle product; s in [0, 4q), d in (0, 4q).
__device__ __forceinline__ void gs_first_sd(u64 x, u64 y, const Tw& t, u64& s, u64& d) {
  if (x < t.q2 && y < t.q2) {
    s = x + y;
    d = x - y + t.q2;
  } else {
    s = ref_reduce64(x + y, t.q, t.mu, t.qbits);
    const u64 xr = ref_reduce64(x, t.q, t.mu, t.qbits);
    const u64 yr = ref_reduce64(y, t.q, t.mu, t.qbits);
    d = xr >= yr ? xr - yr : xr + t.q - yr;
  }
}

// ---------------------------------------------------------------------------
// Register-resident radix-2^KK groups.  A group holds 2^KK words v[G0 + j]
// at stride t_min of the transform, all inside one block of the first stage
// of the pass; `base` = (tw_mult * m0 + block) so that the root of sub-stage u
// and sub-block r is table[(base << u) + r].

template <int KK, int U0, int G0, int NV>
__device__ __forceinline__ void ct_group(u64 (&v)[NV], const ulonglong2* tw, u32 base, const Tw& t) {
  static_for<U0, KK>([&](auto uc) {
    constexpr int u = decltype(uc)::value;
    constexpr int half = 1 << (KK - 1 - u);
    static_for<0, (1 << u)>([&](auto rc) {
      constexpr int r = decltype(rc)::value;
      const ulonglong2 w = ld_tw(tw + ((base << u) + r));
#pragma unroll
      for (int jj = 0; jj < half; jj++)
        ct_bfly(v[G0 + r * 2 * half + jj], v[G0 + r * 2 * half + jj + half], w.x, w.y, t.q, t.q2);
    });
  });
}

// Forward sub-stage 0 of a group with the exact first-stage rule (root index 1).
template <int KK, int G0, int NV>
__device__ __forceinline__ void ct_group_first_exact(u64 (&v)[NV], const Tw& t) {
  constexpr int half = 1 << (KK - 1);
  const ulonglong2 w = ld_tw(t.fwd + 1);
#pragma unroll
  for (int jj = 0; jj < half; jj++) ct_first(v[G0 + jj], v[G0 + jj + half], w.x, w.y, t);
}

// Inverse group: sub-stages KK-1 .. 0.  EXACT_TOP applies the exact rule to
// sub-stage KK-1 (global stage m = n/2); FOLD folds n^-1 into sub-stage 0
// (global stage m = 1, root index 1) and leaves canonical outputs.
template <int KK, int G0, bool EXACT_TOP, bool FOLD, int NV>
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
          gs_first_sd(x, y, t, s, d);
        } else {
          s = x + y;
          d = x - y + t.q2;
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
            gs_first_sd(x, y, t, s, d);
            x = csub(s, t.q2);
            y = shoup_lazy(d, w.x, w.y, t.q);
          } else {
            gs_bfly(x, y, w.x, w.y, t.q, t.q2);
          }
        }
      });
    }
  });
}

// ---------------------------------------------------------------------------
// Pass schedule for n = 2^LOGN held by T = n/E threads.

constexpr int ilog2c(int x) { return x <= 1 ? 0 : 1 + ilog2c(x >> 1); }

template <int LOGN_, int E_>
struct Shape {
  static constexpr int LOGN = LOGN_, E = E_;
  static constexpr int N = 1 << LOGN, T = N / E, K = ilog2c(E);
  static constexpr int LASTK = 4;               // last pass: groups of 16 consecutive words
  static constexpr int HEAD = LOGN - LASTK;     // stages before the last pass
  static constexpr int NHEAD = (HEAD + K - 1) / K;
  static constexpr int FIRSTK = HEAD - K * (NHEAD - 1);
  static constexpr int SMEM_BYTES = (N + N / 16) * 8;
  static_assert(E >= 16 && HEAD >= 1 && T >= 1, "unsupported shape");
  template <int P>
  static constexpr int s0() { return P == 0 ? 0 : FIRSTK + K * (P - 1); }
  template <int P>
  static constexpr int kk() { return P == 0 ? FIRSTK : K; }
};

// Thread-to-group map of a pass starting at stage S0 with KK stages: group
// g = tid + i*T has block b = g / TMIN and offset o = g % TMIN; its words sit
// at b*(n >> S0) + o + j*TMIN.
template <class S, int S0, int KK>
__device__ __forceinline__ void smem_load(u64 (&v)[S::E], const u64* sm) {
  constexpr int G = S::E >> KK, TMIN = S::N >> (S0 + KK), BLK = S::N >> S0;
  static_for<0, G>([&](auto ic) {
    constexpr int i = decltype(ic)::value;
    const int g = threadIdx.x + i * S::T;
    const int a0 = (g / TMIN) * BLK + (g % TMIN);
#pragma unroll
    for (int j = 0; j < (1 << KK); j++) v[i * (1 << KK) + j] = sm[pad(a0 + j * TMIN)];
  });
}

template <class S, int S0, int KK>
__device__ __forceinline__ void smem_store(const u64 (&v)[S::E], u64* sm) {
  constexpr int G = S::E >> KK, TMIN = S::N >> (S0 + KK), BLK = S::N >> S0;
  static_for<0, G>([&](auto ic) {
    constexpr int i = decltype(ic)::value;
    const int g = threadIdx.x + i * S::T;
    const int a0 = (g / TMIN) * BLK + (g % TMIN);
#pragma unroll
    for (int j = 0; j < (1 << KK); j++) sm[pad(a0 + j * TMIN)] = v[i * (1 << KK) + j];
  });
}

template <class S, int S0, int KK>
__device__ __forceinline__ void fwd_compute(u64 (&v)[S::E], const Tw& t, u32 tw_mult) {
  constexpr int G = S::E >> KK, TMIN = S::N >> (S0 + KK);
  static_for<0, G>([&](auto ic) {
    constexpr int i = decltype(ic)::value;
    const int g = threadIdx.x + i * S::T;
    ct_group<KK, 0, i * (1 << KK)>(v, t.fwd, tw_mult * (1u << S0) + (u32)(g / TMIN), t);
  });
}

template <class S, int S0, int KK, bool EXACT_TOP, bool FOLD>
__device__ __forceinline__ void inv_compute(u64 (&v)[S::E], const Tw& t, u32 tw_mult) {
  constexpr int G = S::E >> KK, TMIN = S::N >> (S0 + KK);
  static_for<0, G>([&](auto ic) {
    constexpr int i = decltype(ic)::value;
    const int g = threadIdx.x + i * S::T;
    gs_group<KK, i * (1 << KK), EXACT_TOP, FOLD>(v, t.inv, tw_mult * (1u << S0) + (u32)(g / TMIN), t);
  });
}

// Forward transform of the n words at `in` (stride-1) into registers: on
// return thread tid holds v[16 i + j] = out[16 (tid + i T) + j], lazy [0, 4q).
// EXACT: `in` is caller data and stage 0 of this pass is global stage 0.
template <class S, bool EXACT>
__device__ __forceinline__ void fwd_ntt(u64 (&v)[S::E], u64* sm, const u64* __restrict__ in,
                                        const Tw& t, u32 tw_mult) {
  {
    constexpr int KK = S::FIRSTK, G = S::E >> KK, TMIN = S::N >> KK;
    static_for<0, G>([&](auto ic) {
      constexpr int i = decltype(ic)::value;
      const int g = threadIdx.x + i * S::T;
#pragma unroll
      for (int j = 0; j < (1 << KK); j++) v[i * (1 << KK) + j] = ld_stream(in + g + j * TMIN);
    });
    static_for<0, G>([&](auto ic) {
      constexpr int i = decltype(ic)::value;
      if constexpr (EXACT) {
        ct_group_first_exact<KK, i * (1 << KK)>(v, t);
        ct_group<KK, 1, i * (1 << KK)>(v, t.fwd, tw_mult, t);
      } else {
        ct_group<KK, 0, i * (1 << KK)>(v, t.fwd, tw_mult, t);
      }
    });
    smem_store<S, 0, KK>(v, sm);
    __syncthreads();
  }
  static_for<1, S::NHEAD>([&](auto pc) {
    constexpr int P = decltype(pc)::value;
    constexpr int S0 = S::template s0<P>(), KK = S::template kk<P>();
    smem_load<S, S0, KK>(v, sm);
    fwd_compute<S, S0, KK>(v, t, tw_mult);
    smem_store<S, S0, KK>(v, sm);
    __syncthreads();
  });
  smem_load<S, S::HEAD, S::LASTK>(v, sm);
  fwd_compute<S, S::HEAD, S::LASTK>(v, t, tw_mult);
}

// Inverse transform of register-resident input laid out as fwd_ntt leaves
// it, written to `out` (stride-1).  EXACT: the register values are caller
// data (global stage m = n/2 is sub-stage 3 of the first pass).  FOLD: this is
// the whole transform (tw_mult == 1): n^-1 is folded in, outputs canonical;
// otherwise outputs are lazy [0, 2q).
template <class S, bool EXACT, bool FOLD>
__device__ __forceinline__ void inv_ntt(u64 (&v)[S::E], u64* sm, const Tw& t, u32 tw_mult,
                                        u64* __restrict__ out) {
  inv_compute<S, S::HEAD, S::LASTK, EXACT, false>(v, t, tw_mult);
  smem_store<S, S::HEAD, S::LASTK>(v, sm);
  __syncthreads();
  static_for<1, S::NHEAD>([&](auto pc) {
    constexpr int P = S::NHEAD - decltype(pc)::value;  // NHEAD-1 .. 1
    constexpr int S0 = S::template s0<P>(), KK = S::template kk<P>();
    smem_load<S, S0, KK>(v, sm);
    inv_compute<S, S0, KK, false, false>(v, t, tw_mult);
    smem_store<S, S0, KK>(v, sm);
    __syncthreads();
  });
  {
    constexpr int KK = S::FIRSTK, G = S::E >> KK, TMIN = S::N >> KK;
    smem_load<S, 0, KK>(v, sm);
    inv_compute<S, 0, KK, false, FOLD>(v, t, tw_mult);
    static_for<0, G>([&](auto ic) {
      constexpr int i = decltype(ic)::value;
      const int g = threadIdx.x + i * S::T;
#pragma unroll
      for (int j = 0; j < (1 << KK); j++) out[g + j * TMIN] = v[i * (1 << KK) + j];
    });
  }
}

// Register groups of 16 consecutive words <-> global memory (32-byte vectors).
template <class S>
__device__ __forceinline__ void groups_load(u64 (&v)[S::E], const u64* p) {
  static_for<0, S::E / 16>([&](auto ic) {
    constexpr int i = decltype(ic)::value;
    const u64* q = p + 16 * (threadIdx.x + i * S::T);
#pragma unroll
    for (int h = 0; h < 4; h++)
      ld4(q + 4 * h, v[16 * i + 4 * h], v[16 * i + 4 * h + 1], v[16 * i + 4 * h + 2], v[16 * i + 4 * h + 3]);
  });
}

template <class S>
__device__ __forceinline__ void groups_store(const u64 (&v)[S::E], u64* p) {
  static_for<0, S::E / 16>([&](auto ic) {
    constexpr int i = decltype(ic)::value;
    u64* q = p + 16 * (threadIdx.x + i * S::T);
#pragma unroll
    for (int h = 0; h < 4; h++)
      st4(q + 4 * h, v[16 * i + 4 * h], v[16 * i + 4 * h + 1], v[16 * i + 4 * h + 2], v[16 * i + 4 * h + 3]);
  });
}

// ---------------------------------------------------------------------------
// Kernels.  Jobs come from a device array (persistent loop over
// blockIdx.x, blockIdx.x + gridDim.x, ...) or, for a single job, by value.

template <class J>
__device__ __forceinline__ J fetch_job(const J* jobs, const J& one, int jid) {
  return jobs ? jobs[jid] : one;
}

// sub_log > 0: the job is one 2^LOGN-word sub-block (index jid % 2^sub_log of
// a transform of size 2^(LOGN + sub_log)) after/before the global stages.
template <int LOGN, int E>
__global__ void __launch_bounds__((1 << LOGN) / E)
    k_ntt_fwd(const vkcu_ntt_job* __restrict__ jobs, int njobs, vkcu_ntt_job one, int sub_log) {
  using S = Shape<LOGN, E>;
  extern __shared__ u64 sm[];
  const int total = njobs << sub_log;
  for (int w = blockIdx.x; w < total; w += gridDim.x) {
    const vkcu_ntt_job job = fetch_job(jobs, one, w >> sub_log);
    const int sub = w & ((1 << sub_log) - 1);
    const Tw t = load_tw(job.tw);
    u64 v[S::E];
    const u64* in = reinterpret_cast<const u64*>(sub_log ? job.out : job.in) + ((size_t)sub << LOGN);
    if (sub_log == 0)
      fwd_ntt<S, true>(v, sm, in, t, 1u);
    else
      fwd_ntt<S, false>(v, sm, in, t, (1u << sub_log) + sub);
#pragma unroll
    for (int i = 0; i < S::E; i++) v[i] = canon4(v[i], t.q, t.q2);
    groups_store<S>(v, reinterpret_cast<u64*>(job.out) + ((size_t)sub << LOGN));
    __syncthreads();
  }
}

template <int LOGN, int E>
__global__ void __launch_bounds__((1 << LOGN) / E)
    k_ntt_inv(const vkcu_ntt_job* __restrict__ jobs, int njobs, vkcu_ntt_job one, int sub_log) {
  using S = Shape<LOGN, E>;
  extern __shared__ u64 sm[];
  const int total = njobs << sub_log;
  for (int w = blockIdx.x; w < total; w += gridDim.x) {
    const vkcu_ntt_job job = fetch_job(jobs, one, w >> sub_log);
    const int sub = w & ((1 << sub_log) - 1);
    const Tw t = load_tw(job.tw);
    u64 v[S::E];
    groups_load<S>(v, reinterpret_cast<const u64*>(job.in) + ((size_t)sub << LOGN));
    u64* out = reinterpret_cast<u64*>(job.out) + ((size_t)sub << LOGN);
    if (sub_log == 0)
      inv_ntt<S, true, true>(v, sm, t, 1u, out);
    else
      inv_ntt<S, true, false>(v, sm, t, (1u << sub_log) + sub, out);
    __syncthreads();
  }
}

// Fused c = INTT(NTT(a) . NTT(b)): NTT(b) goes to job.scratch (canonical),
// NTT(a) stays in registers, the pointwise product reads NTT(b) back at the
// same positions written by the same thread, the INTT writes c.
template <int LOGN, int E>
__global__ void __launch_bounds__((1 << LOGN) / E)
    k_polymul(const vkcu_poly_job* __restrict__ jobs, int njobs, vkcu_poly_job one) {
  using S = Shape<LOGN, E>;
  extern __shared__ u64 sm[];
  for (int w = blockIdx.x; w < njobs; w += gridDim.x) {
    const vkcu_poly_job job = fetch_job(jobs, one, w);
    const Tw t = load_tw(job.tw);
    u64* scratch = reinterpret_cast<u64*>(job.scratch);
    u64 v[S::E];
    fwd_ntt<S, true>(v, sm, reinterpret_cast<const u64*>(job.b), t, 1u);
#pragma unroll
    for (int i = 0; i < S::E; i++) v[i] = canon4(v[i], t.q, t.q2);
    groups_store<S>(v, scratch);
    __syncthreads();
    fwd_ntt<S, true>(v, sm, reinterpret_cast<const u64*>(job.a), t, 1u);
    static_for<0, S::E / 16>([&](auto ic) {
      constexpr int i = decltype(ic)::value;
      const u64* q = scratch + 16 * (threadIdx.x + i * S::T);
#pragma unroll
      for (int h = 0; h < 4; h++) {
        u64 b0, b1, b2, b3;
        ld4(q + 4 * h, b0, b1, b2, b3);
        const u64 bb[4] = {b0, b1, b2, b3};
#pragma unroll
        for (int e = 0; e < 4; e++) {
          u64& x = v[16 * i + 4 * h + e];
          x = barrett_mul_lazy(canon4(x, t.q, t.q2), bb[e], t.q, t.q2, t.mu, t.qbits);
        }
      }
    });
    inv_ntt<S, false, true>(v, sm, t, 1u, reinterpret_cast<u64*>(job.c));
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Simple kernels: one CTA per job, whole vector in shared memory, one
// radix-2 stage per __syncthreads.  Used for n < 256, for n <= 2^14 when a
// pointer is not 32-byte aligned, and as an independent cross-check.

__global__ void k_ntt_fwd_simple(const vkcu_ntt_job* __restrict__ jobs, int njobs, vkcu_ntt_job one,
                                 int log_n) {
  extern __shared__ u64 sm[];
  const int n = 1 << log_n;
  for (int w = blockIdx.x; w < njobs; w += gridDim.x) {
    const vkcu_ntt_job job = fetch_job(jobs, one, w);
    const Tw t = load_tw(job.tw);
    const u64* in = reinterpret_cast<const u64*>(job.in);
    for (int i = threadIdx.x; i < n; i += blockDim.x) sm[i] = in[i];
    __syncthreads();
    for (int s = 0; s < log_n; s++) {
      const int half = n >> (s + 1);
      for (int p = threadIdx.x; p < n / 2; p += blockDim.x) {
        const int blk = p >> (log_n - 1 - s);
        const int x = blk * 2 * half + (p & (half - 1));
        const ulonglong2 wt = ld_tw(t.fwd + (1 << s) + blk);
        if (s == 0)
          ct_first(sm[x], sm[x + half], wt.x, wt.y, t);
        else
          ct_bfly(sm[x], sm[x + half], wt.x, wt.y, t.q, t.q2);
      }
      __syncthreads();
    }
    u64* out = reinterpret_cast<u64*>(job.out);
    for (int i = threadIdx.x; i < n; i += blockDim.x) out[i] = canon4(sm[i], t.q, t.q2);
    __syncthreads();
  }
}

__global__ void k_ntt_inv_simple(const vkcu_ntt_job* __restrict__ jobs, int njobs, vkcu_ntt_job one,
                                 int log_n) {
  extern __shared__ u64 sm[];
  const int n = 1 << log_n;
  for (int w = blockIdx.x; w < njobs; w += gridDim.x) {
    const vkcu_ntt_job job = fetch_job(jobs, one, w);
    const Tw t = load_tw(job.tw);
    const u64* in = reinterpret_cast<const u64*>(job.in);
    for (int i = threadIdx.x; i < n; i += blockDim.x) sm[i] = in[i];
    __syncthreads();
    for (int s = log_n - 1; s >= 0; s--) {
      const int half = n >> (s + 1);
      for (int p = threadIdx.x; p < n / 2; p += blockDim.x) {
        const int blk = p >> (log_n - 1 - s);
        const int x = blk * 2 * half + (p & (half - 1));
        u64 sum, dif;
        if (s == log_n - 1) {
          gs_first_sd(sm[x], sm[x + half], t, sum, dif);
        } else {
          sum = sm[x] + sm[x + half];
          dif = sm[x] - sm[x + half] + t.q2;
        }
        if (s == 0) {
          sm[x] = shoup(sum, t.ninv, t.ninv_s, t.q);
          sm[x + half] = shoup(dif, t.w1ninv, t.w1ninv_s, t.q);
        } else {
          const ulonglong2 wt = ld_tw(t.inv + (1 << s) + blk);
          sm[x] = csub(sum, t.q2);
          sm[x + half] = shoup_lazy(dif, wt.x, wt.y, t.q);
        }
      }
      __syncthreads();
    }
    u64* out = reinterpret_cast<u64*>(job.out);
    for (int i = threadIdx.x; i < n; i += blockDim.x) out[i] = sm[i];
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Global-memory passes for n > 2^14 (KK = log2(n) - 14 stages, KK <= 4).
// Forward: global stages 0 .. KK-1, in -> out, lazy [0, 4q).  Each thread
// owns one group of 2^KK words at stride n / 2^KK (coalesced).
template <int KK>
__global__ void k_fwd_head_global(const vkcu_ntt_job* __restrict__ jobs, int njobs, vkcu_ntt_job one,
                                  int log_n) {
  const int groups = 1 << (log_n - KK);
  const long total = (long)njobs * groups;
  for (long w = blockIdx.x * (long)blockDim.x + threadIdx.x; w < total; w += (long)gridDim.x * blockDim.x) {
    const vkcu_ntt_job job = fetch_job(jobs, one, (int)(w / groups));
    const int o = (int)(w % groups);
    const Tw t = load_tw(job.tw);
    const u64* in = reinterpret_cast<const u64*>(job.in);
    u64 v[1 << KK];
#pragma unroll
    for (int j = 0; j < (1 << KK); j++) v[j] = ld_stream(in + o + (size_t)j * groups);
    ct_group_first_exact<KK, 0>(v, t);
    ct_group<KK, 1, 0>(v, t.fwd, 1u, t);
    u64* out = reinterpret_cast<u64*>(job.out);
#pragma unroll
    for (int j = 0; j < (1 << KK); j++) out[o + (size_t)j * groups] = v[j];
  }
}

// Inverse: global stages KK-1 .. 0 on `out` in place (after the sub-block
// kernels), with n^-1 folded in, canonical output.
template <int KK>
__global__ void k_inv_tail_global(const vkcu_ntt_job* __restrict__ jobs, int njobs, vkcu_ntt_job one,
                                  int log_n) {
  const int groups = 1 << (log_n - KK);
  const long total = (long)njobs * groups;
  for (long w = blockIdx.x * (long)blockDim.x + threadIdx.x; w < total; w += (long)gridDim.x * blockDim.x) {
    const vkcu_ntt_job job = fetch_job(jobs, one, (int)(w / groups));
    const int o = (int)(w % groups);
    const Tw t = load_tw(job.tw);
    u64* out = reinterpret_cast<u64*>(job.out);
    u64 v[1 << KK];
#pragma unroll
    for (int j = 0; j < (1 << KK); j++) v[j] = out[o + (size_t)j * groups];
    gs_group<KK, 0, false, true>(v, t.inv, 1u, t);
#pragma unroll
    for (int j = 0; j < (1 << KK); j++) out[o + (size_t)j * groups] = v[j];
  }
}

// ---------------------------------------------------------------------------
// Host-side launch helpers.

template <class K>
static int smem_attr(K kernel, int bytes) {
  return (int)cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

template <class K>
static int grid_for(K kernel, int threads, int smem, long work, int sms) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  const long cap = (long)per_sm * (sms > 0 ? sms : 1);
  return (int)(work < cap ? work : cap);
}

template <int LOGN, int E>
static int launch_fwd(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int sub_log,
                      int sms) {
  using S = Shape<LOGN, E>;
  auto kern = k_ntt_fwd<LOGN, E>;
  if (int e = smem_attr(kern, S::SMEM_BYTES)) return e;
  const int grid = grid_for(kern, S::T, S::SMEM_BYTES, (long)njobs << sub_log, sms);
  kern<<<grid, S::T, S::SMEM_BYTES, st>>>(jobs, njobs, one, sub_log);
  vkcu_count_launches(1);
  return (int)cudaGetLastError();
}

template <int LOGN, int E>
static int launch_inv(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int sub_log,
                      int sms) {
  using S = Shape<LOGN, E>;
  auto kern = k_ntt_inv<LOGN, E>;
  if (int e = smem_attr(kern, S::SMEM_BYTES)) return e;
  const int grid = grid_for(kern, S::T, S::SMEM_BYTES, (long)njobs << sub_log, sms);
  kern<<<grid, S::T, S::SMEM_BYTES, st>>>(jobs, njobs, one, sub_log);
  vkcu_count_launches(1);
  return (int)cudaGetLastError();
}

template <int LOGN, int E>
static int launch_poly(cudaStream_t st, const vkcu_poly_job* jobs, int njobs, const vkcu_poly_job& one, int sms) {
  using S = Shape<LOGN, E>;
  auto kern = k_polymul<LOGN, E>;
  if (int e = smem_attr(kern, S::SMEM_BYTES)) return e;
  const int grid = grid_for(kern, S::T, S::SMEM_BYTES, njobs, sms);
  kern<<<grid, S::T, S::SMEM_BYTES, st>>>(jobs, njobs, one);
  vkcu_count_launches(1);
  return (int)cudaGetLastError();
}

static constexpr int kMaxFused = 14;

// Dispatch over log_n for the CTA kernels.
#define VK_FOR_LOGN(X)                       \
  switch (log_n) {                           \
    case 8: return X(8, 16);                 \
    case 9: return X(9, 16);                 \
    case 10: return X(10, 16);               \
    case 11: return X(11, 16);               \
    case 12: return X(12, 16);               \
    case 13: return X(13, 32);               \
    case 14: return X(14, 32);               \
    default: return (int)cudaErrorInvalidValue; \
  }

static int fwd_cta(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int log_n,
                   int sub_log, int sms) {
#define X(L, E) launch_fwd<L, E>(st, jobs, njobs, one, sub_log, sms)
  VK_FOR_LOGN(X)
#undef X
}

static int inv_cta(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int log_n,
                   int sub_log, int sms) {
#define X(L, E) launch_inv<L, E>(st, jobs, njobs, one, sub_log, sms)
  VK_FOR_LOGN(X)
#undef X
}

static int poly_cta(cudaStream_t st, const vkcu_poly_job* jobs, int njobs, const vkcu_poly_job& one, int log_n,
                    int sms) {
#define X(L, E) launch_poly<L, E>(st, jobs, njobs, one, sms)
  VK_FOR_LOGN(X)
#undef X
}

static bool aligned32(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 31) == 0; }

static int simple(cudaStream_t st, bool inverse, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one,
                  int log_n, int sms) {
  const int n = 1 << log_n;
  const int threads = n / 2 < 32 ? 32 : (n / 2 > 512 ? 512 : n / 2);
  const int smem = n * 8;
  auto kern = inverse ? k_ntt_inv_simple : k_ntt_fwd_simple;
  if (int e = smem_attr(kern, smem)) return e;
  const int grid = grid_for(kern, threads, smem, njobs, sms);
  kern<<<grid, threads, smem, st>>>(jobs, njobs, one, log_n);
  vkcu_count_launches(1);
  return (int)cudaGetLastError();
}

template <bool INV>
static int global_pass(cudaStream_t st, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one, int log_n,
                       int kk, int sms) {
  const long work = (long)njobs << (log_n - kk);
  const int threads = 256;
  long blocks = (work + threads - 1) / threads;
  const long cap = (long)sms * 8;
  if (blocks > cap) blocks = cap;
  switch (kk) {
#define G(K)                                                                                \
  case K:                                                                                   \
    if (INV)                                                                                \
      k_inv_tail_global<K><<<(int)blocks, threads, 0, st>>>(jobs, njobs, one, log_n);       \
    else                                                                                    \
      k_fwd_head_global<K><<<(int)blocks, threads, 0, st>>>(jobs, njobs, one, log_n);       \
    break;
    G(1)
    G(2)
    G(3)
    G(4)
#undef G
    default:
      return (int)cudaErrorInvalidValue;
  }
  vkcu_count_launches(1);
  return (int)cudaGetLastError();
}

}  // namespace vk

using namespace vk;

extern "C" uint32_t vkcu_max_fused_log_n(void) { return kMaxFused; }

static bool jobs_aligned(const vkcu_ntt_job* jobs, const vkcu_ntt_job* one) {
  // Device job arrays are built by the library with aligned vectors; a single
  // job is checked here.
  return jobs != nullptr || (aligned32(one->in) && aligned32(one->out));
}

extern "C" int vkcu_ntt_forward(void* stream, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job* one,
                                uint32_t log_n, int sms) {
  cudaStream_t st = (cudaStream_t)stream;
  const vkcu_ntt_job o = one ? *one : vkcu_ntt_job{};
  if (log_n < 1 || njobs < 1) return (int)cudaErrorInvalidValue;
  if (log_n < 8 || (log_n <= (uint32_t)kMaxFused && !jobs_aligned(jobs, one)))
    return simple(st, false, jobs, njobs, o, (int)log_n, sms);
  if (log_n <= (uint32_t)kMaxFused) return fwd_cta(st, jobs, njobs, o, (int)log_n, 0, sms);
  const int kk = (int)log_n - kMaxFused;
  if (kk > 4) return (int)cudaErrorInvalidValue;
  if (int e = global_pass<false>(st, jobs, njobs, o, (int)log_n, kk, sms)) return e;
  return fwd_cta(st, jobs, njobs, o, kMaxFused, kk, sms);
}

extern "C" int vkcu_ntt_inverse(void* stream, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job* one,
                                uint32_t log_n, int sms) {
  cudaStream_t st = (cudaStream_t)stream;
  const vkcu_ntt_job o = one ? *one : vkcu_ntt_job{};
  if (log_n < 1 || njobs < 1) return (int)cudaErrorInvalidValue;
  if (log_n < 8 || (log_n <= (uint32_t)kMaxFused && !jobs_aligned(jobs, one)))
    return simple(st, true, jobs, njobs, o, (int)log_n, sms);
  if (log_n <= (uint32_t)kMaxFused) return inv_cta(st, jobs, njobs, o, (int)log_n, 0, sms);
  const int kk = (int)log_n - kMaxFused;
  if (kk > 4) return (int)cudaErrorInvalidValue;
  if (int e = inv_cta(st, jobs, njobs, o, kMaxFused, kk, sms)) return e;
  return global_pass<true>(st, jobs, njobs, o, (int)log_n, kk, sms);
}

extern "C" int vkcu_polymul(void* stream, const vkcu_poly_job* jobs, int njobs, const vkcu_poly_job* one,
                            uint32_t log_n, int sms) {
  cudaStream_t st = (cudaStream_t)stream;
  const vkcu_poly_job o = one ? *one : vkcu_poly_job{};
  if (log_n < 8 || log_n > (uint32_t)kMaxFused || njobs < 1) return (int)cudaErrorInvalidValue;
  return poly_cta(st, jobs, njobs, o, (int)log_n, sms);
}

// Pointwise step of a composed polymul: c = c * scratch mod q over njobs
// jobs of n words each (both operands canonical NTT outputs).
__global__ void k_pointwise(const vkcu_poly_job* __restrict__ jobs, int njobs, int log_n) {
  const long n = 1L << log_n;
  const long total = (long)njobs * n;
  for (long w = blockIdx.x * (long)blockDim.x + threadIdx.x; w < total; w += (long)gridDim.x * blockDim.x) {
    const vkcu_poly_job job = jobs[w >> log_n];
    const long i = w & (n - 1);
    const Tw t = load_tw(job.tw);
    u64* c = reinterpret_cast<u64*>(job.c);
    const u64 x = c[i], y = reinterpret_cast<const u64*>(job.scratch)[i];
    c[i] = csub(barrett_mul_lazy(x, y, t.q, t.q2, t.mu, t.qbits), t.q);
  }
}

extern "C" int vkcu_pointwise(void* stream, const vkcu_poly_job* jobs, int njobs, uint32_t log_n, int sms) {
  if (njobs < 1 || !jobs) return (int)cudaErrorInvalidValue;
  const long work = (long)njobs << log_n;
  long blocks = (work + 255) / 256;
  if (blocks > (long)sms * 8) blocks = (long)sms * 8;
  k_pointwise<<<(int)blocks, 256, 0, (cudaStream_t)stream>>>(jobs, njobs, (int)log_n);
  vkcu_count_launches(1);
  return (int)cudaGetLastError();
}
