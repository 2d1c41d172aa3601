// Transform dispatch and the kernels outside the CTA-resident families:
// simple one-stage-per-barrier kernels (n < 256, unaligned operands), the
// global-memory passes of n >= 2^18, and the pointwise step of a composed
// polynomial multiply.  Every launcher takes the modulus class of its jobs
// (`wide`: 2^62 <= q < 2^63).  The CTA-resident kernels are in
// ntt_core.cuh with one launcher per family (ntt_fwd.cu, ntt_inv.cu,
// ntt_poly.cu).
#include "elem_ops.cuh"
#include "ntt_core.cuh"

namespace vk {

// ---------------------------------------------------------------------------
// Simple kernels: one CTA per job, whole vector in shared memory, one
// radix-2 stage per __syncthreads.  Used for n < 256, for n <= 2^14 when a
// pointer is not 32-byte aligned, and as an independent cross-check.

template <class M>
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
          ct_first<M>(sm[x], sm[x + half], wt.x, wt.y, t);
        else
          M::ct(sm[x], sm[x + half], wt.x, wt.y, t);
      }
      __syncthreads();
    }
    u64* out = reinterpret_cast<u64*>(job.out);
    for (int i = threadIdx.x; i < n; i += blockDim.x) out[i] = M::canon(sm[i], t);
    __syncthreads();
  }
}

template <class M>
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
        if (s == log_n - 1)
          gs_first_sd<M>(sm[x], sm[x + half], t, sum, dif);
        else
          M::sd(sm[x], sm[x + half], t, sum, dif);
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
// Global-memory passes for n >= 2^18: the first (forward) or last (inverse)
// log2(n) - 14 stages run over HBM in passes of KK <= 4 stages each, and
// one CTA-resident kernel runs the other 14 stages on every 2^14-word
// sub-block (sub-block r uses twiddle multiplier 2^(log2 n - 14) + r).  A
// pass starting at stage s0 gives each thread one radix-2^KK group: the
// 2^KK words at stride t = n >> (s0 + KK) inside one block of stage s0
// (blocks of n >> s0 words), twiddle base 2^s0 + block (root index m + block
// of the reference's stage loop, src/vector.c:536-566).  Consecutive threads
// take consecutive offsets, so every load and store is coalesced.

// Forward: stages s0 .. s0 + KK - 1, in -> out, forward-lazy; stage 0 takes
// the reference's exact first-stage rule; the last pass (handoff) leaves
// words below the sub-block kernels' first-stage fast-path bound.
template <int KK, class M>
__global__ void k_fwd_global(const vkcu_ntt_job* __restrict__ jobs, int njobs, vkcu_ntt_job one, int log_n, int s0,
                             int handoff) {
  const int lt = log_n - s0 - KK;  // log2 of the stride
  const long groups = 1L << (log_n - KK);
  const long total = (long)njobs * groups;
  for (long w = blockIdx.x * (long)blockDim.x + threadIdx.x; w < total; w += (long)gridDim.x * blockDim.x) {
    const vkcu_ntt_job job = fetch_job(jobs, one, (int)(w >> (log_n - KK)));
    const long g = w & (groups - 1);
    const long blk = g >> lt;
    const size_t first = ((size_t)blk << (log_n - s0)) | (size_t)(g & ((1L << lt) - 1));
    const size_t st = (size_t)1 << lt;
    const Tw t = load_tw(job.tw);
    const u64* in = reinterpret_cast<const u64*>(s0 ? job.out : job.in);
    u64 v[1 << KK];
#pragma unroll
    for (int j = 0; j < (1 << KK); j++) v[j] = ld_stream(in + first + j * st);
    const u32 base = (1u << s0) + (u32)blk;
    if (s0 == 0) {
      const ulonglong2 w0 = ld_tw(t.fwd + 1);
#pragma unroll
      for (int jj = 0; jj < (1 << (KK - 1)); jj++) ct_first<M>(v[jj], v[jj + (1 << (KK - 1))], w0.x, w0.y, t);
      ct_group<M, KK, 1, 0>(v, t.fwd, base, t);
    } else {
      ct_group<M, KK, 0, 0>(v, t.fwd, base, t);
    }
    u64* out = reinterpret_cast<u64*>(job.out);
#pragma unroll
    for (int j = 0; j < (1 << KK); j++) out[first + j * st] = handoff ? M::handoff(v[j], t) : v[j];
  }
}

// Inverse: stages s0 + KK - 1 .. s0 on `out` in place (after the sub-block
// kernels, which leave inverse-lazy words); the pass with s0 = 0 folds n^-1
// into stage 0 and writes canonical words.
template <int KK, class M>
__global__ void k_inv_global(const vkcu_ntt_job* __restrict__ jobs, int njobs, vkcu_ntt_job one, int log_n, int s0) {
  const int lt = log_n - s0 - KK;
  const long groups = 1L << (log_n - KK);
  const long total = (long)njobs * groups;
  for (long w = blockIdx.x * (long)blockDim.x + threadIdx.x; w < total; w += (long)gridDim.x * blockDim.x) {
    const vkcu_ntt_job job = fetch_job(jobs, one, (int)(w >> (log_n - KK)));
    const long g = w & (groups - 1);
    const long blk = g >> lt;
    const size_t first = ((size_t)blk << (log_n - s0)) | (size_t)(g & ((1L << lt) - 1));
    const size_t st = (size_t)1 << lt;
    const Tw t = load_tw(job.tw);
    u64* out = reinterpret_cast<u64*>(job.out);
    u64 v[1 << KK];
#pragma unroll
    for (int j = 0; j < (1 << KK); j++) v[j] = out[first + j * st];
    const u32 base = (1u << s0) + (u32)blk;
    if (s0 == 0)
      gs_group<M, KK, 0, false, true>(v, t.inv, base, t);
    else
      gs_group<M, KK, 0, false, false>(v, t.inv, base, t);
#pragma unroll
    for (int j = 0; j < (1 << KK); j++) out[first + j * st] = v[j];
  }
}

static constexpr int kMaxCta = 14;      // one CTA per transform
static constexpr int kMaxCluster = 17;  // one cluster of up to 8 CTAs
static constexpr int kMaxLogN = 26;     // global passes + 2^14-word sub-blocks

static bool aligned32(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 31) == 0; }

template <class M>
static int simple(cudaStream_t st, bool inverse, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one,
                  int log_n, int sms) {
  const int n = 1 << log_n;
  const int threads = n / 2 < 32 ? 32 : (n / 2 > 512 ? 512 : n / 2);
  const int smem = n * 8;
  auto kern = inverse ? k_ntt_inv_simple<M> : k_ntt_fwd_simple<M>;
  // threads and shared memory depend on n: one occupancy per direction and
  // degree; the kernel's shared-memory limit is the largest n (2^14) always
  static KernelSetup setups[2][kMaxCta + 1];
  int per_sm = 1;
  if (int e = setup_cta(kern, threads, smem, setups[inverse ? 1 : 0][log_n], &per_sm, (1 << kMaxCta) * 8)) return e;
  const int grid = grid_from(per_sm, njobs, sms);
  kern<<<grid, threads, smem, st>>>(jobs, njobs, one, log_n);
  vkcu_count_launches(1);
  return (int)cudaGetLastError();
}

// Stages of the global pass p (0-based, in forward order) for log_n: the
// log_n - 14 global stages split into as few passes of <= 4 stages as
// possible, sizes as equal as possible (2^21: 4 + 3).
static int global_passes(int log_n) { return (log_n - kMaxCta + 3) / 4; }
static void global_split(int log_n, int p, int* s0, int* kk) {
  const int g = log_n - kMaxCta, np = global_passes(log_n), small = g / np, big = g % np;
  *s0 = p * small + (p < big ? p : big);
  *kk = small + (p < big ? 1 : 0);
}

template <class M>
static int global_pass(cudaStream_t st, bool inverse, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one,
                       int log_n, int s0, int kk, int handoff, int sms) {
  const long work = (long)njobs << (log_n - kk);
  const int threads = 256;
  long blocks = (work + threads - 1) / threads;
  const long cap = (long)sms * 8;
  if (blocks > cap) blocks = cap;
  switch (kk) {
#define G(K)                                                                                          \
  case K:                                                                                             \
    if (inverse)                                                                                      \
      k_inv_global<K, M><<<(int)blocks, threads, 0, st>>>(jobs, njobs, one, log_n, s0);               \
    else                                                                                              \
      k_fwd_global<K, M><<<(int)blocks, threads, 0, st>>>(jobs, njobs, one, log_n, s0, handoff);      \
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

extern "C" uint32_t vkcu_max_fused_log_n(void) { return kMaxCluster; }
extern "C" uint32_t vkcu_max_log_n(void) { return kMaxLogN; }

static bool jobs_aligned(const vkcu_ntt_job* jobs, const vkcu_ntt_job* one) {
  // Device job arrays are built by the library with aligned vectors; a single
  // job is checked here.
  return jobs != nullptr || (aligned32(one->in) && aligned32(one->out));
}

// Few jobs of n = 2^12 .. 2^16 (at most one per 8 SMs, e.g. a single call):
// each runs on a cluster of 8 CTAs with 2^9 .. 2^13-word sub-blocks instead
// of one CTA (n <= 2^14) or a cluster of 2 / 4 CTAs (n = 2^15 / 2^16), so it
// uses 8 SMs.  Tuning entry (family 3, log_n 1) = 1 turns this off.
// Cluster size (log2) for a few jobs of n = 2^12 .. 2^16, 0 for none: 8
// CTAs when there is at most one job per 8 SMs; 16 for a single call (one
// job passed by value) of n >= 2^14 (tuning entry (3, 3) = 1 keeps it on 8).
// Batches and server micro-batches keep 8: their classes run beside other
// kernels, and a 16-CTA cluster can only start once 16 SMs of one GPC are
// free at the same time.
static int split_small(int njobs, uint32_t log_n, int sms, bool single) {
  if (log_n < 12 || log_n > 16 || vkh_variant(3, 1) != 0) return 0;
  if (single && log_n >= 14 && (long)njobs * 16 <= (long)sms && vkh_variant(3, 3) == 0) return 4;
  return (long)njobs * 8 <= (long)sms ? 3 : 0;
}

extern "C" int vkcu_ntt_forward(void* stream, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job* one,
                                uint32_t log_n, int wide, int sms) {
  cudaStream_t st = (cudaStream_t)stream;
  const vkcu_ntt_job o = one ? *one : vkcu_ntt_job{};
  if (log_n < 1 || log_n > (uint32_t)kMaxLogN || njobs < 1) return (int)cudaErrorInvalidValue;
  const bool aligned = jobs_aligned(jobs, one);
  if (log_n < 8 || (log_n <= (uint32_t)kMaxCta && !aligned))
    return wide ? simple<Mod63>(st, false, jobs, njobs, o, (int)log_n, sms)
                : simple<Mod62>(st, false, jobs, njobs, o, (int)log_n, sms);
  if (!aligned) return (int)cudaErrorMisalignedAddress;
  if (wide) {
    if (log_n <= (uint32_t)kMaxCta) return fwd_cta_wide(st, jobs, njobs, o, (int)log_n, 0, sms);
    if (log_n <= (uint32_t)kMaxCluster) return fwd_cluster_wide(st, jobs, njobs, o, (int)log_n - kMaxCta);
  } else {
    if (const int lc = split_small(njobs, log_n, sms, jobs == nullptr)) {
      const int e = fwd_cluster(st, jobs, njobs, o, lc, (int)log_n - lc);
      // a GPU that cannot host 16-CTA clusters: the set-up refuses before any launch
      return e == (int)cudaErrorInvalidConfiguration && lc == 4 ? fwd_cluster(st, jobs, njobs, o, 3, (int)log_n - 3)
                                                                : e;
    }
    if (log_n <= (uint32_t)kMaxCta) return fwd_cta(st, jobs, njobs, o, (int)log_n, 0, sms, vkh_variant_jobs(1, (int)log_n, njobs, sms));
    if (log_n <= (uint32_t)kMaxCluster) return fwd_cluster(st, jobs, njobs, o, (int)log_n - kMaxCta, kMaxCta);
  }
  const int np = global_passes((int)log_n);
  for (int p = 0; p < np; p++) {
    int s0, kk;
    global_split((int)log_n, p, &s0, &kk);
    const int e = wide ? global_pass<Mod63>(st, false, jobs, njobs, o, (int)log_n, s0, kk, p == np - 1, sms)
                       : global_pass<Mod62>(st, false, jobs, njobs, o, (int)log_n, s0, kk, p == np - 1, sms);
    if (e) return e;
  }
  const int sub_log = (int)log_n - kMaxCta;
  return wide ? fwd_cta_wide(st, jobs, njobs, o, kMaxCta, sub_log, sms)
              : fwd_cta(st, jobs, njobs, o, kMaxCta, sub_log, sms, vkh_variant_jobs(1, kMaxCta, (long)njobs << sub_log, sms));
}

static bool has_lift(const vkcu_lift* lift) { return lift && lift->count > 0; }

extern "C" int vkcu_ntt_inverse_lift(void* stream, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job* one,
                                     uint32_t log_n, int wide, int sms, const vkcu_lift* lift) {
  cudaStream_t st = (cudaStream_t)stream;
  const vkcu_ntt_job o = one ? *one : vkcu_ntt_job{};
  if (log_n < 1 || log_n > (uint32_t)kMaxLogN || njobs < 1) return (int)cudaErrorInvalidValue;
  if (has_lift(lift) && lift->count > VKCU_MAX_LIFT) return (int)cudaErrorInvalidValue;
  const bool aligned = jobs_aligned(jobs, one);
  const bool lifted = has_lift(lift);
  const vkcu_lift* lp = lifted ? lift : nullptr;
  int e;
  if (log_n < 8 || (log_n <= (uint32_t)kMaxCta && !aligned)) {
    e = wide ? simple<Mod63>(st, true, jobs, njobs, o, (int)log_n, sms)
             : simple<Mod62>(st, true, jobs, njobs, o, (int)log_n, sms);
  } else if (!aligned) {
    return (int)cudaErrorMisalignedAddress;
  } else if (wide && log_n <= (uint32_t)kMaxCta) {
    return inv_cta_wide(st, jobs, njobs, o, (int)log_n, 0, sms, lp);
  } else if (wide && log_n <= (uint32_t)kMaxCluster) {
    return inv_cluster_wide(st, jobs, njobs, o, (int)log_n - kMaxCta, lp);
  } else if (!wide && split_small(njobs, log_n, sms, jobs == nullptr)) {
    const int lc = split_small(njobs, log_n, sms, jobs == nullptr);
    const int e = inv_cluster(st, jobs, njobs, o, lc, (int)log_n - lc, lp);
    return e == (int)cudaErrorInvalidConfiguration && lc == 4 ? inv_cluster(st, jobs, njobs, o, 3, (int)log_n - 3, lp)
                                                              : e;
  } else if (!wide && log_n <= (uint32_t)kMaxCta) {
    if (lifted) return inv_cta_lift(st, jobs, njobs, o, (int)log_n, sms, *lift);
    return inv_cta(st, jobs, njobs, o, (int)log_n, 0, sms, vkh_variant_jobs(2, (int)log_n, njobs, sms));
  } else if (!wide && log_n <= (uint32_t)kMaxCluster) {
    return inv_cluster(st, jobs, njobs, o, (int)log_n - kMaxCta, kMaxCta, lp);
  } else {
    const int sub_log = (int)log_n - kMaxCta;
    e = wide ? inv_cta_wide(st, jobs, njobs, o, kMaxCta, sub_log, sms, nullptr)
             : inv_cta(st, jobs, njobs, o, kMaxCta, sub_log, sms, vkh_variant_jobs(2, kMaxCta, (long)njobs << sub_log, sms));
    for (int p = global_passes((int)log_n) - 1; !e && p >= 0; p--) {
      int s0, kk;
      global_split((int)log_n, p, &s0, &kk);
      e = wide ? global_pass<Mod63>(st, true, jobs, njobs, o, (int)log_n, s0, kk, 0, sms)
               : global_pass<Mod62>(st, true, jobs, njobs, o, (int)log_n, s0, kk, 0, sms);
    }
  }
  // the multi-launch paths take the epilogue as one more element-wise launch
  if (!e && lifted) e = vkcu_lift_jobs(stream, jobs, njobs, one, log_n, sms, lift);
  return e;
}

extern "C" int vkcu_ntt_inverse(void* stream, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job* one,
                                uint32_t log_n, int wide, int sms) {
  return vkcu_ntt_inverse_lift(stream, jobs, njobs, one, log_n, wide, sms, nullptr);
}

extern "C" int vkcu_polymul_lift(void* stream, const vkcu_poly_job* jobs, int njobs, const vkcu_poly_job* one,
                                 uint32_t log_n, int wide, int sms, const vkcu_lift* lift, int b_ntt) {
  cudaStream_t st = (cudaStream_t)stream;
  const vkcu_poly_job o = one ? *one : vkcu_poly_job{};
  if (log_n < 8 || log_n > (uint32_t)kMaxCluster || njobs < 1) return (int)cudaErrorInvalidValue;
  if (has_lift(lift) && lift->count > VKCU_MAX_LIFT) return (int)cudaErrorInvalidValue;
  static const vkcu_lift kNoSteps{};  // the epilogue instantiations with nothing to apply
  const vkcu_lift* lp = has_lift(lift) ? lift : b_ntt ? &kNoSteps : nullptr;
  if (wide) {
    if (log_n <= (uint32_t)kMaxCta) return poly_cta_wide(st, jobs, njobs, o, (int)log_n, sms, lp);
    return poly_cluster_wide(st, jobs, njobs, o, (int)log_n - kMaxCta, lp);
  }
  if (const int lc = split_small(njobs, log_n, sms, jobs == nullptr)) {
    const int e = poly_cluster(st, jobs, njobs, o, lc, (int)log_n - lc, lp);
    return e == (int)cudaErrorInvalidConfiguration && lc == 4 ? poly_cluster(st, jobs, njobs, o, 3, (int)log_n - 3, lp)
                                                              : e;
  }
  if (log_n <= (uint32_t)kMaxCta) {
    if (lp) return poly_cta_lift(st, jobs, njobs, o, (int)log_n, sms, vkh_variant_jobs(0, (int)log_n, njobs, sms), *lp);
    return poly_cta(st, jobs, njobs, o, (int)log_n, sms, vkh_variant_jobs(0, (int)log_n, njobs, sms));
  }
  return poly_cluster(st, jobs, njobs, o, (int)log_n - kMaxCta, kMaxCta, lp);
}

extern "C" int vkcu_polymul(void* stream, const vkcu_poly_job* jobs, int njobs, const vkcu_poly_job* one,
                            uint32_t log_n, int wide, int sms) {
  return vkcu_polymul_lift(stream, jobs, njobs, one, log_n, wide, sms, nullptr, 0);
}

// The epilogue as its own element-wise pass: over `len` words at p, or over
// the n output words of each job (q from the job's twiddle set).  Words move
// as 16-byte pairs, two pairs per thread per round, software pipelined (the
// next round's loads are issued before this round's four words walk the
// step list together and are stored); a word before the first 16-byte
// boundary and an odd last word are done alone, and a job whose output is
// not 16-byte aligned word by word.  The grid is one wave of resident blocks.
__device__ __forceinline__ void lift_pairs(u64* __restrict__ a, long lo, long hi, long stride, const LiftRun& lr) {
  ulonglong2 x0 = make_ulonglong2(0, 0), x1 = x0;
  if (lo < hi) x0 = ld2(a + 2 * lo);
  if (lo + stride < hi) x1 = ld2(a + 2 * (lo + stride));
  for (long p = lo; p < hi; p += 2 * stride) {
    const long n0 = p + 2 * stride, n1 = n0 + stride;
    ulonglong2 y0 = x0, y1 = x1;
    if (n0 < hi) y0 = ld2(a + 2 * n0);
    if (n1 < hi) y1 = ld2(a + 2 * n1);
    u64 v[4] = {x0.x, x0.y, x1.x, x1.y};
    lr.apply(v);
    st2(a + 2 * p, v[0], v[1]);
    if (p + stride < hi) st2(a + 2 * (p + stride), v[2], v[3]);
    x0 = y0;
    x1 = y1;
  }
}

__global__ void __launch_bounds__(256) k_lift_range(u64* __restrict__ p, u64 len, u64 q,
                                                    const __grid_constant__ vkcu_lift lift) {
  const LiftRun lr(&lift, q);
  const u64 head = (reinterpret_cast<uintptr_t>(p) & 15) ? 1 : 0;
  const bool first = blockIdx.x == 0 && threadIdx.x == 0;
  if (head && len && first) p[0] = lr(p[0]);
  u64* a = p + head;
  const u64 rest = len > head ? len - head : 0;
  lift_pairs(a, (long)(blockIdx.x * blockDim.x + threadIdx.x), (long)(rest >> 1), (long)gridDim.x * blockDim.x, lr);
  if ((rest & 1) && first) a[rest - 1] = lr(a[rest - 1]);
}

// Jobs of up to 2^11 words: one block per job (grid-stride over the jobs),
// blockDim sized to the job; longer jobs take k_lift_stream below.
static constexpr int kLiftSmallLog = 11;

template <class L>
__device__ __forceinline__ void lift_segment(u64* __restrict__ out, long words, const L& lr) {
  if ((reinterpret_cast<uintptr_t>(out) & 15) == 0) {
    lift_pairs(out, threadIdx.x, words >> 1, blockDim.x, lr);
    if ((words & 1) && threadIdx.x == 0) out[words - 1] = lr(out[words - 1]);
  } else {
    for (long i = threadIdx.x; i < words; i += blockDim.x) out[i] = lr(out[i]);
  }
}

__global__ void __launch_bounds__(256) k_lift_jobs(const vkcu_ntt_job* __restrict__ jobs, int njobs, vkcu_ntt_job one,
                                                   int log_n, const __grid_constant__ vkcu_lift lift) {
  for (int w = blockIdx.x; w < njobs; w += gridDim.x) {
    const vkcu_ntt_job job = fetch_job(jobs, one, w);
    const LiftRun lr(&lift, load_tw(job.tw).q);
    lift_segment(reinterpret_cast<u64*>(job.out), 1L << log_n, lr);
  }
}

// Long jobs (n >= 2^12), up to kLiftStreamJobs per launch: the jobs' words
// laid end to end are walked in 128-word warp chunks, chunk c by warp c mod W
// (W warps in the grid), so that the whole grid streams through adjacent
// memory at any time (a block per contiguous range, 608 blocks reading from
// 608 places, reached 0.71 of HBM against 0.91 so on 32 jobs of 2^20
// words); each job's output pointer and step constants are staged in shared
// memory once per block.  Two pairs per lane per chunk, the next chunk's
// loads issued before this chunk is lifted; word by word when an output is
// off the 16-byte grid.
static constexpr int kLiftStreamJobs = 256;

__global__ void __launch_bounds__(256) k_lift_stream(const vkcu_ntt_job* __restrict__ jobs, int njobs,
                                                     vkcu_ntt_job one, int log_n,
                                                     const __grid_constant__ vkcu_lift lift) {
  __shared__ u64 s_out[kLiftStreamJobs];
  __shared__ u64 s_c[kLiftStreamJobs][2 * VKCU_MAX_LIFT];
  __shared__ int s_unaligned;
  if (threadIdx.x == 0) s_unaligned = 0;
  __syncthreads();
  for (int j = threadIdx.x; j < njobs; j += blockDim.x) {
    const vkcu_ntt_job job = fetch_job(jobs, one, j);
    const LiftRun lr(&lift, load_tw(job.tw).q);
    s_out[j] = reinterpret_cast<u64>(job.out);
    if (s_out[j] & 15) atomicOr(&s_unaligned, 1);
#pragma unroll
    for (int k = 0; k < VKCU_MAX_LIFT; k++) {
      s_c[j][k] = lr.bound[k];
      s_c[j][VKCU_MAX_LIFT + k] = lr.d[k];
    }
  }
  __syncthreads();
  const int cl = log_n - 7;  // log2 of the chunks of a job
  const long chunks = (long)njobs << cl;
  const long nw = (long)gridDim.x * (blockDim.x >> 5);
  const int lane = threadIdx.x & 31;
  auto base = [&](long c) {
    return reinterpret_cast<u64*>(s_out[c >> cl]) + ((c & ((1L << cl) - 1)) << 7) + 2 * lane;
  };
  long c = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (s_unaligned) {  // an output off the 16-byte grid: word by word
    for (; c < chunks; c += nw) {
      u64* pw = base(c);
      const u64* cj = s_c[c >> cl];
      const LiftRun lr(&lift, cj, cj + VKCU_MAX_LIFT);
      pw[0] = lr(pw[0]);
      pw[1] = lr(pw[1]);
      pw[64] = lr(pw[64]);
      pw[65] = lr(pw[65]);
    }
    return;
  }
  if (c >= chunks) return;
  u64* p = base(c);
  ulonglong2 x0 = ld2(p), x1 = ld2(p + 64);
  for (; c < chunks; c += nw) {
    const long cn = c + nw;
    u64* pn = p;
    ulonglong2 y0 = x0, y1 = x1;
    if (cn < chunks) {
      pn = base(cn);
      y0 = ld2(pn);
      y1 = ld2(pn + 64);
    }
    const u64* cj = s_c[c >> cl];
    const LiftRun lr(&lift, cj, cj + VKCU_MAX_LIFT);
    u64 v[4] = {x0.x, x0.y, x1.x, x1.y};
    lr.apply(v);
    st2(p, v[0], v[1]);
    st2(p + 64, v[2], v[3]);
    p = pn;
    x0 = y0;
    x1 = y1;
  }
}

template <auto kernel>
static long resident_blocks(int sms) {
  static const int per_sm = [] {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, 256, 0) != cudaSuccess || b < 1) b = 1;
    return b;
  }();
  return (long)(sms > 0 ? sms : 1) * per_sm;
}

extern "C" int vkcu_lift_range(void* stream, uint64_t* p, uint64_t len, uint64_t q, int sms, const vkcu_lift* lift) {
  if (!has_lift(lift) || len == 0) return 0;
  if (lift->count > VKCU_MAX_LIFT) return (int)cudaErrorInvalidValue;
  long blocks = (long)((len + 1023) / 1024);  // four words per thread per round
  const long cap = resident_blocks<k_lift_range>(sms);
  if (blocks > cap) blocks = cap;
  k_lift_range<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<u64*>(p), len, q, *lift);
  vkcu_count_launches(1);
  return (int)cudaGetLastError();
}

extern "C" int vkcu_lift_jobs(void* stream, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job* one,
                              uint32_t log_n, int sms, const vkcu_lift* lift) {
  if (!has_lift(lift)) return 0;
  if (njobs < 1 || log_n > (uint32_t)kMaxLogN || lift->count > VKCU_MAX_LIFT) return (int)cudaErrorInvalidValue;
  const vkcu_ntt_job o = one ? *one : vkcu_ntt_job{};
  if ((int)log_n <= kLiftSmallLog) {  // one block per job, a thread per pair up to 256
    const long pairs = (1L << log_n) / 2;
    const int threads = pairs <= 32 ? 32 : pairs >= 256 ? 256 : (int)pairs;
    const long cap = (long)(sms > 0 ? sms : 1) * 16;
    const long blocks = njobs < cap ? njobs : cap;
    k_lift_jobs<<<(unsigned)blocks, threads, 0, (cudaStream_t)stream>>>(jobs, njobs, o, (int)log_n, *lift);
    vkcu_count_launches(1);
    return (int)cudaGetLastError();
  }
  // long jobs: one streaming launch per kLiftStreamJobs jobs (a single job by value: one)
  for (int g = 0; g < njobs; g += kLiftStreamJobs) {
    const int cnt = njobs - g < kLiftStreamJobs ? njobs - g : kLiftStreamJobs;
    long blocks = (((long)cnt << log_n) + 1023) / 1024;
    const long cap = resident_blocks<k_lift_stream>(sms);
    if (blocks > cap) blocks = cap;
    k_lift_stream<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(jobs ? jobs + g : nullptr, cnt, o, (int)log_n,
                                                                     *lift);
    vkcu_count_launches(1);
    if (const int e = (int)cudaGetLastError()) return e;
  }
  return 0;
}

// Pointwise step of a composed polymul: c = c * scratch mod q over njobs
// jobs of n words each, the word the reference's elemmul stores: c is a
// canonical NTT output, scratch one too or the caller's NTT(b), reduced as
// elemmul reduces its operands.  A block takes chunks of up to 2048 words of
// one job (the job's constants loaded once per chunk, not per word), each
// thread two 16-byte pairs of c and of scratch per round, loads first.
template <class M>
__global__ void __launch_bounds__(256) k_pointwise(const vkcu_poly_job* __restrict__ jobs, int njobs, int log_n) {
  const int lw = log_n < 11 ? log_n : 11;  // log2 of the words of a chunk
  const long cpj = 1L << (log_n - lw);    // chunks per job
  const long total = (long)njobs * cpj;
  const int pairs = 1 << (lw - 1);         // n >= 2
  for (long ch = blockIdx.x; ch < total; ch += gridDim.x) {
    const vkcu_poly_job job = jobs[ch >> (log_n - lw)];
    const Tw t = load_tw(job.tw);
    const long base = (ch & (cpj - 1)) << lw;
    u64* c = reinterpret_cast<u64*>(job.c) + base;
    const u64* y = reinterpret_cast<const u64*>(job.scratch) + base;
    auto prod = [&](u64 x, u64 b) { return M::product_out(x, ref_reduce64_maybe(b, t.q, t.mu, t.qbits), t); };
    for (int p = (int)threadIdx.x; p < pairs; p += 2 * (int)blockDim.x) {
      const int p1 = p + (int)blockDim.x;
      const bool two = p1 < pairs;
      const ulonglong2 x0 = ld2(c + 2 * p), y0 = ld2(y + 2 * p);
      ulonglong2 x1 = x0, y1 = y0;
      if (two) {
        x1 = ld2(c + 2 * p1);
        y1 = ld2(y + 2 * p1);
      }
      st2(c + 2 * p, prod(x0.x, y0.x), prod(x0.y, y0.y));
      if (two) st2(c + 2 * p1, prod(x1.x, y1.x), prod(x1.y, y1.y));
    }
  }
}

extern "C" int vkcu_pointwise(void* stream, const vkcu_poly_job* jobs, int njobs, uint32_t log_n, int wide, int sms) {
  if (njobs < 1 || !jobs || log_n < 1) return (int)cudaErrorInvalidValue;
  const long chunks = (long)njobs << (log_n > 11 ? log_n - 11 : 0);
  long blocks = chunks;
  if (blocks > (long)sms * 8) blocks = (long)sms * 8;
  if (wide)
    k_pointwise<Mod63><<<(int)blocks, 256, 0, (cudaStream_t)stream>>>(jobs, njobs, (int)log_n);
  else
    k_pointwise<Mod62><<<(int)blocks, 256, 0, (cudaStream_t)stream>>>(jobs, njobs, (int)log_n);
  vkcu_count_launches(1);
  return (int)cudaGetLastError();
}
