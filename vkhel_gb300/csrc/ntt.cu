// Transform dispatch and the kernels outside the CTA-resident families:
// simple one-stage-per-barrier kernels (n < 256, unaligned operands), the
// global-memory head/tail passes of n > 2^14, and the pointwise step of a
// composed polynomial multiply.  The CTA-resident kernels are in
// ntt_core.cuh with one launcher per family (ntt_fwd.cu, ntt_inv.cu,
// ntt_poly.cu).
#include "ntt_core.cuh"

namespace vk {

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
// Forward: global stages 0 .. KK-1, in -> out, lazy [0, 2q).  Each thread
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
    const ulonglong2 w0 = ld_tw(t.fwd + 1);
#pragma unroll
    for (int jj = 0; jj < (1 << (KK - 1)); jj++) ct_first(v[jj], v[jj + (1 << (KK - 1))], w0.x, w0.y, t);
    ct_group<KK, 1, 0>(v, t.fwd, 1u, t);
    u64* out = reinterpret_cast<u64*>(job.out);
    // below 2q, so the sub-block kernels' first stage stays on its fast path
#pragma unroll
    for (int j = 0; j < (1 << KK); j++) out[o + (size_t)j * groups] = csub(v[j], t.q2);
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

static constexpr int kMaxCta = 14;      // one CTA per transform
static constexpr int kMaxCluster = 17;  // one cluster of up to 8 CTAs
static constexpr int kMaxLogN = 18;     // one global pass + 2^14 sub-blocks

static bool aligned32(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 31) == 0; }

static int simple(cudaStream_t st, bool inverse, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job& one,
                  int log_n, int sms) {
  const int n = 1 << log_n;
  const int threads = n / 2 < 32 ? 32 : (n / 2 > 512 ? 512 : n / 2);
  const int smem = n * 8;
  auto kern = inverse ? k_ntt_inv_simple : k_ntt_fwd_simple;
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
static bool split_small(int njobs, uint32_t log_n, int sms) {
  return log_n >= 12 && log_n <= 16 && (long)njobs * 8 <= (long)sms && vkh_variant(3, 1) == 0;
}

extern "C" int vkcu_ntt_forward(void* stream, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job* one,
                                uint32_t log_n, int sms) {
  cudaStream_t st = (cudaStream_t)stream;
  const vkcu_ntt_job o = one ? *one : vkcu_ntt_job{};
  if (log_n < 1 || log_n > (uint32_t)kMaxLogN || njobs < 1) return (int)cudaErrorInvalidValue;
  const bool aligned = jobs_aligned(jobs, one);
  if (log_n < 8 || (log_n <= (uint32_t)kMaxCta && !aligned)) return simple(st, false, jobs, njobs, o, (int)log_n, sms);
  if (!aligned) return (int)cudaErrorMisalignedAddress;
  if (split_small(njobs, log_n, sms)) return fwd_cluster(st, jobs, njobs, o, 3, (int)log_n - 3);
  if (log_n <= (uint32_t)kMaxCta) return fwd_cta(st, jobs, njobs, o, (int)log_n, 0, sms, vkh_variant(1, (int)log_n));
  if (log_n <= (uint32_t)kMaxCluster) return fwd_cluster(st, jobs, njobs, o, (int)log_n - kMaxCta, kMaxCta);
  const int kk = (int)log_n - kMaxCta;
  if (int e = global_pass<false>(st, jobs, njobs, o, (int)log_n, kk, sms)) return e;
  return fwd_cta(st, jobs, njobs, o, kMaxCta, kk, sms, vkh_variant(1, kMaxCta));
}

static bool has_lift(const vkcu_lift* lift) { return lift && lift->count > 0; }

extern "C" int vkcu_ntt_inverse_lift(void* stream, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job* one,
                                     uint32_t log_n, int sms, const vkcu_lift* lift) {
  cudaStream_t st = (cudaStream_t)stream;
  const vkcu_ntt_job o = one ? *one : vkcu_ntt_job{};
  if (log_n < 1 || log_n > (uint32_t)kMaxLogN || njobs < 1) return (int)cudaErrorInvalidValue;
  if (has_lift(lift) && lift->count > VKCU_MAX_LIFT) return (int)cudaErrorInvalidValue;
  const bool aligned = jobs_aligned(jobs, one);
  const bool lifted = has_lift(lift);
  int e;
  if (log_n < 8 || (log_n <= (uint32_t)kMaxCta && !aligned)) {
    e = simple(st, true, jobs, njobs, o, (int)log_n, sms);
  } else if (!aligned) {
    return (int)cudaErrorMisalignedAddress;
  } else if (split_small(njobs, log_n, sms)) {
    return inv_cluster(st, jobs, njobs, o, 3, (int)log_n - 3, lifted ? lift : nullptr);
  } else if (log_n <= (uint32_t)kMaxCta) {
    if (lifted) return inv_cta_lift(st, jobs, njobs, o, (int)log_n, sms, *lift);
    return inv_cta(st, jobs, njobs, o, (int)log_n, 0, sms, vkh_variant(2, (int)log_n));
  } else if (log_n <= (uint32_t)kMaxCluster) {
    return inv_cluster(st, jobs, njobs, o, (int)log_n - kMaxCta, kMaxCta, lifted ? lift : nullptr);
  } else {
    const int kk = (int)log_n - kMaxCta;
    e = inv_cta(st, jobs, njobs, o, kMaxCta, kk, sms, vkh_variant(2, kMaxCta));
    if (!e) e = global_pass<true>(st, jobs, njobs, o, (int)log_n, kk, sms);
  }
  // the multi-launch paths take the epilogue as one more element-wise launch
  if (!e && lifted) e = vkcu_lift_jobs(stream, jobs, njobs, one, log_n, sms, lift);
  return e;
}

extern "C" int vkcu_ntt_inverse(void* stream, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job* one,
                                uint32_t log_n, int sms) {
  return vkcu_ntt_inverse_lift(stream, jobs, njobs, one, log_n, sms, nullptr);
}

extern "C" int vkcu_polymul_lift(void* stream, const vkcu_poly_job* jobs, int njobs, const vkcu_poly_job* one,
                                 uint32_t log_n, int sms, const vkcu_lift* lift) {
  cudaStream_t st = (cudaStream_t)stream;
  const vkcu_poly_job o = one ? *one : vkcu_poly_job{};
  if (log_n < 8 || log_n > (uint32_t)kMaxCluster || njobs < 1) return (int)cudaErrorInvalidValue;
  if (has_lift(lift) && lift->count > VKCU_MAX_LIFT) return (int)cudaErrorInvalidValue;
  if (split_small(njobs, log_n, sms)) return poly_cluster(st, jobs, njobs, o, 3, (int)log_n - 3, has_lift(lift) ? lift : nullptr);
  if (log_n <= (uint32_t)kMaxCta) {
    if (has_lift(lift)) return poly_cta_lift(st, jobs, njobs, o, (int)log_n, sms, vkh_variant(0, (int)log_n), *lift);
    return poly_cta(st, jobs, njobs, o, (int)log_n, sms, vkh_variant(0, (int)log_n));
  }
  return poly_cluster(st, jobs, njobs, o, (int)log_n - kMaxCta, kMaxCta, has_lift(lift) ? lift : nullptr);
}

extern "C" int vkcu_polymul(void* stream, const vkcu_poly_job* jobs, int njobs, const vkcu_poly_job* one,
                            uint32_t log_n, int sms) {
  return vkcu_polymul_lift(stream, jobs, njobs, one, log_n, sms, nullptr);
}

// The epilogue as its own element-wise pass: over `len` words at p, or over
// the n output words of each job (q from the job's twiddle set).
__global__ void k_lift_range(u64* __restrict__ p, u64 len, u64 q, const __grid_constant__ vkcu_lift lift) {
  const LiftRun lr(&lift, q);
  for (u64 i = blockIdx.x * (u64)blockDim.x + threadIdx.x; i < len; i += (u64)gridDim.x * blockDim.x)
    p[i] = lr(p[i]);
}

__global__ void k_lift_jobs(const vkcu_ntt_job* __restrict__ jobs, int njobs, vkcu_ntt_job one, int log_n,
                            const __grid_constant__ vkcu_lift lift) {
  const long n = 1L << log_n;
  const long per = (n + gridDim.y - 1) / gridDim.y;  // words of a job per block row
  for (int w = blockIdx.x; w < njobs; w += gridDim.x) {
    const vkcu_ntt_job job = fetch_job(jobs, one, w);
    const LiftRun lr(&lift, load_tw(job.tw).q);
    u64* out = reinterpret_cast<u64*>(job.out);
    const long lo = (long)blockIdx.y * per, hi = lo + per < n ? lo + per : n;
    for (long i = lo + threadIdx.x; i < hi; i += blockDim.x) out[i] = lr(out[i]);
  }
}

extern "C" int vkcu_lift_range(void* stream, uint64_t* p, uint64_t len, uint64_t q, const vkcu_lift* lift) {
  if (!has_lift(lift) || len == 0) return 0;
  if (lift->count > VKCU_MAX_LIFT) return (int)cudaErrorInvalidValue;
  uint64_t blocks = (len + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  k_lift_range<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(reinterpret_cast<u64*>(p), len, q, *lift);
  vkcu_count_launches(1);
  return (int)cudaGetLastError();
}

extern "C" int vkcu_lift_jobs(void* stream, const vkcu_ntt_job* jobs, int njobs, const vkcu_ntt_job* one,
                              uint32_t log_n, int sms, const vkcu_lift* lift) {
  if (!has_lift(lift)) return 0;
  if (njobs < 1 || log_n > (uint32_t)kMaxLogN || lift->count > VKCU_MAX_LIFT) return (int)cudaErrorInvalidValue;
  const vkcu_ntt_job o = one ? *one : vkcu_ntt_job{};
  const long n = 1L << log_n;
  const int threads = n < 256 ? (int)((n + 31) / 32 * 32) : 256;
  const long want = (long)(sms > 0 ? sms : 1) * 8;
  const int gx = njobs < want ? njobs : (int)want;
  long gy = (want + gx - 1) / gx;  // split each job when there are few
  const long max_gy = (n + threads - 1) / threads;
  if (gy > max_gy) gy = max_gy;
  k_lift_jobs<<<dim3((unsigned)gx, (unsigned)gy), threads, 0, (cudaStream_t)stream>>>(jobs, njobs, o, (int)log_n,
                                                                                      *lift);
  vkcu_count_launches(1);
  return (int)cudaGetLastError();
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
