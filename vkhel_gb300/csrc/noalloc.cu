// Fused polynomial multiply for callers that cannot allocate device memory.
//
// vkhel_vector_polymul parks NTT(b) in the result vector, or in a temporary
// buffer from the context's pool when the result aliases a.  Some callers
// cannot let the library allocate at the point where they multiply: a host
// program that has already handed all the device memory it may use to its
// own allocator (another framework's caching allocator, a fixed reservation
// per tenant), so that a pool allocation would fail or push it over its
// limit; or a latency-critical loop that must not call cudaMalloc / cudaFree,
// which can stall until work already queued on the device has drained.
// vkhel_vector_polymul_noalloc runs the same kernel (k_polymul) with its
// scratch in this file's static device array instead, so it allocates
// nothing: the caller passes inputs and outputs.
//
// Limits and rules:
//   * degree 256 <= n <= kNoallocMaxWords (16384): the fused range; the
//     scratch array is kNoallocMaxWords words (128 KiB) on every device that
//     loads libvkhel, held until the process exits; larger n is rejected with
//     VKHEL_ERR_UNSUPPORTED;
//   * the twiddle tables must already be resident on the context (any
//     transform, polymul or batch call with them uploads them); otherwise the
//     call fails with VKHEL_ERR_INVALID_ARGUMENT instead of uploading (which
//     would allocate);
//   * every call on a device shares the one array and the kernel overwrites
//     the n words it uses before reading them (nothing needs clearing), so
//     calls that overlap on the GPU -- two contexts or threads running it at
//     once -- race on the array; calls must not overlap;
//   * the first call on each device resolves the array's device address with
//     cudaGetSymbolAddress (host code cannot use the array's name as a device
//     pointer) and is the first launch of the kernel for its degree; make
//     that first call during set-up, before any stream capture.
#include <cuda_runtime.h>

#include <mutex>

#include "internal.h"

namespace {

constexpr unsigned long long kNoallocMaxWords = 16384;

__device__ __align__(256) unsigned long long g_polymul_scratch[kNoallocMaxWords];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void* g_scratch_addr[kMaxDevices];

// Device address of g_polymul_scratch on `device`, resolved once per device
// with that device current.
int scratch_address(int device, void** out) {
  if (device < 0 || device >= kMaxDevices) return (int)cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_scratch_addr[device]) {
    int prev = -1;
    cudaError_t e = cudaGetDevice(&prev);
    if (e == cudaSuccess && prev != device) e = cudaSetDevice(device);
    void* p = nullptr;
    if (e == cudaSuccess) e = cudaGetSymbolAddress(&p, g_polymul_scratch);
    if (prev >= 0 && prev != device) cudaSetDevice(prev);
    if (e != cudaSuccess) return (int)e;
    g_scratch_addr[device] = p;
  }
  *out = g_scratch_addr[device];
  return 0;
}

}  // namespace

extern "C" VKHEL_EXPORT int vkhel_vector_polymul_noalloc(const struct vkhel_vector* a, const struct vkhel_vector* b,
                                            struct vkhel_vector* result, const struct vkhel_ntt_tables* t) {
  if (!a || !b || !result || !t)
    return vkh_fail(result ? result->ctx : NULL, VKHEL_ERR_INVALID_ARGUMENT, "polymul_noalloc: NULL argument");
  struct vkhel_ctx* ctx = result->ctx;
  if (a->ctx != ctx || b->ctx != ctx)
    return vkh_fail(ctx, VKHEL_ERR_INVALID_ARGUMENT, "polymul_noalloc: vectors belong to different contexts");
  if (t->n > kNoallocMaxWords || t->log_n < 8 || t->log_n > vkcu_max_fused_log_n())
    return vkh_fail(ctx, VKHEL_ERR_UNSUPPORTED,
                    "polymul_noalloc: n=%llu outside 256..%llu (static scratch of %llu words)",
                    (unsigned long long)t->n, kNoallocMaxWords, kNoallocMaxWords);
  if (t->q < 3 || t->q >= (1ull << 63) || t->unreduced)
    return vkh_fail(ctx, VKHEL_ERR_UNSUPPORTED, "polymul_noalloc: q outside [3, 2^63) or tables not reduced");
  if (a->length < t->n || b->length < t->n || result->length < t->n)
    return vkh_fail(ctx, VKHEL_ERR_INVALID_ARGUMENT, "polymul_noalloc: vectors shorter than n");
  const struct vkh_devtab* d = vkh_devtab_find(ctx, t);
  if (!d)
    return vkh_fail(ctx, VKHEL_ERR_INVALID_ARGUMENT,
                    "polymul_noalloc: tables not resident on this context (run any transform or polymul "
                    "with them first)");
  void* scratch = nullptr;
  int e = scratch_address(ctx->device, &scratch);
  if (e) return vkh_cuda(ctx, e, "polymul_noalloc: scratch address");
  const vkcu_poly_job job = {a->dev, b->dev, result->dev, static_cast<uint64_t*>(scratch), d->dev_set};
  e = vkcu_polymul(ctx->stream, nullptr, 1, &job, t->log_n, vkcu_wide(t->q), ctx->sms);
  if (!e) e = vkcu_sync(ctx->stream);
  return vkh_cuda(ctx, e, "polymul_noalloc");
}
