// CUDA runtime layer of libvkhel: the part of the reference's src/vulkan.c
// (instance/device/queue/command-pool set-up, src/vulkan.c:153-206) and of its
// VMA allocations (src/vector.c:60-90) that a CUDA device needs.
//
//  * one device, selected by VKHEL_DEVICE (default 0);
//  * one non-blocking stream per context (the reference's single queue);
//  * a per-context cudaMemPool with an unbounded release threshold, so
//    vector create/destroy recycles device memory instead of calling the
//    driver (the role VMA plays in the reference);
//  * plain stream-ordered copies; pinned host memory for mapped windows.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <cstdint>

#include "kernels.h"

static std::atomic<uint64_t> g_launches{0};

extern "C" uint64_t vkcu_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }
extern "C" void vkcu_count_launches(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

extern "C" const char* vkcu_error_string(int code) { return cudaGetErrorString((cudaError_t)code); }

extern "C" int vkcu_device_count(int* count) {
  *count = 0;
  return (int)cudaGetDeviceCount(count);
}

extern "C" int vkcu_set_device(int device) { return (int)cudaSetDevice(device); }

extern "C" int vkcu_sm_count(int device, int* sms) {
  return (int)cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, device);
}

extern "C" int vkcu_stream_create(void** stream) {
  cudaStream_t s = nullptr;
  const cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  *stream = s;
  return (int)e;
}

extern "C" int vkcu_stream_destroy(void* stream) { return (int)cudaStreamDestroy((cudaStream_t)stream); }

extern "C" int vkcu_pool_create(int device, void** pool) {
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  cudaMemPool_t p = nullptr;
  cudaError_t e = cudaMemPoolCreate(&p, &props);
  if (e != cudaSuccess) return (int)e;
  uint64_t keep = UINT64_MAX;
  e = cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
  *pool = p;
  return (int)e;
}

// NVTX ranges around the library's entry points (header-only NVTX v3: no
// cost unless a profiler is attached).
extern "C" void vkcu_range_push(const char* name) { nvtxRangePushA(name); }
extern "C" void vkcu_range_pop(void) { nvtxRangePop(); }

extern "C" int vkcu_pool_destroy(void* pool) { return (int)cudaMemPoolDestroy((cudaMemPool_t)pool); }

// Memory freed on one stream is reused by an allocation on another stream
// only once the free has completed: the pool then never makes the allocating
// stream wait for the freeing one (it grows instead).
extern "C" int vkcu_pool_independent_streams(void* pool) {
  int no = 0;
  return (int)cudaMemPoolSetAttribute((cudaMemPool_t)pool, cudaMemPoolReuseAllowInternalDependencies, &no);
}

extern "C" int vkcu_alloc(void* pool, void* stream, size_t bytes, void** ptr) {
  *ptr = nullptr;
  return (int)cudaMallocFromPoolAsync(ptr, bytes ? bytes : 8, (cudaMemPool_t)pool, (cudaStream_t)stream);
}

extern "C" int vkcu_free(void* stream, void* ptr) {
  if (!ptr) return 0;
  return (int)cudaFreeAsync(ptr, (cudaStream_t)stream);
}

extern "C" int vkcu_memset0(void* stream, void* ptr, size_t bytes) {
  if (!bytes) return 0;
  return (int)cudaMemsetAsync(ptr, 0, bytes, (cudaStream_t)stream);
}

extern "C" int vkcu_h2d(void* stream, void* dst, const void* src, size_t bytes) {
  if (!bytes) return 0;
  return (int)cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, (cudaStream_t)stream);
}

extern "C" int vkcu_d2h(void* stream, void* dst, const void* src, size_t bytes) {
  if (!bytes) return 0;
  return (int)cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream);
}

extern "C" int vkcu_d2d(void* stream, void* dst, const void* src, size_t bytes) {
  if (!bytes) return 0;
  return (int)cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, (cudaStream_t)stream);
}

extern "C" int vkcu_sync(void* stream) { return (int)cudaStreamSynchronize((cudaStream_t)stream); }

extern "C" int vkcu_host_alloc(void** ptr, size_t bytes) {
  *ptr = nullptr;
  return (int)cudaMallocHost(ptr, bytes ? bytes : 8);
}

extern "C" int vkcu_host_free(void* ptr) { return ptr ? (int)cudaFreeHost(ptr) : 0; }

// ---- CUDA graphs: capture the launches of a batch once, replay them ----
extern "C" int vkcu_capture_begin(void* stream) {
  return (int)cudaStreamBeginCapture((cudaStream_t)stream, cudaStreamCaptureModeThreadLocal);
}

extern "C" int vkcu_capture_end(void* stream, void** exec) {
  cudaGraph_t g = nullptr;
  *exec = nullptr;
  cudaError_t e = cudaStreamEndCapture((cudaStream_t)stream, &g);
  if (e != cudaSuccess) return (int)e;
  cudaGraphExec_t x = nullptr;
  e = cudaGraphInstantiate(&x, g, 0);
  cudaGraphDestroy(g);
  *exec = x;
  return (int)e;
}

extern "C" int vkcu_graph_launch(void* exec, void* stream) {
  return (int)cudaGraphLaunch((cudaGraphExec_t)exec, (cudaStream_t)stream);
}

extern "C" int vkcu_graph_destroy(void* exec) {
  return exec ? (int)cudaGraphExecDestroy((cudaGraphExec_t)exec) : 0;
}

// ---- events: cross-stream ordering and completion polling (serving loop) ----
extern "C" int vkcu_event_create(void** ev) {
  cudaEvent_t e = nullptr;
  const cudaError_t r = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  *ev = e;
  return (int)r;
}

extern "C" int vkcu_event_destroy(void* ev) { return ev ? (int)cudaEventDestroy((cudaEvent_t)ev) : 0; }

extern "C" int vkcu_event_record(void* ev, void* stream) {
  return (int)cudaEventRecord((cudaEvent_t)ev, (cudaStream_t)stream);
}

extern "C" int vkcu_stream_wait(void* stream, void* ev) {
  return (int)cudaStreamWaitEvent((cudaStream_t)stream, (cudaEvent_t)ev, 0);
}

// 0 = completed, 1 = not yet, anything else = CUDA error
// Runs fn(arg) on a driver thread once the stream's earlier work has
// completed (fn must make no CUDA calls).
extern "C" int vkcu_launch_host_func(void* stream, void (*fn)(void*), void* arg) {
  return (int)cudaLaunchHostFunc((cudaStream_t)stream, fn, arg);
}

extern "C" int vkcu_event_query(void* ev) {
  const cudaError_t r = cudaEventQuery((cudaEvent_t)ev);
  if (r == cudaSuccess) return 0;
  if (r == cudaErrorNotReady) return 1;
  return (int)r;
}

extern "C" int vkcu_host_is_pinned(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return a.type == cudaMemoryTypeHost;
}
