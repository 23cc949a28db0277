// Device runtime: one GB300, one stream, a stream-ordered memory pool.
// Replaces SkelCL's OpenCL device layer -- skelcl::init / terminate
// (src/SkelCL.cpp:51-85), DeviceList (src/DeviceList.cpp:82-123), Device
// (src/Device.cpp:95-330: context + profiling queue, enqueueWrite/Read/Copy
// with flush), DeviceBuffer (src/DeviceBuffer.cpp:60-135) and Event
// (src/Event.cpp).  Reference behaviour kept: asynchronous enqueue on one
// in-order queue; host reads wait for completion.  Completion callbacks
// holding buffers alive (keepAlive, KernelUtil.h:287-360) become
// stream-ordered frees.
#include <cstdio>
#include <cstring>
#include <string>

#include "internal.h"

namespace scl {

namespace {
thread_local std::string g_last_error;
Runtime g_rt;
}  // namespace

Runtime& rt() { return g_rt; }

int fail(int status, const std::string& msg) {
  g_last_error = msg;
  return status;
}

int cuda_fail(cudaError_t e, const char* what) {
  cudaGetLastError();  // clear sticky-free errors
  int st = (e == cudaErrorMemoryAllocation) ? SCL_ERR_OOM : SCL_ERR_CUDA;
  return fail(st, std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
}

int cu_fail(CUresult r, const char* what) {
  const char* s = "unknown";
  if (g_rt.drv.cuGetErrorString) g_rt.drv.cuGetErrorString(r, &s);
  int st = (r == CUDA_ERROR_OUT_OF_MEMORY) ? SCL_ERR_OOM
           : (r == CUDA_ERROR_LAUNCH_FAILED || r == CUDA_ERROR_INVALID_VALUE ||
              r == CUDA_ERROR_LAUNCH_OUT_OF_RESOURCES)
               ? SCL_ERR_LAUNCH
               : SCL_ERR_CUDA;
  return fail(st, std::string(what) + ": CUresult " + std::to_string((int)r) + " (" + s + ")");
}

int require_init() {
  if (!g_rt.initialized) return fail(SCL_ERR_NOT_INIT, "scl_init() has not been called");
  return SCL_OK;
}

namespace {
template <typename F>
int resolve(const char* sym, F* fn) {
  void* p = nullptr;
  cudaDriverEntryPointQueryResult q;
  cudaError_t e = cudaGetDriverEntryPointByVersion(sym, &p, CUDA_VERSION, cudaEnableDefault, &q);
  if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !p)
    return fail(SCL_ERR_CUDA, std::string("driver entry point not found: ") + sym);
  *fn = reinterpret_cast<F>(p);
  return SCL_OK;
}

// Test hook: a wait on a flag nothing sets, bounded by `polls`.
__global__ void scl_bounded_wait_kernel(const unsigned int* flag, unsigned int polls,
                                        unsigned int* status) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  unsigned int n = 0;
  while (*(const volatile unsigned int*)flag == 0u) {
    if (++n > polls) {
      *status = SCL_ERR_TIMEOUT;
      return;
    }
    __nanosleep(100);
  }
  *status = SCL_OK;
}

// FP32 peak probe: 16 independent FMA chains per thread (scalar fma.rn.f32,
// or packed fma.rn.f32x2 on 8 pairs), `iters` rounds, no memory traffic
// but one float per thread at the end.  m and c arrive as arguments so the
// chains cannot be folded.
template <int PACKED>
__global__ void __launch_bounds__(256) scl_fma_peak_kernel(float* sink, unsigned int iters, float m,
                                                           float c) {
  const float base = (float)(threadIdx.x & 31) * 1e-3f;
  float r = 0.0f;
  if constexpr (PACKED) {
    unsigned long long a[8], mm, cc;
    asm("mov.b64 %0, {%1, %1};" : "=l"(mm) : "f"(m));
    asm("mov.b64 %0, {%1, %1};" : "=l"(cc) : "f"(c));
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const float lo = base + (float)(2 * k), hi = base + (float)(2 * k + 1);
      asm("mov.b64 %0, {%1, %2};" : "=l"(a[k]) : "f"(lo), "f"(hi));
    }
    for (unsigned int i = 0; i < iters; ++i) {
#pragma unroll
      for (int k = 0; k < 8; ++k)
        asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(a[k]) : "l"(mm), "l"(cc));
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      float lo, hi;
      asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(a[k]));
      r += lo + hi;
    }
  } else {
    float a[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) a[k] = base + (float)k;
    for (unsigned int i = 0; i < iters; ++i) {
#pragma unroll
      for (int k = 0; k < 16; ++k) a[k] = fmaf(a[k], m, c);
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) r += a[k];
  }
  sink[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = r;
}
}  // namespace

}  // namespace scl

using namespace scl;

extern "C" int scl_abi_version(void) { return SCL_ABI_VERSION; }

extern "C" const char* scl_last_error_string(void) { return g_last_error.c_str(); }

extern "C" int scl_is_initialized(void) { return g_rt.initialized ? 1 : 0; }

extern "C" int scl_init(int device) {
  if (g_rt.initialized) {
    if (device == g_rt.device) return SCL_OK;
    return fail(SCL_ERR_ARG, "already initialised on another device; call scl_terminate first");
  }
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0)
    return fail(SCL_ERR_CUDA, std::string("no CUDA device available: ") + cudaGetErrorString(e));
  if (device < 0 || device >= count) return fail(SCL_ERR_ARG, "device index out of range");
  SCL_CUDA(cudaSetDevice(device));
  SCL_CUDA(cudaFree(nullptr));  // create the primary context
  Driver& d = g_rt.drv;
  if (int st = resolve("cuModuleLoadData", &d.cuModuleLoadData)) return st;
  if (int st = resolve("cuModuleUnload", &d.cuModuleUnload)) return st;
  if (int st = resolve("cuModuleGetFunction", &d.cuModuleGetFunction)) return st;
  if (int st = resolve("cuModuleGetGlobal", &d.cuModuleGetGlobal)) return st;
  if (int st = resolve("cuFuncSetAttribute", &d.cuFuncSetAttribute)) return st;
  if (int st = resolve("cuFuncGetAttribute", &d.cuFuncGetAttribute)) return st;
  if (int st = resolve("cuLaunchKernel", &d.cuLaunchKernel)) return st;
  if (resolve("cuLaunchKernelEx", &d.cuLaunchKernelEx) != SCL_OK) d.cuLaunchKernelEx = nullptr;
  if (int st = resolve("cuOccupancyMaxActiveBlocksPerMultiprocessor",
                       &d.cuOccupancyMaxActiveBlocksPerMultiprocessor))
    return st;
  if (int st = resolve("cuTensorMapEncodeTiled", &d.cuTensorMapEncodeTiled)) return st;
  if (int st = resolve("cuGetErrorString", &d.cuGetErrorString)) return st;
  if (resolve("cuFuncGetParamInfo", &d.cuFuncGetParamInfo) != SCL_OK) d.cuFuncGetParamInfo = nullptr;

  cudaDeviceProp prop;
  SCL_CUDA(cudaGetDeviceProperties(&prop, device));
  g_rt.device = device;
  g_rt.sm_count = prop.multiProcessorCount;
  g_rt.cc_major = prop.major;
  g_rt.cc_minor = prop.minor;
  g_rt.smem_optin = prop.sharedMemPerBlockOptin;
  g_rt.global_mem = prop.totalGlobalMem;
  g_rt.name = prop.name;
  SCL_CUDA(cudaStreamCreateWithFlags(&g_rt.stream, cudaStreamNonBlocking));
  for (cudaStream_t& c : g_rt.copy_streams) SCL_CUDA(cudaStreamCreateWithFlags(&c, cudaStreamNonBlocking));
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t thresh = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thresh);
  }
  SCL_CUDA(cudaMalloc(&g_rt.dev_err, 64));
  SCL_CUDA(cudaMemset(g_rt.dev_err, 0, 64));
  SCL_CUDA(cudaMallocHost(&g_rt.host_err, 64));
  std::memset(g_rt.host_err, 0, 64);
  g_rt.launches = 0;
  g_rt.pdl_launches = 0;
  {
    const char* e = std::getenv("SKELCL_PDL");
    g_rt.pdl = d.cuLaunchKernelEx != nullptr && !(e && std::string(e) == "0");
  }
  g_rt.initialized = true;
  return SCL_OK;
}

extern "C" int scl_terminate(void) {
  if (!g_rt.initialized) return SCL_OK;
  cudaStreamSynchronize(g_rt.stream);
  cudaFree(g_rt.dev_err);
  cudaFreeHost(g_rt.host_err);
  for (cudaStream_t& c : g_rt.copy_streams) {
    cudaStreamSynchronize(c);
    cudaStreamDestroy(c);
    c = nullptr;
  }
  cudaStreamDestroy(g_rt.stream);
  g_rt.dev_err = nullptr;
  g_rt.host_err = nullptr;
  g_rt.stream = nullptr;
  g_rt.initialized = false;
  return SCL_OK;
}

extern "C" int scl_device_info(int* sm_count, size_t* global_mem, char* name, size_t name_cap) {
  if (int st = require_init()) return st;
  if (sm_count) *sm_count = g_rt.sm_count;
  if (global_mem) *global_mem = g_rt.global_mem;
  if (name && name_cap) {
    std::strncpy(name, g_rt.name.c_str(), name_cap - 1);
    name[name_cap - 1] = '\0';
  }
  return SCL_OK;
}

// ---- memory -------------------------------------------------------------------
extern "C" int scl_alloc(size_t bytes, void** dptr) {
  if (int st = require_init()) return st;
  if (!dptr) return fail(SCL_ERR_ARG, "scl_alloc: null out pointer");
  *dptr = nullptr;
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMallocAsync(dptr, bytes, g_rt.stream);
  g_rt.device_allocs++;
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(SCL_ERR_OOM, "scl_alloc: cannot allocate " + std::to_string(bytes) + " bytes (" +
                                 cudaGetErrorString(e) + ")");
  }
  return SCL_OK;
}

extern "C" int scl_free(void* dptr) {
  if (!dptr) return SCL_OK;
  if (!g_rt.initialized) return SCL_OK;  // context already gone
  SCL_CUDA(cudaFreeAsync(dptr, g_rt.stream));
  return SCL_OK;
}

namespace {
int check_device_status() {
  // called after the stream is idle
  SCL_CUDA(cudaMemcpy(g_rt.host_err, g_rt.dev_err, sizeof(unsigned int), cudaMemcpyDeviceToHost));
  unsigned int v = g_rt.host_err[0];
  if (v) {
    SCL_CUDA(cudaMemset(g_rt.dev_err, 0, sizeof(unsigned int)));
    if (v & 1u) return fail(SCL_ERR_TIMEOUT, "a bounded device-side wait gave up (decoupled look-back or TMA barrier)");
    if (v & kDevErrSegments)
      return fail(SCL_ERR_ARG, "segment offsets were decreasing or beyond the vector (clamped)");
    return fail(SCL_ERR_CUDA, "device reported status " + std::to_string(v));
  }
  return SCL_OK;
}

int copy(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, bool wait) {
  if (int st = require_init()) return st;
  if (bytes == 0) return SCL_OK;
  if (!dst || !src) return fail(SCL_ERR_ARG, "copy: null pointer");
  SCL_CUDA(cudaMemcpyAsync(dst, src, bytes, kind, g_rt.stream));
  if (wait) {
    SCL_CUDA(cudaStreamSynchronize(g_rt.stream));
    if (kind == cudaMemcpyDeviceToHost) return check_device_status();
  }
  return SCL_OK;
}
}  // namespace

extern "C" int scl_h2d(void* dst, const void* src, size_t bytes) {
  return copy(dst, src, bytes, cudaMemcpyHostToDevice, true);
}
extern "C" int scl_d2h(void* dst, const void* src, size_t bytes) {
  return copy(dst, src, bytes, cudaMemcpyDeviceToHost, true);
}
extern "C" int scl_d2d(void* dst, const void* src, size_t bytes) {
  return copy(dst, src, bytes, cudaMemcpyDeviceToDevice, false);
}
extern "C" int scl_h2d_async(void* dst, const void* src, size_t bytes) {
  return copy(dst, src, bytes, cudaMemcpyHostToDevice, false);
}
extern "C" int scl_d2h_async(void* dst, const void* src, size_t bytes) {
  return copy(dst, src, bytes, cudaMemcpyDeviceToHost, false);
}
extern "C" int scl_memset(void* dst, int value, size_t bytes) {
  if (int st = require_init()) return st;
  if (bytes == 0) return SCL_OK;
  SCL_CUDA(cudaMemsetAsync(dst, value, bytes, g_rt.stream));
  return SCL_OK;
}
extern "C" int scl_host_alloc(size_t bytes, void** hptr) {
  if (int st = require_init()) return st;
  if (!hptr) return fail(SCL_ERR_ARG, "scl_host_alloc: null out pointer");
  SCL_CUDA(cudaMallocHost(hptr, bytes ? bytes : 16));
  return SCL_OK;
}
extern "C" int scl_host_free(void* hptr) {
  if (!hptr || !g_rt.initialized) return SCL_OK;
  SCL_CUDA(cudaFreeHost(hptr));
  return SCL_OK;
}
extern "C" int scl_sync(void) {
  if (int st = require_init()) return st;
  for (cudaStream_t c : g_rt.copy_streams) SCL_CUDA(cudaStreamSynchronize(c));
  SCL_CUDA(cudaStreamSynchronize(g_rt.stream));
  return check_device_status();
}

// ---- copy streams ----------------------------------------------------------------
namespace {
int stream_of(int s, cudaStream_t* out) {
  if (s == 0) *out = g_rt.stream;
  else if (s == 1 || s == 2) *out = g_rt.copy_streams[s - 1];
  else return fail(SCL_ERR_ARG, "stream must be 0 (launches), 1 or 2 (copies)");
  return SCL_OK;
}
int copy_on(int s, void* dst, const void* src, size_t bytes, cudaMemcpyKind kind) {
  if (int st = require_init()) return st;
  if (bytes == 0) return SCL_OK;
  if (!dst || !src) return fail(SCL_ERR_ARG, "copy: null pointer");
  cudaStream_t cs;
  if (int st = stream_of(s, &cs)) return st;
  SCL_CUDA(cudaMemcpyAsync(dst, src, bytes, kind, cs));
  return SCL_OK;
}
}  // namespace

extern "C" int scl_h2d_on(int stream, void* dst, const void* src, size_t bytes) {
  return copy_on(stream, dst, src, bytes, cudaMemcpyHostToDevice);
}
extern "C" int scl_d2h_on(int stream, void* dst, const void* src, size_t bytes) {
  return copy_on(stream, dst, src, bytes, cudaMemcpyDeviceToHost);
}

// ---- events -------------------------------------------------------------------
struct scl_event {
  cudaEvent_t ev;
};
extern "C" int scl_event_create(scl_event** ev) {
  if (int st = require_init()) return st;
  if (!ev) return fail(SCL_ERR_ARG, "null out pointer");
  scl_event* e = new scl_event;
  cudaError_t r = cudaEventCreate(&e->ev);
  if (r != cudaSuccess) {
    delete e;
    return cuda_fail(r, "cudaEventCreate");
  }
  *ev = e;
  return SCL_OK;
}
extern "C" int scl_event_record(scl_event* ev) {
  if (int st = require_init()) return st;
  if (!ev) return fail(SCL_ERR_ARG, "null event");
  SCL_CUDA(cudaEventRecord(ev->ev, g_rt.stream));
  return SCL_OK;
}
extern "C" int scl_event_record_on(scl_event* ev, int stream) {
  if (int st = require_init()) return st;
  if (!ev) return fail(SCL_ERR_ARG, "null event");
  cudaStream_t cs;
  if (int st = stream_of(stream, &cs)) return st;
  SCL_CUDA(cudaEventRecord(ev->ev, cs));
  return SCL_OK;
}
extern "C" int scl_stream_wait(int stream, scl_event* ev) {
  if (int st = require_init()) return st;
  if (!ev) return fail(SCL_ERR_ARG, "null event");
  cudaStream_t cs;
  if (int st = stream_of(stream, &cs)) return st;
  SCL_CUDA(cudaStreamWaitEvent(cs, ev->ev, 0));
  return SCL_OK;
}
extern "C" int scl_event_elapsed_ms(scl_event* a, scl_event* b, float* ms) {
  if (!a || !b || !ms) return fail(SCL_ERR_ARG, "null argument");
  SCL_CUDA(cudaEventSynchronize(b->ev));
  SCL_CUDA(cudaEventElapsedTime(ms, a->ev, b->ev));
  return SCL_OK;
}
extern "C" int scl_event_destroy(scl_event* ev) {
  if (!ev) return SCL_OK;
  if (g_rt.initialized) cudaEventDestroy(ev->ev);
  delete ev;
  return SCL_OK;
}

// ---- graphs ---------------------------------------------------------------------
struct scl_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};
extern "C" int scl_graph_begin(void) {
  if (int st = require_init()) return st;
  if (g_rt.capturing) return fail(SCL_ERR_ARG, "a capture is already active");
  SCL_CUDA(cudaStreamBeginCapture(g_rt.stream, cudaStreamCaptureModeRelaxed));
  g_rt.capturing = true;
  return SCL_OK;
}
extern "C" int scl_graph_end(scl_graph** out) {
  if (int st = require_init()) return st;
  if (!out) return fail(SCL_ERR_ARG, "null out pointer");
  if (!g_rt.capturing) return fail(SCL_ERR_ARG, "no capture is active");
  g_rt.capturing = false;
  scl_graph* g = new scl_graph;
  cudaError_t e = cudaStreamEndCapture(g_rt.stream, &g->graph);
  if (e != cudaSuccess) {
    delete g;
    return cuda_fail(e, "cudaStreamEndCapture");
  }
  e = cudaGraphInstantiate(&g->exec, g->graph, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g->graph);
    delete g;
    return cuda_fail(e, "cudaGraphInstantiate");
  }
  *out = g;
  return SCL_OK;
}
extern "C" int scl_graph_launch(scl_graph* g) {
  if (int st = require_init()) return st;
  if (!g) return fail(SCL_ERR_ARG, "null graph");
  SCL_CUDA(cudaGraphLaunch(g->exec, g_rt.stream));
  return SCL_OK;
}
extern "C" int scl_graph_destroy(scl_graph* g) {
  if (!g) return SCL_OK;
  if (g_rt.initialized) {
    cudaStreamSynchronize(g_rt.stream);
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
  }
  delete g;
  return SCL_OK;
}

extern "C" int scl_launch_count(uint64_t* count) {
  if (!count) return fail(SCL_ERR_ARG, "null argument");
  *count = g_rt.launches;
  return SCL_OK;
}

extern "C" int scl_pdl_set(int enable, int* previous) {
  if (int st = require_init()) return st;
  if (previous) *previous = g_rt.pdl ? 1 : 0;
  if (enable && !g_rt.drv.cuLaunchKernelEx)
    return fail(SCL_ERR_ARG, "this driver has no cuLaunchKernelEx: launches cannot overlap");
  g_rt.pdl = enable != 0;
  return SCL_OK;
}

extern "C" int scl_pdl_launch_count(uint64_t* count) {
  if (!count) return fail(SCL_ERR_ARG, "null argument");
  *count = g_rt.pdl_launches;
  return SCL_OK;
}

extern "C" int scl_debug_counters(uint64_t* device_allocs, uint64_t* module_loads) {
  if (device_allocs) *device_allocs = g_rt.device_allocs;
  if (module_loads) *module_loads = g_rt.module_loads;
  return SCL_OK;
}

extern "C" int scl_debug_fp32_peak(int packed, uint32_t iters, float* sink, uint64_t sink_floats,
                                   uint64_t* flops) {
  if (int st = require_init()) return st;
  const unsigned int blocks = (unsigned int)g_rt.sm_count * 8u;  // 2048 threads per SM
  const uint64_t threads = (uint64_t)blocks * 256u;
  if (!sink || sink_floats < threads)
    return fail(SCL_ERR_ARG, "scl_debug_fp32_peak: the sink needs " + std::to_string(threads) + " floats");
  if (packed) scl_fma_peak_kernel<1><<<blocks, 256, 0, g_rt.stream>>>(sink, iters, 0.9999f, 1e-4f);
  else scl_fma_peak_kernel<0><<<blocks, 256, 0, g_rt.stream>>>(sink, iters, 0.9999f, 1e-4f);
  SCL_CUDA(cudaGetLastError());
  ++g_rt.launches;
  if (flops) *flops = threads * (uint64_t)iters * 16u * 2u;
  return SCL_OK;
}

extern "C" int scl_debug_bounded_wait(uint32_t polls, int* status) {
  if (int st = require_init()) return st;
  if (!status) return fail(SCL_ERR_ARG, "null argument");
  unsigned int* buf = nullptr;
  g_rt.device_allocs++;
  SCL_CUDA(cudaMalloc(&buf, 2 * sizeof(unsigned int)));
  SCL_CUDA(cudaMemset(buf, 0, 2 * sizeof(unsigned int)));
  unsigned int init = 0xffffffffu;
  SCL_CUDA(cudaMemcpy(buf + 1, &init, sizeof(init), cudaMemcpyHostToDevice));
  scl_bounded_wait_kernel<<<1, 32, 0, g_rt.stream>>>(buf, polls, buf + 1);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    cudaFree(buf);
    return cuda_fail(e, "scl_bounded_wait_kernel launch");
  }
  ++g_rt.launches;
  unsigned int st = 0;
  SCL_CUDA(cudaMemcpyAsync(&st, buf + 1, sizeof(st), cudaMemcpyDeviceToHost, g_rt.stream));
  SCL_CUDA(cudaStreamSynchronize(g_rt.stream));
  cudaFree(buf);
  *status = (int)st;
  return SCL_OK;
}
