// Library-wide runtime pieces: per-thread error string, version, the
// per-thread device staging pool used by the reference-ABI entry points, and
// small device utilities.
#include <stdlib.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <mutex>

#include "gb_common.cuh"
#include "gb_runtime.cuh"

namespace {
thread_local char g_err[1024] = "";
}

void gb_set_error(int code, const char* fmt, ...) {
  char msg[960];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(msg, sizeof(msg), fmt, ap);
  va_end(ap);
  snprintf(g_err, sizeof(g_err), "[%d] %s", code, msg);
}

extern "C" const char* gb_last_error(void) { return g_err; }
extern "C" const char* gb_version(void) { return "rc_gb300 0.1 (sm_103a)"; }

namespace gb {

// ---------------------------------------------------------------- staging pool
// One per host thread: the reference ABI is synchronous and may be called from
// several Haskell capabilities at once (foreign import ccall unsafe from a
// -threaded program), so every thread gets its own stream and buffers.
struct Staging {
  cudaStream_t stream = nullptr;
  cudaStream_t stream2 = nullptr;  // overlaps copies with kernels inside one call
  cudaEvent_t events[kAuxEvents] = {};
  int device = -1;
  void* buf[kStageSlots] = {};
  size_t cap[kStageSlots] = {};
  void release_aux() {
    for (cudaEvent_t& e : events) {
      if (e) cudaEventDestroy(e);
      e = nullptr;
    }
    if (stream2) cudaStreamDestroy(stream2);
    stream2 = nullptr;
  }
  ~Staging() {
    // Released at thread exit; errors are ignored because the context may
    // already be gone at process teardown.
    for (int i = 0; i < kStageSlots; i++)
      if (buf[i]) cudaFree(buf[i]);
    release_aux();
    if (stream) cudaStreamDestroy(stream);
  }
};

static thread_local Staging t_stage;

int stage_stream(cudaStream_t* out) {
  int dev = 0;
  GB_CUDA_TRY(cudaGetDevice(&dev));
  if (t_stage.stream && t_stage.device != dev) {
    // device switched on this thread: drop the old resources
    for (int i = 0; i < kStageSlots; i++) {
      if (t_stage.buf[i]) cudaFree(t_stage.buf[i]);
      t_stage.buf[i] = nullptr;
      t_stage.cap[i] = 0;
    }
    t_stage.release_aux();
    cudaStreamDestroy(t_stage.stream);
    t_stage.stream = nullptr;
  }
  if (!t_stage.stream) {
    GB_CUDA_TRY(cudaStreamCreateWithFlags(&t_stage.stream, cudaStreamNonBlocking));
    t_stage.device = dev;
  }
  *out = t_stage.stream;
  return GB_OK;
}

int stage_aux(cudaStream_t* s2, cudaEvent_t** ev) {
  cudaStream_t s;
  int rc;
  if ((rc = stage_stream(&s))) return rc;  // also drops the aux objects of another device
  if (!t_stage.stream2)
    GB_CUDA_TRY(cudaStreamCreateWithFlags(&t_stage.stream2, cudaStreamNonBlocking));
  for (cudaEvent_t& e : t_stage.events)
    if (!e) GB_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  *s2 = t_stage.stream2;
  *ev = t_stage.events;
  return GB_OK;
}

// ---------------------------------------------------------------- allocations
// Host-side fault injection for tests: let `g_fail_after` more allocations
// succeed, then fail the next `g_fail_count` (no GPU fault involved).
static std::mutex g_fail_mu;
static int g_fail_after = 0, g_fail_count = 0;

int dev_alloc(void** p, size_t bytes, const char* what) {
  *p = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_fail_mu);
    if (g_fail_count > 0) {
      if (g_fail_after > 0) {
        g_fail_after--;
      } else {
        g_fail_count--;
        gb_set_error(GB_ERR_NOMEM, "%s: allocation of %zu bytes failed (injected)", what, bytes);
        return GB_ERR_NOMEM;
      }
    }
  }
  const cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
  if (e != cudaSuccess) {
    *p = nullptr;
    gb_set_error(GB_ERR_NOMEM, "%s: cudaMalloc(%zu): %s", what, bytes, cudaGetErrorString(e));
    return GB_ERR_NOMEM;
  }
  return GB_OK;
}

int stage_buffer(int slot, size_t bytes, void** out) {
  if (slot < 0 || slot >= kStageSlots) {
    gb_set_error(GB_ERR_ARG, "staging slot %d out of range", slot);
    return GB_ERR_ARG;
  }
  if (bytes == 0) bytes = 16;
  if (t_stage.cap[slot] < bytes) {
    if (t_stage.buf[slot]) GB_CUDA_TRY(cudaFree(t_stage.buf[slot]));
    t_stage.buf[slot] = nullptr;
    t_stage.cap[slot] = 0;
    size_t grow = bytes + bytes / 4;
    const int rc = dev_alloc(&t_stage.buf[slot], grow, "staging buffer");
    if (rc) return rc;
    t_stage.cap[slot] = grow;
  }
  *out = t_stage.buf[slot];
  return GB_OK;
}

// ---------------------------------------------------------------- utilities
__global__ void k_zero_f32x2(float2* __restrict__ p, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = make_float2(0.f, 0.f);
}

int sm_count() {
  static int cached = 0;
  static std::once_flag once;
  std::call_once(once, [] {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    cached = n > 0 ? n : 1;
  });
  return cached;
}

static bool host_direct_device() {
  static int cached[64];
  static std::once_flag once[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
  std::call_once(once[dev], [dev] {
    int pma = 0, pmh = 0;
    cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, dev);
    cudaDeviceGetAttribute(&pmh, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev);
    const char* env = getenv("RC_GB300_HOST_DIRECT");
    cached[dev] = pma == 1 && pmh == 1 && !(env && env[0] == '0');
  });
  return cached[dev] != 0;
}

bool host_direct(const void* host, int64_t row_doubles) {
  return host && (reinterpret_cast<uintptr_t>(host) & 15) == 0 && (row_doubles & 1) == 0 &&
         host_direct_device();
}

}  // namespace gb

extern "C" int gb_grid_zero_f32(float* d_grid, int64_t n_complex, void* stream) {
  if (!d_grid || n_complex < 0) {
    gb_set_error(GB_ERR_ARG, "gb_grid_zero_f32: bad arguments");
    return GB_ERR_ARG;
  }
  if (n_complex == 0) return GB_OK;
  GB_CUDA_TRY(cudaMemsetAsync(d_grid, 0, (size_t)n_complex * 8, (cudaStream_t)stream));
  return GB_OK;
}

extern "C" int gb_host_direct(void) { return gb::host_direct_device() ? 1 : 0; }

extern "C" int gb_debug_fail_allocs(int32_t after, int32_t count) {
  if (after < 0 || count < 0) {
    gb_set_error(GB_ERR_ARG, "gb_debug_fail_allocs: negative argument");
    return GB_ERR_ARG;
  }
  std::lock_guard<std::mutex> lk(gb::g_fail_mu);
  gb::g_fail_after = after;
  gb::g_fail_count = count;
  return GB_OK;
}
