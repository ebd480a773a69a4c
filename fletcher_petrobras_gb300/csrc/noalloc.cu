// Field read-back that allocates nothing: FLETCHER_ReadFieldNoAlloc.
//
// Who needs it: a caller that owns all device memory itself -- a seismic
// imaging or inversion code that reserves the whole GPU for its wavefields
// and coefficient volumes up front (at 504^3 those alone are 11+ GB), or
// that runs its time loop where a new cudaMalloc would fail or would stall
// the stream -- and that still wants p or q of a (p, q) pair volume on the
// host.  The regular read-back (FLETCHER_GetField) stages through a full
// volume the library allocated; this one stages through a fixed array that
// is part of the library image instead.
//
// Scratch: `g_stage`, a file-scope __device__ array of
// FLETCHER_NOALLOC_MAX_CELLS floats (16 MiB).  Every GPU that loads the
// library holds it until the process exits.  A grid with more cells than
// that is rejected.  All calls share the array: two calls whose work
// overlaps on the GPU (from concurrent host threads, or on different
// streams) race on it.
//
// Ordering: the unpack runs on FLETCHER_GetStream().  The caller's writes to
// the pair volume must be ordered before it: issued on that stream (name the
// caller's stream with FLETCHER_SetStream) or complete before the call.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdio.h>

#include "../../include/fletcher_gb300.h"

int flt_record_error(int code, const char *msg);

namespace {

static __device__ __align__(256) float g_stage[FLETCHER_NOALLOC_MAX_CELLS];

constexpr int kMaxDevices = 64;

// Device address of g_stage, looked up once per device and context: a
// context that was reset (cudaDeviceReset) reloads the module, so the
// address is looked up again when the current context's id changes.
struct StageAddr {
  unsigned long long ctx_id;
  float *addr;
};
StageAddr g_stage_addr[kMaxDevices] = {};

typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

// Unique id of the calling thread's current context (0 if unknown).
unsigned long long current_context_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(p);
    looked_up = true;
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current && get_id && get_current(&ctx) == CUDA_SUCCESS && ctx && get_id(ctx, &id) == CUDA_SUCCESS)
    return id;
  return 0;
}

// One component of a pitched (p, q) pair volume -> `stage` (unpitched).
__global__ void k_unpack_to_stage(const float2 *__restrict__ pairs, float *__restrict__ stage, int comp, int sx,
                                  int sy, int sz, int pitch) {
  const size_t n = (size_t)sx * sy * sz;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t x = i % sx, yz = i / sx;
    const float2 v = pairs[yz * pitch + x];
    stage[i] = comp ? v.y : v.x;
  }
}

int err(int code, const char *what, cudaError_t e) {
  char msg[256];
  snprintf(msg, sizeof(msg), "FLETCHER_ReadFieldNoAlloc: %s%s%s", what, e == cudaSuccess ? "" : ": ",
           e == cudaSuccess ? "" : cudaGetErrorString(e));
  return flt_record_error(code, msg);
}

}  // namespace

extern "C" int FLETCHER_ReadFieldNoAlloc(const void *dev_pairs, int sx, int sy, int sz, int pitch, int comp,
                                         float *host_out) {
  if (!dev_pairs || !host_out) return err(FLETCHER_ERR_ARGS, "null pointer", cudaSuccess);
  if (sx <= 0 || sy <= 0 || sz <= 0 || pitch < sx || (comp != 0 && comp != 1))
    return err(FLETCHER_ERR_ARGS, "bad sizes, pitch or component", cudaSuccess);
  const size_t n = (size_t)sx * sy * sz;
  if (n > (size_t)FLETCHER_NOALLOC_MAX_CELLS) {
    char msg[160];
    snprintf(msg, sizeof(msg), "grid of %zu cells exceeds the %u-cell staging array", n,
             (unsigned)FLETCHER_NOALLOC_MAX_CELLS);
    return err(FLETCHER_ERR_ARGS, msg, cudaSuccess);
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return err(FLETCHER_ERR_CUDA, "cudaGetDevice", e);
  if (dev < 0 || dev >= kMaxDevices) return err(FLETCHER_ERR_ARGS, "device ordinal out of range", cudaSuccess);
  // First call on this device (or in a new context of it): find the array's
  // device address (host code cannot use the symbol itself as a device
  // pointer).  cudaSetDevice makes the device's primary context current
  // first (it initialises the context since CUDA 12).
  e = cudaSetDevice(dev);
  if (e != cudaSuccess) return err(FLETCHER_ERR_CUDA, "cudaSetDevice", e);
  const unsigned long long ctx = current_context_id();
  if (!g_stage_addr[dev].addr || ctx == 0 || g_stage_addr[dev].ctx_id != ctx) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_stage);
    if (e != cudaSuccess) return err(FLETCHER_ERR_CUDA, "cudaGetSymbolAddress", e);
    g_stage_addr[dev].addr = static_cast<float *>(p);
    g_stage_addr[dev].ctx_id = ctx;
  }
  float *stage = g_stage_addr[dev].addr;
  cudaStream_t s = static_cast<cudaStream_t>(FLETCHER_GetStream());
  const int grid = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
  k_unpack_to_stage<<<grid, 256, 0, s>>>(static_cast<const float2 *>(dev_pairs), stage, comp, sx, sy, sz, pitch);
  e = cudaGetLastError();
  if (e != cudaSuccess) return err(FLETCHER_ERR_CUDA, "unpack kernel launch", e);
  e = cudaMemcpyAsync(host_out, stage, n * sizeof(float), cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return err(FLETCHER_ERR_CUDA, "device-to-host copy", e);
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return err(FLETCHER_ERR_CUDA, "stream synchronisation", e);
  return FLETCHER_OK;
}
