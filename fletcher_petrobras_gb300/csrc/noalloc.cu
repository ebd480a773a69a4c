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
// overlaps on the GPU (on different streams) race on it.
#include <cuda_runtime.h>
#include <stdio.h>

#include "../../include/fletcher_gb300.h"

int flt_record_error(int code, const char *msg);

namespace {

static __device__ __align__(256) float g_stage[FLETCHER_NOALLOC_MAX_CELLS];

constexpr int kMaxDevices = 64;
float *g_stage_addr[kMaxDevices] = {nullptr};  // device address of g_stage, per device

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
  // First call on this device: find the array's device address (host code
  // cannot use the symbol itself as a device pointer).
  if (!g_stage_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_stage);
    if (e != cudaSuccess) return err(FLETCHER_ERR_CUDA, "cudaGetSymbolAddress", e);
    g_stage_addr[dev] = static_cast<float *>(p);
  }
  float *stage = g_stage_addr[dev];
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
