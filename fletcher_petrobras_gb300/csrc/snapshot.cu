// Output path: asynchronous snapshots of the resident fields and the RSF
// (Madagascar) slice files of original/utils.c:7-227.
//
// A snapshot unpacks (or, in the 16-bit forms, decodes) the field into a
// device buffer on the library's stream, then copies it to the host on a
// side stream, so later steps overlap the copy.  A destination that is
// page-locked (cudaHostAlloc / cudaHostRegister / FLETCHER_PinHost) is
// written by the copy itself; any other host buffer through a page-locked
// staging buffer and a host callback.  One device buffer serves every
// snapshot and slice: each use waits (on the device) for the previous copy
// out of it.
//
// The RSF writers produce the reference's files byte for byte: a text
// header `<name>.rsf` and a binary `<name>.rsf@` of native floats, x
// fastest.  A slice file is appended to step after step, from host arrays
// (FLETCHER_DumpSliceFile) or asynchronously from the resident state
// (FLETCHER_SliceAppend), and its header is written when it is closed.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/fletcher_gb300.h"
#include "fletcher_internal.h"

int flt_record_error(int code, const char *msg);

namespace flt {

// Box [x0..x1] x [y0..y1] x [z0..z1] (inclusive) of an unpitched sx*sy*sz
// volume -> compact, x fastest.
__global__ void k_gather_box(const float *__restrict__ v, float *__restrict__ out, int sx, int sy, int x0, int nx,
                             int y0, int ny, int z0, int nz) {
  const long n = (long)nx * ny * nz;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const long x = i % nx, y = (i / nx) % ny, z = i / ((long)nx * ny);
    out[i] = v[((z0 + z) * (long)sy + (y0 + y)) * sx + (x0 + x)];
  }
}

namespace {

// Two device buffers of one unpacked field each, used in turn by the
// full-field snapshots: a snapshot waits only for the copy out of the buffer
// it reuses, two snapshots back, so a copy that runs longer than the steps
// between two snapshots does not hold up the steps.  Slices use buffer 0.
struct Snap {
  cudaStream_t side = nullptr;
  float *dev[2] = {nullptr, nullptr};
  float *staging = nullptr;  // page-locked, for unregistered destinations
  size_t n = 0;
  cudaEvent_t dev_free[2] = {nullptr, nullptr}, ready = nullptr, done = nullptr;
  int next = 0;              // buffer of the next full-field snapshot
  bool inflight = false;
};
Snap S;

int err(int code, const char *msg) { return flt_record_error(code, msg); }

#define CKS(call)                                                                                       \
  do {                                                                                                  \
    cudaError_t e_ = (call);                                                                            \
    if (e_ != cudaSuccess) {                                                                            \
      cudaGetLastError(); /* not sticky: a later launch check must not see it */                        \
      char b_[256];                                                                                     \
      snprintf(b_, sizeof(b_), "%s failed: %s", #call, cudaGetErrorString(e_));                        \
      return err(e_ == cudaErrorMemoryAllocation ? FLETCHER_ERR_NOMEM : FLETCHER_ERR_CUDA, b_);         \
    }                                                                                                   \
  } while (0)

int ensure(size_t n) {
  if (!S.side) {
    CKS(cudaStreamCreateWithFlags(&S.side, cudaStreamNonBlocking));
    for (int k = 0; k < 2; ++k) CKS(cudaEventCreateWithFlags(&S.dev_free[k], cudaEventDisableTiming));
    CKS(cudaEventCreateWithFlags(&S.ready, cudaEventDisableTiming));
    CKS(cudaEventCreateWithFlags(&S.done, cudaEventDisableTiming));
  }
  if (S.n != n) {
    if (S.inflight) CKS(cudaEventSynchronize(S.done));
    for (int k = 0; k < 2; ++k) {
      if (S.dev[k]) cudaFree(S.dev[k]);
      S.dev[k] = nullptr;
    }
    if (S.staging) cudaFreeHost(S.staging);
    S.staging = nullptr;
    S.n = 0;
    for (int k = 0; k < 2; ++k) CKS(cudaMalloc(&S.dev[k], n * sizeof(float)));
    S.n = n;
    S.next = 0;
    for (int k = 0; k < 2; ++k) CKS(cudaEventRecord(S.dev_free[k], resident_stream()));
  }
  return FLETCHER_OK;
}

bool page_locked(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

struct CopyOut {
  float *dst;
  const float *src;  // staging (null: already copied into dst)
  size_t n;
  long fix_idx;
  float fix_val;
};

void CUDART_CB copy_out(void *arg) {
  CopyOut *c = static_cast<CopyOut *>(arg);
  if (c->src) memcpy(c->dst, c->src, c->n * sizeof(float));
  if (c->fix_idx >= 0) c->dst[c->fix_idx] = c->dst[c->fix_idx] + c->fix_val;
  delete c;
}

}  // namespace

void snapshot_release() {
  if (S.side) cudaStreamSynchronize(S.side);
  for (int k = 0; k < 2; ++k) {
    if (S.dev[k]) cudaFree(S.dev[k]);
    S.dev[k] = nullptr;
  }
  if (S.staging) cudaFreeHost(S.staging);
  S.staging = nullptr;
  S.n = 0;
  S.inflight = false;
}

}  // namespace flt

using namespace flt;

// ---- snapshots ------------------------------------------------------------------

extern "C" int FLETCHER_SnapshotBegin(int which, float *host) {
  const size_t n = resident_cells();
  if (!n) return err(FLETCHER_ERR_ARGS, "FLETCHER_SnapshotBegin before DRIVER_Initialize");
  if (!host || which < 0 || which > 3) return err(FLETCHER_ERR_ARGS, "FLETCHER_SnapshotBegin: bad arguments");
  if (ensure(n)) return FLETCHER_GetLastError();
  cudaStream_t s = resident_stream();
  const int k = S.next;
  S.next ^= 1;
  // The copy out of this buffer two snapshots back must be done before it
  // is overwritten (a device-side wait; the host does not block).
  CKS(cudaStreamWaitEvent(s, S.dev_free[k], 0));
  long fix_idx = -1;
  float fix_val = 0.f;
  if (resident_field_to_device(which, S.dev[k], &fix_idx, &fix_val)) return FLETCHER_GetLastError();
  CKS(cudaEventRecord(S.ready, s));
  CKS(cudaStreamWaitEvent(S.side, S.ready, 0));
  CopyOut *c = new CopyOut{host, nullptr, n, fix_idx, fix_val};
  if (page_locked(host)) {
    CKS(cudaMemcpyAsync(host, S.dev[k], n * sizeof(float), cudaMemcpyDeviceToHost, S.side));
  } else {
    // One staging buffer: the side stream runs its copies and host-side
    // copy-outs in order, so a staging copy never overtakes the last one.
    if (!S.staging) CKS(cudaHostAlloc(&S.staging, n * sizeof(float), cudaHostAllocDefault));
    CKS(cudaMemcpyAsync(S.staging, S.dev[k], n * sizeof(float), cudaMemcpyDeviceToHost, S.side));
    c->src = S.staging;
  }
  CKS(cudaEventRecord(S.dev_free[k], S.side));
  if (c->src || c->fix_idx >= 0) {
    CKS(cudaLaunchHostFunc(S.side, copy_out, c));
  } else {
    delete c;
  }
  CKS(cudaEventRecord(S.done, S.side));
  S.inflight = true;
  return FLETCHER_OK;
}

extern "C" int FLETCHER_SnapshotWait(void) {
  if (!S.inflight) return FLETCHER_OK;
  CKS(cudaEventSynchronize(S.done));
  S.inflight = false;
  return FLETCHER_OK;
}

extern "C" int FLETCHER_PinHost(void *ptr, size_t bytes) {
  if (!ptr || !bytes) return err(FLETCHER_ERR_ARGS, "FLETCHER_PinHost: bad arguments");
  CKS(cudaHostRegister(ptr, bytes, cudaHostRegisterDefault));
  return FLETCHER_OK;
}

extern "C" int FLETCHER_UnpinHost(void *ptr) {
  if (!ptr) return err(FLETCHER_ERR_ARGS, "FLETCHER_UnpinHost: bad arguments");
  CKS(cudaHostUnregister(ptr));
  return FLETCHER_OK;
}

// ---- RSF files (original/utils.c:7-227) ----------------------------------------

struct FletcherSlice {
  int dir;  // 0 x-slice, 1 y-slice, 2 z-slice, 3 full section (original/utils.h: XSLICE..FULL)
  int x0, x1, y0, y1, z0, z1;
  int itCnt;
  float dx, dy, dz, dt;
  FILE *head, *bin;
  char headName[160], binName[168];
  // asynchronous appends
  float *dev = nullptr, *staging = nullptr;
  size_t count = 0;
  cudaEvent_t dev_free = nullptr;
};

namespace {
struct SliceWrite {
  FletcherSlice *s;
};
void CUDART_CB slice_write(void *arg) {
  FletcherSlice *s = static_cast<SliceWrite *>(arg)->s;
  fwrite(s->staging, sizeof(float), s->count, s->bin);
  s->itCnt++;
  delete static_cast<SliceWrite *>(arg);
}

// Rows of the box of an sx*sy*sz host array, x fastest (the reference's
// fwrite loop, one row per call).
void write_box(FILE *f, const float *a, int sx, int sy, int x0, int x1, int y0, int y1, int z0, int z1) {
  for (int iz = z0; iz <= z1; iz++)
    for (int iy = y0; iy <= y1; iy++)
      fwrite(a + ((long)iz * sy + iy) * sx + x0, sizeof(float), (size_t)(x1 - x0 + 1), f);
}

bool box_ok(int sx, int sy, int sz, int x0, int x1, int y0, int y1, int z0, int z1) {
  return x0 >= 0 && x0 <= x1 && x1 < sx && y0 >= 0 && y0 <= y1 && y1 < sy && z0 >= 0 && z0 <= z1 && z1 < sz;
}
}  // namespace

extern "C" int FLETCHER_DumpFieldToFile(int sx, int sy, int sz, int ixStart, int ixEnd, int iyStart, int iyEnd,
                                        int izStart, int izEnd, float d1, float d2, float d3, const float *arr,
                                        const char *fName) {
  if (!arr || !fName || strlen(fName) > 120 || !box_ok(sx, sy, sz, ixStart, ixEnd, iyStart, iyEnd, izStart, izEnd))
    return err(FLETCHER_ERR_ARGS, "FLETCHER_DumpFieldToFile: bad arguments");
  char head[160], bin[168];
  snprintf(head, sizeof(head), "%s.rsf", fName);
  snprintf(bin, sizeof(bin), "%s@", head);
  FILE *fp = fopen(head, "w+");
  if (!fp) return err(FLETCHER_ERR_ARGS, "FLETCHER_DumpFieldToFile: cannot create the header file");
  fprintf(fp, "in=\"./%s\"\n", bin);
  fprintf(fp, "data_format=\"native_float\"\n");
  fprintf(fp, "esize=%lu\n", (unsigned long)sizeof(float));
  fprintf(fp, "n1=%d\n", ixEnd - ixStart + 1);
  fprintf(fp, "d1=%f\n", d1);
  fprintf(fp, "n2=%d\n", iyEnd - iyStart + 1);
  fprintf(fp, "d2=%f\n", d2);
  fprintf(fp, "n3=%d\n", izEnd - izStart + 1);
  fprintf(fp, "d3=%f\n", d3);
  fclose(fp);
  fp = fopen(bin, "w+b");
  if (!fp) return err(FLETCHER_ERR_ARGS, "FLETCHER_DumpFieldToFile: cannot create the binary file");
  write_box(fp, arr, sx, sy, ixStart, ixEnd, iyStart, iyEnd, izStart, izEnd);
  fclose(fp);
  return FLETCHER_OK;
}

extern "C" FletcherSlice *FLETCHER_OpenSliceFile(int ixStart, int ixEnd, int iyStart, int iyEnd, int izStart,
                                                 int izEnd, float dx, float dy, float dz, float dt,
                                                 const char *fName) {
  if (!fName || strlen(fName) > 120 || ixStart > ixEnd || iyStart > iyEnd || izStart > izEnd || ixStart < 0 ||
      iyStart < 0 || izStart < 0) {
    err(FLETCHER_ERR_ARGS, "FLETCHER_OpenSliceFile: bad arguments");
    return nullptr;
  }
  FletcherSlice *s = new FletcherSlice();
  s->dir = ixStart == ixEnd ? 0 : (iyStart == iyEnd ? 1 : (izStart == izEnd ? 2 : 3));
  s->x0 = ixStart; s->x1 = ixEnd; s->y0 = iyStart; s->y1 = iyEnd; s->z0 = izStart; s->z1 = izEnd;
  s->itCnt = 0;
  s->dx = dx; s->dy = dy; s->dz = dz; s->dt = dt;
  snprintf(s->headName, sizeof(s->headName), "%s.rsf", fName);
  snprintf(s->binName, sizeof(s->binName), "./%s@", s->headName);
  s->head = fopen(s->headName, "w+");
  s->bin = fopen(s->binName, "w+");
  if (!s->head || !s->bin) {
    if (s->head) fclose(s->head);
    if (s->bin) fclose(s->bin);
    delete s;
    err(FLETCHER_ERR_ARGS, "FLETCHER_OpenSliceFile: cannot create the files");
    return nullptr;
  }
  s->count = (size_t)(ixEnd - ixStart + 1) * (iyEnd - iyStart + 1) * (izEnd - izStart + 1);
  return s;
}

extern "C" int FLETCHER_DumpSliceFile(int sx, int sy, int sz, const float *arr, FletcherSlice *s) {
  if (!s || !arr || !box_ok(sx, sy, sz, s->x0, s->x1, s->y0, s->y1, s->z0, s->z1))
    return err(FLETCHER_ERR_ARGS, "FLETCHER_DumpSliceFile: bad arguments");
  if (s->dev) CKS(cudaStreamSynchronize(S.side));  // keep the order of earlier asynchronous appends
  write_box(s->bin, arr, sx, sy, s->x0, s->x1, s->y0, s->y1, s->z0, s->z1);
  s->itCnt++;
  return FLETCHER_OK;
}

extern "C" int FLETCHER_SliceAppend(FletcherSlice *s, int which) {
  const size_t n = resident_cells();
  if (!s) return err(FLETCHER_ERR_ARGS, "FLETCHER_SliceAppend: no slice");
  if (!n) return err(FLETCHER_ERR_ARGS, "FLETCHER_SliceAppend before DRIVER_Initialize");
  int sx = 0, sy = 0, sz = 0;
  resident_dims(&sx, &sy, &sz);
  if (!box_ok(sx, sy, sz, s->x0, s->x1, s->y0, s->y1, s->z0, s->z1))
    return err(FLETCHER_ERR_ARGS, "FLETCHER_SliceAppend: the slice box lies outside the grid");
  if (ensure(n)) return FLETCHER_GetLastError();
  if (!s->dev) {
    CKS(cudaMalloc(&s->dev, s->count * sizeof(float)));
    CKS(cudaHostAlloc(&s->staging, s->count * sizeof(float), cudaHostAllocDefault));
    CKS(cudaEventCreateWithFlags(&s->dev_free, cudaEventDisableTiming));
    CKS(cudaEventRecord(s->dev_free, resident_stream()));
  }
  cudaStream_t st = resident_stream();
  CKS(cudaStreamWaitEvent(st, S.dev_free[0], 0));
  CKS(cudaStreamWaitEvent(st, s->dev_free, 0));
  long fi;
  float fv;
  if (resident_field_to_device(which, S.dev[0], &fi, &fv)) return FLETCHER_GetLastError();
  const int nx = s->x1 - s->x0 + 1, ny = s->y1 - s->y0 + 1, nz = s->z1 - s->z0 + 1;
  long blocks = ((long)s->count + 255) / 256;
  k_gather_box<<<(int)(blocks < 4096 ? blocks : 4096), 256, 0, st>>>(S.dev[0], s->dev, sx, sy, s->x0, nx, s->y0,
                                                                     ny, s->z0, nz);
  CKS(cudaGetLastError());
  CKS(cudaEventRecord(S.dev_free[0], st));
  CKS(cudaEventRecord(S.ready, st));
  CKS(cudaStreamWaitEvent(S.side, S.ready, 0));
  CKS(cudaMemcpyAsync(s->staging, s->dev, s->count * sizeof(float), cudaMemcpyDeviceToHost, S.side));
  CKS(cudaEventRecord(s->dev_free, S.side));
  if (fi >= 0) {
    // The cell whose stored value lacks a pending source, if it is in the box.
    const long fx = fi % sx, fy = (fi / sx) % sy, fz = fi / ((long)sx * sy);
    if (fx >= s->x0 && fx <= s->x1 && fy >= s->y0 && fy <= s->y1 && fz >= s->z0 && fz <= s->z1) {
      const long k = ((fz - s->z0) * (long)ny + (fy - s->y0)) * nx + (fx - s->x0);
      CopyOut *c = new CopyOut{s->staging, nullptr, 0, k, fv};
      CKS(cudaLaunchHostFunc(S.side, copy_out, c));
    }
  }
  CKS(cudaLaunchHostFunc(S.side, slice_write, new SliceWrite{s}));
  CKS(cudaEventRecord(S.done, S.side));
  S.inflight = true;
  return FLETCHER_OK;
}

extern "C" int FLETCHER_CloseSliceFile(FletcherSlice *s) {
  if (!s) return err(FLETCHER_ERR_ARGS, "FLETCHER_CloseSliceFile: no slice");
  if (s->dev && S.side) cudaStreamSynchronize(S.side);
  FILE *h = s->head;
  fprintf(h, "in=\"%s\"\n", s->binName);
  fprintf(h, "data_format=\"native_float\"\n");
  fprintf(h, "esize=%lu\n", (unsigned long)sizeof(float));
  const int nx = s->x1 - s->x0 + 1, ny = s->y1 - s->y0 + 1, nz = s->z1 - s->z0 + 1;
  switch (s->dir) {
    case 0:
      fprintf(h, "n1=%d\nn2=%d\nn3=%d\n", ny, nz, s->itCnt);
      fprintf(h, "d1=%f\nd2=%f\nd3=%f\n", s->dy, s->dz, s->dt);
      break;
    case 1:
      fprintf(h, "n1=%d\nn2=%d\nn3=%d\n", nx, nz, s->itCnt);
      fprintf(h, "d1=%f\nd2=%f\nd3=%f\n", s->dx, s->dz, s->dt);
      break;
    case 2:
      fprintf(h, "n1=%d\nn2=%d\nn3=%d\n", nx, ny, s->itCnt);
      fprintf(h, "d1=%f\nd2=%f\nd3=%f\n", s->dx, s->dy, s->dt);
      break;
    default:
      fprintf(h, "n1=%d\nn2=%d\nn3=%d\nn4=%d\n", nx, ny, nz, s->itCnt);
      fprintf(h, "d1=%f\nd2=%f\nd3=%f\nd4=%f\n", s->dx, s->dy, s->dz, s->dt);
      break;
  }
  fclose(s->head);
  fclose(s->bin);
  if (s->dev) cudaFree(s->dev);
  if (s->staging) cudaFreeHost(s->staging);
  if (s->dev_free) cudaEventDestroy(s->dev_free);
  delete s;
  return FLETCHER_OK;
}

extern "C" int FLETCHER_SliceFrames(const FletcherSlice *s) { return s ? s->itCnt : -1; }

extern "C" int FLETCHER_DumpSliceSummary(int sx, int sy, int sz, const FletcherSlice *s, float dt, int it,
                                         const float *arr, float src) {
  if (!s || !arr || !box_ok(sx, sy, sz, s->x0, s->x1, s->y0, s->y1, s->z0, s->z1))
    return err(FLETCHER_ERR_ARGS, "FLETCHER_DumpSliceSummary: bad arguments");
  float mx = arr[((long)s->z0 * sy + s->y0) * sx + s->x0], mn = mx;
  for (int iz = s->z0; iz <= s->z1; iz++)
    for (int iy = s->y0; iy <= s->y1; iy++)
      for (int ix = s->x0; ix <= s->x1; ix++) {
        const float v = arr[((long)iz * sy + iy) * sx + ix];
        mx = fmaxf(mx, v);
        mn = fminf(mn, v);
      }
  printf("Slice of %s at iteration; %5.5d; time(s); %f; max; %9.2e; min; %9.2e; src; %9.2e;\n", s->headName, it,
         dt * (float)it, mx, mn, src);
  return FLETCHER_OK;
}
