// ORACLE -- measurement infrastructure only (not part of the library).
//
// Times the reference's own CUDA back-end kernel (kernel_Propagate of
// original/CUDA/cuda_propagate.cu, compiled unmodified for sm_103a into
// oracle/_ref/ref_propagate.cubin by `make -C oracle ref_cuda`) on this GPU,
// launched as original/CUDA/cuda_propagate.cu:64-75 launches it: 16 x 16
// blocks over (sx/16, sy/16), one step per launch, buffers rotated between
// steps.  Its accesses stay inside the arrays for bord >= 4 and sx, sy
// multiples of 16 (the z loop runs over [bord+1, sz-bord-1)), which this
// program checks before any launch.
//
//   nvcc -O2 -o oracle/_build/ref_cuda_bench oracle/ref_cuda_bench.cu -lcuda
//   oracle/_build/ref_cuda_bench oracle/_ref/ref_propagate.cubin SX SY SZ BORD STEPS WARMUP
//
// Coefficients hold one homogeneous TTI medium and the fields start at zero:
// the kernel has no data-dependent branch, so its time does not depend on
// the values.  Prints one JSON line: ms per step and MSamples/s by the
// reference's definition (original/model.c:44, (sx-2 bord)(sy-2 bord)(sz-2 bord)
// cells per step).
#include <cuda.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define CK(x)                                                                  \
  do {                                                                         \
    CUresult r_ = (x);                                                         \
    if (r_ != CUDA_SUCCESS) {                                                  \
      const char *s_ = nullptr;                                                \
      cuGetErrorString(r_, &s_);                                               \
      fprintf(stderr, "%s failed: %s\n", #x, s_ ? s_ : "?");                   \
      return 1;                                                                \
    }                                                                          \
  } while (0)

int main(int argc, char **argv) {
  if (argc < 8) {
    fprintf(stderr, "usage: %s cubin sx sy sz bord steps warmup\n", argv[0]);
    return 2;
  }
  const char *cubin = argv[1];
  int sx = atoi(argv[2]), sy = atoi(argv[3]), sz = atoi(argv[4]), bord = atoi(argv[5]);
  const int steps = atoi(argv[6]), warmup = atoi(argv[7]);
  if (bord < 4 || sx % 16 || sy % 16 || sz <= 2 * bord + 2 || steps < 1) {
    fprintf(stderr, "refused: needs bord >= 4, sx and sy multiples of 16, sz > 2 bord + 2\n");
    return 2;
  }
  CK(cuInit(0));
  CUdevice dev;
  CK(cuDeviceGet(&dev, 0));
  CUcontext ctx;
  CK(cuDevicePrimaryCtxRetain(&ctx, dev));
  CK(cuCtxSetCurrent(ctx));
  CUmodule mod;
  CK(cuModuleLoad(&mod, cubin));
  unsigned int nf = 0;
  CK(cuModuleGetFunctionCount(&nf, mod));
  CUfunction fns[16], kern = nullptr;
  if (nf > 16) nf = 16;
  CK(cuModuleEnumerateFunctions(fns, nf, mod));
  for (unsigned i = 0; i < nf; ++i) {
    const char *name = nullptr;
    CK(cuFuncGetName(&name, fns[i]));
    if (name && strstr(name, "kernel_Propagate")) kern = fns[i];
  }
  if (!kern) {
    fprintf(stderr, "kernel_Propagate not found in %s\n", cubin);
    return 1;
  }
  const size_t n = (size_t)sx * sy * sz;
  // ch1dxx ch1dyy ch1dzz ch1dxy ch1dyz ch1dxz v2px v2pz v2sz v2pn (a homogeneous TTI medium)
  const float cval[10] = {0.2165f, 0.0722f, 0.5f, 0.25f, 0.433f, 0.75f, 1.332e7f, 9.0e6f, 2.25e6f, 1.08e7f};
  CUdeviceptr coef[10], f[4];
  for (int k = 0; k < 10; ++k) {
    CK(cuMemAlloc(&coef[k], n * sizeof(float)));
    unsigned bits;
    memcpy(&bits, &cval[k], 4);
    CK(cuMemsetD32(coef[k], bits, n));
  }
  for (int k = 0; k < 4; ++k) {
    CK(cuMemAlloc(&f[k], n * sizeof(float)));
    CK(cuMemsetD32(f[k], 0u, n));
  }
  float dx = 12.5f, dy = 12.5f, dz = 12.5f, dt = 0.0006f;
  CUdeviceptr pp = f[0], pc = f[1], qp = f[2], qc = f[3];
  CUevent e0, e1;
  CK(cuEventCreate(&e0, CU_EVENT_DEFAULT));
  CK(cuEventCreate(&e1, CU_EVENT_DEFAULT));
  auto launch = [&](int it) -> CUresult {
    void *args[] = {&sx, &sy, &sz, &bord, &dx, &dy, &dz, &dt, &it, &coef[0], &coef[1], &coef[2], &coef[3],
                    &coef[4], &coef[5], &coef[6], &coef[7], &coef[8], &coef[9], &pp, &pc, &qp, &qc};
    CUresult r = cuLaunchKernel(kern, sx / 16, sy / 16, 1, 16, 16, 1, 0, nullptr, args, nullptr);
    CUdeviceptr t = pp;
    pp = pc;
    pc = t;
    t = qp;
    qp = qc;
    qc = t;
    return r;
  };
  for (int it = 1; it <= warmup; ++it) CK(launch(it));
  CK(cuCtxSynchronize());
  CK(cuEventRecord(e0, nullptr));
  for (int it = 1; it <= steps; ++it) CK(launch(it));
  CK(cuEventRecord(e1, nullptr));
  CK(cuEventSynchronize(e1));
  float ms = 0.f;
  CK(cuEventElapsedTime(&ms, e0, e1));
  const double cells = (double)(sx - 2 * bord) * (sy - 2 * bord) * (sz - 2 * bord);
  printf("{\"kernel\": \"reference kernel_Propagate (original/CUDA/cuda_propagate.cu), sm_103a\", \"grid\": [%d, %d, %d], "
         "\"bord\": %d, \"steps\": %d, \"ms_per_step\": %.4f, \"msamples\": %.1f}\n",
         sx, sy, sz, bord, steps, ms / steps, cells * steps / (ms / 1e3) / 1e6);
  for (int k = 0; k < 10; ++k) cuMemFree(coef[k]);
  for (int k = 0; k < 4; ++k) cuMemFree(f[k]);
  cuModuleUnload(mod);
  cuDevicePrimaryCtxRelease(dev);
  return 0;
}
