/*
 * ORACLE -- test infrastructure only.
 *
 * Harness around the reference's own, unmodified canonical tree: it is
 * compiled together with original/{boundary,source,utils,map,walltime,model}.c
 * and original/OpenMP/*.c (see oracle/Makefile) into oracle/_ref/, where it
 * runs the reference's FP32 OpenMP path on arrays the caller prepares.
 * Nothing in the product uses it; the golden fixtures under tests/golden/
 * are its outputs.
 *
 * Entry points (ctypes from tests/golden/make_golden.py, or the ref_cli
 * executable built from this file with -DREF_CLI):
 *   ref_boundary    srand(seed) + RandomVelocityBoundary (original/boundary.c:7-98)
 *   ref_precompute  precomp.h MODEL_INITIALIZE (original/precomp.h:14-58)
 *   ref_source      Source (original/source.c:7-15, FCUT = 40)
 *   ref_run         the Model() time loop (original/model.c:71-88) driving the
 *                   reference's DRIVER_* OpenMP back-end, with a source cut
 *                   frequency parameter (the reference's own Source() when
 *                   fcut == 40)
 *   ref_model       the reference's Model() itself (FCUT = 40 only)
 */
#include <stdio.h>
#include <stdlib.h>
#include <math.h>
#include <string.h>
#include "map.h"
#include "boundary.h"
#include "source.h"
#include "utils.h"
#include "driver.h"
#include "model.h"

/* The coefficient globals are defined by the reference's model.c
 * (MODEL_GLOBALVARS); the OpenMP back-end reads them. */
extern float *ch1dxx, *ch1dyy, *ch1dzz, *ch1dxy, *ch1dyz, *ch1dxz, *v2px, *v2pz, *v2sz, *v2pn;

void ref_boundary(int sx, int sy, int sz, int nx, int ny, int nz, int bord, int absorb,
                  float *vpz, float *vsv, unsigned seed) {
  srand(seed);
  RandomVelocityBoundary(sx, sy, sz, nx, ny, nz, bord, absorb, vpz, vsv);
}

static void precompute_globals(int sx, int sy, int sz, int bord, float *vpz, float *vsv,
                               float *epsilon, float *delta, float *phi, float *theta) {
#define MODEL_INITIALIZE
#include "precomp.h"
#undef MODEL_INITIALIZE
  (void)bord;
}

static void free_globals(void) {
  free(ch1dxx); free(ch1dyy); free(ch1dzz); free(ch1dxy); free(ch1dyz); free(ch1dxz);
  free(v2px); free(v2pz); free(v2sz); free(v2pn);
  ch1dxx = ch1dyy = ch1dzz = ch1dxy = ch1dyz = ch1dxz = v2px = v2pz = v2sz = v2pn = NULL;
}

/* out: 10 arrays of sx*sy*sz floats in the order
 * ch1dxx ch1dyy ch1dzz ch1dxy ch1dyz ch1dxz v2px v2pz v2sz v2pn. */
void ref_precompute(int sx, int sy, int sz, int bord, float *vpz, float *vsv, float *epsilon,
                    float *delta, float *phi, float *theta, float *out) {
  const long n = (long)sx * sy * sz;
  precompute_globals(sx, sy, sz, bord, vpz, vsv, epsilon, delta, phi, theta);
  float *src[10] = {ch1dxx, ch1dyy, ch1dzz, ch1dxy, ch1dyz, ch1dxz, v2px, v2pz, v2sz, v2pn};
  for (int c = 0; c < 10; c++) memcpy(out + c * n, src[c], n * sizeof(float));
  free_globals();
}

float ref_source(float dt, int it) { return Source(dt, it); }

/* Source with a cut frequency other than the compiled-in FCUT: the same
 * formula as original/source.c:7-15. */
static float source_fcut(float dt, int it, double fcut) {
  float tf, fc, fct, expo;
  tf = TWOSQRTPI / fcut;
  fc = fcut / THREESQRTPI;
  fct = fc * (((float)it) * dt - tf);
  expo = PICUBE * fct * fct;
  return ((1.0f - 2.0f * expo) * expf(-expo));
}

/* Returns 1 when the final current field is in the caller's pp/qp. */
int ref_run(int sx, int sy, int sz, int bord, float dx, float dy, float dz, float dt, int st,
            int iSource, double fcut, float *vpz, float *vsv, float *epsilon, float *delta,
            float *phi, float *theta, float *pp, float *pc, float *qp, float *qc) {
  precompute_globals(sx, sy, sz, bord, vpz, vsv, epsilon, delta, phi, theta);
  DRIVER_Initialize(sx, sy, sz, bord, dx, dy, dz, dt, vpz, vsv, epsilon, delta, phi, theta, pp,
                    pc, qp, qc);
  float *p0 = pp;
  for (int it = 1; it <= st; it++) {
    float src = (fcut == FCUT) ? Source(dt, it - 1) : source_fcut(dt, it - 1, fcut);
    DRIVER_InsertSource(dt, it - 1, iSource, pc, qc, src);
    DRIVER_Propagate(sx, sy, sz, bord, dx, dy, dz, dt, it, pp, pc, qp, qc);
    SwapArrays(&pp, &pc, &qp, &qc);
  }
  DRIVER_Finalize();
  free_globals();
  return pc == p0;
}

/* The reference's Model() (prints its report and writes Report.csv in the
 * working directory).  Returns 1 when the final current field is in pp/qp. */
int ref_model(int st, int iSource, int sx, int sy, int sz, int bord, float dx, float dy, float dz,
              float dt, float *vpz, float *vsv, float *epsilon, float *delta, float *phi,
              float *theta, float *pp, float *pc, float *qp, float *qc) {
  SlicePtr sPtr = NULL;
  Model(st, iSource, 0.01f, sPtr, sx, sy, sz, bord, dx, dy, dz, dt, 0, pp, pc, qp, qc, vpz, vsv,
        epsilon, delta, phi, theta);
  return st & 1;
}

#ifdef REF_CLI
/*
 * ref_cli IN OUT sx sy sz nx ny nz bord absorb dx dy dz dt st ix iy iz fcut seed stride
 * IN holds vpz vsv epsilon delta phi theta (sx*sy*sz float32 each, before
 * the boundary); OUT receives the final current p then q, subsampled every
 * `stride` cells in x, y and z (stride 1 = full fields), followed by the
 * per-z-plane sums of p*p and q*q (double, full resolution), and prints
 * the reference's MSamples/s for the run.
 */
#include <sys/time.h>
static double now(void) { struct timeval tv; gettimeofday(&tv, NULL); return tv.tv_sec + 1e-6 * tv.tv_usec; }
int main(int argc, char **argv) {
  if (argc < 22) { fprintf(stderr, "usage: ref_cli IN OUT sx sy sz nx ny nz bord absorb dx dy dz dt st ix iy iz fcut seed stride\n"); return 2; }
  const char *fin = argv[1], *fout = argv[2];
  int sx = atoi(argv[3]), sy = atoi(argv[4]), sz = atoi(argv[5]);
  int nx = atoi(argv[6]), ny = atoi(argv[7]), nz = atoi(argv[8]);
  int bord = atoi(argv[9]), absorb = atoi(argv[10]);
  float dx = atof(argv[11]), dy = atof(argv[12]), dz = atof(argv[13]), dt = atof(argv[14]);
  int st = atoi(argv[15]), ix = atoi(argv[16]), iy = atoi(argv[17]), iz = atoi(argv[18]);
  double fcut = atof(argv[19]);
  unsigned seed = (unsigned)strtoul(argv[20], NULL, 10);
  int stride = atoi(argv[21]);
  const long n = (long)sx * sy * sz;
  float *a[6];
  FILE *f = fopen(fin, "rb");
  if (!f) { perror(fin); return 1; }
  for (int k = 0; k < 6; k++) {
    a[k] = (float *)malloc(n * sizeof(float));
    if (fread(a[k], sizeof(float), n, f) != (size_t)n) { fprintf(stderr, "short read\n"); return 1; }
  }
  fclose(f);
  ref_boundary(sx, sy, sz, nx, ny, nz, bord, absorb, a[0], a[1], seed);
  float *pp = calloc(n, 4), *pc = calloc(n, 4), *qp = calloc(n, 4), *qc = calloc(n, 4);
  const int iSource = (iz * sy + iy) * sx + ix;
  double t0 = now();
  int odd = ref_run(sx, sy, sz, bord, dx, dy, dz, dt, st, iSource, fcut, a[0], a[1], a[2], a[3], a[4], a[5], pp, pc, qp, qc);
  double t1 = now();
  float *P = odd ? pp : pc, *Q = odd ? qp : qc;
  f = fopen(fout, "wb");
  for (int which = 0; which < 2; which++) {
    float *F = which ? Q : P;
    for (int z = 0; z < sz; z += stride)
      for (int y = 0; y < sy; y += stride)
        for (int x = 0; x < sx; x += stride) fwrite(&F[((long)z * sy + y) * sx + x], 4, 1, f);
  }
  for (int which = 0; which < 2; which++) {
    float *F = which ? Q : P;
    for (int z = 0; z < sz; z++) {
      double s = 0.0;
      for (long i = (long)z * sx * sy; i < (long)(z + 1) * sx * sy; i++) s += (double)F[i] * F[i];
      fwrite(&s, 8, 1, f);
    }
  }
  fclose(f);
  const double samples = (double)(sx - 2 * bord) * (sy - 2 * bord) * (sz - 2 * bord) * st;
  printf("ref_cli: %d steps in %.3f s, %.1f MSamples/s\n", st, t1 - t0, 1e-6 * samples / (t1 - t0));
  return 0;
}
#endif
