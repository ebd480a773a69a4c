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
#include "walltime.h"

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

/* The Model() time loop (original/model.c:71-88) over the reference's
 * DRIVER_* OpenMP back-end, with a source cut-frequency parameter.  The
 * timed region is the reference's own: wtime() around DRIVER_Propagate and
 * SwapArrays (original/model.c:82-88), summed over the steps after the first
 * `warmup` ones into *prop_seconds (may be NULL).  Returns 1 when the final
 * current field is in the caller's pp/qp. */
int ref_run_timed(int sx, int sy, int sz, int bord, float dx, float dy, float dz, float dt, int st,
                  int iSource, double fcut, int warmup, float *vpz, float *vsv, float *epsilon, float *delta,
                  float *phi, float *theta, float *pp, float *pc, float *qp, float *qc, double *prop_seconds) {
  precompute_globals(sx, sy, sz, bord, vpz, vsv, epsilon, delta, phi, theta);
  DRIVER_Initialize(sx, sy, sz, bord, dx, dy, dz, dt, vpz, vsv, epsilon, delta, phi, theta, pp,
                    pc, qp, qc);
  float *p0 = pp;
  double walltime = 0.0;
  for (int it = 1; it <= st; it++) {
    float src = (fcut == FCUT) ? Source(dt, it - 1) : source_fcut(dt, it - 1, fcut);
    DRIVER_InsertSource(dt, it - 1, iSource, pc, qc, src);
    const double t0 = wtime();
    DRIVER_Propagate(sx, sy, sz, bord, dx, dy, dz, dt, it, pp, pc, qp, qc);
    SwapArrays(&pp, &pc, &qp, &qc);
    if (it > warmup) walltime += wtime() - t0;
  }
  DRIVER_Finalize();
  free_globals();
  if (prop_seconds) *prop_seconds = walltime;
  return pc == p0;
}

int ref_run(int sx, int sy, int sz, int bord, float dx, float dy, float dz, float dt, int st,
            int iSource, double fcut, float *vpz, float *vsv, float *epsilon, float *delta,
            float *phi, float *theta, float *pp, float *pc, float *qp, float *qc) {
  return ref_run_timed(sx, sy, sz, bord, dx, dy, dz, dt, st, iSource, fcut, 0, vpz, vsv, epsilon, delta, phi,
                       theta, pp, pc, qp, qc, NULL);
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
 * ref_cli MODEL OUT sx sy sz nx ny nz bord absorb dx dy dz dt st ix iy iz fcut seed stride [warmup]
 *
 * MODEL is a file holding vpz vsv epsilon delta phi theta (sx*sy*sz float32
 * each, before the boundary), or "layered:<layers>:<vmin>:<vmax>:<vs_ratio>"
 * for the layered test medium generated here (oracle/model_layered.c) with
 * `seed`.  srand(seed) + RandomVelocityBoundary is applied, then the Model()
 * loop runs `st` steps.  OUT ("-": none) receives the final current p then
 * q, subsampled every `stride` cells in x, y and z (stride 1 = full
 * fields), followed by the per-z-plane sums of p*p and q*q (double, full
 * resolution).  Prints one line with the reference's MSamples/s over the
 * timed steps (all steps after the first `warmup`), the seconds of that
 * region, the set-up seconds and the OpenMP thread count.
 */
#include <omp.h>
#include <stdint.h>
#include <sys/time.h>
void orc_model_layered(int sx, int sy, int sz, int bord, int absorb, int nlayers, uint64_t seed, float vmin,
                       float vmax, float vs_ratio, float *model);
static double now(void) { struct timeval tv; gettimeofday(&tv, NULL); return tv.tv_sec + 1e-6 * tv.tv_usec; }
int main(int argc, char **argv) {
  if (argc < 22) {
    fprintf(stderr, "usage: ref_cli MODEL OUT sx sy sz nx ny nz bord absorb dx dy dz dt st ix iy iz fcut seed "
                    "stride [warmup]\n");
    return 2;
  }
  const double t_start = now();
  const char *fin = argv[1], *fout = argv[2];
  int sx = atoi(argv[3]), sy = atoi(argv[4]), sz = atoi(argv[5]);
  int nx = atoi(argv[6]), ny = atoi(argv[7]), nz = atoi(argv[8]);
  int bord = atoi(argv[9]), absorb = atoi(argv[10]);
  float dx = atof(argv[11]), dy = atof(argv[12]), dz = atof(argv[13]), dt = atof(argv[14]);
  int st = atoi(argv[15]), ix = atoi(argv[16]), iy = atoi(argv[17]), iz = atoi(argv[18]);
  double fcut = atof(argv[19]);
  unsigned seed = (unsigned)strtoul(argv[20], NULL, 10);
  int stride = atoi(argv[21]);
  int warmup = argc > 22 ? atoi(argv[22]) : 0;
  if (warmup < 0 || warmup >= st) warmup = 0;
  const long n = (long)sx * sy * sz;
  float *a[6];
  float *model = (float *)malloc(6 * n * sizeof(float));
  if (!model) { fprintf(stderr, "out of memory\n"); return 1; }
  for (int k = 0; k < 6; k++) a[k] = model + k * n;
  if (strncmp(fin, "layered:", 8) == 0) {
    int layers = 8;
    float vmin = 1500.0f, vmax = 4000.0f, vsr = 0.5f;
    if (sscanf(fin + 8, "%d:%f:%f:%f", &layers, &vmin, &vmax, &vsr) != 4) {
      fprintf(stderr, "bad model spec %s\n", fin);
      return 2;
    }
    orc_model_layered(sx, sy, sz, bord, absorb, layers, (uint64_t)seed, vmin, vmax, vsr, model);
  } else {
    FILE *f = fopen(fin, "rb");
    if (!f) { perror(fin); return 1; }
    if (fread(model, sizeof(float), 6 * n, f) != (size_t)(6 * n)) { fprintf(stderr, "short read\n"); return 1; }
    fclose(f);
  }
  ref_boundary(sx, sy, sz, nx, ny, nz, bord, absorb, a[0], a[1], seed);
  float *pp = calloc(n, 4), *pc = calloc(n, 4), *qp = calloc(n, 4), *qc = calloc(n, 4);
  if (!pp || !pc || !qp || !qc) { fprintf(stderr, "out of memory\n"); return 1; }
  const int iSource = (iz * sy + iy) * sx + ix;
  const double t0 = now();
  double prop_s = 0.0;
  int odd = ref_run_timed(sx, sy, sz, bord, dx, dy, dz, dt, st, iSource, fcut, warmup, a[0], a[1], a[2], a[3], a[4],
                          a[5], pp, pc, qp, qc, &prop_s);
  const double t1 = now();
  float *P = odd ? pp : pc, *Q = odd ? qp : qc;
  if (strcmp(fout, "-") != 0) {
    FILE *f = fopen(fout, "wb");
    if (!f) { perror(fout); return 1; }
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
  }
  const double samples = (double)(sx - 2 * bord) * (sy - 2 * bord) * (sz - 2 * bord) * (st - warmup);
  printf("ref_cli: steps %d warmup %d timed_s %.6f msamples %.4f threads %d setup_s %.3f run_s %.3f\n", st, warmup,
         prop_s, prop_s > 0 ? 1e-6 * samples / prop_s : 0.0, omp_get_max_threads(), t0 - t_start, t1 - t0);
  free(model); free(pp); free(pc); free(qp); free(qc);
  return 0;
}
#endif
