/*
 * ORACLE -- test infrastructure only.
 *
 * The layered TTI test medium, restated for the oracle side so that the
 * reference arm of the benchmark and the reference harness (ref_cli) build
 * their inputs without loading the product library.  It must produce the
 * same floats as FLETCHER_ModelLayered of libfletcher_gb300.so
 * (fletcher_petrobras_gb300/csrc/host/fletcher_host.c); a CPU test checks
 * that bit for bit.
 *
 * Medium: `nlayers` horizontal layers of seeded random thickness tiling the
 * interior depth; per layer vpz ~ U[vmin, vmax] (sorted to increase with
 * depth), epsilon ~ U[0, 0.3], delta ~ U[0, epsilon], theta ~ U[0, 45 deg],
 * phi ~ U[0, 90 deg], vsv = vs_ratio * vpz; the planes above and below the
 * interior repeat the first and last layer.  Draws come from splitmix64
 * (seed ^ 0x5DEECE66D), so every platform gives the same model.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

static uint64_t ml_next(uint64_t *state) {
  uint64_t z = (*state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

/* Uniform double in [0, 1) from the top 53 bits of a draw. */
static double ml_uniform(uint64_t *state) { return (double)(ml_next(state) >> 11) / 9007199254740992.0; }

static int ml_less(const void *a, const void *b) {
  const float u = *(const float *)a, v = *(const float *)b;
  return u < v ? -1 : (u > v ? 1 : 0);
}

/* model: six consecutive arrays of sx*sy*sz floats (vpz vsv epsilon delta
 * phi theta), before any boundary. */
void orc_model_layered(int sx, int sy, int sz, int bord, int absorb, int nlayers, uint64_t seed, float vmin,
                       float vmax, float vs_ratio, float *model) {
  const long plane = (long)sx * sy;
  const long n = plane * sz;
  const int depth = sz - 2 * bord - 2 * absorb;
  const int first = bord + absorb;
  int L = nlayers < 1 ? 1 : nlayers;
  if (L > depth) L = depth;
  uint64_t st = seed ^ 0x5DEECE66Dull;

  /* Layer boundaries from cumulative weights in [0.5, 1.5), rounded to the
   * nearest plane, each layer at least one plane thick. */
  double *weight = malloc(sizeof(double) * L);
  int *start = malloc(sizeof(int) * (L + 1));
  double total = 0.0;
  for (int l = 0; l < L; l++) {
    weight[l] = 0.5 + ml_uniform(&st);
    total += weight[l];
  }
  double run = 0.0;
  start[0] = 0;
  for (int l = 1; l < L; l++) {
    run += weight[l - 1];
    int b = (int)floor(depth * run / total + 0.5);
    const int lo = start[l - 1] + 1, hi = depth - (L - l);
    b = b < lo ? lo : (b > hi ? hi : b);
    start[l] = b;
  }
  start[L] = depth;

  /* Per-layer values, in the generator's draw order: all velocities first,
   * then (epsilon, delta, theta, phi) layer by layer. */
  float *vel = malloc(sizeof(float) * L);
  float *lay = malloc(sizeof(float) * 4 * L); /* eps, delta, theta, phi */
  for (int l = 0; l < L; l++) vel[l] = (float)(vmin + (vmax - vmin) * ml_uniform(&st));
  qsort(vel, L, sizeof(float), ml_less);
  const double rad = 3.14159265358979323846 / 180.0;
  for (int l = 0; l < L; l++) {
    const float e = (float)(0.3 * ml_uniform(&st));
    lay[4 * l + 0] = e;
    lay[4 * l + 1] = (float)(e * ml_uniform(&st));
    lay[4 * l + 2] = (float)(45.0 * rad * ml_uniform(&st));
    lay[4 * l + 3] = (float)(90.0 * rad * ml_uniform(&st));
  }

  int l = 0;
  for (int iz = 0; iz < sz; iz++) {
    const int zi = iz < first ? 0 : (iz - first > depth - 1 ? depth - 1 : iz - first);
    while (l + 1 < L && zi >= start[l + 1]) l++;
    const float v[6] = {vel[l], vs_ratio * vel[l], lay[4 * l], lay[4 * l + 1], lay[4 * l + 3], lay[4 * l + 2]};
    for (int a = 0; a < 6; a++) {
      float *dst = model + a * n + iz * plane;
      for (long i = 0; i < plane; i++) dst[i] = v[a];
    }
  }
  free(weight);
  free(start);
  free(vel);
  free(lay);
}
