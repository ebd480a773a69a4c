/*
 * fletcher_gb300 -- command-line front-end with the reference executable's
 * arguments (original/main.c:47-60):
 *
 *   fletcher_gb300 FORM nx ny nz absorb dx dy dz dt tmax
 *
 * FORM is ISO, VTI or TTI with the reference's homogeneous media
 * (original/main.c:168-221), bord = 4, the source at the grid centre with
 * the reference's 40 Hz cut frequency, the random-velocity boundary drawn
 * from rand()'s default seed, and snapshots every 0.01 s of simulated time
 * (original/model.c:98-107).  Prints the reference's metrics
 * (original/model.c:130-132).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../../include/fletcher_gb300.h"

#define SIGMA 0.75     /* original/fletcher.h:10 */
#define MAX_SIGMA 10.0 /* original/fletcher.h:11 */

int main(int argc, char **argv) {
  if (argc < 11) {
    printf("program requires %d input arguments; execution halted\n", 10);
    return 1;
  }
  const char *form = argv[1];
  const int nx = atoi(argv[2]), ny = atoi(argv[3]), nz = atoi(argv[4]), absorb = atoi(argv[5]);
  const float dx = atof(argv[6]), dy = atof(argv[7]), dz = atof(argv[8]), dt = atof(argv[9]);
  const float tmax = atof(argv[10]);
  int kind;
  if (strcmp(form, "ISO") == 0) kind = 0;
  else if (strcmp(form, "VTI") == 0) kind = 1;
  else if (strcmp(form, "TTI") == 0) kind = 2;
  else {
    printf("Input problem formulation (%s) is unknown\n", form);
    return 1;
  }
  const int bord = 4;
  const int sx = nx + 2 * bord + 2 * absorb, sy = ny + 2 * bord + 2 * absorb, sz = nz + 2 * bord + 2 * absorb;
  const int st = ceil(tmax / dt);
  const long n = (long)sx * sy * sz;
  const long iSource = ((long)(sz / 2) * sy + sy / 2) * sx + sx / 2;
  float *model = (float *)malloc(6 * n * sizeof(float));
  float *f = (float *)calloc(4 * n, sizeof(float));
  if (!model || !f) {
    printf("out of host memory\n");
    return 1;
  }
  const float eps = kind == 0 ? 0.0f : 0.24f, del = kind == 0 ? 0.0f : 0.1f;
  const float phi = kind == 2 ? 1.0f : 0.0f, theta = kind == 2 ? atanf(1.0) : 0.0f;
  float vsv = 0.0f;
  if (kind != 0 && !(SIGMA > MAX_SIGMA)) vsv = 3000.0f * sqrtf(fabsf(eps - del) / SIGMA);
  FLETCHER_ModelHomogeneous(n, 3000.0f, vsv, eps, del, phi, theta, model);
  printf("Recomended maximum time step is %f; used time step is %f\n",
         FLETCHER_RecommendedDt(n, model, model + 2 * n, dx, dy, dz), dt);
  FLETCHER_RandomVelocityBoundary(sx, sy, sz, nx, ny, nz, bord, absorb, model, model + n, 1u);
  double stats[5];
  const int rc = FLETCHER_Model(st, iSource, 40.0, 0.01f, sx, sy, sz, bord, dx, dy, dz, dt, f, f + n, f + 2 * n,
                                f + 3 * n, model, model + n, model + 2 * n, model + 3 * n, model + 4 * n,
                                model + 5 * n, stats);
  if (rc) {
    printf("run failed: %s\n", FLETCHER_GetLastErrorString());
    return 1;
  }
  printf("Execution time (s) is %lf\n", stats[0]);
  printf("MSamples/s %.0lf\n", stats[1]);
  free(model);
  free(f);
  return 0;
}
