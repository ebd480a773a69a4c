/*
 * Host side of libfletcher_gb300.so: model preparation and the time loop,
 * following the reference front-end's call sequence (original/main.c,
 * original/boundary.c, original/source.c, original/model.c) over the
 * DRIVER_* interface.  Compiled with -ffp-contract=off so that every float
 * expression rounds as the reference's x86-64 build does.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>

#include "../../../include/fletcher_gb300.h"

#define IND(ix, iy, iz) ((((long)(iz)) * sy + (iy)) * (long)sx + (ix))

static double wall_seconds(void) {
  struct timeval tv;
  gettimeofday(&tv, NULL);
  return tv.tv_sec + 1.0e-6 * tv.tv_usec;
}

void FLETCHER_ModelHomogeneous(long n, float vpz, float vsv, float epsilon, float delta, float phi,
                               float theta, float *model) {
  for (long i = 0; i < n; i++) {
    model[i] = vpz;
    model[n + i] = vsv;
    model[2 * n + i] = epsilon;
    model[3 * n + i] = delta;
    model[4 * n + i] = phi;
    model[5 * n + i] = theta;
  }
}

/* splitmix64: a fixed, portable generator for the layered-model draws. */
static uint64_t splitmix64(uint64_t *s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static double unif(uint64_t *s) { return (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

static int cmp_float(const void *a, const void *b) {
  const float x = *(const float *)a, y = *(const float *)b;
  return (x > y) - (x < y);
}

void FLETCHER_ModelLayered(int sx, int sy, int sz, int bord, int absorb, int nlayers, uint64_t seed,
                           float vmin, float vmax, float vs_ratio, float *model, int *layer_top) {
  const long n = (long)sx * sy * sz;
  const int nz = sz - 2 * bord - 2 * absorb;
  const int z_in = bord + absorb;
  if (nlayers < 1) nlayers = 1;
  if (nlayers > nz) nlayers = nz;
  uint64_t s = seed ^ 0x5DEECE66Dull;
  /* Thicknesses: weights in [0.5, 1.5), cumulative boundaries rounded, at
   * least one cell each. */
  double *w = (double *)malloc(sizeof(double) * nlayers);
  double tot = 0.0;
  for (int l = 0; l < nlayers; l++) tot += (w[l] = 0.5 + unif(&s));
  int *top = (int *)malloc(sizeof(int) * (nlayers + 1));
  double acc = 0.0;
  top[0] = 0;
  for (int l = 1; l < nlayers; l++) {
    acc += w[l - 1];
    int t = (int)floor(nz * acc / tot + 0.5);
    if (t < top[l - 1] + 1) t = top[l - 1] + 1;
    if (t > nz - (nlayers - l)) t = nz - (nlayers - l);
    top[l] = t;
  }
  top[nlayers] = nz;
  float *vp = (float *)malloc(sizeof(float) * nlayers);
  for (int l = 0; l < nlayers; l++) vp[l] = (float)(vmin + (vmax - vmin) * unif(&s));
  qsort(vp, nlayers, sizeof(float), cmp_float);
  const double deg = 3.14159265358979323846 / 180.0;
  float *eps = (float *)malloc(sizeof(float) * nlayers), *del = (float *)malloc(sizeof(float) * nlayers);
  float *th = (float *)malloc(sizeof(float) * nlayers), *ph = (float *)malloc(sizeof(float) * nlayers);
  for (int l = 0; l < nlayers; l++) {
    eps[l] = (float)(0.3 * unif(&s));
    del[l] = (float)(eps[l] * unif(&s));
    th[l] = (float)(45.0 * deg * unif(&s));
    ph[l] = (float)(90.0 * deg * unif(&s));
  }
  for (int iz = 0; iz < sz; iz++) {
    int zi = iz - z_in;
    if (zi < 0) zi = 0;
    if (zi > nz - 1) zi = nz - 1;
    int l = 0;
    while (l + 1 < nlayers && zi >= top[l + 1]) l++;
    const float vs = vs_ratio * vp[l];
    for (long i = (long)iz * sx * sy; i < (long)(iz + 1) * sx * sy; i++) {
      model[i] = vp[l];
      model[n + i] = vs;
      model[2 * n + i] = eps[l];
      model[3 * n + i] = del[l];
      model[4 * n + i] = ph[l];
      model[5 * n + i] = th[l];
    }
  }
  if (layer_top)
    for (int l = 0; l < nlayers; l++) layer_top[l] = top[l] + z_in;
  free(w); free(top); free(vp); free(eps); free(del); free(th); free(ph);
}

/* RandomVelocityBoundary, original/boundary.c:7-98. */
void FLETCHER_RandomVelocityBoundary(int sx, int sy, int sz, int nx, int ny, int nz, int bord,
                                     int absorb, float *vpz, float *vsv, unsigned seed) {
  srand(seed);
  /* Maximum P and S speeds of the interior (original/boundary.c:20-29). */
  float maxP = 0.0, maxS = 0.0;
  for (int iz = bord + absorb; iz < nz + bord + absorb; iz++)
    for (int iy = bord + absorb; iy < ny + bord + absorb; iy++)
      for (long i = IND(bord + absorb, iy, iz); i < IND(nx + bord + absorb, iy, iz); i++) {
        maxP = fmaxf(vpz[i], maxP);
        maxS = fmaxf(vsv[i], maxS);
      }
  const int last_low = bord + absorb - 1; /* last index of the low absorbing zone */
  const int first_in = last_low + 1;      /* first interior index */
  const float frac = 1.0 / (float)(absorb);
  for (int iz = 0; iz < sz; iz++)
    for (int iy = 0; iy < sy; iy++)
      for (int ix = 0; ix < sx; ix++) {
        const long i = IND(ix, iy, iz);
        const int inside_z = iz >= first_in && iz <= last_low + nz;
        const int inside_y = iy >= first_in && iy <= last_low + ny;
        const int inside_x = ix >= first_in && ix <= last_low + nx;
        if (inside_z && inside_y && inside_x) continue;
        const int zone_z = iz >= bord && iz <= 2 * last_low + nz;
        const int zone_y = iy >= bord && iy <= 2 * last_low + ny;
        const int zone_x = ix >= bord && ix <= 2 * last_low + nx;
        if (!(zone_z && zone_y && zone_x)) { /* zero speed in the border shell */
          vpz[i] = 0.0;
          vsv[i] = 0.0;
          continue;
        }
        /* distance to the interior along each axis, and the nearest
         * interior index whose velocity the cell starts from */
        int dz_ = 0, vz = iz, dy_ = 0, vy = iy, dx_ = 0, vx = ix;
        if (iz > last_low + nz) { dz_ = iz - last_low - nz; vz = last_low + nz; }
        else if (iz < first_in) { dz_ = first_in - iz; vz = first_in; }
        if (iy > last_low + ny) { dy_ = iy - last_low - ny; vy = last_low + ny; }
        else if (iy < first_in) { dy_ = first_in - iy; vy = first_in; }
        if (ix > last_low + nx) { dx_ = ix - last_low - nx; vx = last_low + nx; }
        else if (ix < first_in) { dx_ = first_in - ix; vx = first_in; }
        int dist = dy_ > dz_ ? dy_ : dz_;
        dist = dist > dx_ ? dist : dx_;
        const float bdist = (float)(dist)*frac;
        const float r = (float)rand() / (float)RAND_MAX;
        vpz[i] = vpz[IND(vx, vy, vz)] * (1.0 - bdist) + maxP * r * bdist;
        vsv[i] = vsv[IND(vx, vy, vz)] * (1.0 - bdist) + maxS * r * bdist;
      }
}

/* Ricker wavelet, original/source.c:7-15 (constants of original/source.h:12-14). */
float FLETCHER_Source(float dt, int it, double fcut) {
  const double pi_cube = 31.00627668029982017537;
  const double two_sqrt_pi = 3.54490770181103205458;
  const double three_sqrt_pi = 5.31736155271654808184;
  const float tf = two_sqrt_pi / fcut;
  const float fc = fcut / three_sqrt_pi;
  const float fct = fc * (((float)it) * dt - tf);
  const float expo = pi_cube * fct * fct;
  return ((1.0f - 2.0f * expo) * expf(-expo));
}

float FLETCHER_RecommendedDt(long n, const float *vpz, const float *epsilon, float dx, float dy,
                             float dz) {
  float maxvel = vpz[0] * sqrt(1.0 + 2 * epsilon[0]);
  for (long i = 1; i < n; i++) maxvel = fmaxf(maxvel, vpz[i] * sqrt(1.0 + 2 * epsilon[i]));
  float mindelta = dx;
  if (dy < mindelta) mindelta = dy;
  if (dz < mindelta) mindelta = dz;
  return (0.2 * mindelta) / maxvel;
}

/* Phases of the last FLETCHER_Model call, in seconds. */
static double g_phases[4];

void FLETCHER_ModelPhases(double *phases) {
  for (int k = 0; k < 4; k++) phases[k] = g_phases[k];
}

int FLETCHER_Model(int st, long iSource, double fcut, float dt_output, int sx, int sy, int sz,
                   int bord, float dx, float dy, float dz, float dt, float *pp, float *pc,
                   float *qp, float *qc, float *vpz, float *vsv, float *epsilon, float *delta,
                   float *phi, float *theta, double *stats) {
  const long n = (long)sx * sy * sz;
  float *pc0 = pc, *qc0 = qc;
  const double t_start = wall_seconds();
  FLETCHER_ClearError();
  DRIVER_Initialize(sx, sy, sz, bord, dx, dy, dz, dt, vpz, vsv, epsilon, delta, phi, theta, pp,
                    pc, qp, qc);
  if (FLETCHER_GetLastError()) return FLETCHER_GetLastError();
  double h2d = 10.0 * n * sizeof(float), d2h = 0.0;
  /* Snapshots go straight into the two host p arrays (page-locked for the
   * call) while the steps continue. */
  const int pinned = dt_output > 0.0f && !FLETCHER_PinHost(pp, n * sizeof(float)) &&
                     !FLETCHER_PinHost(pc, n * sizeof(float));
  if (dt_output > 0.0f && !pinned) FLETCHER_ClearError();
  const double t_loop = wall_seconds();
  double walltime = 0.0;
  float tSim = 0.0;
  int nOut = 1;
  float tOut = nOut * dt_output;
  for (int it = 1; it <= st; it++) {
    const float src = FLETCHER_Source(dt, it - 1, fcut);
    DRIVER_InsertSource(dt, it - 1, (int)iSource, pc, qc, src);
    const double t0 = wall_seconds();
    DRIVER_Propagate(sx, sy, sz, bord, dx, dy, dz, dt, it, pp, pc, qp, qc);
    float *t = pp; pp = pc; pc = t;
    t = qp; qp = qc; qc = t;
    walltime += wall_seconds() - t0;
    if (FLETCHER_GetLastError()) break;
    tSim = it * dt;
    if (dt_output > 0.0f && tSim >= tOut) {
      /* DRIVER_Update_pointers(pc) of original/model.c:100, without waiting. */
      if (FLETCHER_SnapshotBegin(0, pc)) break;
      d2h += (double)n * sizeof(float);
      tOut = (++nOut) * dt_output;
    }
  }
  const double t_drain = wall_seconds();
  FLETCHER_SnapshotWait();
  const double t_read = wall_seconds();
  if (FLETCHER_GetLastError()) {
    const int e = FLETCHER_GetLastError();
    if (pinned) {
      FLETCHER_UnpinHost(pp);
      FLETCHER_UnpinHost(pc);
    }
    DRIVER_Finalize();
    return e;
  }
  /* The final p and q go into page-locked destinations too (the copy
   * engine writes them at full speed; into pageable memory the copy is
   * staged by the driver, and memory the caller never touched is faulted
   * in during it).  pc0 is one of the two p arrays. */
  const int pin_p = !pinned && !FLETCHER_PinHost(pc0, n * sizeof(float));
  const int pin_q = !FLETCHER_PinHost(qc0, n * sizeof(float));
  FLETCHER_ClearError(); /* a destination that could not be locked is copied to as it is */
  int rc = FLETCHER_GetField(0, pc0);
  if (!rc) rc = FLETCHER_GetField(1, qc0);
  d2h += 2.0 * n * sizeof(float);
  if (pin_q) FLETCHER_UnpinHost(qc0);
  if (pin_p) FLETCHER_UnpinHost(pc0);
  if (pinned) {
    FLETCHER_UnpinHost(pp);
    FLETCHER_UnpinHost(pc);
  }
  DRIVER_Finalize();
  const double t_end = wall_seconds();
  g_phases[0] = t_loop - t_start;
  g_phases[1] = t_drain - t_loop;
  g_phases[2] = t_read - t_drain;
  g_phases[3] = t_end - t_read;
  if (stats) {
    const double samples = (double)(sx - 2 * bord) * (sy - 2 * bord) * (sz - 2 * bord) * st;
    stats[0] = walltime;
    stats[1] = walltime > 0 ? 1.0e-6 * samples / walltime : 0.0;
    stats[2] = t_end - t_start;
    stats[3] = h2d;
    stats[4] = d2h;
  }
  return rc ? rc : FLETCHER_GetLastError();
}
