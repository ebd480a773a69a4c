/*
 * ORACLE -- test infrastructure only.
 *
 * A CPU restatement of the Fletcher TTI pseudo-acoustic propagator as the
 * reference implements it in its canonical tree (`original/`).  It is the
 * checker for the GPU library: only the tests, the smoke check and the CPU
 * baseline leg of the benchmark may load it.  Nothing in the product links,
 * imports or calls this file.
 *
 * Pinning: `oracle/Makefile` target `ref` compiles the reference's own
 * OpenMP back-end and front-end sources into `oracle/_ref/`, and
 * `tests/golden/make_golden.py` records their outputs as fixtures; the CPU
 * test suite checks this restatement bit-for-bit against those fixtures.
 *
 * FP32 path: every expression keeps the operand order of the reference so
 * that the result is bit-identical when compiled without floating-point
 * contraction (-ffp-contract=off; x86-64 without -mfma never contracts).
 * FP64 path: the same stencil with exact rational weights, in double,
 * used as the error oracle for the reduced-precision storage form.
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_IND(ix, iy, iz) ((((long)(iz)) * sy + (iy)) * (long)sx + (ix))

/* ---- stencil weights: original/derivatives.h:13-41 -------------------- */
#define L1f 0.8f
#define L2f -0.2f
#define L3f 0.0380952380952381f
#define L4f -0.0035714285714285713f
#define L11f 0.64f
#define L12f -0.16f
#define L13f 0.03047619047619047618f
#define L14f -0.00285714285714285713f
#define L22f 0.04f
#define L23f -0.00761904761904761904f
#define L24f 0.00071428571428571428f
#define L33f 0.00145124716553287981f
#define L34f -0.00013605442176870748f
#define L44f 0.00001275510204081632f
#define K0f -2.84722222222222222222f
#define K1f 1.6f
#define K2f -0.2f
#define K3f 0.02539682539682539682f
#define K4f -0.00178571428571428571f

/* Der2, original/derivatives.h:53: 9-point second derivative, summed in
 * the macro's order and scaled last. */
static inline float der2_f(const float *p, long i, long s, float d2inv) {
  return ((K0f * p[i] + K1f * (p[i + s] + p[i - s]) + K2f * (p[i + 2 * s] + p[i - 2 * s]) +
           K3f * (p[i + 3 * s] + p[i - 3 * s]) + K4f * (p[i + 4 * s] + p[i - 4 * s])) *
          (d2inv));
}

/* Groups of DerCross, original/derivatives.h:59-68, with a = ka*s11 and
 * b = kb*s21.  DC4 is the four-term difference p[+b+a] - p[+b-a] - p[-b+a]
 * + p[-b-a]; DC8 is a mixed bracket (e.g. L12): the (a1,b1) and (a2,b2)
 * groups written as ONE flat eight-term expression, summed left to right as
 * the macro does. */
#define DC4(p, i, a, b) ((p)[(i) + (b) + (a)] - (p)[(i) + (b) - (a)] - (p)[(i) - (b) + (a)] + (p)[(i) - (b) - (a)])
#define DC8(p, i, a1, b1, a2, b2)                                                                  \
  ((p)[(i) + (b1) + (a1)] - (p)[(i) + (b1) - (a1)] - (p)[(i) - (b1) + (a1)] + (p)[(i) - (b1) - (a1)] + \
   (p)[(i) + (b2) + (a2)] - (p)[(i) + (b2) - (a2)] - (p)[(i) - (b2) + (a2)] + (p)[(i) - (b2) - (a2)])

/* DerCross, original/derivatives.h:59-68, s11 = first stride, s21 = second.
 * Each mixed bracket lists (s21, k*s11) first, then (k*s21, s11). */
static inline float dercross_f(const float *p, long i, long s11, long s21, float dinv) {
  return ((L11f * (DC4(p, i, s11, s21)) +
           L12f * (DC8(p, i, 2 * s11, s21, s11, 2 * s21)) +
           L13f * (DC8(p, i, 3 * s11, s21, s11, 3 * s21)) +
           L14f * (DC8(p, i, 4 * s11, s21, s11, 4 * s21)) +
           L22f * (DC4(p, i, 2 * s11, 2 * s21)) +
           L23f * (DC8(p, i, 3 * s11, 2 * s21, 2 * s11, 3 * s21)) +
           L24f * (DC8(p, i, 4 * s11, 2 * s21, 2 * s11, 4 * s21)) +
           L33f * (DC4(p, i, 3 * s11, 3 * s21)) +
           L34f * (DC8(p, i, 4 * s11, 3 * s21, 3 * s11, 4 * s21)) +
           L44f * (DC4(p, i, 4 * s11, 4 * s21))) *
          (dinv));
}

/* Coefficient order used everywhere in this file (and in the fixtures). */
enum { C_XX = 0, C_YY, C_ZZ, C_XY, C_YZ, C_XZ, C_V2PX, C_V2PZ, C_V2SZ, C_V2PN, NCOEF };

/*
 * Coefficient precompute, original/precomp.h:14-38 (ch1d**) and :49-58
 * (v2**).  Trigonometry in double, results stored to float, products of the
 * float values in float, velocity terms in double.  `coef` holds NCOEF
 * arrays of n floats each, in the enum order above.
 */
void orc_precompute(long n, const float *vpz, const float *vsv, const float *epsilon,
                    const float *delta, const float *phi, const float *theta, float *coef) {
  float *ch1dxx = coef + C_XX * n, *ch1dyy = coef + C_YY * n, *ch1dzz = coef + C_ZZ * n;
  float *ch1dxy = coef + C_XY * n, *ch1dyz = coef + C_YZ * n, *ch1dxz = coef + C_XZ * n;
  float *v2px = coef + C_V2PX * n, *v2pz = coef + C_V2PZ * n, *v2sz = coef + C_V2SZ * n;
  float *v2pn = coef + C_V2PN * n;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; i++) {
    float sinTheta = sin(theta[i]);
    float cosTheta = cos(theta[i]);
    float sin2Theta = sin(2.0 * theta[i]);
    float sinPhi = sin(phi[i]);
    float cosPhi = cos(phi[i]);
    float sin2Phi = sin(2.0 * phi[i]);
    ch1dxx[i] = sinTheta * sinTheta * cosPhi * cosPhi;
    ch1dyy[i] = sinTheta * sinTheta * sinPhi * sinPhi;
    ch1dzz[i] = cosTheta * cosTheta;
    ch1dxy[i] = sinTheta * sinTheta * sin2Phi;
    ch1dyz[i] = sin2Theta * sinPhi;
    ch1dxz[i] = sin2Theta * cosPhi;
  }
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; i++) {
    v2sz[i] = vsv[i] * vsv[i];
    v2pz[i] = vpz[i] * vpz[i];
    v2px[i] = v2pz[i] * (1.0 + 2.0 * epsilon[i]);
    v2pn[i] = v2pz[i] * (1.0 + 2.0 * delta[i]);
  }
}

/* FP64 coefficients for the double-precision oracle (same formulas, no
 * intermediate rounding to float). */
void orc_precompute_f64(long n, const float *vpz, const float *vsv, const float *epsilon,
                        const float *delta, const float *phi, const float *theta, double *coef) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; i++) {
    double st = sin((double)theta[i]), ct = cos((double)theta[i]), s2t = sin(2.0 * theta[i]);
    double sp = sin((double)phi[i]), cp = cos((double)phi[i]), s2p = sin(2.0 * phi[i]);
    coef[C_XX * n + i] = st * st * cp * cp;
    coef[C_YY * n + i] = st * st * sp * sp;
    coef[C_ZZ * n + i] = ct * ct;
    coef[C_XY * n + i] = st * st * s2p;
    coef[C_YZ * n + i] = s2t * sp;
    coef[C_XZ * n + i] = s2t * cp;
    double vp = vpz[i], vs = vsv[i];
    coef[C_V2SZ * n + i] = vs * vs;
    coef[C_V2PZ * n + i] = vp * vp;
    coef[C_V2PX * n + i] = vp * vp * (1.0 + 2.0 * (double)epsilon[i]);
    coef[C_V2PN * n + i] = vp * vp * (1.0 + 2.0 * (double)delta[i]);
  }
}

/*
 * RandomVelocityBoundary, original/boundary.c:7-98.  Absorbing zone: linear
 * blend of the nearest interior velocity toward maxP/maxS times a glibc
 * rand() draw, by Chebyshev distance; outer `bord` shell: zero velocity.
 * The draw order is the x-fastest sweep of the whole grid.
 */
void orc_random_velocity_boundary(int sx, int sy, int sz, int nx, int ny, int nz, int bord,
                                  int absorb, float *vpz, float *vsv) {
  float maxP = 0.0, maxS = 0.0;
  for (int iz = bord + absorb; iz < nz + bord + absorb; iz++)
    for (int iy = bord + absorb; iy < ny + bord + absorb; iy++)
      for (long i = ORC_IND(bord + absorb, iy, iz); i < ORC_IND(nx + bord + absorb, iy, iz); i++) {
        maxP = fmaxf(vpz[i], maxP);
        maxS = fmaxf(vsv[i], maxS);
      }
  const int bordLen = bord + absorb - 1;
  const int firstIn = bordLen + 1;
  const float frac = 1.0 / (float)(absorb);
  for (int iz = 0; iz < sz; iz++)
    for (int iy = 0; iy < sy; iy++)
      for (int ix = 0; ix < sx; ix++) {
        long i = ORC_IND(ix, iy, iz);
        if ((iz >= firstIn && iz <= bordLen + nz) && (iy >= firstIn && iy <= bordLen + ny) &&
            (ix >= firstIn && ix <= bordLen + nx)) {
          continue;
        } else if ((iz >= bord && iz <= 2 * bordLen + nz) && (iy >= bord && iy <= 2 * bordLen + ny) &&
                   (ix >= bord && ix <= 2 * bordLen + nx)) {
          int distx, disty, distz, ivelx, ively, ivelz;
          if (iz > bordLen + nz) { distz = iz - bordLen - nz; ivelz = bordLen + nz; }
          else if (iz < firstIn) { distz = firstIn - iz; ivelz = firstIn; }
          else { distz = 0; ivelz = iz; }
          if (iy > bordLen + ny) { disty = iy - bordLen - ny; ively = bordLen + ny; }
          else if (iy < firstIn) { disty = firstIn - iy; ively = firstIn; }
          else { disty = 0; ively = iy; }
          if (ix > bordLen + nx) { distx = ix - bordLen - nx; ivelx = bordLen + nx; }
          else if (ix < firstIn) { distx = firstIn - ix; ivelx = firstIn; }
          else { distx = 0; ivelx = ix; }
          int dist = (disty > distz) ? disty : distz;
          dist = (dist > distx) ? dist : distx;
          float bordDist = (float)(dist)*frac;
          float rfac = (float)rand() / (float)RAND_MAX;
          vpz[i] = vpz[ORC_IND(ivelx, ively, ivelz)] * (1.0 - bordDist) + maxP * rfac * bordDist;
          vsv[i] = vsv[ORC_IND(ivelx, ively, ivelz)] * (1.0 - bordDist) + maxS * rfac * bordDist;
        } else {
          vpz[i] = 0.0;
          vsv[i] = 0.0;
        }
      }
}

void orc_srand(unsigned seed) { srand(seed); }

/* Source, original/source.c:7-15 with the cut frequency FCUT
 * (original/source.h:11) as a parameter; peak frequency = fcut/3. */
float orc_source(float dt, int it, double fcut) {
  const double PICUBE = 31.00627668029982017537;
  const double TWOSQRTPI = 3.54490770181103205458;
  const double THREESQRTPI = 5.31736155271654808184;
  float tf, fc, fct, expo;
  tf = TWOSQRTPI / fcut;
  fc = fcut / THREESQRTPI;
  fct = fc * (((float)it) * dt - tf);
  expo = PICUBE * fct * fct;
  return ((1.0f - 2.0f * expo) * expf(-expo));
}

/*
 * One FP32 step: original/OpenMP/openmp_propagate.c:9-41 (loop nest over
 * [bord, s-bord) in z, y, x) with original/sample.h:1-29 (strides and
 * inverse spacings) and :32-89 (the coupled p/q update) as the body.
 */
void orc_propagate_f32(int sx, int sy, int sz, int bord, float dx, float dy, float dz, float dt,
                       float *restrict pp, const float *restrict pc, float *restrict qp,
                       const float *restrict qc, const float *restrict coef) {
  const long n = (long)sx * sy * sz;
  const float *ch1dxx = coef + C_XX * n, *ch1dyy = coef + C_YY * n, *ch1dzz = coef + C_ZZ * n;
  const float *ch1dxy = coef + C_XY * n, *ch1dyz = coef + C_YZ * n, *ch1dxz = coef + C_XZ * n;
  const float *v2px = coef + C_V2PX * n, *v2pz = coef + C_V2PZ * n, *v2sz = coef + C_V2SZ * n;
  const float *v2pn = coef + C_V2PN * n;
  const long strideX = 1, strideY = sx, strideZ = (long)sx * sy;
  const float dxxinv = 1.0f / (dx * dx);
  const float dyyinv = 1.0f / (dy * dy);
  const float dzzinv = 1.0f / (dz * dz);
  const float dxyinv = 1.0f / (dx * dy);
  const float dxzinv = 1.0f / (dx * dz);
  const float dyzinv = 1.0f / (dy * dz);
#pragma omp parallel for schedule(static)
  for (int iz = bord; iz < sz - bord; iz++)
    for (int iy = bord; iy < sy - bord; iy++)
      for (int ix = bord; ix < sx - bord; ix++) {
        const long i = ORC_IND(ix, iy, iz);
        const float pxx = der2_f(pc, i, strideX, dxxinv);
        const float pyy = der2_f(pc, i, strideY, dyyinv);
        const float pzz = der2_f(pc, i, strideZ, dzzinv);
        const float pxy = dercross_f(pc, i, strideX, strideY, dxyinv);
        const float pyz = dercross_f(pc, i, strideY, strideZ, dyzinv);
        const float pxz = dercross_f(pc, i, strideX, strideZ, dxzinv);
        const float cpxx = ch1dxx[i] * pxx;
        const float cpyy = ch1dyy[i] * pyy;
        const float cpzz = ch1dzz[i] * pzz;
        const float cpxy = ch1dxy[i] * pxy;
        const float cpxz = ch1dxz[i] * pxz;
        const float cpyz = ch1dyz[i] * pyz;
        const float h1p = cpxx + cpyy + cpzz + cpxy + cpxz + cpyz;
        const float h2p = pxx + pyy + pzz - h1p;
        const float qxx = der2_f(qc, i, strideX, dxxinv);
        const float qyy = der2_f(qc, i, strideY, dyyinv);
        const float qzz = der2_f(qc, i, strideZ, dzzinv);
        const float qxy = dercross_f(qc, i, strideX, strideY, dxyinv);
        const float qyz = dercross_f(qc, i, strideY, strideZ, dyzinv);
        const float qxz = dercross_f(qc, i, strideX, strideZ, dxzinv);
        const float cqxx = ch1dxx[i] * qxx;
        const float cqyy = ch1dyy[i] * qyy;
        const float cqzz = ch1dzz[i] * qzz;
        const float cqxy = ch1dxy[i] * qxy;
        const float cqxz = ch1dxz[i] * qxz;
        const float cqyz = ch1dyz[i] * qyz;
        const float h1q = cqxx + cqyy + cqzz + cqxy + cqxz + cqyz;
        const float h2q = qxx + qyy + qzz - h1q;
        const float h1pmq = h1p - h1q;
        const float h2pmq = h2p - h2q;
        const float rhsp = v2px[i] * h2p + v2pz[i] * h1q + v2sz[i] * h1pmq;
        const float rhsq = v2pn[i] * h2p + v2pz[i] * h1q - v2sz[i] * h2pmq;
        pp[i] = 2.0f * pc[i] - pp[i] + rhsp * dt * dt;
        qp[i] = 2.0f * qc[i] - qp[i] + rhsq * dt * dt;
      }
}

/* ---- FP64 oracle ------------------------------------------------------ */
static const double LD[5] = {0.0, 4.0 / 5.0, -1.0 / 5.0, 4.0 / 105.0, -1.0 / 280.0};
static const double KD[5] = {-205.0 / 72.0, 8.0 / 5.0, -1.0 / 5.0, 8.0 / 315.0, -1.0 / 560.0};

static inline double der2_d(const double *p, long i, long s, double d2inv) {
  double acc = KD[0] * p[i];
  for (int k = 1; k <= 4; k++) acc += KD[k] * (p[i + k * s] + p[i - k * s]);
  return acc * d2inv;
}
static inline double dercross_d(const double *p, long i, long s1, long s2, double dinv) {
  double acc = 0.0;
  for (int a = 1; a <= 4; a++)
    for (int b = 1; b <= 4; b++)
      acc += LD[a] * LD[b] *
             (p[i + b * s2 + a * s1] - p[i + b * s2 - a * s1] - p[i - b * s2 + a * s1] + p[i - b * s2 - a * s1]);
  return acc * dinv;
}

/* One FP64 step of the same update (exact rational stencil weights,
 * double inverse spacings and time step). */
void orc_propagate_f64(int sx, int sy, int sz, int bord, double dx, double dy, double dz, double dt,
                       double *restrict pp, const double *restrict pc, double *restrict qp,
                       const double *restrict qc, const double *restrict coef) {
  const long n = (long)sx * sy * sz;
  const long sX = 1, sY = sx, sZ = (long)sx * sy;
  const double ixx = 1.0 / (dx * dx), iyy = 1.0 / (dy * dy), izz = 1.0 / (dz * dz);
  const double ixy = 1.0 / (dx * dy), ixz = 1.0 / (dx * dz), iyz = 1.0 / (dy * dz);
#pragma omp parallel for schedule(static)
  for (int iz = bord; iz < sz - bord; iz++)
    for (int iy = bord; iy < sy - bord; iy++)
      for (int ix = bord; ix < sx - bord; ix++) {
        const long i = ORC_IND(ix, iy, iz);
        double h1[2], h2[2];
        const double *f[2] = {pc, qc};
        for (int k = 0; k < 2; k++) {
          double xx = der2_d(f[k], i, sX, ixx), yy = der2_d(f[k], i, sY, iyy), zz = der2_d(f[k], i, sZ, izz);
          double xy = dercross_d(f[k], i, sX, sY, ixy), yz = dercross_d(f[k], i, sY, sZ, iyz);
          double xz = dercross_d(f[k], i, sX, sZ, ixz);
          h1[k] = coef[C_XX * n + i] * xx + coef[C_YY * n + i] * yy + coef[C_ZZ * n + i] * zz +
                  coef[C_XY * n + i] * xy + coef[C_XZ * n + i] * xz + coef[C_YZ * n + i] * yz;
          h2[k] = xx + yy + zz - h1[k];
        }
        const double rhsp = coef[C_V2PX * n + i] * h2[0] + coef[C_V2PZ * n + i] * h1[1] +
                            coef[C_V2SZ * n + i] * (h1[0] - h1[1]);
        const double rhsq = coef[C_V2PN * n + i] * h2[0] + coef[C_V2PZ * n + i] * h1[1] -
                            coef[C_V2SZ * n + i] * (h2[0] - h2[1]);
        pp[i] = 2.0 * pc[i] - pp[i] + rhsp * dt * dt;
        qp[i] = 2.0 * qc[i] - qp[i] + rhsq * dt * dt;
      }
}

/* Source cut frequency as a double-precision Ricker (FP64 oracle only). */
static double source_d(double dt, int it, double fcut) {
  const double fc = fcut / (3.0 * sqrt(M_PI)), tf = 2.0 * sqrt(M_PI) / fcut;
  const double fct = fc * ((double)it * dt - tf);
  const double expo = M_PI * M_PI * M_PI * fct * fct;
  return (1.0 - 2.0 * expo) * exp(-expo);
}

/*
 * Time loop, original/model.c:71-88: for it = 1..st the source value for
 * time (it-1)*dt is added at iSource to the current p and q
 * (original/OpenMP/openmp_insertsource.c:7-13), one step writes the next
 * field into the previous-field buffers, and the buffers swap
 * (original/utils.c:233-243).  Returns 1 when the final current field
 * sits in the caller's pp/qp buffers (odd st), else 0.
 */
int orc_run_f32(int sx, int sy, int sz, int bord, float dx, float dy, float dz, float dt, int st,
                long iSource, double fcut, float *pp, float *pc, float *qp, float *qc,
                const float *coef) {
  for (int it = 1; it <= st; it++) {
    float src = orc_source(dt, it - 1, fcut);
    pc[iSource] += src;
    qc[iSource] += src;
    orc_propagate_f32(sx, sy, sz, bord, dx, dy, dz, dt, pp, pc, qp, qc, coef);
    float *t = pp; pp = pc; pc = t;
    t = qp; qp = qc; qc = t;
  }
  return st & 1;
}

/* Der1 of the Der1-Der1 tree, der1der1/derivatives.h:45: 9-point first
 * derivative, summed in the macro's order and scaled last. */
static inline float der1_f(const float *p, long i, long s, float dinv) {
  return ((L1f * (p[i + s] - p[i - s]) + L2f * (p[i + 2 * s] - p[i - 2 * s]) +
           L3f * (p[i + 3 * s] - p[i - 3 * s]) + L4f * (p[i + 4 * s] - p[i - 4 * s])) *
          (dinv));
}

/*
 * One FP32 step of the Der1-Der1 formulation: der1der1/OpenMP/openmp_propagate.c:9-100
 * with der1der1/sample.h.  First derivatives of p and q are stored
 * (pDx, qDx over x in [bord, sx-bord) for every y and z; pDy, qDy over
 * y in [bord, sy-bord) and x in [bord, sx)), and the mixed derivatives are
 * first derivatives of them: pxy = Der1_y(pDx), pxz = Der1_z(pDx),
 * pyz = Der1_z(pDy).  The rest is the update of original/sample.h:32-89.
 * `work` holds 4 * sx*sy*sz floats (pDx, pDy, qDx, qDy).
 */
void orc_propagate_d1d1_f32(int sx, int sy, int sz, int bord, float dx, float dy, float dz, float dt,
                            float *restrict pp, const float *restrict pc, float *restrict qp,
                            const float *restrict qc, const float *restrict coef, float *restrict work) {
  const long n = (long)sx * sy * sz;
  const float *ch1dxx = coef + C_XX * n, *ch1dyy = coef + C_YY * n, *ch1dzz = coef + C_ZZ * n;
  const float *ch1dxy = coef + C_XY * n, *ch1dyz = coef + C_YZ * n, *ch1dxz = coef + C_XZ * n;
  const float *v2px = coef + C_V2PX * n, *v2pz = coef + C_V2PZ * n, *v2sz = coef + C_V2SZ * n;
  const float *v2pn = coef + C_V2PN * n;
  float *pDx = work, *pDy = work + n, *qDx = work + 2 * n, *qDy = work + 3 * n;
  const long strideX = 1, strideY = sx, strideZ = (long)sx * sy;
  const float dxxinv = 1.0f / (dx * dx);
  const float dyyinv = 1.0f / (dy * dy);
  const float dzzinv = 1.0f / (dz * dz);
  const float dxinv = 1.0f / dx;
  const float dyinv = 1.0f / dy;
  const float dzinv = 1.0f / dz;
#pragma omp parallel
  {
#pragma omp for nowait
    for (int iz = 0; iz < sz; iz++)
      for (int iy = 0; iy < sy; iy++)
        for (long i = ORC_IND(bord, iy, iz); i < ORC_IND(sx - bord, iy, iz); i++) pDx[i] = der1_f(pc, i, strideX, dxinv);
#pragma omp for nowait
    for (int iz = 0; iz < sz; iz++)
      for (int iy = bord; iy < sy - bord; iy++)
        for (long i = ORC_IND(bord, iy, iz); i < ORC_IND(sx, iy, iz); i++) pDy[i] = der1_f(pc, i, strideY, dyinv);
#pragma omp for nowait
    for (int iz = 0; iz < sz; iz++)
      for (int iy = 0; iy < sy; iy++)
        for (long i = ORC_IND(bord, iy, iz); i < ORC_IND(sx - bord, iy, iz); i++) qDx[i] = der1_f(qc, i, strideX, dxinv);
#pragma omp for
    for (int iz = 0; iz < sz; iz++)
      for (int iy = bord; iy < sy - bord; iy++)
        for (long i = ORC_IND(bord, iy, iz); i < ORC_IND(sx, iy, iz); i++) qDy[i] = der1_f(qc, i, strideY, dyinv);
#pragma omp for
    for (int iz = bord; iz < sz - bord; iz++)
      for (int iy = bord; iy < sy - bord; iy++)
        for (int ix = bord; ix < sx - bord; ix++) {
          const long i = ORC_IND(ix, iy, iz);
          const float pxy = der1_f(pDx, i, strideY, dyinv);
          const float pxz = der1_f(pDx, i, strideZ, dzinv);
          const float pyz = der1_f(pDy, i, strideZ, dzinv);
          const float pxx = der2_f(pc, i, strideX, dxxinv);
          const float pyy = der2_f(pc, i, strideY, dyyinv);
          const float pzz = der2_f(pc, i, strideZ, dzzinv);
          const float cpxx = ch1dxx[i] * pxx;
          const float cpyy = ch1dyy[i] * pyy;
          const float cpzz = ch1dzz[i] * pzz;
          const float cpxy = ch1dxy[i] * pxy;
          const float cpxz = ch1dxz[i] * pxz;
          const float cpyz = ch1dyz[i] * pyz;
          const float h1p = cpxx + cpyy + cpzz + cpxy + cpxz + cpyz;
          const float h2p = pxx + pyy + pzz - h1p;
          const float qxy = der1_f(qDx, i, strideY, dyinv);
          const float qxz = der1_f(qDx, i, strideZ, dzinv);
          const float qyz = der1_f(qDy, i, strideZ, dzinv);
          const float qxx = der2_f(qc, i, strideX, dxxinv);
          const float qyy = der2_f(qc, i, strideY, dyyinv);
          const float qzz = der2_f(qc, i, strideZ, dzzinv);
          const float cqxx = ch1dxx[i] * qxx;
          const float cqyy = ch1dyy[i] * qyy;
          const float cqzz = ch1dzz[i] * qzz;
          const float cqxy = ch1dxy[i] * qxy;
          const float cqxz = ch1dxz[i] * qxz;
          const float cqyz = ch1dyz[i] * qyz;
          const float h1q = cqxx + cqyy + cqzz + cqxy + cqxz + cqyz;
          const float h2q = qxx + qyy + qzz - h1q;
          const float h1pmq = h1p - h1q;
          const float h2pmq = h2p - h2q;
          const float rhsp = v2px[i] * h2p + v2pz[i] * h1q + v2sz[i] * h1pmq;
          const float rhsq = v2pn[i] * h2p + v2pz[i] * h1q - v2sz[i] * h2pmq;
          pp[i] = 2.0f * pc[i] - pp[i] + rhsp * dt * dt;
          qp[i] = 2.0f * qc[i] - qp[i] + rhsq * dt * dt;
        }
  }
}

/* The time loop of orc_run_f32 with the Der1-Der1 step. */
int orc_run_d1d1_f32(int sx, int sy, int sz, int bord, float dx, float dy, float dz, float dt, int st,
                     long iSource, double fcut, float *pp, float *pc, float *qp, float *qc, const float *coef) {
  const long n = (long)sx * sy * sz;
  float *work = (float *)calloc((size_t)(4 * n), sizeof(float));
  if (!work) return -1;
  for (int it = 1; it <= st; it++) {
    float src = orc_source(dt, it - 1, fcut);
    pc[iSource] += src;
    qc[iSource] += src;
    orc_propagate_d1d1_f32(sx, sy, sz, bord, dx, dy, dz, dt, pp, pc, qp, qc, coef, work);
    float *t = pp; pp = pc; pc = t;
    t = qp; qp = qc; qc = t;
  }
  free(work);
  return st & 1;
}

/* FP64 time loop: same sequence, double fields, double source values. */
int orc_run_f64(int sx, int sy, int sz, int bord, double dx, double dy, double dz, double dt,
                int st, long iSource, double fcut, double *pp, double *pc, double *qp, double *qc,
                const double *coef) {
  for (int it = 1; it <= st; it++) {
    double src = source_d(dt, it - 1, fcut);
    pc[iSource] += src;
    qc[iSource] += src;
    orc_propagate_f64(sx, sy, sz, bord, dx, dy, dz, dt, pp, pc, qp, qc, coef);
    double *t = pp; pp = pc; pc = t;
    t = qp; qp = qc; qc = t;
  }
  return st & 1;
}

/* Advisory stable time step, original/main.c:225-239 (MI = 0.2,
 * original/fletcher.h:1). */
float orc_recommended_dt(long n, const float *vpz, const float *epsilon, float dx, float dy, float dz) {
  float maxvel = vpz[0] * sqrt(1.0 + 2 * epsilon[0]);
  for (long i = 1; i < n; i++) maxvel = fmaxf(maxvel, vpz[i] * sqrt(1.0 + 2 * epsilon[i]));
  float mindelta = dx;
  if (dy < mindelta) mindelta = dy;
  if (dz < mindelta) mindelta = dz;
  return (0.2 * mindelta) / maxvel;
}

/* Host threads the OpenMP loops use. */
int orc_threads(void) { return omp_get_max_threads(); }

/* ---- FP16-storage emulation -------------------------------------------
 * The reduced-precision form stores p and q as FP16 with one power-of-two
 * scale per z-plane (per field buffer) and does all arithmetic in FP32.
 * `orc_quantize_planes` rounds a field to that storage (round to nearest
 * even, scale 2^k chosen so the plane's largest magnitude lands in
 * [2^13, 2^14)), in place, returning the values the kernel would read.
 * Used by the tests to bound the storage error against the FP64 oracle. */
static float q16(float v, float scale, float inv) {
  _Float16 h = (_Float16)(v * scale);
  return (float)h * inv;
}

void orc_quantize_planes(int sx, int sy, int sz, float *f) {
  const long plane = (long)sx * sy;
#pragma omp parallel for schedule(static)
  for (int z = 0; z < sz; z++) {
    float m = 0.0f;
    for (long i = z * plane; i < (z + 1) * plane; i++) m = fmaxf(m, fabsf(f[i]));
    if (m == 0.0f) continue;
    int e;
    frexpf(m, &e); /* m in [2^(e-1), 2^e) */
    if (e < -100) e = -100; /* keep 2^(14-e) finite; such planes round to zero */
    const float scale = ldexpf(1.0f, 14 - e), inv = ldexpf(1.0f, e - 14);
    for (long i = z * plane; i < (z + 1) * plane; i++) f[i] = q16(f[i], scale, inv);
  }
}

/* Other 16/24-bit storage candidates for the same experiment:
 * mode 1: 16-bit fixed point per plane, value = k * 2^(e-15), |k| <= 32767,
 *         with 2^e >= the plane's largest magnitude (block floating point);
 * mode 2: FP16 plus an 8-bit mantissa extension: the float rounded to 19
 *         significant bits (round to nearest even on the 5 dropped bits). */
static float qfix16(float v, float scale, float inv) {
  float k = rintf(v * scale);
  if (k > 32767.0f) k = 32767.0f;
  if (k < -32767.0f) k = -32767.0f;
  return k * inv;
}
static float q19(float v) {
  uint32_t u;
  memcpy(&u, &v, 4);
  const uint32_t lsb = (u >> 5) & 1u;
  u = (u + 0xFu + lsb) & ~0x1Fu;
  float r;
  memcpy(&r, &u, 4);
  return r;
}
void orc_quantize_planes_mode(int sx, int sy, int sz, float *f, int mode) {
  if (mode == 0) {
    orc_quantize_planes(sx, sy, sz, f);
    return;
  }
  const long plane = (long)sx * sy;
#pragma omp parallel for schedule(static)
  for (int z = 0; z < sz; z++) {
    if (mode == 2) {
      for (long i = z * plane; i < (z + 1) * plane; i++) f[i] = q19(f[i]);
      continue;
    }
    float m = 0.0f;
    for (long i = z * plane; i < (z + 1) * plane; i++) m = fmaxf(m, fabsf(f[i]));
    if (m == 0.0f) continue;
    int e;
    frexpf(m, &e);
    if (e < -100) e = -100;
    const float scale = ldexpf(1.0f, 15 - e), inv = ldexpf(1.0f, e - 15);
    for (long i = z * plane; i < (z + 1) * plane; i++) f[i] = qfix16(f[i], scale, inv);
  }
}
