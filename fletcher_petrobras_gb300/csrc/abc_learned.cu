// Learned absorbing boundary: a thin layer around the interior whose outer
// cells are advanced by a one-way (outgoing-wave) update with a per-cell
// coefficient predicted by a small MLP.
//
// Geometry.  The grid is interior + a layer of L cells + bord zero cells on
// every side; the plain update runs over interior and layer alike (the
// medium is extended into the layer, no random velocities).  A layer cell d
// cells outside the interior along an axis has an update stencil (radius 4)
// reaching d + 4 cells out; for the layer's outer 4 cells (d = L-3 .. L,
// the ghost zone) that reaches the zero border, where an unbounded medium
// would hold the outgoing wave.  After the plain step those cells are
// overwritten with the box-scheme update of the one-way wave equation
// u_t + c u_n = 0 along the outward normal n,
//
//     u_g(t+1) = u_i(t) + k (u_g(t) - u_i(t+1)),   k = (1 - r) / (1 + r),  r = c dt / h
//
// (g the ghost cell, i its inward neighbour), applied outward from d = L-3
// (whose inward neighbour carries the plain update) to d = L, for p and q,
// face by face: the z faces, then the y faces, then the x faces (edge and
// corner cells keep the last face's value).  For r > 0 the box scheme of
// the one-way equation is unconditionally stable and 0 < k < 1.
//
//  * FLETCHER_BOUNDARY_ONEWAY: k from the medium, c = vpz along z and
//    vpz sqrt(1 + 2 epsilon) along x and y (the normal-incidence P-wave
//    velocities of a vertical-axis medium);
//  * FLETCHER_BOUNDARY_LEARNED: (k_p, k_q) = sigmoid(network(inputs)) per
//    ghost cell and step.  The inputs are the 9-point stencils of p and q
//    along the outward normal at t and t-1 (points beyond the layer read as
//    zero) divided by their largest magnitude s, vpz / 4000, epsilon, delta
//    and d / L; the network learns the coefficient with which the update
//    reproduces the unbounded medium's next value (oblique incidence,
//    tilted anisotropy, the wave's own apparent velocity).
//
// Network: 40 -> 32 -> 32 -> 2, tanh, FP16 weights and FP16 activations
// between layers, FP32 accumulation and FP32 biases.
//   * inference runs on the tensor cores (mma.sync m16n8k16, f16 x f16 ->
//     f32) inside the boundary kernel (k_abc_boundary, one cooperative launch
//     after the plain step that also applies the one-way update): one warp
//     evaluates 16 ghost cells, the layer-1 and layer-2 outputs stay in
//     registers as the next layer's A fragments, and k stays in registers
//     until the update uses it; the weights' B fragments are read from a
//     shared-memory copy (in registers they took 62 of 128, and the SM held
//     16 warps instead of 24: 119 against 90 us per evaluating step at
//     256^3);
//   * training (k_abc_train) is a per-sample forward and backward pass in
//     FP32 with the same roundings (straight-through), block sums of the
//     gradients added up in block order (k_abc_reduce: training is
//     reproducible bit for bit), and Adam (k_abc_adam) on FP32 master
//     weights.  The loss of
//     a sample is sum_c (sigmoid(y_c) a_c - b_c)^2 with a = (u_g(t) -
//     u_i(t+1)) / s and b = (u_g(t+1) - u_i(t)) / s: the update's error
//     when the neighbour's next value is the true one.
//
// Training data (k_abc_collect) come from plain-method runs on padded
// domains: around a virtual interior box, the ghost cells' inputs are read
// with everything beyond the virtual layer set to zero, and the next values
// u(t+1) are the plain update on the padded field (an unbounded medium as
// far as the ghost cells can tell).
#include <cuda_fp16.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>

#include <algorithm>
#include <vector>

#include "../../include/fletcher_gb300.h"
#include "device_util.cuh"
#include "fletcher_internal.h"
#include "stencil_common.cuh"

int flt_record_error(int code, const char *msg);

namespace flt {

constexpr int kIn = 40, kHid = 32, kOut = 2;
constexpr int kTgt = 4;   // targets of a sample: a_p, a_q, b_p, b_q
constexpr int kSt = 36;   // stencil inputs (4 x 9)
// Master parameter layout (FP32): W1 [32][40], b1, W2 [32][32], b2, W3 [2][32], b3.
constexpr int oW1 = 0, oB1 = oW1 + kHid * kIn, oW2 = oB1 + kHid, oB2 = oW2 + kHid * kHid, oW3 = oB2 + kHid,
              oB3 = oW3 + kOut * kHid, kNP = oB3 + kOut;
static_assert(kNP == FLETCHER_ABC_PARAMS, "parameter count");
constexpr int kK1 = 48;      // layer-1 K padded to a multiple of 16
constexpr int kXs = 56;      // row stride (halves) of a warp's feature tile: conflict-free A loads
constexpr float kVScale = 1.0f / 4000.0f;
constexpr float kMinScale = 1e-30f;  // smallest stencil magnitude the network sees
constexpr int kGhostD = kRadius;     // ghost cells per ray: the layer's outer 4
constexpr float kInitBias = 0.85f;   // initial output bias: k ~ 0.7 (r ~ 0.18)

// Inference copy of the network: FP16 weights in mma B-operand order
// (row n = output, contiguous k), FP32 biases.
struct NetHalf {
  __half w1[kHid * kK1];
  __half w2[kHid * kHid];
  __half w3[8 * kHid];
  float b1[kHid], b2[kHid], b3[8];
};

// A box [lo, hi) per axis.
struct Box {
  int lo[3], hi[3];
};

// One layer cell (the taper's list): position and distance d.
struct LayerCell {
  int x, y, z, d;
};

// The ghost zone of a layer: the interior box, the layer, the kept box
// (interior grown by L) and the first cell of each face.  Faces 0..5 are
// z-, z+, y-, y+, x-, x+; a face is a set of rays along its outward normal,
// one per transverse position of the kept box (first transverse axis
// fastest), 4 cells per ray (d = L-3 .. L, d fastest).
struct Ghost {
  Box in, keep;
  int L;
  long off[7];
};

__host__ __device__ __forceinline__ int face_axis(int f) { return 2 - f / 2; }
__host__ __device__ __forceinline__ int face_sign(int f) { return (f & 1) ? 1 : -1; }
__host__ __device__ __forceinline__ void transverse(int a, int &t0, int &t1) {
  t0 = a == 0 ? 1 : 0;
  t1 = a == 2 ? 1 : 2;
}

Ghost make_ghost(const Box &in, int L) {
  Ghost G;
  G.in = in;
  G.L = L;
  for (int a = 0; a < 3; ++a) {
    G.keep.lo[a] = in.lo[a] - L;
    G.keep.hi[a] = in.hi[a] + L;
  }
  G.off[0] = 0;
  for (int f = 0; f < 6; ++f) {
    int t0, t1;
    transverse(face_axis(f), t0, t1);
    const long rays = (long)(G.keep.hi[t0] - G.keep.lo[t0]) * (G.keep.hi[t1] - G.keep.lo[t1]);
    G.off[f + 1] = G.off[f] + rays * kGhostD;
  }
  return G;
}

// Ghost cell i: coordinates c, face f, normal axis a, outward sign; returns d.
__host__ __device__ __forceinline__ int ghost_cell(const Ghost &G, long i, int (&c)[3], int &f, int &a, int &sgn) {
  f = 0;
  while (f < 5 && i >= G.off[f + 1]) ++f;
  const long j = i - G.off[f];
  a = face_axis(f);
  sgn = face_sign(f);
  int t0, t1;
  transverse(a, t0, t1);
  const int e0 = G.keep.hi[t0] - G.keep.lo[t0];
  const int ray = (int)(j / kGhostD);  // a face holds fewer than 2^31 rays
  const int d = G.L - kGhostD + 1 + (int)(j % kGhostD);
  c[t0] = G.keep.lo[t0] + ray % e0;
  c[t1] = G.keep.lo[t1] + ray / e0;
  c[a] = sgn < 0 ? G.in.lo[a] - d : G.in.hi[a] - 1 + d;
  return d;
}

__host__ __device__ __forceinline__ int face_of(const Ghost &G, long i) {
  int f = 0;
  while (f < 5 && i >= G.off[f + 1]) ++f;
  return f;
}

// Index step of one cell outward along face f's normal.
__host__ __device__ __forceinline__ int normal_step(int f, int sy, int pitch) {
  const int a = face_axis(f);
  const int s = a == 0 ? 1 : (a == 1 ? pitch : sy * pitch);
  return face_sign(f) > 0 ? s : -s;
}

__host__ __device__ __forceinline__ long cell_index(int x, int y, int z, int sy, int pitch) {
  return ((long)z * sy + y) * pitch + x;
}

// Index in the field of ghost cell i and its face (ghost_cell without an
// indexed coordinate array, for the hot kernels).
__device__ __forceinline__ long ghost_index(const Ghost &G, long i, int sy, int pitch, int &f) {
  f = face_of(G, i);
  const long j = i - G.off[f];
  const int a = face_axis(f);
  const int t0 = a == 0 ? 1 : 0, t1 = a == 2 ? 1 : 2;
  const int e0 = G.keep.hi[t0] - G.keep.lo[t0];
  const int ray = (int)(j / kGhostD);
  const int d = G.L - kGhostD + 1 + (int)(j % kGhostD);
  const int u = G.keep.lo[t0] + ray % e0, v = G.keep.lo[t1] + ray / e0;
  const int n = face_sign(f) < 0 ? G.in.lo[a] - d : G.in.hi[a] - 1 + d;
  const int x = a == 0 ? n : u;
  const int y = a == 1 ? n : (a == 0 ? u : v);
  const int z = a == 2 ? n : v;
  return cell_index(x, y, z, sy, pitch);
}

// ---- features -------------------------------------------------------------------

// vpz, epsilon, delta of a cell from its coefficients (v2pz = vpz^2,
// v2px = vpz^2 (1 + 2 eps), v2pn = vpz^2 (1 + 2 delta): original/precomp.h).
__device__ __forceinline__ float4 medium_of(const float *coef, int x, int y, int z, int sy, int pitch) {
  const size_t plane = (size_t)sy * pitch, row = (size_t)y * pitch + x;
  const size_t base = (size_t)z * kNumCoef * plane + row;
  const float v2px = coef[base + DC_V2PX * plane], v2pz = coef[base + DC_V2PZ * plane];
  const float v2pn = coef[base + DC_V2PN * plane];
  float4 m;
  m.x = sqrtf(v2pz);
  m.y = v2pz > 0.f ? 0.5f * (v2px / v2pz - 1.0f) : 0.f;
  m.z = v2pz > 0.f ? 0.5f * (v2pn / v2pz - 1.0f) : 0.f;
  m.w = 0.f;
  return m;
}

// The 9 (p, q) values of field F along axis a from (x, y, z), offsets
// sign * (-4 .. 4); points outside `keep` read as zero.
__device__ __forceinline__ void normal_stencil(const float2 *F, int x, int y, int z, int a, int sgn, const Box &keep,
                                               int sy, int pitch, float *p9, float *q9) {
#pragma unroll
  for (int j = -kRadius; j <= kRadius; ++j) {
    int c[3] = {x, y, z};
    c[a] += sgn * j;
    float2 v = make_float2(0.f, 0.f);
    if (c[0] >= keep.lo[0] && c[0] < keep.hi[0] && c[1] >= keep.lo[1] && c[1] < keep.hi[1] && c[2] >= keep.lo[2] &&
        c[2] < keep.hi[2])
      v = F[cell_index(c[0], c[1], c[2], sy, pitch)];
    p9[j + kRadius] = v.x;
    q9[j + kRadius] = v.y;
  }
}

// One-way coefficient of the medium along axis a: k = (1 - r) / (1 + r),
// r = c dt / h, c = vpz (z) or vpz sqrt(1 + 2 eps) (x, y).
__host__ __device__ __forceinline__ float oneway_k(float vpz, float eps, int a, float dt, float h) {
  const float c = a == 2 ? vpz : vpz * sqrtf(1.0f + 2.0f * eps);
  const float r = c * dt / h;
  return (1.0f - r) / (1.0f + r);
}

// ---- the plain update's rhs over the cells outside a box (an empty box: every cell) ----

// (p, q) of the current field at a cell, if it lies outside `keep`.
__device__ __forceinline__ float2 outer(const float2 *F, int x, int y, int z, const Box &keep, int sy, int pitch) {
  const bool in = x >= keep.lo[0] && x < keep.hi[0] && y >= keep.lo[1] && y < keep.hi[1] && z >= keep.lo[2] &&
                  z < keep.hi[2];
  if (in) return make_float2(0.f, 0.f);
  return F[((size_t)z * sy + y) * pitch + x];
}

// dt^2 * (rhsp, rhsq) of original/sample.h:32-89 evaluated on the field
// outside `keep` (it is linear in the field; an empty `keep` gives the
// whole update).
__device__ float2 outer_update(const float2 *F, const float *coef, int x, int y, int z, const Box &keep, int sy,
                               int pitch, float dx, float dy, float dz, float dt) {
  const float K[5] = {cK0, cK1, cK2, cK3, cK4};
  const float Lw[5] = {0.f, cL1, cL2, cL3, cL4};
  // The centre term counts when the cell itself lies outside `keep`.
  const float2 u0 = outer(F, x, y, z, keep, sy, pitch);
  float2 d2[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) d2[a] = make_float2(K[0] * u0.x, K[0] * u0.y);
  const int cx[3] = {1, 0, 0}, cy[3] = {0, 1, 0}, cz[3] = {0, 0, 1};
#pragma unroll
  for (int a = 0; a < 3; ++a)
    for (int k = 1; k <= kRadius; ++k) {
      const float2 u = outer(F, x + k * cx[a], y + k * cy[a], z + k * cz[a], keep, sy, pitch);
      const float2 w = outer(F, x - k * cx[a], y - k * cy[a], z - k * cz[a], keep, sy, pitch);
      d2[a].x += K[k] * (u.x + w.x);
      d2[a].y += K[k] * (u.y + w.y);
    }
  // Mixed derivatives: xy, yz, xz.
  const int pa[3] = {0, 1, 0}, pb[3] = {1, 2, 2};
  float2 dc[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
#pragma unroll
  for (int m = 0; m < 3; ++m)
    for (int i = 1; i <= kRadius; ++i)
      for (int j = 1; j <= kRadius; ++j) {
        int o1[3] = {0, 0, 0}, o2[3] = {0, 0, 0};
        o1[pa[m]] = i;
        o2[pb[m]] = j;
        const float2 pp = outer(F, x + o1[0] + o2[0], y + o1[1] + o2[1], z + o1[2] + o2[2], keep, sy, pitch);
        const float2 pm = outer(F, x + o1[0] - o2[0], y + o1[1] - o2[1], z + o1[2] - o2[2], keep, sy, pitch);
        const float2 mp = outer(F, x - o1[0] + o2[0], y - o1[1] + o2[1], z - o1[2] + o2[2], keep, sy, pitch);
        const float2 mm = outer(F, x - o1[0] - o2[0], y - o1[1] - o2[1], z - o1[2] - o2[2], keep, sy, pitch);
        const float w = Lw[i] * Lw[j];
        dc[m].x += w * (pp.x - pm.x - mp.x + mm.x);
        dc[m].y += w * (pp.y - pm.y - mp.y + mm.y);
      }
  const float sx2 = 1.0f / (dx * dx), sy2 = 1.0f / (dy * dy), sz2 = 1.0f / (dz * dz);
  const float sxy = 1.0f / (dx * dy), syz = 1.0f / (dy * dz), sxz = 1.0f / (dx * dz);
  const float pxx = d2[0].x * sx2, pyy = d2[1].x * sy2, pzz = d2[2].x * sz2;
  const float qxx = d2[0].y * sx2, qyy = d2[1].y * sy2, qzz = d2[2].y * sz2;
  const float pxy = dc[0].x * sxy, pyz = dc[1].x * syz, pxz = dc[2].x * sxz;
  const float qxy = dc[0].y * sxy, qyz = dc[1].y * syz, qxz = dc[2].y * sxz;
  const size_t plane = (size_t)sy * pitch, base = (size_t)z * kNumCoef * plane + (size_t)y * pitch + x;
  auto C = [&](int k) { return coef[base + k * plane]; };
  const float cxx = C(DC_XX), cyy = C(DC_YY), czz = C(DC_ZZ), cxy = C(DC_XY), cyz = C(DC_YZ), cxz = C(DC_XZ);
  const float h1p = cxx * pxx + cyy * pyy + czz * pzz + cxy * pxy + cyz * pyz + cxz * pxz;
  const float h1q = cxx * qxx + cyy * qyy + czz * qzz + cxy * qxy + cyz * qyz + cxz * qxz;
  const float h2p = pxx + pyy + pzz - h1p, h2q = qxx + qyy + qzz - h1q;
  const float rhsp = C(DC_V2PX) * h2p + C(DC_V2PZ) * h1q + C(DC_V2SZ) * (h1p - h1q);
  const float rhsq = C(DC_V2PN) * h2p + C(DC_V2PZ) * h1q - C(DC_V2SZ) * (h2p - h2q);
  const float dt2 = dt * dt;
  return make_float2(rhsp * dt2, rhsq * dt2);
}

__device__ __forceinline__ uint32_t mix32(uint32_t a, uint32_t b) {
  uint32_t h = a * 0x9E3779B1u ^ (b + 0x7F4A7C15u + (a << 6) + (a >> 2));
  h ^= h >> 16;
  h *= 0x85EBCA6Bu;
  h ^= h >> 13;
  h *= 0xC2B2AE35u;
  h ^= h >> 16;
  return h;
}

// Training samples from the ghost cells of the layer around a virtual
// interior box: features, targets (a_p, a_q, b_p, b_q) over s, and the
// cell (x, y, z, face + 8 d).  A random fraction `keep_frac` of the cells is
// taken; cells whose stencils are below `min_scale` carry no wave and are
// skipped.  The next values are the plain update of original/sample.h:32-89
// (u(t+1) = 2 u(t) - u(t-1) + dt^2 rhs) on the padded field.
//
// The samples land in cell order, so the training set does not depend on
// thread timing: block b takes the cells [b per, (b+1) per); a counting
// pass gives each block's number of samples, their prefix sums (host) its
// first slot, and the writing pass ranks each cell inside its block with
// warp ballots.

// Whether ghost cell i becomes a sample; its stencils and scale.
__device__ __forceinline__ bool collect_cell(const float2 *cur, const float2 *prev, const Ghost &G, long i, int sy,
                                             int pitch, float keep_frac, uint32_t seed, float min_scale, float (&v)[kSt],
                                             float &s, int (&c)[3], int &f, int &a, int &sgn, int &d) {
  if ((mix32(seed, (uint32_t)i) >> 8) * (1.0f / 16777216.0f) >= keep_frac) return false;
  d = ghost_cell(G, i, c, f, a, sgn);
  normal_stencil(cur, c[0], c[1], c[2], a, sgn, G.keep, sy, pitch, v, v + 9);
  normal_stencil(prev, c[0], c[1], c[2], a, sgn, G.keep, sy, pitch, v + 18, v + 27);
  s = 0.f;
#pragma unroll
  for (int k = 0; k < kSt; ++k) s = fmaxf(s, fabsf(v[k]));
  return (s > min_scale) && (s > kMinScale);
}

constexpr int kCollectBlock = 256;

__global__ void __launch_bounds__(kCollectBlock) k_abc_collect_count(const float2 *cur, const float2 *prev,
                                                                     const __grid_constant__ Ghost G, int sy,
                                                                     int pitch, float keep_frac, uint32_t seed,
                                                                     float min_scale, long per, int *block_count) {
  __shared__ int cnt;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  const long n = G.off[6];
  const long lo = blockIdx.x * per, hi = min(n, lo + per);
  int mine = 0;
  for (long i = lo + threadIdx.x; i < hi; i += kCollectBlock) {
    float v[kSt], sc;
    int c[3], f, a, sgn, d;
    mine += collect_cell(cur, prev, G, i, sy, pitch, keep_frac, seed, min_scale, v, sc, c, f, a, sgn, d) ? 1 : 0;
  }
  atomicAdd(&cnt, mine);  // an integer count: the order does not matter
  __syncthreads();
  if (threadIdx.x == 0) block_count[blockIdx.x] = cnt;
}

__global__ void __launch_bounds__(kCollectBlock) k_abc_collect(const float2 *cur, const float2 *prev,
                                                               const float *coef, const __grid_constant__ Ghost G,
                                                               int sy, int pitch, float dx, float dy, float dz,
                                                               float dt, float keep_frac, uint32_t seed,
                                                               float min_scale, long per, const long *block_first,
                                                               float *feat, float *tgt, int4 *pos, long cap) {
  __shared__ int warp_sum[kCollectBlock / 32];
  const long n = G.off[6];
  const long lo = blockIdx.x * per, hi = min(n, lo + per);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const Box all = {{0, 0, 0}, {0, 0, 0}};  // empty kept box: the whole field counts
  long next = block_first[blockIdx.x];  // slot of this block's next sample
  for (long c0 = lo; c0 < hi; c0 += kCollectBlock) {
    const long i = c0 + threadIdx.x;
    float v[kSt], s = 0.f;
    int c[3] = {0, 0, 0}, f = 0, a = 0, sgn = 1, d = 0;
    const bool keep =
        i < hi && collect_cell(cur, prev, G, i, sy, pitch, keep_frac, seed, min_scale, v, s, c, f, a, sgn, d);
    // Rank in cell order: lanes before this one in the warp, then warps before it.
    const unsigned ball = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) warp_sum[warp] = __popc(ball);
    __syncthreads();
    int before = __popc(ball & ((1u << lane) - 1u)), total = 0;
#pragma unroll
    for (int w = 0; w < kCollectBlock / 32; ++w) {
      before += w < warp ? warp_sum[w] : 0;
      total += warp_sum[w];
    }
    __syncthreads();
    const long slot = next + before;
    next += total;
    if (!keep || slot >= cap) continue;
    pos[slot] = make_int4(c[0], c[1], c[2], f + 8 * d);
    const float inv = 1.0f / s;
    float *fr = feat + slot * kIn;
#pragma unroll
    for (int k = 0; k < kSt; ++k) fr[k] = v[k] * inv;
    const float4 m = medium_of(coef, c[0], c[1], c[2], sy, pitch);
    fr[36] = m.x * kVScale;
    fr[37] = m.y;
    fr[38] = m.z;
    fr[39] = (float)d / (float)G.L;
    int ci[3] = {c[0], c[1], c[2]};
    ci[a] -= sgn;
    const long g = cell_index(c[0], c[1], c[2], sy, pitch), gi = cell_index(ci[0], ci[1], ci[2], sy, pitch);
    const float2 ug = cur[g], ui = cur[gi], ugm = prev[g], uim = prev[gi];
    const float2 rg = outer_update(cur, coef, c[0], c[1], c[2], all, sy, pitch, dx, dy, dz, dt);
    const float2 ri = outer_update(cur, coef, ci[0], ci[1], ci[2], all, sy, pitch, dx, dy, dz, dt);
    const float ugx = 2.0f * ug.x - ugm.x + rg.x, ugy = 2.0f * ug.y - ugm.y + rg.y;
    const float uix = 2.0f * ui.x - uim.x + ri.x, uiy = 2.0f * ui.y - uim.y + ri.y;
    float *t = tgt + slot * kTgt;
    t[0] = (ug.x - uix) * inv;
    t[1] = (ug.y - uiy) * inv;
    t[2] = (ugx - ui.x) * inv;
    t[3] = (ugy - ui.y) * inv;
  }
}

// ---- inference on the tensor cores ---------------------------------------------

__device__ __forceinline__ void mma16816(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_h2(float lo_v, float hi_v) {
  const __half2 h = __floats2half2_rn(lo_v, hi_v);
  return *reinterpret_cast<const uint32_t *>(&h);
}

// tanh of two pre-activations, rounded to FP16 first, as one packed
// half2 tanh.approx (the activations feed the next MMA as FP16 anyway).
__device__ __forceinline__ uint32_t tanh_h2(float lo_v, float hi_v) {
  uint32_t x = pack_h2(lo_v, hi_v), y;
  asm("tanh.approx.f16x2 %0, %1;" : "=r"(y) : "r"(x));
  return y;
}

// A lane's share of the network for mma.sync m16n8k16: the B fragments of
// the three layers and the biases of the output columns it holds (g = lane
// / 4 selects the row of B, t = lane % 4 the column pair).  Loaded once per
// warp, kept in registers.
struct Frags {
  uint32_t w1[4][3][2];  // layer 1: n-tile, k-step, (k 2t, k 2t+8)
  uint32_t w2[4][2][2];  // layer 2
  uint32_t w3[2][2];     // layer 3 (n-tile 0)
  float b1[4][2], b2[4][2], b3[2];
};

__device__ __forceinline__ void load_frags(const NetHalf *__restrict__ N, Frags &F) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const uint32_t *w1 = reinterpret_cast<const uint32_t *>(N->w1);
  const uint32_t *w2 = reinterpret_cast<const uint32_t *>(N->w2);
  const uint32_t *w3 = reinterpret_cast<const uint32_t *>(N->w3);
#pragma unroll
  for (int nt = 0; nt < 4; ++nt) {
#pragma unroll
    for (int ks = 0; ks < 3; ++ks) {
      const int o = ((8 * nt + g) * kK1 + 16 * ks + 2 * t) / 2;
      F.w1[nt][ks][0] = w1[o];
      F.w1[nt][ks][1] = w1[o + 4];
    }
#pragma unroll
    for (int kt = 0; kt < 2; ++kt) {
      const int o = ((8 * nt + g) * kHid + 16 * kt + 2 * t) / 2;
      F.w2[nt][kt][0] = w2[o];
      F.w2[nt][kt][1] = w2[o + 4];
    }
    F.b1[nt][0] = N->b1[8 * nt + 2 * t];
    F.b1[nt][1] = N->b1[8 * nt + 2 * t + 1];
    F.b2[nt][0] = N->b2[8 * nt + 2 * t];
    F.b2[nt][1] = N->b2[8 * nt + 2 * t + 1];
  }
#pragma unroll
  for (int kt = 0; kt < 2; ++kt) {
    const int o = (g * kHid + 16 * kt + 2 * t) / 2;
    F.w3[kt][0] = w3[o];
    F.w3[kt][1] = w3[o + 4];
  }
  F.b3[0] = N->b3[2 * t];
  F.b3[1] = N->b3[2 * t + 1];
}

// The network on the warp's 16-row feature tile Xs (FP16, row stride kXs).
// Lanes with (lane & 3) == 0 return the outputs of rows lane/4 and lane/4+8.
__device__ __forceinline__ void mlp16(const __half *Xs, const Frags &F, float (&y_lo)[2], float (&y_hi)[2]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  uint32_t a[3][4];
#pragma unroll
  for (int ks = 0; ks < 3; ++ks) {
    a[ks][0] = *reinterpret_cast<const uint32_t *>(Xs + g * kXs + 16 * ks + 2 * t);
    a[ks][1] = *reinterpret_cast<const uint32_t *>(Xs + (g + 8) * kXs + 16 * ks + 2 * t);
    a[ks][2] = *reinterpret_cast<const uint32_t *>(Xs + g * kXs + 16 * ks + 2 * t + 8);
    a[ks][3] = *reinterpret_cast<const uint32_t *>(Xs + (g + 8) * kXs + 16 * ks + 2 * t + 8);
  }
  float h[4][4];
#pragma unroll
  for (int nt = 0; nt < 4; ++nt) {
    h[nt][0] = F.b1[nt][0]; h[nt][1] = F.b1[nt][1]; h[nt][2] = F.b1[nt][0]; h[nt][3] = F.b1[nt][1];
#pragma unroll
    for (int ks = 0; ks < 3; ++ks) mma16816(h[nt], a[ks], F.w1[nt][ks][0], F.w1[nt][ks][1]);
  }
  uint32_t a2[2][4];
#pragma unroll
  for (int kt = 0; kt < 2; ++kt) {
    a2[kt][0] = tanh_h2(h[2 * kt][0], h[2 * kt][1]);
    a2[kt][1] = tanh_h2(h[2 * kt][2], h[2 * kt][3]);
    a2[kt][2] = tanh_h2(h[2 * kt + 1][0], h[2 * kt + 1][1]);
    a2[kt][3] = tanh_h2(h[2 * kt + 1][2], h[2 * kt + 1][3]);
  }
#pragma unroll
  for (int nt = 0; nt < 4; ++nt) {
    h[nt][0] = F.b2[nt][0]; h[nt][1] = F.b2[nt][1]; h[nt][2] = F.b2[nt][0]; h[nt][3] = F.b2[nt][1];
#pragma unroll
    for (int kt = 0; kt < 2; ++kt) mma16816(h[nt], a2[kt], F.w2[nt][kt][0], F.w2[nt][kt][1]);
  }
#pragma unroll
  for (int kt = 0; kt < 2; ++kt) {
    a2[kt][0] = tanh_h2(h[2 * kt][0], h[2 * kt][1]);
    a2[kt][1] = tanh_h2(h[2 * kt][2], h[2 * kt][3]);
    a2[kt][2] = tanh_h2(h[2 * kt + 1][0], h[2 * kt + 1][1]);
    a2[kt][3] = tanh_h2(h[2 * kt + 1][2], h[2 * kt + 1][3]);
  }
  float o[4] = {F.b3[0], F.b3[1], F.b3[0], F.b3[1]};
#pragma unroll
  for (int kt = 0; kt < 2; ++kt) mma16816(o, a2[kt], F.w3[kt][0], F.w3[kt][1]);
  y_lo[0] = o[0];
  y_lo[1] = o[1];
  y_hi[0] = o[2];
  y_hi[1] = o[3];
}

// The same fragments in shared memory, lane-minor with a lane's two words
// side by side ([..][lane][2]: one 8-byte load per MMA operand or bias
// pair, a warp's 32 lanes reading 256 consecutive bytes, no bank conflict),
// for the boundary kernel: there the 62 registers of Frags would hold the
// SM to 16 warps.
struct FragsSmem {
  uint2 w1[4][3][32];
  uint2 w2[4][2][32];
  uint2 w3[2][32];
  float2 b1[4][32], b2[4][32], b3[32];
};

// Fills S from the network, warp 0 writing its lanes' fragments.
__device__ __forceinline__ void frags_to_smem(const NetHalf *__restrict__ N, FragsSmem &S) {
  if (threadIdx.x >= 32) return;
  const int lane = threadIdx.x;
  Frags F;
  load_frags(N, F);
#pragma unroll
  for (int nt = 0; nt < 4; ++nt) {
#pragma unroll
    for (int ks = 0; ks < 3; ++ks) S.w1[nt][ks][lane] = make_uint2(F.w1[nt][ks][0], F.w1[nt][ks][1]);
#pragma unroll
    for (int kt = 0; kt < 2; ++kt) S.w2[nt][kt][lane] = make_uint2(F.w2[nt][kt][0], F.w2[nt][kt][1]);
    S.b1[nt][lane] = make_float2(F.b1[nt][0], F.b1[nt][1]);
    S.b2[nt][lane] = make_float2(F.b2[nt][0], F.b2[nt][1]);
  }
#pragma unroll
  for (int kt = 0; kt < 2; ++kt) S.w3[kt][lane] = make_uint2(F.w3[kt][0], F.w3[kt][1]);
  S.b3[lane] = make_float2(F.b3[0], F.b3[1]);
}

// mlp16 with the B fragments and biases read from shared memory.
__device__ __forceinline__ void mlp16_smem(const __half *Xs, const FragsSmem &S, float (&y_lo)[2],
                                           float (&y_hi)[2]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  uint32_t a[3][4];
#pragma unroll
  for (int ks = 0; ks < 3; ++ks) {
    a[ks][0] = *reinterpret_cast<const uint32_t *>(Xs + g * kXs + 16 * ks + 2 * t);
    a[ks][1] = *reinterpret_cast<const uint32_t *>(Xs + (g + 8) * kXs + 16 * ks + 2 * t);
    a[ks][2] = *reinterpret_cast<const uint32_t *>(Xs + g * kXs + 16 * ks + 2 * t + 8);
    a[ks][3] = *reinterpret_cast<const uint32_t *>(Xs + (g + 8) * kXs + 16 * ks + 2 * t + 8);
  }
  float h[4][4];
#pragma unroll
  for (int nt = 0; nt < 4; ++nt) {
    const float2 c = S.b1[nt][lane];
    h[nt][0] = c.x; h[nt][1] = c.y; h[nt][2] = c.x; h[nt][3] = c.y;
#pragma unroll
    for (int ks = 0; ks < 3; ++ks) {
      const uint2 w = S.w1[nt][ks][lane];
      mma16816(h[nt], a[ks], w.x, w.y);
    }
  }
  uint32_t a2[2][4];
#pragma unroll
  for (int kt = 0; kt < 2; ++kt) {
    a2[kt][0] = tanh_h2(h[2 * kt][0], h[2 * kt][1]);
    a2[kt][1] = tanh_h2(h[2 * kt][2], h[2 * kt][3]);
    a2[kt][2] = tanh_h2(h[2 * kt + 1][0], h[2 * kt + 1][1]);
    a2[kt][3] = tanh_h2(h[2 * kt + 1][2], h[2 * kt + 1][3]);
  }
#pragma unroll
  for (int nt = 0; nt < 4; ++nt) {
    const float2 c = S.b2[nt][lane];
    h[nt][0] = c.x; h[nt][1] = c.y; h[nt][2] = c.x; h[nt][3] = c.y;
#pragma unroll
    for (int kt = 0; kt < 2; ++kt) {
      const uint2 w = S.w2[nt][kt][lane];
      mma16816(h[nt], a2[kt], w.x, w.y);
    }
  }
#pragma unroll
  for (int kt = 0; kt < 2; ++kt) {
    a2[kt][0] = tanh_h2(h[2 * kt][0], h[2 * kt][1]);
    a2[kt][1] = tanh_h2(h[2 * kt][2], h[2 * kt][3]);
    a2[kt][2] = tanh_h2(h[2 * kt + 1][0], h[2 * kt + 1][1]);
    a2[kt][3] = tanh_h2(h[2 * kt + 1][2], h[2 * kt + 1][3]);
  }
  const float2 ob = S.b3[lane];
  float o[4] = {ob.x, ob.y, ob.x, ob.y};
#pragma unroll
  for (int kt = 0; kt < 2; ++kt) {
    const uint2 w = S.w3[kt][lane];
    mma16816(o, a2[kt], w.x, w.y);
  }
  y_lo[0] = o[0];
  y_lo[1] = o[1];
  y_hi[0] = o[2];
  y_hi[1] = o[3];
}

constexpr int kInferWarps = 8;

__device__ __forceinline__ float sigmoid(float y) { return 1.0f / (1.0f + __expf(-y)); }

// The network on given features (rows of 40 floats), raw outputs.
__global__ void __launch_bounds__(32 * kInferWarps) k_abc_forward(const float *feat, long n, const NetHalf *net,
                                                                   float *out) {
  __shared__ __align__(16) __half Xs[kInferWarps][16 * kXs];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  Frags F;
  load_frags(net, F);
  __half *X = Xs[warp];
  const long ntiles = (n + 15) / 16;
  for (long tile = blockIdx.x * (long)kInferWarps + warp; tile < ntiles; tile += (long)gridDim.x * kInferWarps) {
    for (int e = lane; e < 16 * kK1; e += 32) {
      const int r = e / kK1, k = e % kK1;
      const long row = tile * 16 + r;
      X[r * kXs + k] = __float2half_rn((row < n && k < kIn) ? feat[row * kIn + k] : 0.f);
    }
    __syncwarp();
    float ylo[2], yhi[2];
    mlp16(X, F, ylo, yhi);
    const int g = lane >> 2;
    if ((lane & 3) == 0) {
      const long c0 = tile * 16 + g, c1 = tile * 16 + g + 8;
      if (c0 < n) {
        out[c0 * 2] = ylo[0];
        out[c0 * 2 + 1] = ylo[1];
      }
      if (c1 < n) {
        out[c1 * 2] = yhi[0];
        out[c1 * 2 + 1] = yhi[1];
      }
    }
    __syncwarp();
  }
}

// ---- the boundary step: one cooperative launch after the plain step -----------
//
// Two kernels, one launch per step: k_abc_boundary on the steps where the
// learned form evaluates its network, k_abc_rays_coop on the other steps and
// for the medium's fixed coefficients.  Both run the face pairs normal to z,
// then y, then x, with a bounded grid-wide barrier between them (a pass
// reads the next values the previous pass wrote at edge cells).
//
// k_abc_boundary: every warp takes groups of 4 consecutive rays (16 ghost
// cells):
//  1. lane 8 r + q loads point q (d = L-7+q) of ray r's outward normal line
//     at t from the current field and at t-1 from the line buffer the
//     previous launch filled; it stores the t line when the next step
//     evaluates the network too;
//  2. the 16 cells' features and the network on the tensor cores
//     (mma.sync m16n8k16), two lanes per cell building the t and t-1
//     stencils; k = sigmoid(y) stays in registers (it is written to the
//     coefficient buffer only when later steps reuse it);
//  3. lanes 4 r + j (j = 0..3: d = L-3+j) apply the box-scheme update
//     next_g = cur_i + k (cur_g - next_i) outward along ray r, an inclusive
//     scan of affine maps over the ray's 4 lanes.
// The line buffer replaces the read of the t-1 field, which the plain step
// has overwritten by the time this kernel runs.
struct BoundaryArgs {
  Ghost G;
  const float2 *cur;        // field at t
  float2 *next;             // field at t+1 (the plain step's result)
  int sy, pitch;
  const float4 *med;        // per ghost cell: vpz, epsilon, delta, field index (int bits)
  const NetHalf *net;
  const float2 *line_in;    // per ray: the 8 line points at t-1 (learned form)
  float2 *line_out;         // per ray: the 8 line points at t, for the next launch (learned form)
  float2 *k;                // per ghost cell: (k_p, k_q), read unless the network runs, written when it is kept
  int eval;                 // the network runs at this step
  int keep;                 // store the network's k for the steps that reuse it
  int save;                 // store the t lines (the next step evaluates the network)
  unsigned *bar;            // grid barrier: arrival count, generation
  unsigned *err;            // error word (bit 0: a bounded wait gave up)
  unsigned long long wait_ns;
};

constexpr int kBoundaryWarps = 8;
constexpr int kBoundaryBlocks = 3;  // resident blocks of the network kernel per SM (at most 85 registers)

// Field index of cell d = L-3+j of ray `ray` of the face pair normal to axis
// A (rays [r0, rmid) on the low face, [rmid, ...) on the high one, each face
// in ghost-cell order: first transverse coordinate fastest), and the step
// one cell outward.  The coordinates come from the ray index alone, so the
// field loads do not wait for a table lookup.
__device__ __forceinline__ int ray_cell(const Ghost &G, int A, long ray, long r0, long rmid, int j, int sy, int pitch,
                                        int stride, int &step) {
  const bool high = ray >= rmid;
  const int rs = (int)(ray - (high ? rmid : r0));  // a face holds fewer than 2^31 rays
  const int t0 = A == 0 ? 1 : 0, t1 = A == 2 ? 1 : 2;
  const int e0 = G.keep.hi[t0] - G.keep.lo[t0];
  const int u = G.keep.lo[t0] + rs % e0, v = G.keep.lo[t1] + rs / e0;
  const int d = G.L - kGhostD + 1 + j;
  const int n = high ? G.in.hi[A] - 1 + d : G.in.lo[A] - d;
  const int x = A == 0 ? n : u;
  const int y = A == 0 ? u : (A == 1 ? n : v);
  const int z = A == 2 ? n : v;
  step = high ? stride : -stride;
  return (z * sy + y) * pitch + x;
}

// Grid-wide barrier of a cooperative launch (every block is resident),
// bounded: false when the other blocks have not all arrived within limit_ns
// (bit 0 of the error word is then set).
__device__ __forceinline__ bool grid_barrier(unsigned *bar, unsigned nblocks, uint64_t limit_ns, unsigned *err) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned *gen = bar + 1;
    const unsigned g0 = *gen;
    __threadfence();
    int ok = 1;
    if (atomicAdd(bar, 1u) == nblocks - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      const uint64_t t0 = global_ns();
      while (*gen == g0) {
        if (global_ns() - t0 > limit_ns) {
          ok = 0;
          atomicOr(err, 1u);
          break;
        }
        __nanosleep(100);
      }
    }
    __threadfence();
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

__global__ void __launch_bounds__(32 * kBoundaryWarps, kBoundaryBlocks) k_abc_boundary(const __grid_constant__ BoundaryArgs B) {
  __shared__ __align__(16) __half Xs[kBoundaryWarps][16 * kXs];
  __shared__ float2 Ln[kBoundaryWarps][2][4][8];  // [time: t, t-1][ray][point] (p, q)
  __shared__ FragsSmem F;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const Ghost &G = B.G;
  frags_to_smem(B.net, F);
  __syncthreads();
  const long wg = (long)blockIdx.x * kBoundaryWarps + warp, nw = (long)gridDim.x * kBoundaryWarps;
  for (int A = 2; A >= 0; --A) {
    const int fa = 2 * (2 - A);                       // the low face; fa + 1 is the high one
    const long r0 = G.off[fa] / kGhostD, rmid = G.off[fa + 1] / kGhostD, r1 = G.off[fa + 2] / kGhostD;
    const long ngroups = (r1 - r0 + 3) / 4;
    const int stride = A == 0 ? 1 : (A == 1 ? B.pitch : B.sy * B.pitch);
    // A group's loads (lane 8 r + q: point q of ray r at t and t-1; lane
    // 2 c + h: the medium of cell c), issued a group ahead of their use.
    // Lane 8 r + 3 also loads next at d = L-4, the value the update of ray r
    // starts from (no cell a pass writes: it is final when the pass begins).
    auto load_group = [&](long grp, float2 &a, float2 &b, float4 &m, float2 &n) {
      const long ray0 = r0 + 4 * grp;
      const long ray = ray0 + (lane >> 3);
      const int q = lane & 7, c = lane >> 1;
      a = b = n = make_float2(0.f, 0.f);
      m = make_float4(0.f, 0.f, 0.f, 0.f);
      if (grp >= ngroups) return;
      if (ray < r1) {
        int step;
        const int idx0 = ray_cell(G, A, ray, r0, rmid, 0, B.sy, B.pitch, stride, step);  // d = L-3 (point 4)
        a = __ldcg(B.cur + idx0 + (q - kGhostD) * step);
        b = __ldcg(B.line_in + ray * 8 + q);
        if (q == kGhostD - 1) n = __ldcg(B.next + idx0 - step);
      }
      if (ray0 + (c >> 2) < r1) m = B.med[ray0 * kGhostD + c];
    };
    float2 pa, pb, pn;
    float4 pm;
    load_group(wg, pa, pb, pm, pn);
    for (long grp = wg; grp < ngroups; grp += nw) {
      const long ray0 = r0 + 4 * grp;
      // 1. the rays' lines into shared memory, the t line kept for the next
      //    step when it evaluates too; then the next group's loads.
      const float4 m = pm;
      const float2 nq = pn;
      {
        const int r = lane >> 3, q = lane & 7;
        const long ray = ray0 + r;
        if (B.save && ray < r1) __stcg(B.line_out + ray * 8 + q, pa);
        Ln[warp][0][r][q] = pa;
        Ln[warp][1][r][q] = pb;
      }
      load_group(grp + nw, pa, pb, pm, pn);
      __syncwarp();
      // 2. the coefficient of update lane u = 4 r + j (cell 4 r + j of the group).
      const int u = lane & 15;
      const long cell = ray0 * kGhostD + u;
      const bool live = lane < 16 && ray0 + (u >> 2) < r1;
      float2 kc;
      {
        // Features of cell c = lane / 2 (ray c / 4, d = L-3 + c % 4); the
        // lane pair builds the t (even lane) and t-1 (odd lane) stencils.
        const int c = lane >> 1, half_t = lane & 1, j = c & 3;
        const bool clive = ray0 + (c >> 2) < r1;
        const float2 *line = Ln[warp][half_t][c >> 2];
        float vv[18];
#pragma unroll
        for (int o = 0; o < 9; ++o) {
          const int qq = j + o;  // line points j .. j+8; past 7 (beyond the layer): zero
          const float2 v = (qq < 8 && clive) ? line[qq < 8 ? qq : 7] : make_float2(0.f, 0.f);
          vv[o] = v.x;
          vv[9 + o] = v.y;
        }
        float s = 0.f;
#pragma unroll
        for (int k = 0; k < 18; ++k) s = fmaxf(s, fabsf(vv[k]));
        s = fmaxf(s, __shfl_xor_sync(0xffffffffu, s, 1));
        // Stencils this small carry no wave (the first cells a front reaches
        // hold values near the FP32 underflow, whose reciprocal overflows).
        if (!(s > kMinScale)) s = 0.f;
        const float inv = s > 0.f ? 1.0f / s : 0.f;
        __half *X = Xs[warp];
        __half *row = X + c * kXs + 18 * half_t;
#pragma unroll
        for (int k = 0; k < 18; k += 2)
          *reinterpret_cast<__half2 *>(row + k) = __floats2half2_rn(vv[k] * inv, vv[k + 1] * inv);
        if (half_t == 0) {
          const int d = G.L - kGhostD + 1 + j;
          *reinterpret_cast<__half2 *>(X + c * kXs + 36) = __floats2half2_rn(m.x * kVScale, m.y);
          *reinterpret_cast<__half2 *>(X + c * kXs + 38) = __floats2half2_rn(m.z, (float)d / (float)G.L);
        } else {
#pragma unroll
          for (int k = 40; k < kK1; k += 2) *reinterpret_cast<__half2 *>(X + c * kXs + k) = __floats2half2_rn(0.f, 0.f);
        }
        __syncwarp();
        float ylo[2], yhi[2];
        mlp16_smem(X, F, ylo, yhi);
        // Rows g and g + 8 sit in lane 4 g: cell u comes from lane 4 (u % 8).
        const int src = 4 * (u & 7);
        const float a0 = __shfl_sync(0xffffffffu, ylo[0], src), a1 = __shfl_sync(0xffffffffu, ylo[1], src);
        const float b0 = __shfl_sync(0xffffffffu, yhi[0], src), b1 = __shfl_sync(0xffffffffu, yhi[1], src);
        kc = u < 8 ? make_float2(sigmoid(a0), sigmoid(a1)) : make_float2(sigmoid(b0), sigmoid(b1));
        if (B.keep && live) B.k[cell] = kc;
      }
      // 3. the update along each ray (lanes 0 .. 15).
      const int r = u >> 2, j = u & 3;
      const float2 cg = Ln[warp][0][r][kGhostD + j];      // the cell at t
      const float2 ci = Ln[warp][0][r][kGhostD - 1 + j];  // its inward neighbour at t
      int gidx = 0;
      float2 ni = make_float2(0.f, 0.f);
      {
        // next of d = L-4, loaded a group ahead by lane 8 r + 3.
        const float nx = __shfl_sync(0xffffffffu, nq.x, 8 * r + kGhostD - 1);
        const float ny = __shfl_sync(0xffffffffu, nq.y, 8 * r + kGhostD - 1);
        if (j == 0) ni = make_float2(nx, ny);
      }
      if (live) {
        int step;
        gidx = ray_cell(G, A, ray0 + r, r0, rmid, j, B.sy, B.pitch, stride, step);
      }
      // a_d = cur_(d-1) + k_d cur_d, next_d = a_d - k_d next_(d-1): lane j
      // folds in lanes j-1 .. 0 of its ray (the first one brings next_(L-4)).
      float ax = __fmaf_rn(kc.x, cg.x, ci.x), ay = __fmaf_rn(kc.y, cg.y, ci.y);
      float mx = -kc.x, my = -kc.y;  // coefficient of next_(start-1) in the running value
      if (j == 0) {
        ax = __fmaf_rn(mx, ni.x, ax);
        ay = __fmaf_rn(my, ni.y, ay);
        mx = 0.f;
        my = 0.f;
      }
#pragma unroll
      for (int o = 1; o < kGhostD; o <<= 1) {
        const float px = __shfl_up_sync(0xffffffffu, ax, o), py = __shfl_up_sync(0xffffffffu, ay, o);
        const float qx = __shfl_up_sync(0xffffffffu, mx, o), qy = __shfl_up_sync(0xffffffffu, my, o);
        if (j >= o) {
          // value = a + m * (previous value) with the previous one = p + q * (...)
          ax = __fmaf_rn(mx, px, ax);
          ay = __fmaf_rn(my, py, ay);
          mx *= qx;
          my *= qy;
        }
      }
      if (live) __stcg(B.next + gidx, make_float2(ax, ay));
      __syncwarp();
    }
    if (A > 0 && !grid_barrier(B.bar, gridDim.x, B.wait_ns, B.err)) return;
  }
}

// k_abc_rays_coop: the update with coefficients from the buffer (the
// medium's, or the network's from its last evaluation), four lanes per ray
// (j = 0..3: d = L-3+j), eight rays per warp.  Each lane loads its cell's
// coefficient and value at t, the lane of d = L-3 also the inward
// neighbour's values at t and t+1; the outward dependence is an inclusive
// scan of affine maps over the ray's 4 lanes.  SAVE: the step before an
// evaluation also stores the rays' 8 line points at t (lane j: points j
// and j+4), which the evaluating step reads as its t-1 lines.
template <bool SAVE>
__global__ void __launch_bounds__(256) k_abc_rays_coop(const __grid_constant__ BoundaryArgs B) {
  const Ghost &G = B.G;
  const int lane = threadIdx.x & 31, j = lane & 3;
  const long tid = (long)blockIdx.x * blockDim.x + threadIdx.x, nth = (long)gridDim.x * blockDim.x;
  for (int A = 2; A >= 0; --A) {
    const int fa = 2 * (2 - A);
    const long r0 = G.off[fa] / kGhostD, rmid = G.off[fa + 1] / kGhostD, r1 = G.off[fa + 2] / kGhostD;
    const int stride = A == 0 ? 1 : (A == 1 ? B.pitch : B.sy * B.pitch);
    const long total = ((r1 - r0) * kGhostD + 31) / 32 * 32;  // whole warps iterate together
    // kU cells per thread and iteration, all their loads issued before any
    // of them is used (whether a cell lies below `total` is the same for
    // every lane of a warp, so the shuffles below see whole warps).
    constexpr int kU = 4;
    for (long t0 = tid; t0 < total; t0 += kU * nth) {
      float2 kk[kU], cg[kU], ci[kU], ni[kU], far[kU];
      int gidx[kU];
      bool live[kU];
#pragma unroll
      for (int w = 0; w < kU; ++w) {
        const long t = t0 + w * nth;
        const long ray = r0 + (t >> 2);
        live[w] = t < total && ray < r1;
        kk[w] = cg[w] = ci[w] = ni[w] = far[w] = make_float2(0.f, 0.f);
        gidx[w] = 0;
        if (live[w]) {
          int step;
          kk[w] = B.k[ray * kGhostD + j];
          gidx[w] = ray_cell(G, A, ray, r0, rmid, j, B.sy, B.pitch, stride, step);
          cg[w] = __ldcg(B.cur + gidx[w]);
          if (SAVE) far[w] = __ldcg(B.cur + gidx[w] - kGhostD * step);  // line point j (d = L-7+j)
          if (j == 0) {
            if (!SAVE) ci[w] = __ldcg(B.cur + gidx[w] - step);
            ni[w] = __ldcg(B.next + gidx[w] - step);  // next of d = L-4
          }
          if (SAVE) {
            __stcg(B.line_out + ray * 8 + j, far[w]);
            __stcg(B.line_out + ray * 8 + kGhostD + j, cg[w]);
          }
        }
      }
#pragma unroll
      for (int w = 0; w < kU; ++w) {
        if (t0 - lane + w * nth >= total) break;  // the warp's first cell (uniform)
        // The inward cell of lanes 1 .. 3 is the cell of the lane before; that
        // of lane 0 is line point 3, which lane 3 loaded when saving.
        {
          const float ux = __shfl_up_sync(0xffffffffu, cg[w].x, 1), uy = __shfl_up_sync(0xffffffffu, cg[w].y, 1);
          const float fx = __shfl_sync(0xffffffffu, far[w].x, lane | 3);
          const float fy = __shfl_sync(0xffffffffu, far[w].y, lane | 3);
          if (j != 0) ci[w] = make_float2(ux, uy);
          else if (SAVE) ci[w] = make_float2(fx, fy);
        }
        float ax = __fmaf_rn(kk[w].x, cg[w].x, ci[w].x), ay = __fmaf_rn(kk[w].y, cg[w].y, ci[w].y);
        float mx = -kk[w].x, my = -kk[w].y;
        if (j == 0) {
          ax = __fmaf_rn(mx, ni[w].x, ax);
          ay = __fmaf_rn(my, ni[w].y, ay);
          mx = 0.f;
          my = 0.f;
        }
#pragma unroll
        for (int o = 1; o < kGhostD; o <<= 1) {
          const float px = __shfl_up_sync(0xffffffffu, ax, o), py = __shfl_up_sync(0xffffffffu, ay, o);
          const float qx = __shfl_up_sync(0xffffffffu, mx, o), qy = __shfl_up_sync(0xffffffffu, my, o);
          if (j >= o) {
            ax = __fmaf_rn(mx, px, ax);
            ay = __fmaf_rn(my, py, ay);
            mx *= qx;
            my *= qy;
          }
        }
        if (live[w]) __stcg(B.next + gidx[w], make_float2(ax, ay));
      }
    }
    if (A > 0 && !grid_barrier(B.bar, gridDim.x, B.wait_ns, B.err)) return;
  }
}

// The t-1 line points of every ray from the previous field, before the
// first boundary step (later steps carry them over themselves).
__global__ void k_abc_lines(const __grid_constant__ Ghost G, const float2 *__restrict__ prev, int sy, int pitch,
                            const float4 *__restrict__ med, float2 *__restrict__ lines) {
  const long nrays = G.off[6] / kGhostD;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < nrays * 8; i += (long)gridDim.x * blockDim.x) {
    const long ray = i >> 3;
    const int q = (int)(i & 7);
    const int f = face_of(G, ray * kGhostD);
    const int idx0 = __float_as_int(med[ray * kGhostD].w);
    lines[i] = prev[idx0 + (q - kGhostD) * normal_step(f, sy, pitch)];
  }
}

// Taper of the layer cells after the step: next *= exp(-(damping d)^2).
__global__ void k_abc_taper(const LayerCell *cells, long ncells, float2 *next, int sy, int pitch, float damping) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < ncells; i += (long)gridDim.x * blockDim.x) {
    const LayerCell c = cells[i];
    float2 *p = next + cell_index(c.x, c.y, c.z, sy, pitch);
    const float a = damping * (float)c.d;
    const float w = __expf(-a * a);
    float2 v = *p;
    v.x *= w;
    v.y *= w;
    *p = v;
  }
}

// Medium of every ghost cell (inputs of the network) with the cell's index
// in the field in .w (as int bits), and the medium's one-way coefficients.
__global__ void k_abc_fill(const __grid_constant__ Ghost G, const float *coef, int sy, int pitch, float dt, float hx, float hy, float hz,
                           float4 *med, float2 *kfix) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < G.off[6]; i += (long)gridDim.x * blockDim.x) {
    int c[3], f, a, sgn;
    ghost_cell(G, i, c, f, a, sgn);
    float4 m = medium_of(coef, c[0], c[1], c[2], sy, pitch);
    m.w = __int_as_float((int)cell_index(c[0], c[1], c[2], sy, pitch));
    med[i] = m;
    if (kfix) {
      const float kf = oneway_k(m.x, m.y, a, dt, a == 0 ? hx : (a == 1 ? hy : hz));
      kfix[i] = make_float2(kf, kf);
    }
  }
}

// ---- training -------------------------------------------------------------------

constexpr int kTB = 128;  // samples per training block
constexpr int sX = 41, sH = 33;

__device__ __forceinline__ float h16(float v) { return __half2float(__float2half_rn(v)); }

// Forward and backward of B samples (index b of the batch: a random sample,
// or b itself when seed is 0): each block writes its part of the loss
// sum_c (sigmoid(y_c) a_c - b_c)^2 / (2 B) and of the gradient to its own
// slots of lpartial and partial.  Weights are used FP16-rounded, hidden
// pre-activations and activations are rounded to FP16 (as inference does),
// the derivatives treat the roundings as the identity.  noise > 0 perturbs the
// stencil inputs.
__global__ void __launch_bounds__(kTB) k_abc_train(const float *feat, const float *tgt, long nsamp, int B,
                                                    uint32_t seed, const float *P, float noise, float *partial,
                                                    float *lpartial) {
  extern __shared__ float sm[];
  float *W1 = sm, *b1 = W1 + kHid * kIn, *W2 = b1 + kHid, *b2 = W2 + kHid * kHid, *W3 = b2 + kHid,
        *b3 = W3 + kOut * kHid;
  float *X = b3 + 4;
  float *H1 = X + kTB * sX, *D1 = H1 + kTB * sH, *H2 = D1 + kTB * sH, *D2 = H2 + kTB * sH, *DY = D2 + kTB * sH;
  for (int i = threadIdx.x; i < kNP; i += blockDim.x) {
    const bool w = (i < oB1) || (i >= oW2 && i < oB2) || (i >= oW3 && i < oB3);
    sm[i] = w ? h16(P[i]) : P[i];
  }
  const int tid = threadIdx.x;
  const int b = blockIdx.x * kTB + tid;
  const bool live = b < B;
  long si = 0;
  if (live)
    si = seed ? (long)((((uint64_t)mix32(seed, (uint32_t)b) << 16) ^ mix32(seed + 1u, (uint32_t)b)) % (uint64_t)nsamp)
              : b;
  float *x = X + tid * sX;
  for (int k = 0; k < kIn; ++k) {
    float f = live ? feat[si * kIn + k] : 0.f;
    if (noise > 0.f && k < kSt && live) {
      // Input noise (approximately normal, from four uniforms).
      float u = 0.f;
      for (int r = 0; r < 4; ++r) u += (float)(mix32(seed ^ (0x51ED27u * (r + 1)), (uint32_t)(b * kIn + k)) >> 8);
      f += noise * 1.7320508f * (u * (1.0f / 16777216.0f) - 2.0f);
    }
    x[k] = live ? h16(f) : 0.f;
  }
  __syncthreads();
  float *h1 = H1 + tid * sH, *d1v = D1 + tid * sH, *h2 = H2 + tid * sH, *d2v = D2 + tid * sH, *dy = DY + tid * 2;
  float a1[kHid], a2[kHid];
  for (int o = 0; o < kHid; ++o) {
    float z = b1[o];
    for (int k = 0; k < kIn; ++k) z = fmaf(W1[o * kIn + k], x[k], z);
    a1[o] = tanhf(h16(z));  // inference rounds the pre-activation to FP16 for its half2 tanh
    h1[o] = live ? h16(a1[o]) : 0.f;
  }
  for (int o = 0; o < kHid; ++o) {
    float z = b2[o];
    for (int k = 0; k < kHid; ++k) z = fmaf(W2[o * kHid + k], h1[k], z);
    a2[o] = tanhf(h16(z));
    h2[o] = live ? h16(a2[o]) : 0.f;
  }
  float l = 0.f;
  for (int o = 0; o < kOut; ++o) {
    float y = b3[o];
    for (int k = 0; k < kHid; ++k) y = fmaf(W3[o * kHid + k], h2[k], y);
    float g = 0.f;
    if (live) {
      const float kk = 1.0f / (1.0f + expf(-y));
      const float ta = tgt[si * kTgt + o], tb = tgt[si * kTgt + 2 + o];
      const float e = fmaf(kk, ta, -tb);
      l += e * e;
      g = e * ta * kk * (1.0f - kk);
    }
    dy[o] = g / (float)B;
  }
  for (int k = 0; k < kHid; ++k) {
    float g = 0.f;
    for (int o = 0; o < kOut; ++o) g = fmaf(W3[o * kHid + k], dy[o], g);
    d2v[k] = g * (1.0f - a2[k] * a2[k]);
  }
  for (int k = 0; k < kHid; ++k) {
    float g = 0.f;
    for (int o = 0; o < kHid; ++o) g = fmaf(W2[o * kHid + k], d2v[o], g);
    d1v[k] = g * (1.0f - a1[k] * a1[k]);
  }
  // The block's loss and gradient sums go to its own slots (summed over the
  // blocks in order by k_abc_reduce: the result does not depend on timing).
  __shared__ float wl[kTB / 32];
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((tid & 31) == 0) wl[tid >> 5] = l;
  __syncthreads();
  if (tid == 0) {
    float bl = 0.f;
    for (int w = 0; w < kTB / 32; ++w) bl += wl[w];
    lpartial[blockIdx.x] = bl / (2.0f * (float)B);
  }
  // Block sums of the per-sample gradient terms.
  for (int e = tid; e < kNP; e += kTB) {
    float s = 0.f;
    if (e < oB1) {
      const int o = e / kIn, k = e % kIn;
      for (int q = 0; q < kTB; ++q) s = fmaf(D1[q * sH + o], X[q * sX + k], s);
    } else if (e < oW2) {
      const int o = e - oB1;
      for (int q = 0; q < kTB; ++q) s += D1[q * sH + o];
    } else if (e < oB2) {
      const int o = (e - oW2) / kHid, k = (e - oW2) % kHid;
      for (int q = 0; q < kTB; ++q) s = fmaf(D2[q * sH + o], H1[q * sH + k], s);
    } else if (e < oW3) {
      const int o = e - oB2;
      for (int q = 0; q < kTB; ++q) s += D2[q * sH + o];
    } else if (e < oB3) {
      const int o = (e - oW3) / kHid, k = (e - oW3) % kHid;
      for (int q = 0; q < kTB; ++q) s = fmaf(DY[q * 2 + o], H2[q * sH + k], s);
    } else {
      const int o = e - oB3;
      for (int q = 0; q < kTB; ++q) s += DY[q * 2 + o];
    }
    partial[(size_t)blockIdx.x * kNP + e] = s;
  }
}

// Sums of the training blocks' partial gradients and losses, in block order.
__global__ void k_abc_reduce(const float *partial, const float *lpartial, int nblocks, float *grad, float *loss) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < kNP) {
    float g = 0.f;
    for (int b = 0; b < nblocks; ++b) g += partial[(size_t)b * kNP + e];
    grad[e] = g;
  }
  if (e == 0) {
    float l = 0.f;
    for (int b = 0; b < nblocks; ++b) l += lpartial[b];
    *loss = l;
  }
}

constexpr size_t kTrainSmem = sizeof(float) * (kNP + 4 + kTB * (sX + 4 * sH + 2));

// Adam step on the master weights; clears the gradient.
__global__ void k_abc_adam(float *P, float *grad, float *m, float *v, int n, float lr, float b1, float b2, float eps,
                           float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float g = grad[i];
  grad[i] = 0.f;
  const float mi = b1 * m[i] + (1.f - b1) * g, vi = b2 * v[i] + (1.f - b2) * g * g;
  m[i] = mi;
  v[i] = vi;
  P[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// FP32 master weights -> inference copy.
__global__ void k_abc_pack(const float *P, NetHalf *N) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kHid * kK1) {
    const int o = i / kK1, k = i % kK1;
    N->w1[i] = __float2half_rn(k < kIn ? P[oW1 + o * kIn + k] : 0.f);
  }
  if (i < kHid * kHid) N->w2[i] = __float2half_rn(P[oW2 + i]);
  if (i < 8 * kHid) N->w3[i] = __float2half_rn(i < kOut * kHid ? P[oW3 + i] : 0.f);
  if (i < kHid) {
    N->b1[i] = P[oB1 + i];
    N->b2[i] = P[oB2 + i];
  }
  if (i < 8) N->b3[i] = i < kOut ? P[oB3 + i] : 0.f;
}

// ---- host state -------------------------------------------------------------------

namespace {

struct Trainer {
  float *P = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;  // master weights and Adam state
  NetHalf *net = nullptr;
  bool weights = false;
  long adam_t = 0;
  float *feat = nullptr, *tgt = nullptr;
  int4 *pos = nullptr;  // grid cell, face and distance of every sample
  long nsamp = 0;       // samples held (at most cap)
  long cap = 0;
  bool reserved = false;
};

struct ResidentLayer {
  bool on = false;
  int mode = 0;
  int interval = 1;  // learned form: network every `interval` steps
  long steps = 0;    // steps since SetBoundary
  float damping = 0.f;
  Ghost G;
  float4 *med = nullptr;       // medium of every ghost cell (one-way modes)
  float2 *k = nullptr;         // one-way coefficients of every ghost cell (fixed, or the network's kept ones)
  float2 *lines[2] = {nullptr, nullptr};  // learned form: t-1 line points of every ray, by step parity
  unsigned *bar = nullptr;     // the boundary kernels' grid barrier (count, generation)
  int grid_net = 0, grid_rays = 0;  // their cooperative grids
  LayerCell *cells = nullptr;  // every layer cell (taper), z, y, x order
  long ncells = 0;
};

Trainer T;
ResidentLayer R;

int err(int code, const char *msg) { return flt_record_error(code, msg); }

#define CKA(call)                                                                                       \
  do {                                                                                                  \
    cudaError_t e_ = (call);                                                                            \
    if (e_ != cudaSuccess) {                                                                            \
      cudaGetLastError(); /* not sticky: a later launch check must not see it */                        \
      char b_[256];                                                                                     \
      snprintf(b_, sizeof(b_), "%s failed: %s", #call, cudaGetErrorString(e_));                        \
      return err(e_ == cudaErrorMemoryAllocation ? FLETCHER_ERR_NOMEM : FLETCHER_ERR_CUDA, b_);         \
    }                                                                                                   \
  } while (0)

cudaStream_t stream_of() {
  const ResidentView v = resident_view();
  return v.init ? v.stream : (cudaStream_t)FLETCHER_GetStream();
}

int ensure_trainer() {
  if (T.P) return FLETCHER_OK;
  CKA(cudaMalloc(&T.P, kNP * sizeof(float)));
  CKA(cudaMalloc(&T.grad, kNP * sizeof(float)));
  CKA(cudaMalloc(&T.m, kNP * sizeof(float)));
  CKA(cudaMalloc(&T.v, kNP * sizeof(float)));
  CKA(cudaMalloc(&T.net, sizeof(NetHalf)));
  CKA(cudaMemset(T.grad, 0, kNP * sizeof(float)));
  CKA(cudaMemset(T.m, 0, kNP * sizeof(float)));
  CKA(cudaMemset(T.v, 0, kNP * sizeof(float)));
  CKA(cudaMemset(T.net, 0, sizeof(NetHalf)));
  return FLETCHER_OK;
}

int pack_net(cudaStream_t s) {
  k_abc_pack<<<(kHid * kK1 + 255) / 256, 256, 0, s>>>(T.P, T.net);
  CKA(cudaGetLastError());
  return FLETCHER_OK;
}

uint64_t splitmix(uint64_t &x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

int grid_of(long n, int block) {
  long b = (n + block - 1) / block;
  return (int)(b < 1 ? 1 : (b > 4096 ? 4096 : b));
}

int train_attr() {
  static bool done = false;
  if (!done) {
    CKA(cudaFuncSetAttribute(k_abc_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmem));
    done = true;
  }
  return FLETCHER_OK;
}

bool oneway_mode(int mode) { return mode == FLETCHER_BOUNDARY_LEARNED || mode == FLETCHER_BOUNDARY_ONEWAY; }

}  // namespace

bool abc_active() { return R.on; }

void abc_release_resident() {
  if (R.med) cudaFree(R.med);
  if (R.k) cudaFree(R.k);
  if (R.lines[0]) cudaFree(R.lines[0]);
  if (R.lines[1]) cudaFree(R.lines[1]);
  if (R.bar) cudaFree(R.bar);
  if (R.cells) cudaFree(R.cells);
  R = ResidentLayer();
}

int g_interval = 1;  // FLETCHER_AbcSetInterval

// After the plain step: the ghost zone's one-way update (with the network
// on the learned form's evaluation steps) in one cooperative launch, then
// the taper if any.
cudaError_t abc_after_step(const ResidentView &v) {
  if (!R.on) return cudaSuccess;
  if (oneway_mode(R.mode)) {
    const bool learned = R.mode == FLETCHER_BOUNDARY_LEARNED;
    BoundaryArgs a;
    memset(&a, 0, sizeof(a));
    a.G = R.G;
    a.cur = v.cur;
    a.next = v.next;
    a.sy = v.sy;
    a.pitch = v.pitch;
    a.med = R.med;
    a.net = T.net;
    a.line_in = R.lines[R.steps & 1];
    a.line_out = R.lines[(R.steps + 1) & 1];
    a.k = R.k;
    a.eval = learned && R.steps % R.interval == 0;        // the last coefficients stay in between
    a.keep = learned && R.interval > 1;
    a.save = learned && (R.steps + 1) % R.interval == 0;  // the next step evaluates
    a.bar = R.bar;
    a.err = v.err;
    a.wait_ns = kWaitLimitNs;
    ++R.steps;
    void *args[] = {&a};
    const void *kern = a.eval ? (const void *)k_abc_boundary
                              : (a.save ? (const void *)k_abc_rays_coop<true> : (const void *)k_abc_rays_coop<false>);
    const int grid = a.eval ? R.grid_net : R.grid_rays;
    const cudaError_t e = cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(256), args, 0, v.stream);
    if (e != cudaSuccess) return e;
  }
  if (R.damping > 0.f && R.ncells)
    k_abc_taper<<<grid_of(R.ncells, 256), 256, 0, v.stream>>>(R.cells, R.ncells, v.next, v.sy, v.pitch, R.damping);
  return cudaGetLastError();
}

}  // namespace flt

using namespace flt;

// ===== Part 4: learned absorbing boundary =========================================

extern "C" int FLETCHER_AbcSetWeights(const float *params) {
  if (!params) return err(FLETCHER_ERR_ARGS, "AbcSetWeights: bad arguments");
  if (ensure_trainer()) return FLETCHER_GetLastError();
  CKA(cudaMemcpy(T.P, params, kNP * sizeof(float), cudaMemcpyHostToDevice));
  CKA(cudaMemset(T.m, 0, kNP * sizeof(float)));
  CKA(cudaMemset(T.v, 0, kNP * sizeof(float)));
  T.adam_t = 0;
  T.weights = true;
  if (pack_net(nullptr)) return FLETCHER_GetLastError();
  CKA(cudaDeviceSynchronize());
  return FLETCHER_OK;
}

extern "C" int FLETCHER_AbcInit(unsigned seed) {
  std::vector<float> p(kNP, 0.f);
  uint64_t s = 0x1234567ull ^ ((uint64_t)seed << 20);
  auto unif = [&]() { return (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); };
  auto fill = [&](int off, int fan_out, int fan_in) {
    const double a = sqrt(6.0 / (fan_in + fan_out));
    for (int i = 0; i < fan_out * fan_in; ++i) p[off + i] = (float)((2.0 * unif() - 1.0) * a);
  };
  fill(oW1, kHid, kIn);
  fill(oW2, kHid, kHid);
  fill(oW3, kOut, kHid);
  for (int o = 0; o < kOut; ++o) p[oB3 + o] = kInitBias;
  return FLETCHER_AbcSetWeights(p.data());
}

extern "C" int FLETCHER_AbcGetWeights(float *params) {
  if (!T.weights) return err(FLETCHER_ERR_ARGS, "AbcGetWeights: no network");
  if (!params) return err(FLETCHER_ERR_ARGS, "AbcGetWeights: bad arguments");
  CKA(cudaDeviceSynchronize());
  CKA(cudaMemcpy(params, T.P, kNP * sizeof(float), cudaMemcpyDeviceToHost));
  return FLETCHER_OK;
}

extern "C" int FLETCHER_AbcReserve(long capacity) {
  if (capacity < 0) return err(FLETCHER_ERR_ARGS, "AbcReserve: negative capacity");
  if (T.feat) cudaFree(T.feat);
  if (T.tgt) cudaFree(T.tgt);
  if (T.pos) cudaFree(T.pos);
  T.feat = T.tgt = nullptr;
  T.pos = nullptr;
  T.nsamp = 0;
  T.reserved = true;
  T.cap = capacity;
  if (capacity) {
    CKA(cudaMalloc(&T.feat, (size_t)capacity * kIn * sizeof(float)));
    CKA(cudaMalloc(&T.tgt, (size_t)capacity * kTgt * sizeof(float)));
    CKA(cudaMalloc(&T.pos, (size_t)capacity * sizeof(int4)));
  }
  return FLETCHER_OK;
}

extern "C" long FLETCHER_AbcSamples(void) { return T.nsamp; }

extern "C" int FLETCHER_AbcCollect(const int *interior_lo, const int *interior_hi, int layer, float keep_frac,
                                   unsigned seed, float min_scale) {
  const ResidentView v = resident_view();
  if (!v.init) return err(FLETCHER_ERR_ARGS, "AbcCollect needs an FP32 resident state");
  if (!T.reserved || !T.cap) return err(FLETCHER_ERR_ARGS, "AbcCollect: call FLETCHER_AbcReserve first");
  if (!interior_lo || !interior_hi || layer < kRadius + 1)
    return err(FLETCHER_ERR_ARGS, "AbcCollect: bad box or layer");
  Box in;
  const int dims[3] = {v.sx, v.sy, v.sz};
  for (int a = 0; a < 3; ++a) {
    in.lo[a] = interior_lo[a];
    in.hi[a] = interior_hi[a];
    // The next values read 4 cells beyond the kept box; all of it must be updated grid.
    if (in.hi[a] <= in.lo[a] || in.lo[a] - layer - kRadius < v.bord || in.hi[a] + layer + kRadius > dims[a] - v.bord)
      return err(FLETCHER_ERR_ARGS, "AbcCollect: the box and its layer must lie 4 cells inside the updated region");
  }
  const Ghost G = make_ghost(in, layer);
  const long n = G.off[6];
  const int nb = (int)std::max(1L, std::min(1024L, (n + kCollectBlock - 1) / kCollectBlock));
  const long per = (n + nb - 1) / nb;
  std::vector<int> cnt(nb);
  std::vector<long> first(nb);
  int *d_cnt = nullptr;
  long *d_first = nullptr;
  CKA(cudaMalloc(&d_cnt, nb * sizeof(int)));
  CKA(cudaMalloc(&d_first, nb * sizeof(long)));
  k_abc_collect_count<<<nb, kCollectBlock, 0, v.stream>>>(v.cur, v.prev, G, v.sy, v.pitch, keep_frac, seed, min_scale,
                                                          per, d_cnt);
  CKA(cudaGetLastError());
  CKA(cudaMemcpyAsync(cnt.data(), d_cnt, nb * sizeof(int), cudaMemcpyDeviceToHost, v.stream));
  CKA(cudaStreamSynchronize(v.stream));
  long total = 0;
  for (int b = 0; b < nb; ++b) {
    first[b] = T.nsamp + total;
    total += cnt[b];
  }
  CKA(cudaMemcpyAsync(d_first, first.data(), nb * sizeof(long), cudaMemcpyHostToDevice, v.stream));
  k_abc_collect<<<nb, kCollectBlock, 0, v.stream>>>(v.cur, v.prev, v.coef, G, v.sy, v.pitch, v.dx, v.dy, v.dz, v.dt,
                                                    keep_frac, seed, min_scale, per, d_first, T.feat, T.tgt, T.pos,
                                                    T.cap);
  CKA(cudaGetLastError());
  CKA(cudaStreamSynchronize(v.stream));
  cudaFree(d_cnt);
  cudaFree(d_first);
  T.nsamp = std::min(T.cap, T.nsamp + total);
  return FLETCHER_OK;
}

extern "C" int FLETCHER_AbcGetSamples(long start, long n, float *feat, float *tgt, int *pos) {
  const long have = FLETCHER_AbcSamples();
  if (start < 0 || n < 0 || start + n > have)
    return err(FLETCHER_ERR_ARGS, "AbcGetSamples: range outside the samples");
  if (feat) CKA(cudaMemcpy(feat, T.feat + start * kIn, n * kIn * sizeof(float), cudaMemcpyDeviceToHost));
  if (tgt) CKA(cudaMemcpy(tgt, T.tgt + start * kTgt, n * kTgt * sizeof(float), cudaMemcpyDeviceToHost));
  if (pos) CKA(cudaMemcpy(pos, T.pos + start, n * sizeof(int4), cudaMemcpyDeviceToHost));
  return FLETCHER_OK;
}

extern "C" int FLETCHER_AbcTrain(int iters, int batch, float lr, unsigned seed, float noise, float *loss_out) {
  const long ns = FLETCHER_AbcSamples();
  if (ns <= 0) return err(FLETCHER_ERR_ARGS, "AbcTrain: no samples");
  if (!T.weights) return err(FLETCHER_ERR_ARGS, "AbcTrain: call FLETCHER_AbcInit or AbcSetWeights first");
  if (iters < 1 || batch < 1 || !(lr > 0.f) || !(noise >= 0.f))
    return err(FLETCHER_ERR_ARGS, "AbcTrain: bad arguments");
  cudaStream_t s = stream_of();
  if (train_attr()) return FLETCHER_GetLastError();
  const int blocks = (batch + kTB - 1) / kTB;
  float *loss = nullptr, *partial = nullptr, *lpartial = nullptr;
  CKA(cudaMalloc(&loss, iters * sizeof(float)));
  CKA(cudaMalloc(&partial, (size_t)blocks * kNP * sizeof(float)));
  CKA(cudaMalloc(&lpartial, blocks * sizeof(float)));
  const float b1 = 0.9f, b2 = 0.999f;
  for (int it = 0; it < iters; ++it) {
    uint64_t st = (uint64_t)seed * 1000003ull + (uint64_t)it;
    const uint32_t sd = (uint32_t)splitmix(st) | 1u;
    k_abc_train<<<blocks, kTB, kTrainSmem, s>>>(T.feat, T.tgt, ns, batch, sd, T.P, noise, partial, lpartial);
    k_abc_reduce<<<(kNP + 255) / 256, 256, 0, s>>>(partial, lpartial, blocks, T.grad, loss + it);
    ++T.adam_t;
    const float lr_t = lr * 0.5f * (1.0f + cosf(3.14159265f * (float)it / (float)iters));
    k_abc_adam<<<(kNP + 255) / 256, 256, 0, s>>>(T.P, T.grad, T.m, T.v, kNP, lr_t, b1, b2, 1e-8f,
                                                 1.0f - powf(b1, (float)T.adam_t), 1.0f - powf(b2, (float)T.adam_t));
  }
  CKA(cudaGetLastError());
  if (pack_net(s)) return FLETCHER_GetLastError();
  if (loss_out) CKA(cudaMemcpyAsync(loss_out, loss, iters * sizeof(float), cudaMemcpyDeviceToHost, s));
  CKA(cudaStreamSynchronize(s));
  cudaFree(loss);
  cudaFree(partial);
  cudaFree(lpartial);
  return FLETCHER_OK;
}

extern "C" int FLETCHER_AbcGradient(const float *feat, const float *tgt, int n, float *grad, float *loss) {
  if (!T.weights) return err(FLETCHER_ERR_ARGS, "AbcGradient: no network");
  if (!feat || !tgt || !grad || n < 1) return err(FLETCHER_ERR_ARGS, "AbcGradient: bad arguments");
  if (train_attr()) return FLETCHER_GetLastError();
  const int blocks = (n + kTB - 1) / kTB;
  float *df = nullptr, *dt = nullptr, *dl = nullptr, *dg = nullptr, *partial = nullptr, *lpartial = nullptr;
  CKA(cudaMalloc(&df, (size_t)n * kIn * sizeof(float)));
  CKA(cudaMalloc(&dt, (size_t)n * kTgt * sizeof(float)));
  CKA(cudaMalloc(&dl, sizeof(float)));
  CKA(cudaMalloc(&dg, kNP * sizeof(float)));
  CKA(cudaMalloc(&partial, (size_t)blocks * kNP * sizeof(float)));
  CKA(cudaMalloc(&lpartial, blocks * sizeof(float)));
  CKA(cudaMemcpy(df, feat, (size_t)n * kIn * sizeof(float), cudaMemcpyHostToDevice));
  CKA(cudaMemcpy(dt, tgt, (size_t)n * kTgt * sizeof(float), cudaMemcpyHostToDevice));
  k_abc_train<<<blocks, kTB, kTrainSmem>>>(df, dt, n, n, 0u, T.P, 0.f, partial, lpartial);
  k_abc_reduce<<<(kNP + 255) / 256, 256>>>(partial, lpartial, blocks, dg, dl);
  CKA(cudaGetLastError());
  CKA(cudaMemcpy(grad, dg, kNP * sizeof(float), cudaMemcpyDeviceToHost));
  if (loss) CKA(cudaMemcpy(loss, dl, sizeof(float), cudaMemcpyDeviceToHost));
  cudaFree(df);
  cudaFree(dt);
  cudaFree(dl);
  cudaFree(dg);
  cudaFree(partial);
  cudaFree(lpartial);
  return FLETCHER_OK;
}

extern "C" int FLETCHER_AbcForward(const float *feat, int n, float *out) {
  if (!T.weights) return err(FLETCHER_ERR_ARGS, "AbcForward: no network");
  if (!feat || !out || n < 1) return err(FLETCHER_ERR_ARGS, "AbcForward: bad arguments");
  float *df = nullptr, *dout = nullptr;
  CKA(cudaMalloc(&df, (size_t)n * kIn * sizeof(float)));
  CKA(cudaMalloc(&dout, (size_t)n * kOut * sizeof(float)));
  CKA(cudaMemcpy(df, feat, (size_t)n * kIn * sizeof(float), cudaMemcpyHostToDevice));
  const int grid = (int)(((n + 15) / 16 + kInferWarps - 1) / kInferWarps);
  k_abc_forward<<<grid, 32 * kInferWarps>>>(df, n, T.net, dout);
  CKA(cudaGetLastError());
  CKA(cudaMemcpy(out, dout, (size_t)n * kOut * sizeof(float), cudaMemcpyDeviceToHost));
  cudaFree(df);
  cudaFree(dout);
  return FLETCHER_OK;
}

extern "C" int FLETCHER_SetBoundary(int mode, int layer, float damping) {
  const ResidentView v = resident_view();
  if (!v.init) return err(FLETCHER_ERR_ARGS, "SetBoundary needs an initialised FP32 resident state");
  abc_release_resident();
  if (mode == FLETCHER_BOUNDARY_PLAIN) return FLETCHER_OK;
  if (mode != FLETCHER_BOUNDARY_LEARNED && mode != FLETCHER_BOUNDARY_SPONGE && mode != FLETCHER_BOUNDARY_ONEWAY)
    return err(FLETCHER_ERR_ARGS, "SetBoundary: unknown mode");
  if (mode == FLETCHER_BOUNDARY_LEARNED && !T.weights)
    return err(FLETCHER_ERR_ARGS, "SetBoundary: the learned layer needs weights");
  if (layer < kRadius + 1) return err(FLETCHER_ERR_ARGS, "SetBoundary: layer must be at least 5 cells");
  if (!(damping >= 0.f) || (mode == FLETCHER_BOUNDARY_SPONGE && !(damping > 0.f)))
    return err(FLETCHER_ERR_ARGS, "SetBoundary: damping must be >= 0 (> 0 for the sponge)");
  const int dims[3] = {v.sx, v.sy, v.sz};
  Box in, keep;
  for (int a = 0; a < 3; ++a) {
    keep.lo[a] = v.bord;
    keep.hi[a] = dims[a] - v.bord;
    in.lo[a] = v.bord + layer;
    in.hi[a] = dims[a] - v.bord - layer;
    if (in.hi[a] <= in.lo[a]) return err(FLETCHER_ERR_ARGS, "SetBoundary: no interior inside the layer");
  }
  R.G = make_ghost(in, layer);
  if ((long)v.sz * v.sy * v.pitch >= (1l << 31))
    return err(FLETCHER_ERR_ARGS, "SetBoundary: the layer needs a field of fewer than 2^31 cells");
  if (oneway_mode(mode)) {
    const long n = R.G.off[6];
    CKA(cudaMalloc(&R.med, n * sizeof(float4)));
    CKA(cudaMalloc(&R.k, n * sizeof(float2)));
    k_abc_fill<<<grid_of(n, 256), 256, 0, v.stream>>>(R.G, v.coef, v.sy, v.pitch, v.dt, v.dx, v.dy, v.dz, R.med,
                                                      R.k);
    CKA(cudaGetLastError());
    if (mode == FLETCHER_BOUNDARY_LEARNED) {
      // The first step's t-1 lines from the previous field; each boundary
      // launch then stores the t lines for the next one.
      for (int b = 0; b < 2; ++b) CKA(cudaMalloc(&R.lines[b], n * 2 * sizeof(float2)));
      k_abc_lines<<<grid_of(n * 2, 256), 256, 0, v.stream>>>(R.G, v.prev, v.sy, v.pitch, R.med, R.lines[0]);
      CKA(cudaGetLastError());
    }
    CKA(cudaMalloc(&R.bar, 2 * sizeof(unsigned)));
    CKA(cudaMemsetAsync(R.bar, 0, 2 * sizeof(unsigned), v.stream));
    // Cooperative grids: every block resident at once (the grid barrier needs it).
    const int sms = v.num_sms > 0 ? v.num_sms : 1;
    int per_sm = 0;
    CKA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_abc_boundary, 256, 0));
    if (per_sm < 1) return err(FLETCHER_ERR_CUDA, "SetBoundary: the boundary kernel fits no block on an SM");
    R.grid_net = per_sm * sms;
    int per_sm_r = 0, per_sm_s = 0;
    CKA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_r, k_abc_rays_coop<false>, 256, 0));
    CKA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_s, k_abc_rays_coop<true>, 256, 0));
    per_sm_r = std::min(std::min(per_sm_r, per_sm_s), 4);
    if (per_sm_r < 1) return err(FLETCHER_ERR_CUDA, "SetBoundary: the ray kernel fits no block on an SM");
    R.grid_rays = per_sm_r * sms;
  }
  if (damping > 0.f) {
    // Layer cells in z, y, x order (coalesced).
    std::vector<LayerCell> cells;
    for (int z = keep.lo[2]; z < keep.hi[2]; ++z)
      for (int y = keep.lo[1]; y < keep.hi[1]; ++y) {
        const bool inner = z >= in.lo[2] && z < in.hi[2] && y >= in.lo[1] && y < in.hi[1];
        for (int x = keep.lo[0]; x < keep.hi[0]; x = (inner && x == in.lo[0]) ? in.hi[0] : x + 1) {
          if (inner && x >= in.lo[0] && x < in.hi[0]) continue;
          const int c[3] = {x, y, z};
          int d = 0;
          for (int a = 0; a < 3; ++a) {
            const int lo = in.lo[a] - c[a], hi = c[a] - (in.hi[a] - 1);
            d = lo > d ? lo : d;
            d = hi > d ? hi : d;
          }
          if (d > 0) cells.push_back({x, y, z, d});
        }
      }
    R.ncells = (long)cells.size();
    CKA(cudaMalloc(&R.cells, R.ncells * sizeof(LayerCell)));
    CKA(cudaMemcpyAsync(R.cells, cells.data(), R.ncells * sizeof(LayerCell), cudaMemcpyHostToDevice, v.stream));
  }
  CKA(cudaStreamSynchronize(v.stream));
  R.mode = mode;
  R.damping = damping;
  R.interval = g_interval;
  R.steps = 0;
  R.on = true;
  return FLETCHER_OK;
}

extern "C" int FLETCHER_AbcSetInterval(int steps) {
  if (steps < 1) return err(FLETCHER_ERR_ARGS, "AbcSetInterval: steps must be >= 1");
  g_interval = steps;
  if (R.on) R.interval = steps;
  return FLETCHER_OK;
}

extern "C" long FLETCHER_AbcLayerCells(void) { return (R.on && oneway_mode(R.mode)) ? R.G.off[6] : 0; }

extern "C" void FLETCHER_AbcRelease(void) {
  abc_release_resident();
  if (T.P) cudaFree(T.P);
  if (T.grad) cudaFree(T.grad);
  if (T.m) cudaFree(T.m);
  if (T.v) cudaFree(T.v);
  if (T.net) cudaFree(T.net);
  if (T.feat) cudaFree(T.feat);
  if (T.tgt) cudaFree(T.tgt);
  if (T.pos) cudaFree(T.pos);
  T = Trainer();
}
