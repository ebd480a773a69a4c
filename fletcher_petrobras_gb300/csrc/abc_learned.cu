// Learned absorbing boundary: a thin layer around the interior whose outer
// cells get a correction from a small per-cell MLP.
//
// Geometry.  The grid is interior + a layer of L cells + bord zero cells on
// every side; the plain update runs over interior and layer alike (the
// medium is extended into the layer, no random velocities).  A layer cell at
// Chebyshev distance d outside the interior has an update stencil (radius 4)
// that reaches past the layer once d > L - 4; those reads see the zero
// border where an unbounded medium would hold the outgoing wave.  The
// network predicts the missing part of the update, dt^2 * rhs(field beyond
// the layer) (the rhs of original/sample.h:32-89), from what the cell can
// see: the 9-point stencils of p and q along its outward normal at t and
// t-1 (points beyond the layer read as zero), vpz, epsilon, delta and d / L.
// Stencil inputs are divided by their largest magnitude s and the output is
// multiplied by s * out_scale, so the network works on unit-scale values.
// It serves the face cells of the layer (one axis more than L - 4 outside);
// edge and corner cells keep the plain update.
//
// Network: 40 -> 32 -> 32 -> 2, tanh, FP16 weights and FP16 activations
// between layers, FP32 accumulation and FP32 biases.
//   * inference (k_abc_infer) runs on the tensor cores (mma.sync m16n8k16,
//     f16 x f16 -> f32): one warp evaluates 16 cells, the layer-1 and
//     layer-2 outputs stay in registers as the next layer's A fragments;
//   * training (k_abc_train) is a per-sample forward and backward pass in
//     FP32 with the same roundings (straight-through), block sums of the
//     gradients, and Adam (k_abc_adam) on FP32 master weights.
//
// Training data (k_abc_collect) come from plain-method runs on padded
// domains: around a virtual interior box, the layer cells' inputs are read
// with everything beyond the layer set to zero, and the target is the
// update's contribution from the cells beyond the layer.
#include <cuda_fp16.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>

#include <vector>

#include "../../include/fletcher_gb300.h"
#include "device_util.cuh"
#include "fletcher_internal.h"
#include "stencil_common.cuh"

int flt_record_error(int code, const char *msg);

namespace flt {

constexpr int kIn = 40, kHid = 32, kOut = 2;
constexpr int kSt = 36;  // stencil inputs (4 x 9)
// Master parameter layout (FP32): W1 [32][40], b1, W2 [32][32], b2, W3 [2][32], b3.
constexpr int oW1 = 0, oB1 = oW1 + kHid * kIn, oW2 = oB1 + kHid, oB2 = oW2 + kHid * kHid, oW3 = oB2 + kHid,
              oB3 = oW3 + kOut * kHid, kNP = oB3 + kOut;
static_assert(kNP == FLETCHER_ABC_PARAMS, "parameter count");
constexpr int kK1 = 48;      // layer-1 K padded to a multiple of 16
constexpr int kXs = 56;      // row stride (halves) of a warp's feature tile: conflict-free A loads
constexpr float kVScale = 1.0f / 4000.0f;
constexpr float kMinScale = 1e-30f;  // smallest stencil magnitude the network sees

// Inference copy of the network: FP16 weights in mma B-operand order
// (row n = output, contiguous k), FP32 biases.
struct NetHalf {
  __half w1[kHid * kK1];
  __half w2[kHid * kHid];
  __half w3[8 * kHid];
  float b1[kHid], b2[kHid], b3[8];
  float out_scale;
};

// One layer cell: position, outward axis (0 x, 1 y, 2 z), direction
// (+1 / -1), distance d, and its medium.
struct LayerCell {
  int x, y, z, code;  // code = axis | (sign > 0) << 2 | d << 3
  float vpz, eps, del, pad;
};

// A box [lo, hi) per axis.
struct Box {
  int lo[3], hi[3];
};

// ---- features -------------------------------------------------------------------

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
      v = F[((size_t)c[2] * sy + c[1]) * pitch + c[0]];
    p9[j + kRadius] = v.x;
    q9[j + kRadius] = v.y;
  }
}

// Distance outside `in` (Chebyshev), outward axis (first largest) and sign.
__host__ __device__ __forceinline__ int outside_of(const Box &in, int x, int y, int z, int *axis, int *sgn) {
  const int c[3] = {x, y, z};
  int d = 0, a = 0, s = 1;
  for (int k = 0; k < 3; ++k) {
    const int lo = in.lo[k] - c[k], hi = c[k] - (in.hi[k] - 1);
    const int dk = lo > hi ? lo : hi;
    if (dk > d) {
      d = dk;
      a = k;
      s = hi > 0 ? 1 : -1;
    }
  }
  *axis = a;
  *sgn = s;
  return d;
}

// Number of axes along which (x, y, z) lies more than L - 4 cells outside
// `in` (its stencil along that axis reaches past the layer).  The network
// serves face cells (exactly one such axis); its input sees one normal.
__host__ __device__ __forceinline__ int far_axes(const Box &in, int x, int y, int z, int L) {
  const int c[3] = {x, y, z};
  int n = 0;
  for (int k = 0; k < 3; ++k) {
    const int lo = in.lo[k] - c[k], hi = c[k] - (in.hi[k] - 1);
    n += (lo > L - kRadius || hi > L - kRadius) ? 1 : 0;
  }
  return n;
}

// ---- targets: the update's contribution of the cells outside `keep` ----

// (p, q) of the current field at a cell, if it lies outside `keep`.
__device__ __forceinline__ float2 outer(const float2 *F, int x, int y, int z, const Box &keep, int sy, int pitch) {
  const bool in = x >= keep.lo[0] && x < keep.hi[0] && y >= keep.lo[1] && y < keep.hi[1] && z >= keep.lo[2] &&
                  z < keep.hi[2];
  if (in) return make_float2(0.f, 0.f);
  return F[((size_t)z * sy + y) * pitch + x];
}

// dt^2 * (rhsp, rhsq) of original/sample.h:32-89 evaluated on the field
// outside `keep` (it is linear in the field).
__device__ float2 outer_update(const float2 *F, const float *coef, int x, int y, int z, const Box &keep, int sy,
                               int pitch, float dx, float dy, float dz, float dt) {
  const float K[5] = {cK0, cK1, cK2, cK3, cK4};
  const float Lw[5] = {0.f, cL1, cL2, cL3, cL4};
  float2 d2[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
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

// Training samples from the face cells of the layer of a virtual interior
// box `in` (layer L, keep = in grown by L): features, targets / s and the
// cell.  A random fraction `keep_frac` of the cells is taken; cells whose
// stencils are below `min_scale` carry no wave and are skipped.
__global__ void k_abc_collect(const float2 *cur, const float2 *prev, const float *coef, Box in, Box keep, int L,
                              int sy, int pitch, float dx, float dy, float dz, float dt, float keep_frac,
                              uint32_t seed, float min_scale, float *feat, float *tgt, int4 *pos,
                              unsigned long long *count, unsigned long long cap) {
  const int ex = keep.hi[0] - keep.lo[0], ey = keep.hi[1] - keep.lo[1], ez = keep.hi[2] - keep.lo[2];
  const long n = (long)ex * ey * ez;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const int x = keep.lo[0] + (int)(i % ex), y = keep.lo[1] + (int)((i / ex) % ey),
              z = keep.lo[2] + (int)(i / ((long)ex * ey));
    int a, sgn;
    const int d = outside_of(in, x, y, z, &a, &sgn);
    if (d <= L - kRadius || far_axes(in, x, y, z, L) != 1) continue;
    if ((mix32(seed, (uint32_t)i) >> 8) * (1.0f / 16777216.0f) >= keep_frac) continue;
    float v[kSt];
    normal_stencil(cur, x, y, z, a, sgn, keep, sy, pitch, v, v + 9);
    normal_stencil(prev, x, y, z, a, sgn, keep, sy, pitch, v + 18, v + 27);
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < kSt; ++k) s = fmaxf(s, fabsf(v[k]));
    if (!(s > min_scale) || !(s > kMinScale)) continue;
    const unsigned long long slot = atomicAdd(count, 1ull);
    if (slot >= cap) continue;
    pos[slot] = make_int4(x, y, z, d);
    const float inv = 1.0f / s;
    float *f = feat + slot * kIn;
#pragma unroll
    for (int k = 0; k < kSt; ++k) f[k] = v[k] * inv;
    const float4 m = medium_of(coef, x, y, z, sy, pitch);
    f[36] = m.x * kVScale;
    f[37] = m.y;
    f[38] = m.z;
    f[39] = (float)d / (float)L;
    const float2 t = outer_update(cur, coef, x, y, z, keep, sy, pitch, dx, dy, dz, dt);
    tgt[slot * 2] = t.x * inv;
    tgt[slot * 2 + 1] = t.y * inv;
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

__device__ __forceinline__ float tanh_fast(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ uint32_t pack_h2(float lo_v, float hi_v) {
  const __half2 h = __floats2half2_rn(lo_v, hi_v);
  return *reinterpret_cast<const uint32_t *>(&h);
}

// The network on the warp's 16-row feature tile Xs (FP16, row stride kXs).
// Lanes with (lane & 3) == 0 return the outputs of rows lane/4 and lane/4+8.
__device__ __forceinline__ void mlp16(const __half *Xs, const NetHalf &N, float (&y_lo)[2], float (&y_hi)[2]) {
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
    const float b0 = N.b1[8 * nt + 2 * t], b1 = N.b1[8 * nt + 2 * t + 1];
    h[nt][0] = b0; h[nt][1] = b1; h[nt][2] = b0; h[nt][3] = b1;
#pragma unroll
    for (int ks = 0; ks < 3; ++ks) {
      const __half *w = N.w1 + (8 * nt + g) * kK1 + 16 * ks + 2 * t;
      mma16816(h[nt], a[ks], *reinterpret_cast<const uint32_t *>(w), *reinterpret_cast<const uint32_t *>(w + 8));
    }
  }
  uint32_t a2[2][4];
#pragma unroll
  for (int kt = 0; kt < 2; ++kt) {
    a2[kt][0] = pack_h2(tanh_fast(h[2 * kt][0]), tanh_fast(h[2 * kt][1]));
    a2[kt][1] = pack_h2(tanh_fast(h[2 * kt][2]), tanh_fast(h[2 * kt][3]));
    a2[kt][2] = pack_h2(tanh_fast(h[2 * kt + 1][0]), tanh_fast(h[2 * kt + 1][1]));
    a2[kt][3] = pack_h2(tanh_fast(h[2 * kt + 1][2]), tanh_fast(h[2 * kt + 1][3]));
  }
#pragma unroll
  for (int nt = 0; nt < 4; ++nt) {
    const float b0 = N.b2[8 * nt + 2 * t], b1 = N.b2[8 * nt + 2 * t + 1];
    h[nt][0] = b0; h[nt][1] = b1; h[nt][2] = b0; h[nt][3] = b1;
#pragma unroll
    for (int kt = 0; kt < 2; ++kt) {
      const __half *w = N.w2 + (8 * nt + g) * kHid + 16 * kt + 2 * t;
      mma16816(h[nt], a2[kt], *reinterpret_cast<const uint32_t *>(w), *reinterpret_cast<const uint32_t *>(w + 8));
    }
  }
#pragma unroll
  for (int kt = 0; kt < 2; ++kt) {
    a2[kt][0] = pack_h2(tanh_fast(h[2 * kt][0]), tanh_fast(h[2 * kt][1]));
    a2[kt][1] = pack_h2(tanh_fast(h[2 * kt][2]), tanh_fast(h[2 * kt][3]));
    a2[kt][2] = pack_h2(tanh_fast(h[2 * kt + 1][0]), tanh_fast(h[2 * kt + 1][1]));
    a2[kt][3] = pack_h2(tanh_fast(h[2 * kt + 1][2]), tanh_fast(h[2 * kt + 1][3]));
  }
  float o[4] = {N.b3[2 * t], N.b3[2 * t + 1], N.b3[2 * t], N.b3[2 * t + 1]};
#pragma unroll
  for (int kt = 0; kt < 2; ++kt) {
    const __half *w = N.w3 + g * kHid + 16 * kt + 2 * t;
    mma16816(o, a2[kt], *reinterpret_cast<const uint32_t *>(w), *reinterpret_cast<const uint32_t *>(w + 8));
  }
  y_lo[0] = o[0];
  y_lo[1] = o[1];
  y_hi[0] = o[2];
  y_hi[1] = o[3];
}

constexpr int kInferWarps = 8;

// Fused layer-cell step: gathers every listed cell's inputs from the
// current and previous fields, evaluates the network and writes the
// correction (p, q) of the cell.  A warp takes 16 cells: two lanes per cell,
// one reading time t, the other t-1.
__global__ void __launch_bounds__(32 * kInferWarps) k_abc_infer(const LayerCell *cells, long ncells, const float2 *cur,
                                                                 const float2 *prev, Box keep, int L, int sy, int pitch,
                                                                 const NetHalf *net, float2 *corr) {
  __shared__ __align__(16) __half Xs[kInferWarps][16 * kXs];
  __shared__ NetHalf N;
  for (int i = threadIdx.x; i < (int)(sizeof(NetHalf) / 4); i += blockDim.x)
    reinterpret_cast<uint32_t *>(&N)[i] = reinterpret_cast<const uint32_t *>(net)[i];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = lane >> 1, half_t = lane & 1;
  __half *X = Xs[warp];
  const long ntiles = (ncells + 15) / 16;
  for (long tile = blockIdx.x * (long)kInferWarps + warp; tile < ntiles; tile += (long)gridDim.x * kInferWarps) {
    const long ci = tile * 16 + r;
    float v[18];
    float s = 0.f;
    LayerCell lc = {0, 0, 0, 0, 0.f, 0.f, 0.f, 0.f};
    if (ci < ncells) {
      lc = cells[ci];
      const int a = lc.code & 3, sgn = (lc.code & 4) ? 1 : -1;
      normal_stencil(half_t ? prev : cur, lc.x, lc.y, lc.z, a, sgn, keep, sy, pitch, v, v + 9);
#pragma unroll
      for (int k = 0; k < 18; ++k) s = fmaxf(s, fabsf(v[k]));
    } else {
#pragma unroll
      for (int k = 0; k < 18; ++k) v[k] = 0.f;
    }
    s = fmaxf(s, __shfl_xor_sync(0xffffffffu, s, 1));
    // Stencils this small carry no wave (the first cells a front reaches
    // hold values near the FP32 underflow, whose reciprocal overflows).
    if (!(s > kMinScale)) s = 0.f;
    const float inv = s > 0.f ? 1.0f / s : 0.f;
    __half *row = X + r * kXs + 18 * half_t;
#pragma unroll
    for (int k = 0; k < 18; k += 2)
      *reinterpret_cast<__half2 *>(row + k) = __floats2half2_rn(v[k] * inv, v[k + 1] * inv);
    if (half_t == 0) {
      X[r * kXs + 36] = __float2half_rn(lc.vpz * kVScale);
      X[r * kXs + 37] = __float2half_rn(lc.eps);
      X[r * kXs + 38] = __float2half_rn(lc.del);
      X[r * kXs + 39] = __float2half_rn((float)(lc.code >> 3) / (float)L);
    } else {
#pragma unroll
      for (int k = 40; k < kK1; ++k) X[r * kXs + k] = __float2half_rn(0.f);
    }
    __syncwarp();
    float ylo[2], yhi[2];
    mlp16(X, N, ylo, yhi);
    const int g = lane >> 2;
    const float s_lo = __shfl_sync(0xffffffffu, s, 2 * g), s_hi = __shfl_sync(0xffffffffu, s, 2 * (g + 8));
    if ((lane & 3) == 0) {
      const long c0 = tile * 16 + g, c1 = tile * 16 + g + 8;
      const float k0 = s_lo * N.out_scale, k1 = s_hi * N.out_scale;
      if (c0 < ncells) corr[c0] = make_float2(ylo[0] * k0, ylo[1] * k0);
      if (c1 < ncells) corr[c1] = make_float2(yhi[0] * k1, yhi[1] * k1);
    }
    __syncwarp();
  }
}

// The network on given features (rows of 40 floats), raw outputs.
__global__ void __launch_bounds__(32 * kInferWarps) k_abc_forward(const float *feat, long n, const NetHalf *net,
                                                                   float *out) {
  __shared__ __align__(16) __half Xs[kInferWarps][16 * kXs];
  __shared__ NetHalf N;
  for (int i = threadIdx.x; i < (int)(sizeof(NetHalf) / 4); i += blockDim.x)
    reinterpret_cast<uint32_t *>(&N)[i] = reinterpret_cast<const uint32_t *>(net)[i];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
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
    mlp16(X, N, ylo, yhi);
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

// The layer's step after the plain update: next[cell] += corr[cell] for the
// first nnet listed cells (the network's), then every layer cell is scaled
// by its taper weight exp(-(damping * d)^2) (1 when damping is 0).
__global__ void k_abc_add(const LayerCell *cells, long ncells, long nnet, const float2 *corr, float2 *next, int sy,
                          int pitch, float damping) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < ncells; i += (long)gridDim.x * blockDim.x) {
    const LayerCell c = cells[i];
    float2 *p = next + ((size_t)c.z * sy + c.y) * pitch + c.x;
    float2 v = *p;
    if (i < nnet) {
      const float2 d = corr[i];
      v.x += d.x;
      v.y += d.y;
    }
    if (damping > 0.f) {
      const float a = damping * (float)(c.code >> 3);
      const float w = __expf(-a * a);
      v.x *= w;
      v.y *= w;
    }
    *p = v;
  }
}

// Medium of the listed cells from the coefficient block.
__global__ void k_abc_fill_medium(LayerCell *cells, long ncells, const float *coef, int sy, int pitch) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < ncells; i += (long)gridDim.x * blockDim.x) {
    LayerCell c = cells[i];
    const float4 m = medium_of(coef, c.x, c.y, c.z, sy, pitch);
    c.vpz = m.x;
    c.eps = m.y;
    c.del = m.z;
    cells[i] = c;
  }
}

// ---- training -------------------------------------------------------------------

constexpr int kTB = 128;  // samples per training block
constexpr int sX = 41, sH = 33;

__device__ __forceinline__ float h16(float v) { return __half2float(__float2half_rn(v)); }

// Forward and backward of B samples (index b of the batch: a random sample,
// or b itself when seed is 0): loss += sum (y - t * tgt_scale)^2 / (2 B),
// gradients summed into grad.  Weights are used FP16-rounded, activations
// are rounded to FP16 between layers (as inference does), the derivatives
// treat both roundings as the identity.  noise > 0 perturbs the stencil
// inputs.
__global__ void __launch_bounds__(kTB) k_abc_train(const float *feat, const float *tgt, long nsamp, int B,
                                                    uint32_t seed, const float *P, float tgt_scale, float noise,
                                                    float *grad, float *loss) {
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
      // Input noise (approximately normal, from four uniforms): the network
      // learns to respond weakly to perturbations of the layer's fields.
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
    a1[o] = tanhf(z);
    h1[o] = live ? h16(a1[o]) : 0.f;
  }
  for (int o = 0; o < kHid; ++o) {
    float z = b2[o];
    for (int k = 0; k < kHid; ++k) z = fmaf(W2[o * kHid + k], h1[k], z);
    a2[o] = tanhf(z);
    h2[o] = live ? h16(a2[o]) : 0.f;
  }
  float l = 0.f;
  for (int o = 0; o < kOut; ++o) {
    float y = b3[o];
    for (int k = 0; k < kHid; ++k) y = fmaf(W3[o * kHid + k], h2[k], y);
    const float e = live ? y - tgt[si * kOut + o] * tgt_scale : 0.f;
    l += e * e;
    dy[o] = e / (float)B;
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
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((tid & 31) == 0) atomicAdd(loss, l / (2.0f * (float)B));
  __syncthreads();
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
    atomicAdd(&grad[e], s);
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
__global__ void k_abc_pack(const float *P, float out_scale, NetHalf *N) {
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
  if (i == 0) N->out_scale = out_scale;
}

__global__ void k_sumsq(const float *v, long n, double *out) {
  double s = 0.0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    s += (double)v[i] * v[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

// ---- host state -------------------------------------------------------------------

namespace {

struct Trainer {
  float *P = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;  // master weights and Adam state
  NetHalf *net = nullptr;
  float out_scale = 1.0f;
  bool weights = false;
  long adam_t = 0;
  float *feat = nullptr, *tgt = nullptr;
  int4 *pos = nullptr;  // grid cell and distance of every sample
  unsigned long long *count = nullptr;
  long cap = 0;
};

struct ResidentLayer {
  bool on = false;
  int L = 0, mode = 0;
  float damping = 0.f;
  LayerCell *cells = nullptr;  // network cells first, then the other layer cells; z, y, x order in each
  long ncells = 0, nnet = 0;
  float2 *corr = nullptr;
  Box in, keep;
};

Trainer T;
ResidentLayer R;

int err(int code, const char *msg) { return flt_record_error(code, msg); }

#define CKA(call)                                                                                       \
  do {                                                                                                  \
    cudaError_t e_ = (call);                                                                            \
    if (e_ != cudaSuccess) {                                                                            \
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
  k_abc_pack<<<(kHid * kK1 + 255) / 256, 256, 0, s>>>(T.P, T.out_scale, T.net);
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

}  // namespace

bool abc_active() { return R.on; }

void abc_release_resident() {
  if (R.cells) cudaFree(R.cells);
  if (R.corr) cudaFree(R.corr);
  R = ResidentLayer();
}

cudaError_t abc_before_step(const ResidentView &v) {
  if (!R.on || !R.nnet) return cudaSuccess;
  const int grid = (int)(((R.nnet + 15) / 16 + kInferWarps - 1) / kInferWarps);
  const int cap = v.num_sms > 0 ? v.num_sms * 8 : 1024;
  k_abc_infer<<<grid < cap ? grid : cap, 32 * kInferWarps, 0, v.stream>>>(R.cells, R.nnet, v.cur, v.prev, R.keep,
                                                                          R.L, v.sy, v.pitch, T.net, R.corr);
  return cudaGetLastError();
}

cudaError_t abc_after_step(const ResidentView &v) {
  if (!R.on || !R.ncells) return cudaSuccess;
  const long n = R.damping > 0.f ? R.ncells : R.nnet;
  if (!n) return cudaSuccess;
  k_abc_add<<<grid_of(n, 256), 256, 0, v.stream>>>(R.cells, n, R.nnet, R.corr, v.next, v.sy, v.pitch, R.damping);
  return cudaGetLastError();
}

}  // namespace flt

using namespace flt;

// ===== Part 4: learned absorbing boundary =========================================

extern "C" int FLETCHER_AbcSetWeights(const float *params, float out_scale) {
  if (!params || !(out_scale > 0.f)) return err(FLETCHER_ERR_ARGS, "AbcSetWeights: bad arguments");
  if (ensure_trainer()) return FLETCHER_GetLastError();
  CKA(cudaMemcpy(T.P, params, kNP * sizeof(float), cudaMemcpyHostToDevice));
  CKA(cudaMemset(T.m, 0, kNP * sizeof(float)));
  CKA(cudaMemset(T.v, 0, kNP * sizeof(float)));
  T.adam_t = 0;
  T.out_scale = out_scale;
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
  return FLETCHER_AbcSetWeights(p.data(), 1.0f);
}

extern "C" int FLETCHER_AbcGetWeights(float *params, float *out_scale) {
  if (!T.weights) return err(FLETCHER_ERR_ARGS, "AbcGetWeights: no network");
  CKA(cudaDeviceSynchronize());
  if (params) CKA(cudaMemcpy(params, T.P, kNP * sizeof(float), cudaMemcpyDeviceToHost));
  if (out_scale) *out_scale = T.out_scale;
  return FLETCHER_OK;
}

extern "C" int FLETCHER_AbcReserve(long capacity) {
  if (capacity < 0) return err(FLETCHER_ERR_ARGS, "AbcReserve: negative capacity");
  if (T.feat) cudaFree(T.feat);
  if (T.tgt) cudaFree(T.tgt);
  if (T.pos) cudaFree(T.pos);
  T.feat = T.tgt = nullptr;
  T.pos = nullptr;
  if (!T.count) CKA(cudaMalloc(&T.count, sizeof(unsigned long long)));
  CKA(cudaMemset(T.count, 0, sizeof(unsigned long long)));
  T.cap = capacity;
  if (capacity) {
    CKA(cudaMalloc(&T.feat, (size_t)capacity * kIn * sizeof(float)));
    CKA(cudaMalloc(&T.tgt, (size_t)capacity * kOut * sizeof(float)));
    CKA(cudaMalloc(&T.pos, (size_t)capacity * sizeof(int4)));
  }
  return FLETCHER_OK;
}

extern "C" long FLETCHER_AbcSamples(void) {
  if (!T.count) return 0;
  unsigned long long c = 0;
  if (cudaMemcpy(&c, T.count, sizeof(c), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  return (long)(c < (unsigned long long)T.cap ? c : (unsigned long long)T.cap);
}

extern "C" int FLETCHER_AbcCollect(const int *interior_lo, const int *interior_hi, int layer, float keep_frac,
                                   unsigned seed, float min_scale) {
  const ResidentView v = resident_view();
  if (!v.init) return err(FLETCHER_ERR_ARGS, "AbcCollect needs an FP32 resident state");
  if (!T.count || !T.cap) return err(FLETCHER_ERR_ARGS, "AbcCollect: call FLETCHER_AbcReserve first");
  if (!interior_lo || !interior_hi || layer < kRadius + 1)
    return err(FLETCHER_ERR_ARGS, "AbcCollect: bad box or layer");
  Box in, keep;
  const int dims[3] = {v.sx, v.sy, v.sz};
  for (int a = 0; a < 3; ++a) {
    in.lo[a] = interior_lo[a];
    in.hi[a] = interior_hi[a];
    keep.lo[a] = in.lo[a] - layer;
    keep.hi[a] = in.hi[a] + layer;
    // The target reads 4 cells beyond the kept box; all of it must be updated grid.
    if (in.hi[a] <= in.lo[a] || keep.lo[a] - kRadius < v.bord || keep.hi[a] + kRadius > dims[a] - v.bord)
      return err(FLETCHER_ERR_ARGS, "AbcCollect: the box and its layer must lie 4 cells inside the updated region");
  }
  const long n = (long)(keep.hi[0] - keep.lo[0]) * (keep.hi[1] - keep.lo[1]) * (keep.hi[2] - keep.lo[2]);
  k_abc_collect<<<grid_of(n, 256), 256, 0, v.stream>>>(v.cur, v.prev, v.coef, in, keep, layer, v.sy, v.pitch, v.dx,
                                                       v.dy, v.dz, v.dt, keep_frac, seed, min_scale, T.feat, T.tgt,
                                                       T.pos, T.count, (unsigned long long)T.cap);
  CKA(cudaGetLastError());
  CKA(cudaStreamSynchronize(v.stream));
  return FLETCHER_OK;
}

extern "C" int FLETCHER_AbcGetSamples(long start, long n, float *feat, float *tgt, int *pos) {
  const long have = FLETCHER_AbcSamples();
  if (start < 0 || n < 0 || start + n > have)
    return err(FLETCHER_ERR_ARGS, "AbcGetSamples: range outside the samples");
  if (feat) CKA(cudaMemcpy(feat, T.feat + start * kIn, n * kIn * sizeof(float), cudaMemcpyDeviceToHost));
  if (tgt) CKA(cudaMemcpy(tgt, T.tgt + start * kOut, n * kOut * sizeof(float), cudaMemcpyDeviceToHost));
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
  // Output scale: the root mean square of the targets, fixed at the first
  // training of these weights (Adam's state restarts with it).
  if (T.adam_t == 0) {
    double *d = nullptr;
    CKA(cudaMalloc(&d, sizeof(double)));
    CKA(cudaMemsetAsync(d, 0, sizeof(double), s));
    k_sumsq<<<1024, 256, 0, s>>>(T.tgt, ns * kOut, d);
    double sq = 0.0;
    CKA(cudaMemcpyAsync(&sq, d, sizeof(double), cudaMemcpyDeviceToHost, s));
    CKA(cudaStreamSynchronize(s));
    cudaFree(d);
    const double rms = sqrt(sq / (double)(ns * kOut));
    T.out_scale = rms > 0.0 ? (float)rms : 1.0f;
  }
  float *loss = nullptr;
  CKA(cudaMalloc(&loss, iters * sizeof(float)));
  CKA(cudaMemsetAsync(loss, 0, iters * sizeof(float), s));
  CKA(cudaMemsetAsync(T.grad, 0, kNP * sizeof(float), s));
  const float b1 = 0.9f, b2 = 0.999f;
  const int blocks = (batch + kTB - 1) / kTB;
  for (int it = 0; it < iters; ++it) {
    uint64_t st = (uint64_t)seed * 1000003ull + (uint64_t)it;
    const uint32_t sd = (uint32_t)splitmix(st) | 1u;
    k_abc_train<<<blocks, kTB, kTrainSmem, s>>>(T.feat, T.tgt, ns, batch, sd, T.P, 1.0f / T.out_scale, noise,
                                                T.grad, loss + it);
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
  return FLETCHER_OK;
}

extern "C" int FLETCHER_AbcGradient(const float *feat, const float *tgt, int n, float *grad, float *loss) {
  if (!T.weights) return err(FLETCHER_ERR_ARGS, "AbcGradient: no network");
  if (!feat || !tgt || !grad || n < 1) return err(FLETCHER_ERR_ARGS, "AbcGradient: bad arguments");
  if (train_attr()) return FLETCHER_GetLastError();
  float *df = nullptr, *dt = nullptr, *dl = nullptr, *dg = nullptr;
  CKA(cudaMalloc(&df, (size_t)n * kIn * sizeof(float)));
  CKA(cudaMalloc(&dt, (size_t)n * kOut * sizeof(float)));
  CKA(cudaMalloc(&dl, sizeof(float)));
  CKA(cudaMalloc(&dg, kNP * sizeof(float)));
  CKA(cudaMemcpy(df, feat, (size_t)n * kIn * sizeof(float), cudaMemcpyHostToDevice));
  CKA(cudaMemcpy(dt, tgt, (size_t)n * kOut * sizeof(float), cudaMemcpyHostToDevice));
  CKA(cudaMemset(dl, 0, sizeof(float)));
  CKA(cudaMemset(dg, 0, kNP * sizeof(float)));
  k_abc_train<<<(n + kTB - 1) / kTB, kTB, kTrainSmem>>>(df, dt, n, n, 0u, T.P, 1.0f, 0.f, dg, dl);
  CKA(cudaGetLastError());
  CKA(cudaMemcpy(grad, dg, kNP * sizeof(float), cudaMemcpyDeviceToHost));
  if (loss) CKA(cudaMemcpy(loss, dl, sizeof(float), cudaMemcpyDeviceToHost));
  cudaFree(df);
  cudaFree(dt);
  cudaFree(dl);
  cudaFree(dg);
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
  if (mode != FLETCHER_BOUNDARY_LEARNED && mode != FLETCHER_BOUNDARY_SPONGE)
    return err(FLETCHER_ERR_ARGS, "SetBoundary: unknown mode");
  const bool net = mode == FLETCHER_BOUNDARY_LEARNED;
  if (net && !T.weights) return err(FLETCHER_ERR_ARGS, "SetBoundary: the learned layer needs weights");
  if (layer < kRadius + 1) return err(FLETCHER_ERR_ARGS, "SetBoundary: layer must be at least 5 cells");
  if (!(damping >= 0.f) || (!net && !(damping > 0.f)))
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
  // Layer cells in z, y, x order (coalesced gathers): the network's first.
  std::vector<LayerCell> cells[2];
  for (int z = keep.lo[2]; z < keep.hi[2]; ++z)
    for (int y = keep.lo[1]; y < keep.hi[1]; ++y) {
      const bool inner = z >= in.lo[2] && z < in.hi[2] && y >= in.lo[1] && y < in.hi[1];
      for (int x = keep.lo[0]; x < keep.hi[0]; x = (inner && x == in.lo[0]) ? in.hi[0] : x + 1) {
        if (inner && x >= in.lo[0] && x < in.hi[0]) continue;
        int ax, sg;
        const int d = outside_of(in, x, y, z, &ax, &sg);
        if (d == 0) continue;
        LayerCell lc = {x, y, z, ax | (sg > 0 ? 4 : 0) | (d << 3), 0.f, 0.f, 0.f, 0.f};
        cells[(net && d > layer - kRadius && far_axes(in, x, y, z, layer) == 1) ? 0 : 1].push_back(lc);
      }
    }
  R.nnet = (long)cells[0].size();
  R.ncells = R.nnet + (long)cells[1].size();
  cells[0].insert(cells[0].end(), cells[1].begin(), cells[1].end());
  CKA(cudaMalloc(&R.cells, R.ncells * sizeof(LayerCell)));
  CKA(cudaMalloc(&R.corr, (R.nnet ? R.nnet : 1) * sizeof(float2)));
  CKA(cudaMemcpyAsync(R.cells, cells[0].data(), R.ncells * sizeof(LayerCell), cudaMemcpyHostToDevice, v.stream));
  k_abc_fill_medium<<<grid_of(R.ncells, 256), 256, 0, v.stream>>>(R.cells, R.ncells, v.coef, v.sy, v.pitch);
  CKA(cudaGetLastError());
  CKA(cudaStreamSynchronize(v.stream));
  R.in = in;
  R.keep = keep;
  R.L = layer;
  R.mode = mode;
  R.damping = damping;
  R.on = true;
  return FLETCHER_OK;
}

extern "C" long FLETCHER_AbcLayerCells(void) { return R.on ? R.nnet : 0; }

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
  if (T.count) cudaFree(T.count);
  T = Trainer();
}
