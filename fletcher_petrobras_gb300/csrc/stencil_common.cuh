// Stencil pieces shared by the propagate kernels: the reference's weights
// (original/derivatives.h:13-41) as compile-time constants and the packed
// (p, q) first and second derivatives built from them.
#pragma once
#include "device_util.cuh"

namespace flt {

// Stencil weights of original/derivatives.h:13-41 (first derivative L1..L4,
// second derivative K0..K4) as compile-time constants.
constexpr float cL1 = 0.8f, cL2 = -0.2f, cL3 = 0.0380952380952381f, cL4 = -0.0035714285714285713f;
constexpr float cK0 = -2.84722222222222222222f, cK1 = 1.6f, cK2 = -0.2f, cK3 = 0.02539682539682539682f,
                cK4 = -0.00178571428571428571f;

// First derivative (unscaled) from the four (+j, -j) pairs.
__device__ __forceinline__ f2 d1(f2 a1, f2 b1, f2 a2, f2 b2, f2 a3, f2 b3, f2 a4, f2 b4) {
  f2 r = mul2(splat(cL1), sub2(a1, b1));
  r = fma2(splat(cL2), sub2(a2, b2), r);
  r = fma2(splat(cL3), sub2(a3, b3), r);
  return fma2(splat(cL4), sub2(a4, b4), r);
}
// Second derivative (unscaled) from the centre and four (+j, -j) pairs.
__device__ __forceinline__ f2 d2(f2 c, f2 a1, f2 b1, f2 a2, f2 b2, f2 a3, f2 b3, f2 a4, f2 b4) {
  f2 r = mul2(splat(cK0), c);
  r = fma2(splat(cK1), add2(a1, b1), r);
  r = fma2(splat(cK2), add2(a2, b2), r);
  r = fma2(splat(cK3), add2(a3, b3), r);
  return fma2(splat(cK4), add2(a4, b4), r);
}
// (p, q) pairs through the scalar round-to-nearest intrinsics: each
// operation rounded on its own, never contracted into a fused multiply-add
// (unlike plain expressions, which the compiler may fuse).
__device__ __forceinline__ f2 add_rn(f2 a, f2 b) { return mk2(__fadd_rn(lo(a), lo(b)), __fadd_rn(hi(a), hi(b))); }
__device__ __forceinline__ f2 sub_rn(f2 a, f2 b) { return mk2(__fsub_rn(lo(a), lo(b)), __fsub_rn(hi(a), hi(b))); }
__device__ __forceinline__ f2 mul_rn(float s, f2 b) { return mk2(__fmul_rn(s, lo(b)), __fmul_rn(s, hi(b))); }

// The two derivatives in the reference's operation order
// (original/derivatives.h:47,53, the Der1 / Der2 macros): every term
// rounded on its own, the terms summed left to right, the sum multiplied by
// the inverse spacing last -- the floats of a build without contraction.
__device__ __forceinline__ f2 d1_ref(f2 a1, f2 b1, f2 a2, f2 b2, f2 a3, f2 b3, f2 a4, f2 b4, float dinv) {
  f2 r = mul_rn(cL1, sub_rn(a1, b1));
  r = add_rn(r, mul_rn(cL2, sub_rn(a2, b2)));
  r = add_rn(r, mul_rn(cL3, sub_rn(a3, b3)));
  r = add_rn(r, mul_rn(cL4, sub_rn(a4, b4)));
  return mul_rn(dinv, r);
}
__device__ __forceinline__ f2 d2_ref(f2 c, f2 a1, f2 b1, f2 a2, f2 b2, f2 a3, f2 b3, f2 a4, f2 b4, float d2inv) {
  f2 r = mul_rn(cK0, c);
  r = add_rn(r, mul_rn(cK1, add_rn(a1, b1)));
  r = add_rn(r, mul_rn(cK2, add_rn(a2, b2)));
  r = add_rn(r, mul_rn(cK3, add_rn(a3, b3)));
  r = add_rn(r, mul_rn(cK4, add_rn(a4, b4)));
  return mul_rn(d2inv, r);
}

// Applies a spacing factor unless the grid is isotropic (then every factor
// is folded into one dt^2/h^2 at the end).
template <bool ISO>
__device__ __forceinline__ f2 scale(f2 v, float s) {
  if constexpr (ISO) return v;
  else return mul2(splat(s), v);
}

// Adds `s` to the register among {c, a[0..3] (offsets +1..+4), b[0..3]
// (offsets -1..-4)} at offset d from the centre (|d| <= 4).
__device__ __forceinline__ void add_at(f2 &c, f2 (&a)[4], f2 (&b)[4], int d, f2 s) {
  if (d == 0) c = add2(c, s);
#pragma unroll
  for (int j = 1; j <= 4; ++j) {
    if (d == j) a[j - 1] = add2(a[j - 1], s);
    if (d == -j) b[j - 1] = add2(b[j - 1], s);
  }
}

}  // namespace flt
