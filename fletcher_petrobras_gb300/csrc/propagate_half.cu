// Reduced-precision wavefield storage: the step of propagate_fp32.cu with p
// and q stored in 16-bit floats and all arithmetic in FP32.
//
// Storage of one field buffer: (p, q) as a half2 per cell, [z][y][pitch],
// with one power-of-two scale per z-plane: stored = value * 2^e[z].  The
// scale of every new plane is set before the step (k_half_scales) from the
// largest magnitudes of the current field within 4 planes and of the
// previous field at that plane, so the new values stay below 2^14 (2^16 is
// FP16's limit) and far above its subnormal range.
//
// The extended form (EXT) adds one signed byte per value: the rounding error
// of the half in units of 2^-8 of the half's last place, i.e. a 19-bit
// significand for every value (3 bytes per value).
//
// Each step, the CTA decodes the (p, q) halo tile of the arriving plane into
// an FP32 shared-memory tile once per cell, then runs the FP32 stencil of
// propagate_fp32.cu on it.  The updated plane is encoded with its new scale,
// and the CTA's largest magnitude on it is folded (atomicMax) into the
// per-plane maximum that the next step's scales use; a magnitude beyond
// FP16's range there sets bit 2 of the error word.
#include <cuda_fp16.h>

#include "device_util.cuh"
#include "fletcher_internal.h"
#include "stencil_common.cuh"

namespace flt {

template <int TY, bool EXT>
struct GeoH {
  static constexpr int TX = kTileX;
  static constexpr int HX = TX + 2 * kRadius;
  static constexpr int HY = TY + 2 * kRadius;
  static constexpr int HXY = HX * HY;
  static constexpr int NT = TX * TY;
  static constexpr int r128(int b) { return (b + 127) / 128 * 128; }
  static constexpr int HI_B = HXY * 4;                   // half2 halo tile
  static constexpr int LO_B = EXT ? HXY * 2 : 0;         // residual bytes of the halo tile
  static constexpr int ARR_B = kArrivalCoef * NT * 4;
  static constexpr int UPD_B = kUpdateCoef * NT * 4;
  static constexpr int PHI_B = NT * 4;                   // previous field (point box)
  static constexpr int PLO_B = EXT ? HX * TY * 2 : 0;    // its residuals, box from x0-4
  static constexpr int OFF_LO = r128(HI_B);
  static constexpr int OFF_ARR = OFF_LO + r128(LO_B);
  static constexpr int OFF_UPD = OFF_ARR + ARR_B;
  static constexpr int OFF_PHI = OFF_UPD + UPD_B;
  static constexpr int OFF_PLO = OFF_PHI + r128(PHI_B);
  static constexpr int STAGE_B = r128(OFF_PLO + PLO_B);
  static constexpr int H32_B = HXY * 8;                  // one decoded FP32 halo tile
  static constexpr int DBUF_B = 2 * TY * HX * 8;
  static constexpr int OFF_H32 = 0;                      // after the stages
  static constexpr int OFF_DB = 2 * H32_B;
  // 16-row tiles (512 threads, at most 128 registers) keep the per-cell
  // in-plane terms (A, B) of the last 5 planes in shared memory.
  static constexpr bool AB_SMEM = TY >= 16;
  static constexpr int OFF_AB = OFF_DB + DBUF_B;
  static constexpr int AB_B = AB_SMEM ? 5 * NT * 16 : 0;
  static constexpr int OFF_BAR = OFF_AB + AB_B;
  static_assert(TY % 4 == 0, "tile rows must be a multiple of 4");
  static_assert(ARR_B % 128 == 0 && UPD_B % 128 == 0, "stage regions 128-B aligned");
};

// A batched item's per-shot values that the plane loop reads, kept in
// shared memory (two records, by item parity) rather than in registers.
struct HRec {
  const int *e_cur, *e_prev, *e_new;  // exponents of the current, previous and new field
  unsigned *out_hi;                   // the new field
  unsigned short *out_lo;
  long plane;                         // pitch * sy
  int src_z, cor_z;
};

template <int TY, int S, bool EXT>
constexpr size_t smem_bytes_half() {
  using G = GeoH<TY, EXT>;
  // stages, two decoded tiles, D1y exchange, S+1 barriers, control words
  // and item records, alignment slack
  return size_t(S) * G::STAGE_B + G::OFF_BAR + 8 * (S + 1) + 32 + 2 * sizeof(HRec) + 128;
}

// 2^e as a float (|e| <= 126).
__device__ __forceinline__ float exp2i(int e) { return __int_as_float((127 + e) << 23); }

// 2^-8 of the last place of the half h (given as a float), for |h| >= 2^-14;
// 2^-32 below that (FP16's subnormal spacing 2^-24, over 2^8).
__device__ __forceinline__ float ext_unit(float h) {
  const int b = max(__float_as_int(h) & 0x7f800000, (127 - 14) << 23);
  return __int_as_float(b - (18 << 23));
}

// 1 / ext_unit(h), exact (a power of two).
__device__ __forceinline__ float ext_inv_unit(float h) {
  const unsigned b = (unsigned)max(__float_as_int(h) & 0x7f800000, (127 - 14) << 23) - (18u << 23);
  return __uint_as_float((254u << 23) - b);
}

// Value of one stored cell pair: (half + r * unit(half)) * 2^-e.
template <bool EXT>
__device__ __forceinline__ f2 decode(unsigned hv, unsigned short rv, float inv) {
  const float2 h = __half22float2(*reinterpret_cast<const __half2 *>(&hv));
  float a = h.x, b = h.y;
  if constexpr (EXT) {
    a = __fmaf_rn((float)(signed char)(rv & 0xffu), ext_unit(a), a);
    b = __fmaf_rn((float)(signed char)(rv >> 8), ext_unit(b), b);
  }
  return mk2(__fmul_rn(a, inv), __fmul_rn(b, inv));
}

// Stored form of a value pair under scale sc = 2^e.
template <bool EXT>
__device__ __forceinline__ void encode(f2 v, float sc, unsigned &hv, unsigned short &rv) {
  const float a = __fmul_rn(lo(v), sc), b = __fmul_rn(hi(v), sc);
  const __half2 h = __floats2half2_rn(a, b);
  hv = *reinterpret_cast<const unsigned *>(&h);
  rv = 0;
  if constexpr (EXT) {
    const float2 hf = __half22float2(h);
    // a - hf.x is exact, and so is the product by a power of two.
    const float ua = ext_inv_unit(hf.x), ub = ext_inv_unit(hf.y);
    const float ra = fminf(fmaxf(rintf(__fmul_rn(__fsub_rn(a, hf.x), ua)), -127.f), 127.f);
    const float rb = fminf(fmaxf(rintf(__fmul_rn(__fsub_rn(b, hf.y), ub)), -127.f), 127.f);
    rv = (unsigned short)(((unsigned)(int)ra & 0xffu) | (((unsigned)(int)rb & 0xffu) << 8));
  }
}

struct HItem {
  int x0, y0, z0, z1;
};

// Fetches a step's tensor maps into the descriptor cache (the residual
// maps exist in the extended form only).
template <bool EXT>
__device__ __forceinline__ void prefetch_maps(const HalfMaps &m) {
  tma_prefetch_desc(&m.cur_hi);
  tma_prefetch_desc(&m.prev_hi);
  if constexpr (EXT) {
    tma_prefetch_desc(&m.cur_lo);
    tma_prefetch_desc(&m.prev_lo);
  }
  tma_prefetch_desc(&m.arr);
  tma_prefetch_desc(&m.upd);
}

// Segment `item` of the launch's list: {x0, y0, z0, z1}.
__device__ __forceinline__ HItem decode_hitem(int item, const PropParams &P) {
  const int4 w = P.seg[item];
  HItem it;
  it.x0 = w.x;
  it.y0 = w.y;
  it.z0 = w.z;
  it.z1 = w.w;
  return it;
}

// A batched work item {shot, x0, y0, chunk index} as a z range of one shot.
struct BItem : HItem {
  int shot;
};

__device__ __forceinline__ BItem decode_bitem(int item, const PropParams &P) {
  const int4 w = P.items[item];
  const ShotDesc &d = P.shots[w.x];
  BItem it;
  it.x0 = w.y;
  it.y0 = w.z;
  it.z0 = d.bord + w.w * d.chunk;
  it.z1 = min(it.z0 + d.chunk, d.sz - d.bord);
  it.shot = w.x;
  return it;
}

// Loads of step k of an item into one stage: the halo tile of plane k, the
// three in-plane coefficients of plane k while k is in the item's range, and
// for the plane k-4 being updated its seven coefficients and previous field.
template <int TY, bool EXT>
__device__ __forceinline__ void issue_half(unsigned char *stage, uint64_t *bar, const HItem &it, int k,
                                           const HalfMaps &M) {
  using G = GeoH<TY, EXT>;
  const bool center = (k >= it.z0) && (k < it.z1);
  const bool upd = (k - kRadius >= it.z0);
  const uint32_t bytes =
      G::HI_B + G::LO_B + (center ? G::ARR_B : 0) + (upd ? G::UPD_B + G::PHI_B + G::PLO_B : 0);
  mbar_arrive_expect_tx(bar, bytes);
  tma_load_3d(stage, &M.cur_hi, bar, it.x0 - kRadius, it.y0 - kRadius, k);
  if constexpr (EXT) tma_load_3d(stage + G::OFF_LO, &M.cur_lo, bar, it.x0 - kRadius, it.y0 - kRadius, k);
  if (center) tma_load_4d(stage + G::OFF_ARR, &M.arr, bar, it.x0, it.y0, 0, k);
  if (upd) {
    tma_load_4d(stage + G::OFF_UPD, &M.upd, bar, it.x0, it.y0, kArrivalCoef, k - kRadius);
    tma_load_3d(stage + G::OFF_PHI, &M.prev_hi, bar, it.x0, it.y0, k - kRadius);
    // 2-byte elements: this box starts at x0-4 so that x * 2 B is a multiple of 16.
    if constexpr (EXT) tma_load_3d(stage + G::OFF_PLO, &M.prev_lo, bar, it.x0 - kRadius, it.y0, k - kRadius);
  }
}

template <int TY, int S, bool ISO, bool EXT>
__global__ void __launch_bounds__(kTileX *TY, 1)
    k_propagate_half(const __grid_constant__ HalfMaps M, const __grid_constant__ HalfParams H) {
  using G = GeoH<TY, EXT>;
  const PropParams &P = H.p;
  const ShotDesc &sd = P.one;
  constexpr int NTH = kTileX * TY;
  extern __shared__ unsigned char smem_dyn[];
  unsigned char *smem = smem_dyn + ((128u - (smem_addr(smem_dyn) & 127u)) & 127u);
  unsigned char *tail = smem + S * G::STAGE_B;
  f2 *H32 = reinterpret_cast<f2 *>(tail + G::OFF_H32);
  f2 *dbuf = reinterpret_cast<f2 *>(tail + G::OFF_DB);
  float4 *ABs = reinterpret_cast<float4 *>(tail + G::OFF_AB);  // [5][NT] (AB_SMEM)
  uint64_t *full = reinterpret_cast<uint64_t *>(tail + G::OFF_BAR);
  uint64_t *xchg = full + S;
  int *ctl = reinterpret_cast<int *>(xchg + 1);
  int *cur = ctl;                                          // producer cursor: item, k, stage
  volatile int *s_end = ctl + 3;                           // end of this CTA's segments
  unsigned *smax = reinterpret_cast<unsigned *>(ctl + 4);  // CTA max of the plane updated, by step parity
  volatile int *s_pend = ctl + 6;  // plane whose CTA maximum waits in smax[sel ^ 1] (-1: none)

  const int tid = threadIdx.x;
  const int lx = tid & 31;
  const int ly = tid >> 5;
  // This CTA's segments: cta_first[b] .. cta_first[b + 1] - 1.  The end
  // and thread 0's pending plane live in shared memory (no loop registers).
  const int item_first = P.cta_first[blockIdx.x];
  if (item_first >= P.cta_first[blockIdx.x + 1]) return;
  auto item_end = [&]() { return *s_end; };
  const bool producer = tid == (TY - 1) * 32;
  auto produce = [&]() {
    int item = cur[0], k = cur[1], stg = cur[2];
    const HItem it = decode_hitem(item, P);
    issue_half<TY, EXT>(smem + stg * G::STAGE_B, &full[stg], it, k, M);
    if (++stg == S) stg = 0;
    if (++k >= it.z1 + kRadius) {
      ++item;
      if (item < item_end()) k = decode_hitem(item, P).z0 - kRadius;
    }
    cur[0] = item;
    cur[1] = k;
    cur[2] = stg;
  };
  if (tid == 0) {
    for (int s = 0; s < S; ++s) mbar_init(&full[s], 1);
    mbar_init(xchg, TY);
    mbar_fence_init();
    cur[0] = item_first;
    cur[1] = decode_hitem(item_first, P).z0 - kRadius;
    cur[2] = 0;
    *s_end = P.cta_first[blockIdx.x + 1];
    *s_pend = -1;
    smax[0] = smax[1] = 0u;
  }
  __syncthreads();
  if (producer) {
    tma_prefetch_desc(&M.cur_hi);
    tma_prefetch_desc(&M.prev_hi);
    tma_prefetch_desc(&M.arr);
    tma_prefetch_desc(&M.upd);
    // Prologue: S-1 steps; afterwards each step refills the stage freed by
    // the step before it.
    for (int a = 0; a < S - 1 && cur[0] < item_end(); ++a) produce();
  }

  const float sxy = P.inv_dxy, sxz = P.inv_dxz, syz = P.inv_dyz;
  const float sxx = P.inv_dxx, syy = P.inv_dyy, szz = P.inv_dzz;
  const bool halo_warp = ly < TY / 4;
  const int hr = ly * 4 + (lx >> 3);
  const int hxc = (lx & 7) < 4 ? (lx & 7) : G::TX + (lx & 7);
  const int hh = (hr + kRadius) * G::HX + hxc;
  const long plane = (long)sd.pitch * sd.sy;

  int stage = 0;
  uint32_t phase = 0, xphase = 0;
  int sel = 0;
  int abw = 0;  // shared A/B ring slot of the arriving plane (the plane 4 back is at abw + 1)
  bool bad = false;
  for (int item = item_first; item < item_end(); ++item) {
    const HItem it = decode_hitem(item, P);
    const int kbeg = it.z0 - kRadius;
    const int kend = it.z1 + kRadius;
    const int gx = it.x0 + lx;
    const int gy = it.y0 + ly;
    const bool valid = (gx >= sd.bord) && (gx < sd.sx - sd.bord) && (gy >= sd.bord) && (gy < sd.sy - sd.bord);
    const long oidx = (long)gy * sd.pitch + gx;
    const int ci = ly * G::TX + lx;
    const int hc = (ly + kRadius) * G::HX + (lx + kRadius);
    const int src_z = sd.src_z, cor_z = sd.cor_z;

    f2 Pr[9], Dx[9], Dy[9], A[9], B[9];

    for (int kb = kbeg; kb < kend; kb += 9) {
#pragma unroll
      for (int j = 0; j < 9; ++j) {
        const int k = kb + j;
        if (k >= kend) break;
        unsigned char *st = smem + stage * G::STAGE_B;
        bad |= !mbar_wait(&full[stage], phase, kWaitLimitNs);
        f2 *Hs = H32 + sel * G::HXY;
        {
          // Decode the arriving plane once per cell, two cells per thread
          // (one 64-bit load of two half2 cells, one 128-bit store of their
          // FP32 pairs).  The source cell then gains the step's source
          // (original/OpenMP/openmp_insertsource.c:7-13), added by the
          // thread that decoded it.
          const float inv = exp2i(-H.e_cur[k]);
          const uint2 *hv2 = reinterpret_cast<const uint2 *>(st);
          const unsigned *rv2 = reinterpret_cast<const unsigned *>(st + G::OFF_LO);
          float4 *Hs4 = reinterpret_cast<float4 *>(Hs);
#pragma unroll
          for (int c0 = 0; c0 < G::HXY / 2; c0 += NTH) {
            const int c2 = c0 + tid;
            if (c2 < G::HXY / 2) {
              const uint2 h = hv2[c2];
              const unsigned r = EXT ? rv2[c2] : 0u;
              const f2 a = decode<EXT>(h.x, (unsigned short)(r & 0xffffu), inv);
              const f2 b = decode<EXT>(h.y, (unsigned short)(r >> 16), inv);
              Hs4[c2] = make_float4(lo(a), hi(a), lo(b), hi(b));
            }
          }
          if (k == src_z) {
            // Halo-tile index of the source cell, if it lies in this tile.
            const int rx = sd.src_x - (it.x0 - kRadius), ry = sd.src_y - (it.y0 - kRadius);
            if (rx >= 0 && rx < G::HX && ry >= 0 && ry < G::HY) {
              const int src_c = ry * G::HX + rx;
              if (tid == (src_c >> 1) % NTH) Hs[src_c] = add2(Hs[src_c], splat(P.src));
            }
          }
        }
        // Every thread is past the previous step: its stage is free and the
        // CTA maximum of the plane it updated is complete.  Every thread
        // takes the same branch (a wait that gave up anywhere ends the CTA).
        if (__syncthreads_or(bad)) goto aborted;
        if (producer && cur[0] < item_end()) {
          fence_proxy_async_smem();
          produce();
        }
        if (tid == 0 && *s_pend >= 0) {
          const int pend_z = *s_pend;
          const unsigned v = smax[sel ^ 1];
          smax[sel ^ 1] = 0u;
          if (v) {
            atomicMax(&H.m_new[pend_z], v);
            // Beyond FP16's range: the scale bound was exceeded.
            if (!(__fmul_rn(__uint_as_float(v), exp2i(H.e_new[pend_z])) < 65504.0f)) atomicOr(P.err, 4u);
          }
        }
        const bool center = (k >= it.z0) && (k < it.z1);
        const bool upd = (k - kRadius >= it.z0);
        if (tid == 0) *s_pend = upd ? k - kRadius : -1;

        const f2 c = Hs[hc];
        f2 xa[4], xb[4], ya[4], yb[4];
#pragma unroll
        for (int o = 1; o <= 4; ++o) {
          xa[o - 1] = Hs[hc + o];
          xb[o - 1] = Hs[hc - o];
          ya[o - 1] = Hs[hc + o * G::HX];
          yb[o - 1] = Hs[hc - o * G::HX];
        }
        const f2 d1x = d1(xa[0], xb[0], xa[1], xb[1], xa[2], xb[2], xa[3], xb[3]);
        const f2 d1y = d1(ya[0], yb[0], ya[1], yb[1], ya[2], yb[2], ya[3], yb[3]);
        Pr[j] = c;
        Dx[j] = d1x;
        Dy[j] = d1y;
        f2 d2x, d2y;
        f2 *db = dbuf + sel * (TY * G::HX);
        if (center) {
          d2x = scale<ISO>(d2(c, xa[0], xb[0], xa[1], xb[1], xa[2], xb[2], xa[3], xb[3]), sxx);
          d2y = scale<ISO>(d2(c, ya[0], yb[0], ya[1], yb[1], ya[2], yb[2], ya[3], yb[3]), syy);
          db[ly * G::HX + lx + kRadius] = d1y;
          if (halo_warp) {
            f2 ha[4], hb[4];
#pragma unroll
            for (int o = 1; o <= 4; ++o) {
              ha[o - 1] = Hs[hh + o * G::HX];
              hb[o - 1] = Hs[hh - o * G::HX];
            }
            db[hr * G::HX + hxc] = d1(ha[0], hb[0], ha[1], hb[1], ha[2], hb[2], ha[3], hb[3]);
          }
        }
        __syncwarp();
        if (lx == 0) mbar_arrive(xchg);
        if (upd) {
          const int cs = (j + 5) % 9;
#define RP(o) Pr[(cs + (o)) % 9]
#define RX(o) Dx[(cs + (o)) % 9]
#define RY(o) Dy[(cs + (o)) % 9]
          const f2 d2z = scale<ISO>(d2(RP(0), RP(1), RP(8), RP(2), RP(7), RP(3), RP(6), RP(4), RP(5)), szz);
          const f2 dxz = scale<ISO>(d1(RX(1), RX(8), RX(2), RX(7), RX(3), RX(6), RX(4), RX(5)), sxz);
          const f2 dyz = scale<ISO>(d1(RY(1), RY(8), RY(2), RY(7), RY(3), RY(6), RY(4), RY(5)), syz);
#undef RP
#undef RX
#undef RY
          const float *cu = reinterpret_cast<const float *>(st + G::OFF_UPD);
          const float czz = cu[ci], cxz = cu[G::NT + ci], cyz = cu[2 * G::NT + ci];
          const float v2px = cu[3 * G::NT + ci], v2pz = cu[4 * G::NT + ci];
          const float v2sz = cu[5 * G::NT + ci], v2pn = cu[6 * G::NT + ci];
          f2 Ak, Bk;
          if constexpr (G::AB_SMEM) {
            const float4 ab = ABs[(abw == 4 ? 0 : abw + 1) * G::NT + ci];
            Ak = mk2(ab.x, ab.y);
            Bk = mk2(ab.z, ab.w);
          } else {
            Ak = A[cs];
            Bk = B[cs];
          }
          const f2 h1 = fma2(splat(cyz), dyz, fma2(splat(cxz), dxz, fma2(splat(czz), d2z, Ak)));
          const f2 h2 = sub2(add2(Bk, d2z), h1);
          const float h1p = lo(h1), h1q = hi(h1), h2p = lo(h2), h2q = hi(h2);
          const float t = __fmul_rn(v2pz, h1q);
          const float rhsp = __fmaf_rn(v2sz, __fsub_rn(h1p, h1q), __fmaf_rn(v2px, h2p, t));
          const float rhsq = __fmaf_rn(-v2sz, __fsub_rn(h2p, h2q), __fmaf_rn(v2pn, h2p, t));
          const int zc = k - kRadius;
          const unsigned phv = reinterpret_cast<const unsigned *>(st + G::OFF_PHI)[ci];
          unsigned short prv = 0;
          if constexpr (EXT) prv = reinterpret_cast<const unsigned short *>(st + G::OFF_PLO)[ly * G::HX + lx + kRadius];
          f2 old = decode<EXT>(phv, prv, exp2i(-H.e_prev[zc]));
          if (zc == cor_z) {
            if (gx == sd.cor_x && gy == sd.cor_y) old = add2(old, splat(P.cor));
          }
          const f2 curv = Pr[cs];
          const f2 nw = fma2(mk2(rhsp, rhsq), splat(P.dt2), sub2(add2(curv, curv), old));
          const float scl = exp2i(H.e_new[zc]);
          unsigned ohv;
          unsigned short orv;
          encode<EXT>(nw, scl, ohv, orv);
          if (valid) {
            H.out_hi[(long)zc * plane + oidx] = ohv;
            if constexpr (EXT) H.out_lo[(long)zc * plane + oidx] = orv;
          }
          // The warp's largest magnitude: the bits of non-negative floats
          // order like the floats, so one integer warp reduction finds it
          // (a NaN, above every finite value, reaches the range check).
          unsigned mb = 0u;
          if (valid) mb = max(__float_as_uint(fabsf(lo(nw))), __float_as_uint(fabsf(hi(nw))));
          mb = __reduce_max_sync(0xffffffffu, mb);
          if (lx == 0 && mb) atomicMax(&smax[sel], mb);
        }
        bad |= !mbar_wait(xchg, xphase, kWaitLimitNs);
        xphase ^= 1u;
        if (center) {
          const f2 *dr = db + ly * G::HX + lx + kRadius;
          const f2 dxy = scale<ISO>(d1(dr[1], dr[-1], dr[2], dr[-2], dr[3], dr[-3], dr[4], dr[-4]), sxy);
          const float *ca = reinterpret_cast<const float *>(st + G::OFF_ARR);
          const float cxx = ca[ci], cyy = ca[G::NT + ci], cxy = ca[2 * G::NT + ci];
          const f2 av = fma2(splat(cxy), dxy, fma2(splat(cyy), d2y, mul2(splat(cxx), d2x)));
          const f2 bv = add2(d2x, d2y);
          if constexpr (G::AB_SMEM) {
            ABs[abw * G::NT + ci] = make_float4(lo(av), hi(av), lo(bv), hi(bv));
          } else {
            A[j] = av;
            B[j] = bv;
          }
        }
        sel ^= 1;
        abw = abw == 4 ? 0 : abw + 1;
        if (++stage == S) {
          stage = 0;
          phase ^= 1u;
        }
      }
    }
  }
  // The last plane's CTA maximum.
  if (__syncthreads_or(bad)) goto aborted;
  if (tid == 0 && *s_pend >= 0) {
    const int pend_z = *s_pend;
    const unsigned v = smax[sel ^ 1];
    if (v) {
      atomicMax(&H.m_new[pend_z], v);
      if (!(__fmul_rn(__uint_as_float(v), exp2i(H.e_new[pend_z])) < 65504.0f)) atomicOr(P.err, 4u);
    }
  }
  return;
aborted:
  // A bounded wait gave up (every thread of the CTA arrives here together,
  // from a barrier).  Thread 0 waits, bounded, for the loads that may still
  // be in flight into this CTA's stages.
  if (tid == 0) {
    atomicOr(P.err, 1u);
    for (int a = 0; a < S; ++a) {
      const int s2 = (stage + a) % S;
      (void)mbar_wait(&full[s2], phase ^ uint32_t(stage + a >= S), kWaitLimitNs);
    }
  }
}

// The same step for a batch of shots (p.items, p.shots, hshots, hmaps): each
// item is a z-chunk of one tile column of one shot, with that shot's tensor
// maps, buffers and exponents.  It is a kernel of its own because folding
// the batched lookups into k_propagate_half, even behind compile-time
// switches, made the single-shot kernel 9-11% slower at 504^3.
template <int TY, int S, bool ISO, bool EXT>
__global__ void __launch_bounds__(kTileX *TY, 1)
    k_propagate_half_batch(const __grid_constant__ HalfParams H) {
  using G = GeoH<TY, EXT>;
  const PropParams &P = H.p;
  constexpr int NTH = kTileX * TY;
  extern __shared__ unsigned char smem_dyn[];
  unsigned char *smem = smem_dyn + ((128u - (smem_addr(smem_dyn) & 127u)) & 127u);
  unsigned char *tail = smem + S * G::STAGE_B;
  f2 *H32 = reinterpret_cast<f2 *>(tail + G::OFF_H32);
  f2 *dbuf = reinterpret_cast<f2 *>(tail + G::OFF_DB);
  float4 *ABs = reinterpret_cast<float4 *>(tail + G::OFF_AB);  // [5][NT] (AB_SMEM)
  uint64_t *full = reinterpret_cast<uint64_t *>(tail + G::OFF_BAR);
  uint64_t *xchg = full + S;
  int *ctl = reinterpret_cast<int *>(xchg + 1);
  int *cur = ctl;                                          // producer cursor: item, k, stage
  unsigned *smax = reinterpret_cast<unsigned *>(ctl + 4);  // CTA max of the plane updated, by step parity
  volatile int *s_pend = ctl + 6;  // plane whose CTA maximum waits in smax[sel ^ 1] (-1: none)
  volatile int *s_pend_shot = ctl + 7;  // and its shot
  HRec *rec = reinterpret_cast<HRec *>(ctl + 8);  // records of this CTA's current and next item

  const int tid = threadIdx.x;
  const int lx = tid & 31;
  const int ly = tid >> 5;
  // This CTA's items: b, b + grid, ... below nitems.
  const int item_first = blockIdx.x;
  if (item_first >= P.nitems) return;
  auto item_end = [&]() { return P.nitems; };
  auto item_step = [&]() { return (int)gridDim.x; };
  // Tensor maps of an item's shot, for the buffer holding its current field.
  auto maps_of = [&](const BItem &it) -> const HalfMaps & { return H.hmaps[it.shot].m[P.parity]; };
  // Thread 0 fills the record of an item.  The record of a CTA's
  // first item is filled before the start barrier; that of its next item
  // once every thread has passed the first plane of the current one (so no
  // thread still reads the previous item's record, which it replaces).
  auto fill_rec = [&](HRec *r, int item) {
    const int shot = P.items[item].x;
    const ShotDesc &d = P.shots[shot];
    const HalfShot &h = H.hshots[shot];
    r->e_cur = h.E + (H.ecur % 3) * d.sz;
    r->e_new = h.E + ((H.ecur + 1) % 3) * d.sz;
    r->e_prev = h.E + ((H.ecur + 2) % 3) * d.sz;
    r->out_hi = h.hi[1 - P.parity];
    r->out_lo = h.lo[1 - P.parity];
    r->plane = (long)d.pitch * d.sy;
    r->src_z = d.src_z;
    r->cor_z = d.cor_z;
  };
  const bool producer = tid == (TY - 1) * 32;
  auto produce = [&]() {
    int item = cur[0], k = cur[1], stg = cur[2];
    const BItem it = decode_bitem(item, P);
    issue_half<TY, EXT>(smem + stg * G::STAGE_B, &full[stg], it, k, maps_of(it));
    if (++stg == S) stg = 0;
    if (++k >= it.z1 + kRadius) {
      item += item_step();
      if (item < item_end()) {
        k = decode_bitem(item, P).z0 - kRadius;
        // The shots' tensor maps live in global memory: fetch those of the
        // item after this one into the descriptor cache, an item ahead.
        if (item + item_step() < item_end()) prefetch_maps<EXT>(maps_of(decode_bitem(item + item_step(), P)));
      }
    }
    cur[0] = item;
    cur[1] = k;
    cur[2] = stg;
  };
  if (tid == 0) {
    for (int s = 0; s < S; ++s) mbar_init(&full[s], 1);
    mbar_init(xchg, TY);
    mbar_fence_init();
    cur[0] = item_first;
    cur[1] = decode_bitem(item_first, P).z0 - kRadius;
    cur[2] = 0;
    *s_pend = -1;
    *s_pend_shot = 0;
    fill_rec(rec, item_first);
    smax[0] = smax[1] = 0u;
  }
  __syncthreads();
  if (producer) {
    prefetch_maps<EXT>(maps_of(decode_bitem(item_first, P)));
    if (item_first + item_step() < item_end()) prefetch_maps<EXT>(maps_of(decode_bitem(item_first + item_step(), P)));
    // Prologue: S-1 steps; afterwards each step refills the stage freed by
    // the step before it.
    for (int a = 0; a < S - 1 && cur[0] < item_end(); ++a) produce();
  }
  // Exponents and maxima of the new field of a shot: its buffers, where the
  // current field is in buffer parity and exponent slot ecur.
  auto e_new_of = [&](int shot) -> const int * {
    return H.hshots[shot].E + ((H.ecur + 1) % 3) * P.shots[shot].sz;
  };
  auto m_new_of = [&](int shot) -> unsigned * { return H.hshots[shot].Mx + (1 - P.parity) * P.shots[shot].sz; };

  const float sxy = P.inv_dxy, sxz = P.inv_dxz, syz = P.inv_dyz;
  const float sxx = P.inv_dxx, syy = P.inv_dyy, szz = P.inv_dzz;
  const bool halo_warp = ly < TY / 4;
  const int hr = ly * 4 + (lx >> 3);
  const int hxc = (lx & 7) < 4 ? (lx & 7) : G::TX + (lx & 7);
  const int hh = (hr + kRadius) * G::HX + hxc;

  int stage = 0;
  uint32_t phase = 0, xphase = 0;
  int sel = 0;
  int abw = 0;  // shared A/B ring slot of the arriving plane (the plane 4 back is at abw + 1)
  bool bad = false;
  int nloc = 0;  // items this CTA has finished (record slot nloc & 1)
  for (int item = item_first; item < item_end(); item += item_step(), ++nloc) {
    const BItem it = decode_bitem(item, P);
    // The item's shot: its descriptor (read where needed) and its record,
    // read at each use.
    const ShotDesc *sdp = P.shots + it.shot;
    const volatile HRec *vr = rec + (nloc & 1);
    const int kbeg = it.z0 - kRadius;
    const int kend = it.z1 + kRadius;
    const int gx = it.x0 + lx;
    const int gy = it.y0 + ly;
    bool valid;
    long oidx;
    {
      const ShotDesc &sd = *sdp;
      valid = (gx >= sd.bord) && (gx < sd.sx - sd.bord) && (gy >= sd.bord) && (gy < sd.sy - sd.bord);
      oidx = (long)gy * sd.pitch + gx;
    }
    const int ci = ly * G::TX + lx;
    const int hc = (ly + kRadius) * G::HX + (lx + kRadius);

    f2 Pr[9], Dx[9], Dy[9], A[9], B[9];

    for (int kb = kbeg; kb < kend; kb += 9) {
#pragma unroll
      for (int j = 0; j < 9; ++j) {
        const int k = kb + j;
        if (k >= kend) break;
        unsigned char *st = smem + stage * G::STAGE_B;
        bad |= !mbar_wait(&full[stage], phase, kWaitLimitNs);
        f2 *Hs = H32 + sel * G::HXY;
        {
          // Decode the arriving plane once per cell, two cells per thread
          // (one 64-bit load of two half2 cells, one 128-bit store of their
          // FP32 pairs).  The source cell then gains the step's source
          // (original/OpenMP/openmp_insertsource.c:7-13), added by the
          // thread that decoded it.
          const float inv = exp2i(-vr->e_cur[k]);
          const uint2 *hv2 = reinterpret_cast<const uint2 *>(st);
          const unsigned *rv2 = reinterpret_cast<const unsigned *>(st + G::OFF_LO);
          float4 *Hs4 = reinterpret_cast<float4 *>(Hs);
#pragma unroll
          for (int c0 = 0; c0 < G::HXY / 2; c0 += NTH) {
            const int c2 = c0 + tid;
            if (c2 < G::HXY / 2) {
              const uint2 h = hv2[c2];
              const unsigned r = EXT ? rv2[c2] : 0u;
              const f2 a = decode<EXT>(h.x, (unsigned short)(r & 0xffffu), inv);
              const f2 b = decode<EXT>(h.y, (unsigned short)(r >> 16), inv);
              Hs4[c2] = make_float4(lo(a), hi(a), lo(b), hi(b));
            }
          }
          if (k == vr->src_z) {
            // Halo-tile index of the source cell, if it lies in this tile.
            const int rx = sdp->src_x - (it.x0 - kRadius), ry = sdp->src_y - (it.y0 - kRadius);
            if (rx >= 0 && rx < G::HX && ry >= 0 && ry < G::HY) {
              const int src_c = ry * G::HX + rx;
              if (tid == (src_c >> 1) % NTH) Hs[src_c] = add2(Hs[src_c], splat(P.src));
            }
          }
        }
        // Every thread is past the previous step: its stage is free and the
        // CTA maximum of the plane it updated is complete.  Every thread
        // takes the same branch (a wait that gave up anywhere ends the CTA).
        if (__syncthreads_or(bad)) goto aborted;
        if (tid == 0 && k == kbeg && item + item_step() < item_end()) fill_rec(rec + ((nloc + 1) & 1), item + item_step());
        if (producer && cur[0] < item_end()) {
          fence_proxy_async_smem();
          produce();
        }
        if (tid == 0 && *s_pend >= 0) {
          const int pend_z = *s_pend, ps = *s_pend_shot;
          const unsigned v = smax[sel ^ 1];
          smax[sel ^ 1] = 0u;
          if (v) {
            atomicMax(&m_new_of(ps)[pend_z], v);
            // Beyond FP16's range: the scale bound was exceeded.
            if (!(__fmul_rn(__uint_as_float(v), exp2i(e_new_of(ps)[pend_z])) < 65504.0f)) atomicOr(P.err, 4u);
          }
        }
        const bool center = (k >= it.z0) && (k < it.z1);
        const bool upd = (k - kRadius >= it.z0);
        if (tid == 0) {
          *s_pend = upd ? k - kRadius : -1;
          *s_pend_shot = it.shot;
        }

        const f2 c = Hs[hc];
        f2 xa[4], xb[4], ya[4], yb[4];
#pragma unroll
        for (int o = 1; o <= 4; ++o) {
          xa[o - 1] = Hs[hc + o];
          xb[o - 1] = Hs[hc - o];
          ya[o - 1] = Hs[hc + o * G::HX];
          yb[o - 1] = Hs[hc - o * G::HX];
        }
        const f2 d1x = d1(xa[0], xb[0], xa[1], xb[1], xa[2], xb[2], xa[3], xb[3]);
        const f2 d1y = d1(ya[0], yb[0], ya[1], yb[1], ya[2], yb[2], ya[3], yb[3]);
        Pr[j] = c;
        Dx[j] = d1x;
        Dy[j] = d1y;
        f2 d2x, d2y;
        f2 *db = dbuf + sel * (TY * G::HX);
        if (center) {
          d2x = scale<ISO>(d2(c, xa[0], xb[0], xa[1], xb[1], xa[2], xb[2], xa[3], xb[3]), sxx);
          d2y = scale<ISO>(d2(c, ya[0], yb[0], ya[1], yb[1], ya[2], yb[2], ya[3], yb[3]), syy);
          db[ly * G::HX + lx + kRadius] = d1y;
          if (halo_warp) {
            f2 ha[4], hb[4];
#pragma unroll
            for (int o = 1; o <= 4; ++o) {
              ha[o - 1] = Hs[hh + o * G::HX];
              hb[o - 1] = Hs[hh - o * G::HX];
            }
            db[hr * G::HX + hxc] = d1(ha[0], hb[0], ha[1], hb[1], ha[2], hb[2], ha[3], hb[3]);
          }
        }
        __syncwarp();
        if (lx == 0) mbar_arrive(xchg);
        if (upd) {
          const int cs = (j + 5) % 9;
#define RP(o) Pr[(cs + (o)) % 9]
#define RX(o) Dx[(cs + (o)) % 9]
#define RY(o) Dy[(cs + (o)) % 9]
          const f2 d2z = scale<ISO>(d2(RP(0), RP(1), RP(8), RP(2), RP(7), RP(3), RP(6), RP(4), RP(5)), szz);
          const f2 dxz = scale<ISO>(d1(RX(1), RX(8), RX(2), RX(7), RX(3), RX(6), RX(4), RX(5)), sxz);
          const f2 dyz = scale<ISO>(d1(RY(1), RY(8), RY(2), RY(7), RY(3), RY(6), RY(4), RY(5)), syz);
#undef RP
#undef RX
#undef RY
          const float *cu = reinterpret_cast<const float *>(st + G::OFF_UPD);
          const float czz = cu[ci], cxz = cu[G::NT + ci], cyz = cu[2 * G::NT + ci];
          const float v2px = cu[3 * G::NT + ci], v2pz = cu[4 * G::NT + ci];
          const float v2sz = cu[5 * G::NT + ci], v2pn = cu[6 * G::NT + ci];
          f2 Ak, Bk;
          if constexpr (G::AB_SMEM) {
            const float4 ab = ABs[(abw == 4 ? 0 : abw + 1) * G::NT + ci];
            Ak = mk2(ab.x, ab.y);
            Bk = mk2(ab.z, ab.w);
          } else {
            Ak = A[cs];
            Bk = B[cs];
          }
          const f2 h1 = fma2(splat(cyz), dyz, fma2(splat(cxz), dxz, fma2(splat(czz), d2z, Ak)));
          const f2 h2 = sub2(add2(Bk, d2z), h1);
          const float h1p = lo(h1), h1q = hi(h1), h2p = lo(h2), h2q = hi(h2);
          const float t = __fmul_rn(v2pz, h1q);
          const float rhsp = __fmaf_rn(v2sz, __fsub_rn(h1p, h1q), __fmaf_rn(v2px, h2p, t));
          const float rhsq = __fmaf_rn(-v2sz, __fsub_rn(h2p, h2q), __fmaf_rn(v2pn, h2p, t));
          const int zc = k - kRadius;
          const unsigned phv = reinterpret_cast<const unsigned *>(st + G::OFF_PHI)[ci];
          unsigned short prv = 0;
          if constexpr (EXT) prv = reinterpret_cast<const unsigned short *>(st + G::OFF_PLO)[ly * G::HX + lx + kRadius];
          f2 old = decode<EXT>(phv, prv, exp2i(-vr->e_prev[zc]));
          if (zc == vr->cor_z) {
            if (gx == sdp->cor_x && gy == sdp->cor_y) old = add2(old, splat(P.cor));
          }
          const f2 curv = Pr[cs];
          const f2 nw = fma2(mk2(rhsp, rhsq), splat(P.dt2), sub2(add2(curv, curv), old));
          const float scl = exp2i(vr->e_new[zc]);
          unsigned ohv;
          unsigned short orv;
          encode<EXT>(nw, scl, ohv, orv);
          if (valid) {
            const long o = (long)zc * vr->plane + oidx;
            vr->out_hi[o] = ohv;
            if constexpr (EXT) vr->out_lo[o] = orv;
          }
          // The warp's largest magnitude: the bits of non-negative floats
          // order like the floats, so one integer warp reduction finds it
          // (a NaN, above every finite value, reaches the range check).
          unsigned mb = 0u;
          if (valid) mb = max(__float_as_uint(fabsf(lo(nw))), __float_as_uint(fabsf(hi(nw))));
          mb = __reduce_max_sync(0xffffffffu, mb);
          if (lx == 0 && mb) atomicMax(&smax[sel], mb);
        }
        bad |= !mbar_wait(xchg, xphase, kWaitLimitNs);
        xphase ^= 1u;
        if (center) {
          const f2 *dr = db + ly * G::HX + lx + kRadius;
          const f2 dxy = scale<ISO>(d1(dr[1], dr[-1], dr[2], dr[-2], dr[3], dr[-3], dr[4], dr[-4]), sxy);
          const float *ca = reinterpret_cast<const float *>(st + G::OFF_ARR);
          const float cxx = ca[ci], cyy = ca[G::NT + ci], cxy = ca[2 * G::NT + ci];
          const f2 av = fma2(splat(cxy), dxy, fma2(splat(cyy), d2y, mul2(splat(cxx), d2x)));
          const f2 bv = add2(d2x, d2y);
          if constexpr (G::AB_SMEM) {
            ABs[abw * G::NT + ci] = make_float4(lo(av), hi(av), lo(bv), hi(bv));
          } else {
            A[j] = av;
            B[j] = bv;
          }
        }
        sel ^= 1;
        abw = abw == 4 ? 0 : abw + 1;
        if (++stage == S) {
          stage = 0;
          phase ^= 1u;
        }
      }
    }
  }
  // The last plane's CTA maximum.
  if (__syncthreads_or(bad)) goto aborted;
  if (tid == 0 && *s_pend >= 0) {
    const int pend_z = *s_pend, ps = *s_pend_shot;
    const unsigned v = smax[sel ^ 1];
    if (v) {
      atomicMax(&m_new_of(ps)[pend_z], v);
      if (!(__fmul_rn(__uint_as_float(v), exp2i(e_new_of(ps)[pend_z])) < 65504.0f)) atomicOr(P.err, 4u);
    }
  }
  return;
aborted:
  // A bounded wait gave up (every thread of the CTA arrives here together,
  // from a barrier).  Thread 0 waits, bounded, for the loads that may still
  // be in flight into this CTA's stages.
  if (tid == 0) {
    atomicOr(P.err, 1u);
    for (int a = 0; a < S; ++a) {
      const int s2 = (stage + a) % S;
      (void)mbar_wait(&full[s2], phase ^ uint32_t(stage + a >= S), kWaitLimitNs);
    }
  }
}

// Before each step: the exponent of every plane of the new field (its
// largest possible magnitude: 4 x the current field's largest magnitude
// within 4 planes, plus the previous field's at that plane, plus the sources
// near the source plane), and the previous field's maxima, consumed here, are
// cleared for the new field's.
__global__ void k_half_scales(const unsigned *__restrict__ m_cur, unsigned *__restrict__ m_prev, int *__restrict__ e_new,
                              int sz, int src_z, float src_abs) {
  const int z = blockIdx.x * blockDim.x + threadIdx.x;
  if (z >= sz) return;
  float b = 0.0f;
  for (int dz = -kRadius; dz <= kRadius; ++dz)
    if (z + dz >= 0 && z + dz < sz) b = fmaxf(b, __uint_as_float(m_cur[z + dz]));
  b = 4.0f * b + __uint_as_float(m_prev[z]);
  if (abs(z - src_z) <= kRadius) b += 4.0f * src_abs;
  int e = 0;
  if (b > 0.0f) {
    int ex;
    frexpf(b, &ex);  // b < 2^ex
    e = min(max(14 - ex, -100), 100);
  }
  e_new[z] = e;
  m_prev[z] = 0u;
}

// Plane z (= blockIdx.x) of float (p, q) volumes -> stored form, the scale
// from the plane's largest magnitude.
template <bool EXT>
__global__ void k_half_encode_plane(const float *__restrict__ p, const float *__restrict__ q, unsigned *hv,
                                    unsigned short *rv, int *e, unsigned *m, int sx, int sy, int pitch) {
  const int z = blockIdx.x;
  const size_t base = (size_t)z * sx * sy;
  __shared__ float red[32];
  float mx = 0.0f;
  for (int i = threadIdx.x; i < sx * sy; i += blockDim.x) {
    const float a = p ? p[base + i] : 0.f, b = q ? q[base + i] : 0.f;
    mx = fmaxf(mx, fmaxf(fabsf(a), fabsf(b)));
  }
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x < 32) {
    mx = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0f;
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (threadIdx.x == 0) red[0] = mx;
  }
  __syncthreads();
  mx = red[0];
  int ez = 0;
  if (mx > 0.0f) {
    int ex;
    frexpf(mx, &ex);
    ez = min(max(14 - ex, -100), 100);
  }
  if (threadIdx.x == 0) {
    e[z] = ez;
    m[z] = __float_as_uint(mx);
  }
  const float sc = exp2i(ez);
  for (int i = threadIdx.x; i < sx * sy; i += blockDim.x) {
    const int x = i % sx, y = i / sx;
    unsigned h;
    unsigned short l;
    encode<EXT>(mk2(p ? p[base + i] : 0.f, q ? q[base + i] : 0.f), sc, h, l);
    const size_t o = ((size_t)z * sy + y) * pitch + x;
    hv[o] = h;
    if (EXT) rv[o] = l;
  }
}

// One component of a stored volume -> float volume (unpitched).
template <bool EXT>
__global__ void k_half_decode(const unsigned *__restrict__ hv, const unsigned short *__restrict__ rv,
                              const int *__restrict__ e, float *__restrict__ out, int comp, int sx, int sy, int sz,
                              int pitch) {
  const size_t n = (size_t)sx * sy * sz;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t x = i % sx, yz = i / sx, z = yz / sy;
    const size_t o = yz * pitch + x;
    const f2 v = decode<EXT>(hv[o], EXT ? rv[o] : (unsigned short)0, exp2i(-e[z]));
    out[i] = comp ? hi(v) : lo(v);
  }
}

// ---- host side ---------------------------------------------------------------

#define FLT_HALF_SHAPES(X) X(12, 4) X(12, 5) X(12, 6) X(8, 6) X(16, 4) X(16, 5)

// Dynamic shared-memory limit of a kernel shape, single-shot or batched
// (once; outside any stream capture before a captured launch).
template <int TY, int S, bool EXT, bool BATCH>
static cudaError_t prepare_half_t() {
  constexpr int smem = (int)smem_bytes_half<TY, S, EXT>();
  static bool ready = false;
  if (!ready) {
    const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e;
    if constexpr (BATCH) {
      e = cudaFuncSetAttribute(k_propagate_half_batch<TY, S, true, EXT>, a, smem);
      if (e == cudaSuccess) e = cudaFuncSetAttribute(k_propagate_half_batch<TY, S, false, EXT>, a, smem);
    } else {
      e = cudaFuncSetAttribute(k_propagate_half<TY, S, true, EXT>, a, smem);
      if (e == cudaSuccess) e = cudaFuncSetAttribute(k_propagate_half<TY, S, false, EXT>, a, smem);
    }
    if (e != cudaSuccess) return e;
    ready = true;
  }
  return cudaSuccess;
}

template <int TY, int S, bool EXT>
static cudaError_t launch_half_b(const HalfLaunch &L, cudaStream_t s) {
  constexpr size_t smem = smem_bytes_half<TY, S, EXT>();
  const bool iso = L.h.p.iso;
  if (L.batch) {
    const cudaError_t e = prepare_half_t<TY, S, EXT, true>();
    if (e != cudaSuccess) return e;
    auto kern = iso ? k_propagate_half_batch<TY, S, true, EXT> : k_propagate_half_batch<TY, S, false, EXT>;
    kern<<<L.grid, kTileX * TY, smem, s>>>(L.h);
  } else {
    const cudaError_t e = prepare_half_t<TY, S, EXT, false>();
    if (e != cudaSuccess) return e;
    auto kern = iso ? k_propagate_half<TY, S, true, EXT> : k_propagate_half<TY, S, false, EXT>;
    kern<<<L.grid, kTileX * TY, smem, s>>>(L.m, L.h);
  }
  return cudaGetLastError();
}

bool propagate_half_supported(int tile_rows, int stages) {
#define X(a, b) \
  if (tile_rows == a && stages == b) return true;
  FLT_HALF_SHAPES(X)
#undef X
  return false;
}

cudaError_t propagate_half_launch(const HalfLaunch &L, bool ext, cudaStream_t s) {
  // The work description the chosen kernel reads must be present.
  if (L.batch ? (!L.h.p.items || !L.h.p.shots || !L.h.hshots || !L.h.hmaps)
              : (!L.h.p.seg || !L.h.p.cta_first || !L.h.out_hi || !L.h.e_cur))
    return cudaErrorInvalidValue;
#define X(a, b)                          \
  if (L.tile_rows == a && L.stages == b) \
    return ext ? launch_half_b<a, b, true>(L, s) : launch_half_b<a, b, false>(L, s);
  FLT_HALF_SHAPES(X)
#undef X
  return cudaErrorInvalidValue;
}

cudaError_t propagate_half_prepare(int tile_rows, int stages, bool ext, bool batch) {
#define X(a, b)                                                                                  \
  if (tile_rows == a && stages == b)                                                             \
    return ext ? (batch ? prepare_half_t<a, b, true, true>() : prepare_half_t<a, b, true, false>()) \
               : (batch ? prepare_half_t<a, b, false, true>() : prepare_half_t<a, b, false, false>());
  FLT_HALF_SHAPES(X)
#undef X
  return cudaErrorInvalidValue;
}

// Resident CTAs per SM of a shape (registers and shared memory decide:
// the 8-row shapes use over 128 registers a thread, so one 256-thread CTA
// per SM); 0 if the shape is not built or the query fails.
int propagate_half_ctas_per_sm(int tile_rows, int stages, bool ext, bool batch) {
  int n = 0;
#define X(a, b)                                                                                                \
  if (tile_rows == a && stages == b) {                                                                         \
    const int smem = (int)(ext ? smem_bytes_half<a, b, true>() : smem_bytes_half<a, b, false>());              \
    cudaError_t e = ext ? (batch ? prepare_half_t<a, b, true, true>() : prepare_half_t<a, b, true, false>())    \
                        : (batch ? prepare_half_t<a, b, false, true>() : prepare_half_t<a, b, false, false>()); \
    if (e == cudaSuccess) {                                                                                    \
      const void *k = ext ? (batch ? (const void *)k_propagate_half_batch<a, b, true, true>                    \
                                   : (const void *)k_propagate_half<a, b, true, true>)                         \
                          : (batch ? (const void *)k_propagate_half_batch<a, b, true, false>                   \
                                   : (const void *)k_propagate_half<a, b, true, false>);                       \
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, kTileX * a, smem);                              \
    }                                                                                                          \
    if (e != cudaSuccess) {                                                                                    \
      cudaGetLastError();                                                                                      \
      n = 0;                                                                                                   \
    }                                                                                                          \
    return n;                                                                                                  \
  }
  FLT_HALF_SHAPES(X)
#undef X
  return 0;
}

cudaError_t half_scales(const unsigned *m_cur, unsigned *m_prev, int *e_new, int sz, int src_z, float src_abs,
                        cudaStream_t s) {
  k_half_scales<<<(sz + 127) / 128, 128, 0, s>>>(m_cur, m_prev, e_new, sz, src_z, src_abs);
  return cudaGetLastError();
}

// The same for every running shot of a batch (block i: shot order[i]); the
// current field is in buffer c and uses exponent slot ecur.
__global__ void k_half_scales_batch(const HalfShot *__restrict__ hs, const ShotDesc *__restrict__ sd,
                                    const int *__restrict__ order, int c, int ecur, float src_abs) {
  const int shot = order[blockIdx.x];
  const int sz = sd[shot].sz, src_z = sd[shot].src_z;
  const unsigned *m_cur = hs[shot].Mx + c * sz;
  unsigned *m_prev = hs[shot].Mx + (1 - c) * sz;
  int *e_new = hs[shot].E + ((ecur + 1) % 3) * sz;
  for (int z = threadIdx.x; z < sz; z += blockDim.x) {
    float b = 0.0f;
    for (int dz = -kRadius; dz <= kRadius; ++dz)
      if (z + dz >= 0 && z + dz < sz) b = fmaxf(b, __uint_as_float(m_cur[z + dz]));
    b = 4.0f * b + __uint_as_float(m_prev[z]);
    if (abs(z - src_z) <= kRadius) b += 4.0f * src_abs;
    int e = 0;
    if (b > 0.0f) {
      int ex;
      frexpf(b, &ex);
      e = min(max(14 - ex, -100), 100);
    }
    e_new[z] = e;
    m_prev[z] = 0u;
  }
}

cudaError_t half_scales_batch(const HalfShot *hs, const ShotDesc *sd, const int *order, int active, int c, int ecur,
                              float src_abs, cudaStream_t s) {
  k_half_scales_batch<<<active, 256, 0, s>>>(hs, sd, order, c, ecur, src_abs);
  return cudaGetLastError();
}

cudaError_t half_encode(const float *p, const float *q, unsigned *hv, unsigned short *rv, int *e, unsigned *m, int sx,
                        int sy, int sz, int pitch, bool ext, cudaStream_t s) {
  if (ext)
    k_half_encode_plane<true><<<sz, 256, 0, s>>>(p, q, hv, rv, e, m, sx, sy, pitch);
  else
    k_half_encode_plane<false><<<sz, 256, 0, s>>>(p, q, hv, rv, e, m, sx, sy, pitch);
  return cudaGetLastError();
}

cudaError_t half_decode(const unsigned *hv, const unsigned short *rv, const int *e, float *out, int comp, int sx,
                        int sy, int sz, int pitch, bool ext, int grid, cudaStream_t s) {
  if (ext)
    k_half_decode<true><<<grid, 256, 0, s>>>(hv, rv, e, out, comp, sx, sy, sz, pitch);
  else
    k_half_decode<false><<<grid, 256, 0, s>>>(hv, rv, e, out, comp, sx, sy, sz, pitch);
  return cudaGetLastError();
}

}  // namespace flt
