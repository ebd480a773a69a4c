// Plain FP32 Fletcher TTI step for sm_103a.
//
// Computes, for every cell of [bord, s-bord)^3, the coupled p/q update of
// original/sample.h:32-89 (Der2 / DerCross of original/derivatives.h:37-68,
// weighted by the ch1d** and v2** coefficients of original/precomp.h), with
// the source of original/OpenMP/openmp_insertsource.c:7-13 fused in.
//
// Structure (one CTA per SM, persistent):
//  * a work item is a 32 x TY column tile of one z-chunk; the CTA streams
//    its planes k = z0-4 .. z1+3 in z;
//  * thread 0 issues TMA loads S-1 planes ahead into a ring of shared-memory
//    stages: the (p,q) halo tile of plane k (box 40 x (TY+8)), the three
//    in-plane coefficients of plane k, and the seven other coefficients and
//    the previous (p,q) of plane k-4, which is updated at this step;
//  * each thread owns one (x, y) column.  When plane k arrives it reads its
//    9-point x and y neighbourhoods from shared memory and forms Der2x,
//    Der2y and the first derivatives D1x, D1y; DerCross xy is D1x applied to
//    D1y (exchanged through shared memory, including the 4-column x halo);
//    DerCross xz and yz are the z first derivative of the D1x / D1y values,
//    which each thread keeps for 9 planes in registers, as it keeps p and q
//    for Der2z;
//  * both fields travel as one 64-bit (p, q) pair and are updated with the
//    packed .f32x2 add/mul/fma instructions;
//  * plane k-4 is completed at step k and written with coalesced 64-bit
//    stores into the previous-field buffer (in place).
//
// Media-table layout (template parameter MT): instead of the ten coefficient
// planes a stage holds the one-byte medium ids of planes k and k-4 and the
// four velocity terms of plane k-4; the six angle terms come from a table
// of at most 256 media loaded into shared memory once per launch.  The
// floats read are the same as in the plane layout, so results are
// bit-identical; the stream drops from 64 to 41 bytes per cell.
//
// DerCross(p, a, b) equals D1_b(D1_a(p)) exactly in real arithmetic because
// its weights are the products L_i L_j of the first-derivative weights
// (original/derivatives.h:13-31); the FP32 rounding differs from the
// reference's grouped sum, which the parity tolerance covers.
#include "device_util.cuh"
#include "fletcher_internal.h"
#include "propagate_fp32_pipe.cuh"
#include "stencil_common.cuh"

namespace flt {

// D1D1: the Der1-Der1 numerics.  HOOK: the fault-injection variant (waits
// limited to P.wait_ns, CTA 0 skipping the loads of step P.stall_step),
// launched only when a test injects a stall.  MT: the media-table layout of
// the coefficients.
template <int TY, int S, bool ISO, int MODE, int MINB, bool D1D1 = false, bool HOOK = false, bool MT = false>
__global__ void __launch_bounds__(kTileX *TY, MINB)
    k_propagate_fp32(const __grid_constant__ SingleMaps SM, const __grid_constant__ PropParams P) {
  constexpr bool BATCH = MODE == kItemsBatch;
  static_assert(!D1D1 || (!ISO && !BATCH), "the Der1-Der1 numerics scale every derivative, single shot only");
  static_assert(!MT || (!BATCH && !HOOK && !D1D1), "the media-table layout runs single-shot plain steps");
  using G = Geo<TY, D1D1, MT>;
  extern __shared__ unsigned char smem_dyn[];
  // Align in the shared window (pointer arithmetic on the shared array keeps
  // every access below a shared-memory access).
  unsigned char *smem = smem_dyn + ((128u - (smem_addr(smem_dyn) & 127u)) & 127u);
  f2 *dbuf = reinterpret_cast<f2 *>(smem + S * G::STAGE_B);
  float4 *ABs = reinterpret_cast<float4 *>(smem + S * G::STAGE_B + G::DBUF_B);  // [5][NT] (AB_SMEM)
  f2 *Cs = reinterpret_cast<f2 *>(ABs + kABSlots * G::NT);  // [kABSlots][NT] (Der1-Der1 numerics: ch1dxy * pxy)
  float *s_med = reinterpret_cast<float *>(smem + S * G::STAGE_B + G::DBUF_B + G::AB_B);  // [6][256] (MT)
  uint64_t *full = reinterpret_cast<uint64_t *>(smem + S * G::STAGE_B + G::DBUF_B + G::AB_B + G::TAB_B);
  uint64_t *xchg = full + S;  // D1y rows written (one arrival per warp)
  int *s_abort = reinterpret_cast<int *>(xchg + 1);

  const int tid = threadIdx.x;
  const int lx = tid & 31;
  const int ly = tid >> 5;

  // This CTA's items.  A segment run's end lives in shared memory (read once
  // per item), so the loop keeps no register for it.
  const ItemRange R = item_range<MODE>(P);
  if (R.first >= R.end) return;
  volatile int *s_end = s_abort + 1;
  int *s_issued = s_abort + 2;  // fault-injection variant: steps this CTA has issued
  auto item_end = [&]() { return MODE != kItemsTiles ? *s_end : P.nitems; };
  auto item_step = [&]() { return MODE != kItemsTiles ? 1 : (int)gridDim.x; };
  // The producer is lane 0 of the last warp (warps 0 .. TY/4-1 carry the
  // halo-column work).  Its cursor, in shared memory, is the next step to load.
  const bool producer = tid == (TY - 1) * 32;
  auto maps_of = [&](const Item &it) {
    StepMaps m;
    if constexpr (BATCH) {
      const ShotMaps *sm = P.maps + it.shot;
      m.cur = &sm->halo[P.parity];
      m.prev = &sm->pt[P.parity ^ 1];
      m.arr = &sm->arr;
      m.upd = &sm->upd;
    } else {
      m.cur = &SM.cur_halo;
      m.prev = &SM.prev_pt;
      m.arr = &SM.arr;
      m.upd = &SM.upd;
    }
    m.ids = &SM.ids;
    m.vel = &SM.vel;
    return m;
  };
  Cursor *cur = reinterpret_cast<Cursor *>(s_abort + 4);
  // Issues the cursor's step into its stage and advances the cursor.  (Test
  // hook: CTA 0 skips the loads of its P.stall_step-th step, so that the
  // waits for that stage give up and the launch reports a timeout.)
  auto produce = [&]() {
    Cursor c = *cur;
    if constexpr (HOOK) {
      if (*s_issued != P.stall_step || blockIdx.x != 0)
        issue_step<TY, MT>(smem + c.stage * G::STAGE_B, &full[c.stage], c.it, c.k, maps_of(c.it));
      ++*s_issued;
    } else {
      issue_step<TY, MT>(smem + c.stage * G::STAGE_B, &full[c.stage], c.it, c.k, maps_of(c.it));
    }
    if (++c.stage == S) c.stage = 0;
    if (++c.k >= c.it.z1 + kLag) {
      c.item += item_step();
      if (c.item < item_end()) {
        c.it = decode_item<TY, MODE>(c.item, P);
        c.k = c.it.z0 - kRadius;
        if constexpr (BATCH) {
          // Batched shots keep their tensor maps in global memory: fetch
          // those of the item after this one into the descriptor cache now,
          // an item ahead of their first use.
          if (c.item + 1 < item_end()) {
            const StepMaps m = maps_of(decode_item<TY, MODE>(c.item + 1, P));
            tma_prefetch_desc(m.cur);
            tma_prefetch_desc(m.prev);
            tma_prefetch_desc(m.arr);
            tma_prefetch_desc(m.upd);
          }
        }
      }
    }
    *cur = c;
  };
  if (tid == 0) {
    for (int s = 0; s < S; ++s) mbar_init(&full[s], 1);
    mbar_init(xchg, TY);
    mbar_fence_init();
    *s_abort = 0;
    *s_issued = 0;
    if constexpr (MODE != kItemsTiles) *s_end = R.end;
  }
  if constexpr (MT) {
    for (int i = tid; i < kAngleCoef * kMediaMax; i += kTileX * TY) s_med[i] = P.media[i];
  }
  if (producer) {
    Cursor c;
    c.it = decode_item<TY, MODE>(R.first, P);
    c.item = R.first;
    c.k = c.it.z0 - kRadius;
    c.stage = 0;
    *cur = c;
  }
  __syncthreads();
  if (producer) {
    {
      const StepMaps m = maps_of(cur->it);
      tma_prefetch_desc(m.cur);
      tma_prefetch_desc(m.prev);
      if constexpr (MT) {
        tma_prefetch_desc(m.ids);
        tma_prefetch_desc(m.vel);
      } else {
        tma_prefetch_desc(m.arr);
        tma_prefetch_desc(m.upd);
      }
      if (BATCH && cur->item + 1 < item_end()) {
        const StepMaps m2 = maps_of(decode_item<TY, MODE>(cur->item + 1, P));
        tma_prefetch_desc(m2.cur);
        tma_prefetch_desc(m2.prev);
        tma_prefetch_desc(m2.arr);
        tma_prefetch_desc(m2.upd);
      }
    }
    // Prologue: the first S-2 steps of this CTA.
    for (int a = 0; a < S - 2 && cur->item < item_end(); ++a) produce();
  }

  const uint64_t wait_ns = HOOK ? P.wait_ns : kWaitLimitNs;
  // Spacing factors (unused on isotropic grids).
  const float sxy = P.inv_dxy, sxz = P.inv_dxz, syz = P.inv_dyz;
  const float sxx = P.inv_dxx, syy = P.inv_dyy, szz = P.inv_dzz;
  // Halo-column duty: warps 0 .. TY/4-1 evaluate D1y in the 4 columns left
  // and right of the tile for all TY rows (lane -> row 4*warp + lane/8).
  const bool halo_warp = ly < TY / 4;
  const int hr = ly * 4 + (lx >> 3);
  const int hxc = (lx & 7) < 4 ? (lx & 7) : G::TX + (lx & 7);
  const int hh = (hr + kRadius) * G::HX + hxc;

  int stage = 0;
  uint32_t phase = 0, xphase = 0;
  int dsel = 0;
  int abw = 0;  // shared A/B ring slot of the arriving plane (the plane kLag back is at abw + 1)
  for (int item = R.first; item < item_end(); item += item_step()) {
    const Item it = decode_item<TY, MODE>(item, P);
    const ShotDesc &sd = BATCH ? P.shots[it.shot] : P.one;
    const int kbeg = it.z0 - kRadius;
    const int kend = it.z1 + kLag;
    const int gx = it.x0 + lx;
    const int gy = it.y0 + ly;
    const int bord = sd.bord, sxs = sd.sx, sys = sd.sy;
    const bool valid = (gx >= bord) && (gx < sxs - bord) && (gy >= bord) && (gy < sys - bord);
    const long plane = (long)sd.pitch * sys;
    unsigned long long *out = reinterpret_cast<unsigned long long *>(sd.F[P.parity ^ 1]) + ((long)gy * sd.pitch + gx);
    const int src_z = sd.src_z, cor_z = sd.cor_z;  // cells are read from `sd` on the (rare) planes
    const int ci = ly * G::TX + lx;
    const int hc = (ly + kRadius) * G::HX + (lx + kRadius);

    f2 Pr[kRing], Dx[kRing], Dy[kRing], A[kRing], B[kRing];

    for (int kb = kbeg; kb < kend; kb += kRing) {
#pragma unroll
      for (int j = 0; j < kRing; ++j) {
        const int k = kb + j;
        if (k >= kend) break;
        unsigned char *st = smem + stage * G::STAGE_B;
        if (!mbar_wait(&full[stage], phase, wait_ns)) {
          *s_abort = 1;
          atomicOr(P.err, 1u);
          goto aborted;
        }
        const bool center = (k >= it.z0) && (k < it.z1);
        const bool upd = (k - kLag >= it.z0);
        const bool src_plane = (k == src_z);
        const f2 *H = reinterpret_cast<const f2 *>(st);

        f2 c = H[hc];
        f2 xa[4], xb[4], ya[4], yb[4];
#pragma unroll
        for (int o = 1; o <= 4; ++o) {
          xa[o - 1] = H[hc + o];
          xb[o - 1] = H[hc - o];
          ya[o - 1] = H[hc + o * G::HX];
          yb[o - 1] = H[hc - o * G::HX];
        }
        // Fused source (original/OpenMP/openmp_insertsource.c:7-13): the
        // current p and q gain `src` at the source cell before the update
        // reads them; added to this thread's copies of the plane.
        if (src_plane) {
          const int src_x = sd.src_x, src_y = sd.src_y;
          const f2 sv = splat(P.src);
          f2 dummy;
          if (gy == src_y && abs(src_x - gx) <= kRadius) add_at(c, xa, xb, src_x - gx, sv);
          if (gx == src_x && src_y != gy && abs(src_y - gy) <= kRadius) add_at(dummy, ya, yb, src_y - gy, sv);
        }
        f2 d1x, d1y;
        if constexpr (D1D1) {
          // der1der1/sample.h:35-49: pDx = Der1_x(p) / dx and pDy = Der1_y(p) / dy.
          d1x = d1_ref(xa[0], xb[0], xa[1], xb[1], xa[2], xb[2], xa[3], xb[3], P.inv_dx);
          d1y = d1_ref(ya[0], yb[0], ya[1], yb[1], ya[2], yb[2], ya[3], yb[3], P.inv_dy);
        } else {
          d1x = d1(xa[0], xb[0], xa[1], xb[1], xa[2], xb[2], xa[3], xb[3]);
          d1y = d1(ya[0], yb[0], ya[1], yb[1], ya[2], yb[2], ya[3], yb[3]);
        }
        Pr[j] = c;
        Dx[j] = d1x;
        Dy[j] = d1y;
        f2 d2x, d2y;
        constexpr int DB_N = D1D1 ? G::HY * G::TX : TY * G::HX;
        f2 *db = dbuf + dsel * DB_N;
        if constexpr (D1D1) {
          if (center) {
            d2x = d2_ref(c, xa[0], xb[0], xa[1], xb[1], xa[2], xb[2], xa[3], xb[3], sxx);
            d2y = d2_ref(c, ya[0], yb[0], ya[1], yb[1], ya[2], yb[2], ya[3], yb[3], syy);
            // pDx of the tile column and of its 4-row y halo: the row's own
            // value, and warps 0..7 one halo row each (halo-tile rows 0..3 and
            // TY+4..TY+7).
            db[(ly + kRadius) * G::TX + lx] = d1x;
            if (ly < 2 * kRadius) {
              const int hrow = ly < kRadius ? ly : TY + ly;
              const int hb0 = hrow * G::HX + lx + kRadius;
              f2 ha[4], hb[4], dummy;
#pragma unroll
              for (int o = 1; o <= 4; ++o) {
                ha[o - 1] = H[hb0 + o];
                hb[o - 1] = H[hb0 - o];
              }
              if (src_plane && it.y0 - kRadius + hrow == sd.src_y && abs(sd.src_x - gx) <= kRadius)
                add_at(dummy, ha, hb, sd.src_x - gx, splat(P.src));
              db[hrow * G::TX + lx] = d1_ref(ha[0], hb[0], ha[1], hb[1], ha[2], hb[2], ha[3], hb[3], P.inv_dx);
            }
          }
        } else if (center) {
          d2x = scale<ISO>(d2(c, xa[0], xb[0], xa[1], xb[1], xa[2], xb[2], xa[3], xb[3]), sxx);
          d2y = scale<ISO>(d2(c, ya[0], yb[0], ya[1], yb[1], ya[2], yb[2], ya[3], yb[3]), syy);
          db[ly * G::HX + lx + kRadius] = d1y;
          if (halo_warp) {
            f2 ha[4], hb[4];
#pragma unroll
            for (int o = 1; o <= 4; ++o) {
              ha[o - 1] = H[hh + o * G::HX];
              hb[o - 1] = H[hh - o * G::HX];
            }
            if (src_plane) {
              const int src_x = sd.src_x, src_y = sd.src_y;
              const int hgy = it.y0 + hr;
              if (hxc == src_x - (it.x0 - kRadius) && src_y != hgy && abs(src_y - hgy) <= kRadius) {
                f2 dummy;
                add_at(dummy, ha, hb, src_y - hgy, splat(P.src));
              }
            }
            db[hr * G::HX + hxc] = d1(ha[0], hb[0], ha[1], hb[1], ha[2], hb[2], ha[3], hb[3]);
          }
        }
        // Split-phase exchange: announce this warp's D1y (and, by program
        // order, that it has finished the previous step), update plane k-4,
        // which needs no exchanged data, then wait for the other warps.
        __syncwarp();
        if (lx == 0) mbar_arrive(xchg);
        // The producer has passed the exchange of the previous step, so every
        // thread is past the step before it: refill that step's stage with
        // the next step due (S-2 steps ahead of this one).
        if (producer && cur->item < item_end()) {
          fence_proxy_async_smem();
          produce();
        }
        if (upd) {
          const int cs = (j + kRing - kLag) % kRing;  // ring slot of plane k-kLag
          // RP(o): plane k-kLag+o for o = 0..4, k-kLag-(kRing-o) for o > 4.
#define RP(o) Pr[(cs + (o)) % kRing]
#define RX(o) Dx[(cs + (o)) % kRing]
#define RY(o) Dy[(cs + (o)) % kRing]
          constexpr int M1 = kRing - 1, M2 = kRing - 2, M3 = kRing - 3, M4 = kRing - 4;
          f2 d2z, dxz, dyz;
          if constexpr (D1D1) {
            // der1der1/sample.h:58-66: pzz, pxz = Der1_z(pDx) / dz, pyz = Der1_z(pDy) / dz.
            d2z = d2_ref(RP(0), RP(1), RP(M1), RP(2), RP(M2), RP(3), RP(M3), RP(4), RP(M4), szz);
            dxz = d1_ref(RX(1), RX(M1), RX(2), RX(M2), RX(3), RX(M3), RX(4), RX(M4), P.inv_dz);
            dyz = d1_ref(RY(1), RY(M1), RY(2), RY(M2), RY(3), RY(M3), RY(4), RY(M4), P.inv_dz);
          } else {
            d2z = scale<ISO>(d2(RP(0), RP(1), RP(M1), RP(2), RP(M2), RP(3), RP(M3), RP(4), RP(M4)), szz);
            dxz = scale<ISO>(d1(RX(1), RX(M1), RX(2), RX(M2), RX(3), RX(M3), RX(4), RX(M4)), sxz);
            dyz = scale<ISO>(d1(RY(1), RY(M1), RY(2), RY(M2), RY(3), RY(M3), RY(4), RY(M4)), syz);
          }
#undef RP
#undef RX
#undef RY
          const float *cu = reinterpret_cast<const float *>(st + G::OFF_UPD);
          float czz, cxz, cyz, v2px, v2pz, v2sz, v2pn;
          if constexpr (MT) {
            const int md = st[G::OFF_IDU + ci];
            czz = s_med[(DC_ZZ * kMediaMax) + md];
            cxz = s_med[(DC_XZ * kMediaMax) + md];
            cyz = s_med[(DC_YZ * kMediaMax) + md];
            v2px = cu[ci];
            v2pz = cu[G::NT + ci];
            v2sz = cu[2 * G::NT + ci];
            v2pn = cu[3 * G::NT + ci];
          } else {
            czz = cu[ci];
            cxz = cu[G::NT + ci];
            cyz = cu[2 * G::NT + ci];
            v2px = cu[3 * G::NT + ci];
            v2pz = cu[4 * G::NT + ci];
            v2sz = cu[5 * G::NT + ci];
            v2pn = cu[6 * G::NT + ci];
          }
          f2 Ak, Bk;
          if constexpr (G::AB_SMEM) {
            const float4 ab = ABs[(abw == kLag ? 0 : abw + 1) * G::NT + ci];
            Ak = mk2(ab.x, ab.y);
            Bk = mk2(ab.z, ab.w);
          } else {
            Ak = A[cs];
            Bk = B[cs];
          }
          f2 h1, h2;
          float rhsp, rhsq;
          if constexpr (D1D1) {
            // der1der1/sample.h:70-117 in its order, each operation rounded:
            // h1 = cpxx + cpyy + cpzz + cpxy + cpxz + cpyz (A = cpxx + cpyy,
            // C = cpxy from the plane's arrival), h2 = pxx + pyy + pzz - h1.
            const f2 Ck = Cs[(abw == kLag ? 0 : abw + 1) * G::NT + ci];
            h1 = add_rn(add_rn(add_rn(add_rn(Ak, mul_rn(czz, d2z)), Ck), mul_rn(cxz, dxz)), mul_rn(cyz, dyz));
            h2 = sub_rn(add_rn(Bk, d2z), h1);
            const float h1p = lo(h1), h1q = hi(h1), h2p = lo(h2), h2q = hi(h2);
            const float t = __fmul_rn(v2pz, h1q);
            rhsp = __fadd_rn(__fadd_rn(__fmul_rn(v2px, h2p), t), __fmul_rn(v2sz, __fsub_rn(h1p, h1q)));
            rhsq = __fsub_rn(__fadd_rn(__fmul_rn(v2pn, h2p), t), __fmul_rn(v2sz, __fsub_rn(h2p, h2q)));
          } else {
            h1 = fma2(splat(cyz), dyz, fma2(splat(cxz), dxz, fma2(splat(czz), d2z, Ak)));
            h2 = sub2(add2(Bk, d2z), h1);
            const float h1p = lo(h1), h1q = hi(h1), h2p = lo(h2), h2q = hi(h2);
            // Explicit roundings: every unrolled copy computes identical floats.
            const float t = __fmul_rn(v2pz, h1q);
            rhsp = __fmaf_rn(v2sz, __fsub_rn(h1p, h1q), __fmaf_rn(v2px, h2p, t));
            rhsq = __fmaf_rn(-v2sz, __fsub_rn(h2p, h2q), __fmaf_rn(v2pn, h2p, t));
          }
          f2 old = reinterpret_cast<const f2 *>(st + G::OFF_PP)[ci];
          const int zc = k - kLag;
          if (zc == cor_z) {
            if (gx == sd.cor_x && gy == sd.cor_y) old = add2(old, splat(P.cor));
          }
          const f2 cur = Pr[cs];
          f2 nw;
          if constexpr (D1D1) {
            // pp = 2 pc - pp + rhs * dt * dt (der1der1/sample.h:119-120).
            nw = add_rn(sub_rn(add_rn(cur, cur), old), mul_rn(P.dt, mul_rn(P.dt, mk2(rhsp, rhsq))));
          } else {
            nw = fma2(mk2(rhsp, rhsq), splat(P.dt2), sub2(add2(cur, cur), old));
          }
          if (valid) out[(long)zc * plane] = nw.v;
        }
        if (!mbar_wait(xchg, xphase, wait_ns)) {
          // A warp of this CTA stopped arriving (it gave up a wait itself):
          // leave too, so that no thread keeps waiting step after step.
          *s_abort = 1;
          atomicOr(P.err, 2u);
          goto aborted;
        }
        xphase ^= 1u;
        if constexpr (D1D1) {
          if (center) {
            // pxy = Der1_y(pDx) / dy (der1der1/sample.h:55); A = cpxx + cpyy,
            // B = pxx + pyy, C = cpxy.
            const f2 *dc = db + (ly + kRadius) * G::TX + lx;
            constexpr int W = G::TX;
            const f2 pxy = d1_ref(dc[W], dc[-W], dc[2 * W], dc[-2 * W], dc[3 * W], dc[-3 * W], dc[4 * W], dc[-4 * W],
                                  P.inv_dy);
            const float *ca = reinterpret_cast<const float *>(st + G::OFF_ARR);
            const float cxx = ca[ci], cyy = ca[G::NT + ci], cxy = ca[2 * G::NT + ci];
            const f2 av = add_rn(mul_rn(cxx, d2x), mul_rn(cyy, d2y));
            const f2 bv = add_rn(d2x, d2y);
            ABs[abw * G::NT + ci] = make_float4(lo(av), hi(av), lo(bv), hi(bv));
            Cs[abw * G::NT + ci] = mul_rn(cxy, pxy);
          }
        } else if (center) {
          const f2 *dr = db + ly * G::HX + lx + kRadius;
          const f2 dxy = scale<ISO>(d1(dr[1], dr[-1], dr[2], dr[-2], dr[3], dr[-3], dr[4], dr[-4]), sxy);
          float cxx, cyy, cxy;
          if constexpr (MT) {
            const int md = st[G::OFF_IDC + ci];
            cxx = s_med[(DC_XX * kMediaMax) + md];
            cyy = s_med[(DC_YY * kMediaMax) + md];
            cxy = s_med[(DC_XY * kMediaMax) + md];
          } else {
            const float *ca = reinterpret_cast<const float *>(st + G::OFF_ARR);
            cxx = ca[ci];
            cyy = ca[G::NT + ci];
            cxy = ca[2 * G::NT + ci];
          }
          const f2 av = fma2(splat(cxy), dxy, fma2(splat(cyy), d2y, mul2(splat(cxx), d2x)));
          const f2 bv = add2(d2x, d2y);
          if constexpr (G::AB_SMEM) {
            ABs[abw * G::NT + ci] = make_float4(lo(av), hi(av), lo(bv), hi(bv));
          } else {
            A[j] = av;
            B[j] = bv;
          }
        }
        dsel ^= 1;
        abw = abw == kLag ? 0 : abw + 1;
        if (++stage == S) {
          stage = 0;
          phase ^= 1u;
        }
      }
    }
  }
  return;
aborted:
  // A bounded wait gave up.  Every thread leaves (the others give up on
  // their own bounded waits or see the flag); thread 0 first waits, bounded,
  // for the loads that may still be in flight into this CTA's stages.
  *s_abort = 1;
  if (tid == 0) {
    for (int a = 0; a < S - 2; ++a) {
      const int s2 = (stage + a) % S;
      (void)mbar_wait(&full[s2], phase ^ uint32_t(stage + a >= S), kWaitLimitNs);
    }
  }
}

// ---- host side ---------------------------------------------------------------

template <int TY, int S, int MINB>
static cudaError_t prepare_t() {
  constexpr size_t smem = smem_bytes<TY, S>();
  cudaError_t e = cudaSuccess;
  for (auto kern : {k_propagate_fp32<TY, S, true, kItemsTiles, MINB>, k_propagate_fp32<TY, S, false, kItemsTiles, MINB>,
                    k_propagate_fp32<TY, S, true, kItemsBatch, MINB>, k_propagate_fp32<TY, S, false, kItemsBatch, MINB>,
                    k_propagate_fp32<TY, S, true, kItemsSegments, MINB>,
                    k_propagate_fp32<TY, S, false, kItemsSegments, MINB>})
    if (e == cudaSuccess) e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return e;
}

template <int TY, int S, int MINB>
static cudaError_t launch_t(const PropLaunch &L, cudaStream_t s) {
  constexpr size_t smem = smem_bytes<TY, S>();
  static bool ready = false;  // dynamic shared-memory limit set for this shape
  if (!ready) {
    cudaError_t e = prepare_t<TY, S, MINB>();
    if (e != cudaSuccess) return e;
    ready = true;
  }
  const bool iso = L.p.iso != 0;
  auto kern = L.batch      ? (iso ? k_propagate_fp32<TY, S, true, kItemsBatch, MINB>
                                  : k_propagate_fp32<TY, S, false, kItemsBatch, MINB>)
              : L.p.seg    ? (iso ? k_propagate_fp32<TY, S, true, kItemsSegments, MINB>
                                  : k_propagate_fp32<TY, S, false, kItemsSegments, MINB>)
                           : (iso ? k_propagate_fp32<TY, S, true, kItemsTiles, MINB>
                                  : k_propagate_fp32<TY, S, false, kItemsTiles, MINB>);
  kern<<<L.grid, kTileX * TY, smem, s>>>(L.m, L.p);
  return cudaGetLastError();
}

// Supported shapes: rows per tile x stages.  TY = 16 runs one 512-thread CTA
// per SM; TY = 8 runs two 256-thread CTAs per SM.
#define FLT_SHAPES(X) X(12, 4, 1) X(12, 5, 1) X(12, 6, 1) X(16, 4, 1) X(16, 5, 1) X(8, 4, 2) X(8, 5, 2)

size_t propagate_fp32_smem_bytes(int ty, int st) {
#define X(a, b, c) \
  if (ty == a && st == b) return smem_bytes<a, b>();
  FLT_SHAPES(X)
#undef X
  return 0;
}
bool propagate_fp32_supported(int ty, int st) { return propagate_fp32_smem_bytes(ty, st) != 0; }
int propagate_fp32_threads(int ty) { return kTileX * ty; }
int propagate_fp32_ctas_per_sm(int ty) { return ty == 8 ? 2 : 1; }

cudaError_t propagate_fp32_prepare(int ty, int st) {
#define X(a, b, c) \
  if (ty == a && st == b) return prepare_t<a, b, c>();
  FLT_SHAPES(X)
#undef X
  return cudaErrorInvalidValue;
}

// The Der1-Der1 numerics: one shape (kD1D1Rows x kD1D1Stages), single shot.
static cudaError_t launch_d1d1(const PropLaunch &L, cudaStream_t s) {
  constexpr int TY = kD1D1Rows, S = kD1D1Stages;
  constexpr size_t smem = smem_bytes<TY, S, true>();
  static_assert(smem <= 227 * 1024, "Der1-Der1 shape exceeds the shared memory of a CTA");
  auto tiles = k_propagate_fp32<TY, S, false, kItemsTiles, 1, true>;
  auto segs = k_propagate_fp32<TY, S, false, kItemsSegments, 1, true>;
  static bool ready = false;
  if (!ready) {
    for (auto kern : {tiles, segs}) {
      const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    ready = true;
  }
  if (L.batch || L.tile_rows != TY || L.stages != S) return cudaErrorInvalidValue;
  (L.p.seg ? segs : tiles)<<<L.grid, kTileX * TY, smem, s>>>(L.m, L.p);
  return cudaGetLastError();
}

// The fault-injection variant: the default shape, single shot.
static cudaError_t launch_hook(const PropLaunch &L, cudaStream_t s) {
  constexpr int TY = 16, S = 5;
  constexpr size_t smem = smem_bytes<TY, S>();
  auto tiles_i = k_propagate_fp32<TY, S, true, kItemsTiles, 1, false, true>;
  auto tiles_a = k_propagate_fp32<TY, S, false, kItemsTiles, 1, false, true>;
  auto segs_i = k_propagate_fp32<TY, S, true, kItemsSegments, 1, false, true>;
  auto segs_a = k_propagate_fp32<TY, S, false, kItemsSegments, 1, false, true>;
  static bool ready = false;
  if (!ready) {
    for (auto kern : {tiles_i, tiles_a, segs_i, segs_a}) {
      const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    ready = true;
  }
  // Any pipeline depth of the step's own shape: the plan depends on the rows
  // only.  (The coefficient planes are present in either layout.)
  if (L.batch || L.d1d1 || L.tile_rows != TY) return cudaErrorInvalidValue;
  const bool iso = L.p.iso != 0;
  auto kern = L.p.seg ? (iso ? segs_i : segs_a) : (iso ? tiles_i : tiles_a);
  kern<<<L.grid, kTileX * TY, smem, s>>>(L.m, L.p);
  return cudaGetLastError();
}

// The media-table layout: single shot, 16-row tiles.
#define FLT_MEDIA_SHAPES(X) X(16, 5) X(16, 6) X(16, 7)

template <int TY, int S>
static cudaError_t launch_media_t(const PropLaunch &L, cudaStream_t s) {
  constexpr size_t smem = smem_bytes<TY, S, false, true>();
  static_assert(smem <= 227 * 1024, "media-table shape exceeds the shared memory of a CTA");
  auto tiles_i = k_propagate_fp32<TY, S, true, kItemsTiles, 1, false, false, true>;
  auto tiles_a = k_propagate_fp32<TY, S, false, kItemsTiles, 1, false, false, true>;
  auto segs_i = k_propagate_fp32<TY, S, true, kItemsSegments, 1, false, false, true>;
  auto segs_a = k_propagate_fp32<TY, S, false, kItemsSegments, 1, false, false, true>;
  static bool ready = false;
  if (!ready) {
    for (auto kern : {tiles_i, tiles_a, segs_i, segs_a}) {
      const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
    }
    ready = true;
  }
  const bool iso = L.p.iso != 0;
  auto kern = L.p.seg ? (iso ? segs_i : segs_a) : (iso ? tiles_i : tiles_a);
  kern<<<L.grid, kTileX * TY, smem, s>>>(L.m, L.p);
  return cudaGetLastError();
}

bool propagate_fp32_media_supported(int ty, int st) {
#define X(a, b) \
  if (ty == a && st == b) return true;
  FLT_MEDIA_SHAPES(X)
#undef X
  return false;
}

cudaError_t propagate_fp32_launch(const PropLaunch &L, cudaStream_t s) {
  if (L.p.stall_step >= 0) return launch_hook(L, s);
  if (L.d1d1) return launch_d1d1(L, s);
  if (L.media) {
    if (L.batch || !L.p.media) return cudaErrorInvalidValue;
#define X(a, b) \
  if (L.tile_rows == a && L.stages == b) return launch_media_t<a, b>(L, s);
    FLT_MEDIA_SHAPES(X)
#undef X
    return cudaErrorInvalidValue;
  }
#define X(a, b, c) \
  if (L.tile_rows == a && L.stages == b) return launch_t<a, b, c>(L, s);
  FLT_SHAPES(X)
#undef X
  return cudaErrorInvalidValue;
}

}  // namespace flt
