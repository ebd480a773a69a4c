// Pipeline pieces of the FP32 step kernel (propagate_fp32.cu): the
// shared-memory stage layout, the work items of a launch, and the
// producer's TMA issue of one step.
#pragma once
#include "device_util.cuh"
#include "fletcher_internal.h"

namespace flt {

// Plane k arrives at step k; plane k - kLag is updated at that step.  Its
// z stencil (planes k-kLag-4 .. k-kLag+4) lives in per-thread rings of
// kRing planes, and its in-plane terms in kABSlots shared-memory slots.
// kLag = 4 uses the arriving plane at once.  kLag = 5 makes the update
// independent of the same step's arrival work, at one more ring plane (124
// instead of 121 registers) and one more 8 KB slot: bit-identical, and 3%
// slower at 504^3 (2.287 against 2.217 ms per step).
constexpr int kLag = 4;
constexpr int kRing = kLag + 5;
constexpr int kABSlots = kLag + 1;

template <int TY, bool D1D1 = false, bool MT = false>
struct Geo {
  static constexpr int TX = kTileX;
  static constexpr int HX = TX + 2 * kRadius;
  static constexpr int HY = TY + 2 * kRadius;
  static constexpr int NT = TX * TY;
  static constexpr int HALO_B = HX * HY * 8;
  static constexpr int ARR_B = MT ? 0 : kArrivalCoef * NT * 4;
  static constexpr int UPD_B = (MT ? kVelCoef : kUpdateCoef) * NT * 4;  // media table: velocity terms only
  static constexpr int PP_B = NT * 8;
  static constexpr int ID_B = MT ? NT : 0;  // medium ids, one byte per cell
  static constexpr int OFF_ARR = HALO_B;
  static constexpr int OFF_UPD = OFF_ARR + ARR_B;
  static constexpr int OFF_PP = OFF_UPD + UPD_B;
  static constexpr int OFF_IDC = OFF_PP + PP_B;  // ids of plane k
  static constexpr int OFF_IDU = OFF_IDC + ID_B;  // ids of plane k-4
  static constexpr int STAGE_B = (OFF_IDU + ID_B + 127) / 128 * 128;
  static constexpr int TAB_B = MT ? kAngleCoef * kMediaMax * 4 : 0;
  // Exchange buffer, double-buffered: D1y of the tile rows with their 4-column
  // x halo, or (Der1-Der1 numerics) D1x of the tile columns with their 4-row
  // y halo.
  static constexpr int DBUF_B = D1D1 ? 2 * HY * TX * 8 : 2 * TY * HX * 8;
  // Tiles of 16 rows (512 threads, at most 128 registers a thread), and of 8
  // rows (two CTAs per SM), keep the per-cell in-plane terms (A, B; and C
  // for the Der1-Der1 numerics) of the last 5 planes in shared memory
  // instead of a 9-plane register ring.
  static constexpr bool AB_SMEM = TY >= 16 || TY <= 8;  // 8 rows run two CTAs per SM (128 registers)
  static constexpr int AB_B = AB_SMEM ? kABSlots * NT * (D1D1 ? 24 : 16) : 0;
  static_assert(TY % 4 == 0, "tile rows must be a multiple of 4");
  static_assert(!D1D1 || (AB_SMEM && TY >= 8), "the Der1-Der1 numerics keep their in-plane terms in shared memory");
  static_assert(HALO_B % 128 == 0 && ARR_B % 128 == 0 && UPD_B % 128 == 0 && ID_B % 128 == 0,
                "stage regions 128-B aligned");
  static_assert(!(MT && D1D1), "the Der1-Der1 numerics read the coefficient planes");
};

template <int TY, int S, bool D1D1 = false, bool MT = false>
constexpr size_t smem_bytes() {
  using G = Geo<TY, D1D1, MT>;
  return size_t(S) * G::STAGE_B + G::DBUF_B + G::AB_B + G::TAB_B + 8 * S + 8 + 16 + 64 + 128;
}

// A work item resolved against its shot: tile origin, z range, and (batched
// launches) the shot's descriptors.
struct Item {
  int x0, y0, z0, z1;
  int shot;
};

// Work-item kinds of a launch (template parameter MODE):
//  * kItemsTiles: single shot, items = tiles x uniform z-chunks, chunk-major,
//    CTA b takes b, b + grid, ... (decoded arithmetically, no lookups);
//  * kItemsBatch: batched shots, P.seg {x0 + (shot << 16), y0, z0, z1}, CTA
//    b takes its run cta_first[b] .. cta_first[b + 1] - 1 (each running
//    shot's own single-shot plan, stacked);
//  * kItemsSegments: single shot, P.seg {x0, y0, z0, z1}, CTA b takes its run
//    cta_first[b] .. cta_first[b + 1] - 1.
constexpr int kItemsTiles = 0, kItemsBatch = 1, kItemsSegments = 2;

template <int TY, int MODE>
__device__ __forceinline__ Item decode_item(int item, const PropParams &P) {
  Item it;
  if constexpr (MODE == kItemsBatch) {
    const int4 w = P.seg[item];  // {x0 + (shot << 16), y0, z0, z1}
    it.x0 = w.x & 0xffff;
    it.y0 = w.y;
    it.z0 = w.z;
    it.z1 = w.w;
    it.shot = w.x >> 16;
  } else if constexpr (MODE == kItemsSegments) {
    const int4 w = P.seg[item];  // {x0, y0, z0, z1}
    it.x0 = w.x;
    it.y0 = w.y;
    it.z0 = w.z;
    it.z1 = w.w;
    it.shot = 0;
  } else {
    const ShotDesc &d = P.one;
    const int tx = item % d.ntx;
    const int r = item / d.ntx;
    const int ty = r % d.nty;
    const int ch = r / d.nty;
    it.x0 = kRadius + tx * kTileX;
    it.y0 = kRadius + ty * TY;
    it.z0 = d.bord + ch * d.chunk;
    it.z1 = min(it.z0 + d.chunk, d.sz - d.bord);
    it.shot = 0;
  }
  return it;
}

// The items of this CTA: first, end and stride.
struct ItemRange {
  int first, end, step;
};
template <int MODE>
__device__ __forceinline__ ItemRange item_range(const PropParams &P) {
  if constexpr (MODE != kItemsTiles) return {P.cta_first[blockIdx.x], P.cta_first[blockIdx.x + 1], 1};
  else return {(int)blockIdx.x, P.nitems, (int)gridDim.x};
}

// Descriptors used for one step of item `it` (ids, vel: media-table layout).
struct StepMaps {
  const CUtensorMap *cur, *prev, *arr, *upd, *ids, *vel;
};

// The producer's position (next step to load), kept in shared memory so it
// costs no registers in the other threads.
struct Cursor {
  Item it;
  int item, k, stage;
};

// Issues the TMA loads of one step (plane k of item `it`) into `stage`.
// Media-table layout: the id tiles start at column x0 + kIdShift of the id
// volume (x0 = kRadius + 32 t, so a multiple of 16 bytes).
template <int TY, bool MT = false>
__device__ __forceinline__ void issue_step(unsigned char *stage, uint64_t *bar, const Item &it, int k,
                                           const StepMaps &m) {
  using G = Geo<TY, false, MT>;
  const bool center = (k >= it.z0) && (k < it.z1);
  const bool upd = (k - kLag >= it.z0);
  const uint32_t bytes =
      G::HALO_B + (center ? G::ARR_B + G::ID_B : 0) + (upd ? G::UPD_B + G::PP_B + G::ID_B : 0);
  mbar_arrive_expect_tx(bar, bytes);
  tma_load_3d(stage, m.cur, bar, it.x0 - kRadius, it.y0 - kRadius, k);
  if constexpr (MT) {
    if (center) tma_load_3d(stage + G::OFF_IDC, m.ids, bar, it.x0 + kIdShift, it.y0, k);
    if (upd) {
      tma_load_4d(stage + G::OFF_UPD, m.vel, bar, it.x0, it.y0, DC_V2PX, k - kLag);
      tma_load_3d(stage + G::OFF_IDU, m.ids, bar, it.x0 + kIdShift, it.y0, k - kLag);
      tma_load_3d(stage + G::OFF_PP, m.prev, bar, it.x0, it.y0, k - kLag);
    }
  } else {
    if (center) tma_load_4d(stage + G::OFF_ARR, m.arr, bar, it.x0, it.y0, 0, k);
    if (upd) {
      tma_load_4d(stage + G::OFF_UPD, m.upd, bar, it.x0, it.y0, kArrivalCoef, k - kLag);
      tma_load_3d(stage + G::OFF_PP, m.prev, bar, it.x0, it.y0, k - kLag);
    }
  }
}

}  // namespace flt
