// Internal interfaces between the C-ABI layer (driver.cu) and the kernels.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace flt {

constexpr int kRadius = 4;   // stencil half-width of Der2 / DerCross
constexpr int kTileX = 32;   // tile width in x: one warp per tile row
constexpr int kNumCoef = 10;

// Device coefficient block layout: [z][c][y][pitch] with c in this order.
// The first three are read when a plane arrives (in-plane terms), the other
// seven when the plane is updated four planes later.
enum DevCoef {
  DC_XX = 0, DC_YY, DC_XY,                    // arrival: ch1dxx ch1dyy ch1dxy
  DC_ZZ, DC_XZ, DC_YZ, DC_V2PX, DC_V2PZ, DC_V2SZ, DC_V2PN  // update
};
constexpr int kArrivalCoef = 3;
constexpr int kUpdateCoef = 7;

// One plain FP32 step.  The fields are stored as (p, q) pairs of float,
// [z][y][pitch] with x fastest.
struct PropParams {
  float2 *prev;             // pp/qp pairs: read through TMA, written in place
  int sx, sy, sz, pitch, bord;
  int ntx, nty, nchunk, chunk, nitems;
  float inv_dx, inv_dy, inv_dz;     // 1/dx, 1/dy, 1/dz
  float inv_dxx, inv_dyy, inv_dzz;  // 1/(dx*dx), 1/(dy*dy), 1/(dz*dz) as the reference forms them
  int iso;                          // dx == dy == dz: derivatives unscaled, dt2 = dt^2 / h^2
  float dt2;                        // factor of the rhs in the update
  int src_x, src_y, src_z;  // source added to current p,q this step (src_z < 0: none)
  float src;
  int cor_x, cor_y, cor_z;  // last step's source, not stored in the buffer that
  float cor;                //   is now the previous field: added on read
  unsigned int *err;        // error word (bit 0: bounded wait gave up)
};

struct PropLaunch {
  CUtensorMap cur_halo;   // current pairs, box (TX+8, TY+8, 1)
  CUtensorMap prev_pt;    // previous pairs, box (TX, TY, 1)
  CUtensorMap coef_arr;   // coefficients, box (TX, TY, 3, 1)
  CUtensorMap coef_upd;   // coefficients, box (TX, TY, 7, 1)
  PropParams p;
  int tile_rows;          // TY
  int stages;
  int grid;
};

size_t propagate_fp32_smem_bytes(int tile_rows, int stages);
bool propagate_fp32_supported(int tile_rows, int stages);
int propagate_fp32_threads(int tile_rows);
int propagate_fp32_ctas_per_sm(int tile_rows);
cudaError_t propagate_fp32_launch(const PropLaunch &L, cudaStream_t s);

// Time limit of every device-side wait (ns).
constexpr uint64_t kWaitLimitNs = 2000000000ull;

}  // namespace flt
