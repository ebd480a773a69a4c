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

// Media-table layout of the coefficients (FP32 form): the six angle terms
// (DC_XX .. DC_YZ) depend on a cell's (phi, theta) only, so a model with at
// most kMediaMax distinct (phi, theta) pairs stores them once per pair in a
// table [6][kMediaMax] and one byte per cell (the pair's slot) in an id
// volume [z][y][ipitch].  The id of cell x sits in byte x + kIdShift of its
// row: a tile's first column kRadius + 32 t then starts at a multiple of 16
// bytes, as a TMA load of 8-bit elements needs.  The four velocity terms
// (DC_V2PX .. DC_V2PN) stay per cell in the coefficient block.
constexpr int kMediaMax = 256;
constexpr int kAngleCoef = 6;
constexpr int kVelCoef = 4;
constexpr int kIdShift = 12;
constexpr int kMediaStages = 7;  // default pipeline depth of the media-table layout (fastest at 504^3)
static_assert((kRadius + kIdShift) % 16 == 0 && kTileX % 16 == 0, "id tiles must start on 16-byte boundaries");
static_assert(DC_V2PX == kAngleCoef && DC_V2PN == kNumCoef - 1, "velocity terms follow the angle terms");

// One shot's geometry and buffers, in device memory (read by every launch).
// The fields are stored as (p, q) pairs of float, [z][y][pitch] with x fastest.
struct ShotDesc {
  float2 *F[2];                  // the two field buffers
  int sx, sy, sz, pitch, bord;
  int ntx, nty, chunk;           // tiles in x and y, z-chunk length
  int src_x, src_y, src_z;       // cell that gains the step's source (src_z < 0: none)
  int cor_x, cor_y, cor_z;       // cell whose previous-field value lacks the last step's
                                 //   source (added on read; cor_z < 0: none)
  int pad[2];
};

// TMA descriptors of one shot (in device memory; CUtensorMap carries the
// alignment TMA needs).
struct ShotMaps {
  CUtensorMap halo[2];  // field buffer b, box (TX+8, TY+8, 1)
  CUtensorMap pt[2];    // field buffer b, box (TX, TY, 1)
  CUtensorMap arr;      // coefficients, box (TX, TY, 3, 1)
  CUtensorMap upd;      // coefficients, box (TX, TY, 7, 1)
};

// One launch: every active shot advances one step.
//  * batched launches: work items {shot, x0, y0, chunk index}, ordered by
//    shot; CTA b takes items b, b + grid, ... below nitems;
//  * single-shot launches with seg: segments {x0, y0, z0, z1} (a z range of
//    one tile column); CTA b takes segments cta_first[b] .. cta_first[b+1]-1;
//  * single-shot launches without seg: items = tiles x uniform z-chunks of
//    one.chunk planes, chunk-major, CTA b takes b, b + grid, ... below nitems.
struct PropParams {
  ShotDesc one;                     // single-shot launches: the shot itself
  const ShotDesc *shots;            // batched launches: per-shot descriptors
  const ShotMaps *maps;
  const int4 *items;                // batched launches
  int nitems;
  int parity;                       // current field = F[parity], previous = F[1 - parity]
  float inv_dx, inv_dy, inv_dz;     // 1/dx, 1/dy, 1/dz
  float inv_dxx, inv_dyy, inv_dzz;  // 1/(dx*dx), 1/(dy*dy), 1/(dz*dz) as the reference forms them
  float inv_dxy, inv_dxz, inv_dyz;  // 1/(dx*dy), 1/(dx*dz), 1/(dy*dz): factors of the cross derivatives
  int iso;                          // dx == dy == dz: derivatives unscaled, dt2 = dt^2 / h^2
  float dt2;                        // factor of the rhs in the update
  float dt;                         // the time step (Der1-Der1 numerics: rhs * dt * dt)
  float src;                        // value added at each shot's source cell (src_z >= 0)
  float cor;                        // value owed at each shot's cor cell (cor_z >= 0)
  unsigned int *err;                // error word (bit 0: bounded wait gave up)
  const int4 *seg;                  // single-shot launches with a segment list
  const int *cta_first;             // their [grid + 1] first segments
  const float *media;               // media-table layout: angle terms [kAngleCoef][kMediaMax]
  unsigned long long wait_ns;       // limit of the step's waits (ns)
  int stall_step;                   // test hook: CTA 0 skips the loads of its stall_step-th step (-1: none)
};

// The four descriptors a single-shot launch passes as kernel parameters.
struct SingleMaps {
  CUtensorMap cur_halo, prev_pt, arr, upd;
  CUtensorMap ids, vel;  // media-table layout: id volume, box (TX, TY, 1); velocity terms, box (TX, TY, 4, 1)
};

struct PropLaunch {
  PropParams p;
  SingleMaps m;           // single-shot launches
  bool batch;             // true: p.shots / p.maps / p.items describe the work
  bool d1d1;              // Der1-Der1 numerics (single shot, 16 x 4 tiles)
  bool media;             // media-table coefficient layout (single shot)
  int tile_rows;          // TY
  int stages;
  int grid;
};

size_t propagate_fp32_smem_bytes(int tile_rows, int stages);
bool propagate_fp32_supported(int tile_rows, int stages);
// Shapes built for the media-table layout.
bool propagate_fp32_media_supported(int tile_rows, int stages);
int propagate_fp32_threads(int tile_rows);
int propagate_fp32_ctas_per_sm(int tile_rows);
cudaError_t propagate_fp32_prepare(int tile_rows, int stages);
cudaError_t propagate_fp32_launch(const PropLaunch &L, cudaStream_t s);
// Tile shape of the Der1-Der1 numerics (the only one built for it).
constexpr int kD1D1Rows = 16, kD1D1Stages = 4;
// Most concurrent chains of the batched shots' chain schedule, and the
// updated cells from which a shot fills the GPU on its own (measured on
// GB300: at 2.1 M cells a chain and the persistent launch tie; below, the
// persistent launch is 6-7% faster; at 4.7 M cells and more one chain is
// 7% faster).
constexpr int kMaxChains = 8;
constexpr double kChainFillCells = 2.1e6;

// ---- 16-bit field storage (propagate_half.cu) ----
// A field buffer holds (p, q) as half2 per cell ([z][y][pitch]) and, in the
// extended form, one residual byte per value (a ushort per cell), with a
// power-of-two scale per z-plane.
struct HalfMaps {
  CUtensorMap cur_hi, cur_lo;    // current field, halo box (TX+8, TY+8, 1)
  CUtensorMap prev_hi, prev_lo;  // previous field: box (TX, TY, 1) / residuals (TX+8, TY, 1) from x0-4
  CUtensorMap arr, upd;          // coefficients, as in the FP32 form
};

// One batched shot of a 16-bit form (device memory).
struct HalfShot {
  unsigned *hi[2];        // the two field buffers: (p, q) as half2 per cell
  unsigned short *lo[2];  // their residual bytes (extended form; null otherwise)
  int *E;                 // [3][sz] per-plane exponents; the field of step it uses slot it % 3
  unsigned *Mx;           // [2][sz] per-plane max |value| (float bits) of the field in buffer b
};

// A batched shot's tensor maps, by the buffer that holds the current field.
struct HalfShotMaps {
  HalfMaps m[2];
};

struct HalfParams {
  PropParams p;                       // geometry (p.one), spacing, source, error word
  unsigned *out_hi;                   // new field: half2 per cell
  unsigned short *out_lo;             // new field: residual bytes (extended form)
  const int *e_cur, *e_prev, *e_new;  // per-plane exponents of the current, previous and new field
  unsigned *m_new;                    // per-plane max |value| of the new field (float bits), atomicMax
  // Batched launches (p.items, p.shots): per-shot buffers and maps, and the
  // exponent slot of the current field (step % 3).
  const HalfShot *hshots;
  const HalfShotMaps *hmaps;
  int ecur;
};

struct HalfLaunch {
  HalfParams h;
  HalfMaps m;
  int tile_rows, stages, grid;
  bool batch;  // h.p.items / h.p.shots / h.hshots / h.hmaps describe the work
};

bool propagate_half_supported(int tile_rows, int stages);
cudaError_t propagate_half_launch(const HalfLaunch &L, bool ext, cudaStream_t s);
cudaError_t propagate_half_prepare(int tile_rows, int stages, bool ext, bool batch);
int propagate_half_ctas_per_sm(int tile_rows, int stages, bool ext, bool batch);
cudaError_t half_scales(const unsigned *m_cur, unsigned *m_prev, int *e_new, int sz, int src_z, float src_abs,
                        cudaStream_t s);
// Before a batched 16-bit step: the new field's plane exponents and the
// cleared maxima (as half_scales) of the first `active` shots of `order`,
// block i taking shot order[i]; the current field is in buffer c, its
// exponents in slot ecur.
cudaError_t half_scales_batch(const HalfShot *hs, const ShotDesc *sd, const int *order, int active, int c, int ecur,
                              float src_abs, cudaStream_t s);
cudaError_t half_encode(const float *p, const float *q, unsigned *hv, unsigned short *rv, int *e, unsigned *m, int sx,
                        int sy, int sz, int pitch, bool ext, cudaStream_t s);
cudaError_t half_decode(const unsigned *hv, const unsigned short *rv, const int *e, float *out, int comp, int sx,
                        int sy, int sz, int pitch, bool ext, int grid, cudaStream_t s);

// ---- learned absorbing boundary (abc_learned.cu) ----
// The resident single-shot state as the boundary layer sees it.
struct ResidentView {
  bool init = false;
  int sx = 0, sy = 0, sz = 0, bord = 0, pitch = 0;
  float dx = 0, dy = 0, dz = 0, dt = 0;
  const float2 *cur = nullptr, *prev = nullptr;  // current and previous (p, q) fields (FP32 form)
  float2 *next = nullptr;                        // the buffer the step writes
  const float *coef = nullptr;                   // [z][10][y][pitch] (DevCoef order)
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  unsigned *err = nullptr;                       // the error word (bit 0: a bounded wait gave up)
};
ResidentView resident_view();       // driver.cu; cur/prev/next for the next step
bool abc_active();                  // a boundary layer is set on the resident state
cudaError_t abc_after_step(const ResidentView &v);   // the layer's update of next, after the plain step
void abc_release_resident();        // the resident state is re-initialised or finalised

// ---- output path (snapshot.cu) ----
// Field `which` (0 current p, 1 current q, 2 previous p, 3 previous q) of the
// resident state, any storage form, as an unpitched FP32 volume in dev_out,
// issued on the library's stream.  fix_idx / fix_val: the one cell whose
// stored value lacks a source addition the interface shows (-1: none).
int resident_field_to_device(int which, float *dev_out, long *fix_idx, float *fix_val);
size_t resident_cells();             // sx * sy * sz (0 when not initialised)
bool resident_dims(int *sx, int *sy, int *sz);  // grid of the resident state (any form)
cudaStream_t resident_stream();      // the library's stream
void snapshot_release();             // driver.cu calls it when the state goes away

// Time limit of every device-side wait (ns).
constexpr uint64_t kWaitLimitNs = 2000000000ull;

}  // namespace flt
