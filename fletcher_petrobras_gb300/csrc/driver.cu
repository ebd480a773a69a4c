// C-ABI layer of libfletcher_gb300.so: the reference back-end interface
// (original/driver.h:8-22) and the extension entry points declared in
// include/fletcher_gb300.h, over resident device state.
//
// Device layout (single GPU, everything resident in HBM):
//   F[0], F[1]  (p, q) pairs of float, [sz][sy][pitch], pitch = sx rounded
//               up to 32; one buffer holds the current field, the other the
//               previous field, and they swap after every step;
//   coef        ten FP32 coefficient fields, [sz][10][sy][pitch], computed on
//               the GPU in FP64 from the raw model arrays;
//   scratch     one unpitched sx*sy*sz float volume for host transfers;
//   ids, media  media-table layout (FP32 form, when the model has at most 256
//               distinct (phi, theta) pairs): one byte per cell naming its
//               pair, [sz][sy][ipitch] with cell x at byte x + 12, and the six
//               angle coefficients of each pair, [6][256]; the steps then
//               read only the four velocity planes of coef.
// The 16-bit forms replace F by Hh[b] (half2 per cell) and, for FP16X, Hl[b]
// (residual bytes), with per-plane exponents E (three fields: current,
// previous, next) and per-plane maxima Mx (one per buffer).
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <vector>

#include "../../include/fletcher_gb300.h"
#include "fletcher_internal.h"

using namespace flt;

namespace {

struct Source {
  bool on = false;
  long idx = 0;
  float val = 0.f;
};

struct State {
  bool init = false;
  int sx = 0, sy = 0, sz = 0, bord = 0, pitch = 0;
  float dx = 0, dy = 0, dz = 0, dt = 0;
  size_t n = 0;        // sx*sy*sz
  size_t npitch = 0;   // pitch*sy*sz
  float2 *F[2] = {nullptr, nullptr};
  float *coef = nullptr;
  float *scratch = nullptr;
  unsigned *err_host = nullptr, *err_dev = nullptr;
  int cur = 0;
  Source pending;      // registered by DRIVER_InsertSource, applied by the next step
  Source owed;         // source of the last step, missing from the previous-field buffer
  ShotDesc desc;                 // the shot (passed by value to every launch)
  ShotMaps maps;                 // its TMA descriptors
  int tile_rows = 12, stages = 5, zchunks = 0;
  int grid = 0, nitems = 0, ntx = 0, nty = 0, chunk = 0;  // the FP32 launch's items
  bool spread = false;       // the plan shares out its last round (segment list launch)
  int4 *seg = nullptr;       // the plan as work segments {x0, y0, z0, z1}
  int *cta_first = nullptr;  // [seg_grid + 1]: first segment of each CTA
  int nseg = 0, seg_grid = 0;
  long launches = 0;
  size_t dev_bytes = 0;
  int num_sms = 0;
  bool hostmem = false;  // kernels read and write the caller's host arrays directly
  int form = FLETCHER_FORM_FP32;
  unsigned *Hh[2] = {nullptr, nullptr};
  unsigned short *Hl[2] = {nullptr, nullptr};
  int *E = nullptr;        // [3][sz] plane exponents, slot of the current field = ecur
  unsigned *Mx = nullptr;  // [2][sz] plane maxima (float bits) of the field in buffer b
  int ecur = 0;
  HalfMaps hm[2];          // maps of a step whose current field is in buffer b
  int numerics = FLETCHER_NUMERICS_FAST;
  // Media-table layout (FP32 form).
  bool media = false;
  unsigned char *ids = nullptr;  // [sz][sy][ipitch]
  int ipitch = 0;
  float *mtab = nullptr;         // [kAngleCoef][kMediaMax]
  CUtensorMap mids, mvel;        // id tiles (TX, TY, 1); velocity terms (TX, TY, 4, 1)
  unsigned long long *mwork = nullptr;  // set-up only: keys [256], representatives [256], overflow flag
};

State g;

// Online tile-shape tuning (FLETCHER_Autotune): each candidate shape runs
// `per_shape` timed steps after one warm-up step; the steps are real steps.
struct Tuner {
  bool active = false;
  char path[512] = "";
  int per_shape = 0;
  std::vector<int> rows, stages;
  std::vector<float> ms;
  size_t idx = 0;
  int left = 0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
};
Tuner tune;
cudaStream_t g_stream = nullptr;
bool g_own_stream = false;
int g_form = FLETCHER_FORM_FP32;
int g_req_rows = 0, g_req_stages = 0, g_req_chunks = 0;
int g_errmode = FLETCHER_ERRMODE_EXIT;
// 1: kernels read and write the caller's host arrays where the device
// supports it; 0 (default): device buffers and copies.  On GB300 with Grace
// the copies measured faster (e2e 66.3 vs 49.2 GMSamples/s at 504^3).
int g_host_access = 0;
int g_numerics = FLETCHER_NUMERICS_FAST;
// Wall-clock marks of the last DRIVER_Initialize (FLETCHER_InitPhases):
// start, allocations done, host arrays locked and copies issued, device work
// done, state ready, arrays unlocked.
double g_init_mark[6];
double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}
// Coefficient layout of the FP32 form (FLETCHER_SetCoefLayout).  The plane
// layout is the default: at 504^3 the media table, with 36% fewer bytes per
// step, ran 3-5% slower (2.30-2.48 against 2.22 ms per step; the step is
// bound by its per-plane chain of shared-memory reads, not by DRAM).
int g_coef_layout = FLETCHER_COEF_PLANES;
// Fault injection for the failure-path tests (FLETCHER_InjectFault): the
// device allocation that fails (counted down, -1: none), and the stall of
// the next propagate launch (CTA 0's step to skip, -1: none; its wait limit).
int g_fault_alloc = -1;
int g_fault_stall = -1;
unsigned long long g_fault_wait_ns = 0;
int g_last_err = FLETCHER_OK;
char g_errmsg[512] = "";

int fail(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_errmsg, sizeof(g_errmsg), fmt, ap);
  va_end(ap);
  fprintf(stderr, "fletcher_gb300: %s\n", g_errmsg);
  // A CUDA call's failure is now recorded here: clear the runtime's own
  // last-error state (for the errors that are not sticky), so that a later
  // launch check does not report it again.
  if (code == FLETCHER_ERR_CUDA || code == FLETCHER_ERR_NOMEM) cudaGetLastError();
  if (g_last_err == FLETCHER_OK) g_last_err = code;
  if (g_errmode == FLETCHER_ERRMODE_EXIT) exit(1);
  return code;
}

}  // namespace

// Error reporting for other translation units of this library (same sticky
// status and error mode as the DRIVER_* entry points).
int flt_record_error(int code, const char *msg) { return fail(code, "%s", msg); }

namespace flt {
ResidentView resident_view() {
  ResidentView v;
  v.init = g.init && g.form == FLETCHER_FORM_FP32;
  if (!v.init) return v;
  v.sx = g.sx; v.sy = g.sy; v.sz = g.sz; v.bord = g.bord; v.pitch = g.pitch;
  v.dx = g.dx; v.dy = g.dy; v.dz = g.dz; v.dt = g.dt;
  v.cur = g.F[g.cur];
  v.prev = g.F[1 - g.cur];
  v.next = g.F[1 - g.cur];
  v.coef = g.coef;
  v.stream = g_stream;
  v.num_sms = g.num_sms;
  v.err = g.err_dev;
  return v;
}
}  // namespace flt

namespace {

// A failed call is recorded in the library's status; the runtime's own
// last-error state is cleared (for the errors that are not sticky), so a
// later launch check does not report it again.
#define CK(call)                                                                                   \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) {                                                                       \
      cudaGetLastError();                                                                          \
      return fail(e_ == cudaErrorMemoryAllocation ? FLETCHER_ERR_NOMEM : FLETCHER_ERR_CUDA,       \
                  "%s failed at %s:%d: %s", #call, __FILE__, __LINE__, cudaGetErrorString(e_));   \
    }                                                                                              \
  } while (0)

// Device allocation through the fault-injection countdown.
cudaError_t dev_malloc(void **p, size_t bytes) {
  if (g_fault_alloc >= 0 && g_fault_alloc-- == 0) {
    *p = nullptr;
    return cudaErrorMemoryAllocation;
  }
  return cudaMalloc(p, bytes);
}
template <class T>
cudaError_t dev_malloc(T **p, size_t bytes) {
  return dev_malloc(reinterpret_cast<void **>(p), bytes);
}

// ---- auxiliary kernels --------------------------------------------------------

// The six raw model arrays (vpz vsv epsilon delta phi theta): device copies,
// or the caller's host arrays where the GPU reads host memory directly.
struct Raw6 {
  const float *a[6];
};

// First model value that is not finite, as cell * 8 + array (vpz vsv epsilon
// delta phi theta); ~0 when every value is finite.  Set by k_precompute.
__device__ unsigned long long g_bad_model;
const char *const kModelNames[6] = {"vpz", "vsv", "epsilon", "delta", "phi", "theta"};

// Coefficient precompute, original/precomp.h:14-38 and :49-58: trigonometry
// in FP64 rounded to float, products of those floats in float, velocity
// terms in FP64.  A model value that is not finite is recorded in
// g_bad_model (the set-up then rejects the model).
__global__ void k_precompute(Raw6 raw, float *__restrict__ coef, int sx, int sy, int sz, int pitch) {
  const size_t n = (size_t)sx * sy * sz;
  // The trigonometry of the last angles this thread saw: media repeat their
  // angles over many cells (layers), and the same input gives the same floats.
  float last_theta = __int_as_float(0x7fbfffff), last_phi = __int_as_float(0x7fbfffff);  // a NaN pattern no input holds
  float sinTheta = 0.f, cosTheta = 0.f, sin2Theta = 0.f, sinPhi = 0.f, cosPhi = 0.f, sin2Phi = 0.f;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float vpz = raw.a[0][i], vsv = raw.a[1][i], eps = raw.a[2][i], del = raw.a[3][i];
    const float phi = raw.a[4][i], theta = raw.a[5][i];
    const float in6[6] = {vpz, vsv, eps, del, phi, theta};
#pragma unroll
    for (int a = 0; a < 6; ++a)
      if (!isfinite(in6[a])) {
        atomicMin(&g_bad_model, (unsigned long long)i * 8 + a);
        break;
      }
    if (__float_as_int(theta) != __float_as_int(last_theta)) {
      double st, ct;
      sincos((double)theta, &st, &ct);
      sinTheta = (float)st;
      cosTheta = (float)ct;
      sin2Theta = (float)sin(__dmul_rn(2.0, (double)theta));
      last_theta = theta;
    }
    if (__float_as_int(phi) != __float_as_int(last_phi)) {
      double sp, cp;
      sincos((double)phi, &sp, &cp);
      sinPhi = (float)sp;
      cosPhi = (float)cp;
      sin2Phi = (float)sin(__dmul_rn(2.0, (double)phi));
      last_phi = phi;
    }
    const float v2sz = __fmul_rn(vsv, vsv);
    const float v2pz = __fmul_rn(vpz, vpz);
    const float v2px = (float)__dmul_rn((double)v2pz, __dadd_rn(1.0, __dmul_rn(2.0, (double)eps)));
    const float v2pn = (float)__dmul_rn((double)v2pz, __dadd_rn(1.0, __dmul_rn(2.0, (double)del)));
    float c[kNumCoef];
    c[DC_XX] = __fmul_rn(__fmul_rn(__fmul_rn(sinTheta, sinTheta), cosPhi), cosPhi);
    c[DC_YY] = __fmul_rn(__fmul_rn(__fmul_rn(sinTheta, sinTheta), sinPhi), sinPhi);
    c[DC_XY] = __fmul_rn(__fmul_rn(sinTheta, sinTheta), sin2Phi);
    c[DC_ZZ] = __fmul_rn(cosTheta, cosTheta);
    c[DC_XZ] = __fmul_rn(sin2Theta, cosPhi);
    c[DC_YZ] = __fmul_rn(sin2Theta, sinPhi);
    c[DC_V2PX] = v2px;
    c[DC_V2PZ] = v2pz;
    c[DC_V2SZ] = v2sz;
    c[DC_V2PN] = v2pn;
    const size_t x = i % sx, y = (i / sx) % sy, z = i / ((size_t)sx * sy);
#pragma unroll
    for (int k = 0; k < kNumCoef; ++k) coef[((z * kNumCoef + k) * sy + y) * pitch + x] = c[k];
  }
}

// Media table, first pass: each cell's (phi, theta) bit pair gets a slot of
// a 256-slot open-addressing table (keys: phi bits << 32 | theta bits), and
// the slot is the cell's one-byte id.  A slot is claimed by compare-and-swap
// from `kEmptyKey` (a NaN pair, which the set-up rejects anyway); its claimer
// records itself as the slot's representative cell.  `full` is set when a
// pair finds no slot (more than 256 pairs: the layout is not used).
constexpr unsigned long long kEmptyKey = ~0ull;
__global__ void k_media_ids(const float *__restrict__ phi, const float *__restrict__ theta, unsigned char *ids,
                            unsigned long long *keys, unsigned long long *rep, unsigned *full, int sx, int sy,
                            int sz, int ipitch) {
  const size_t n = (size_t)sx * sy * sz;
  unsigned long long last_key = kEmptyKey;
  int last_id = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const unsigned long long key =
        ((unsigned long long)__float_as_uint(phi[i]) << 32) | __float_as_uint(theta[i]);
    int id = last_id;
    if (key != last_key) {
      unsigned long long h = key * 0x9E3779B97F4A7C15ull;
      int slot = (int)(h >> 56);
      id = -1;
      for (int probe = 0; probe < kMediaMax; ++probe, slot = (slot + 1) & (kMediaMax - 1)) {
        const unsigned long long v = *(volatile unsigned long long *)&keys[slot];
        if (v == key) {
          id = slot;
          break;
        }
        if (v == kEmptyKey) {
          const unsigned long long old = atomicCAS(&keys[slot], kEmptyKey, key);
          if (old == kEmptyKey) rep[slot] = i;
          if (old == kEmptyKey || old == key) {
            id = slot;
            break;
          }
        }
      }
      if (id < 0) {
        atomicOr(full, 1u);
        id = 0;
      }
      last_key = key;
      last_id = id;
    }
    const size_t x = i % sx, yz = i / sx;
    ids[yz * ipitch + x + kIdShift] = (unsigned char)id;
  }
}

// Media table, second pass: the angle coefficients of each claimed slot,
// copied from its representative cell's coefficient planes (so the table
// holds exactly the floats of the plane layout).
__global__ void k_media_table(const unsigned long long *keys, const unsigned long long *rep,
                              const float *__restrict__ coef, float *tab, int sx, int sy, int pitch) {
  const int slot = threadIdx.x;
  const bool used = keys[slot] != kEmptyKey;
  const size_t i = used ? rep[slot] : 0;
  const size_t x = i % sx, y = (i / sx) % sy, z = i / ((size_t)sx * sy);
  for (int k = 0; k < kAngleCoef; ++k)
    tab[k * kMediaMax + slot] = used ? coef[((z * kNumCoef + k) * sy + y) * pitch + x] : 0.f;
}

// (p, q) volumes -> pitched pair buffer.  Null p or q gives zeros.
__global__ void k_pack(const float *__restrict__ p, const float *__restrict__ q, float2 *__restrict__ F, int sx,
                       int sy, int sz, int pitch) {
  const size_t n = (size_t)sx * sy * sz;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t x = i % sx, yz = i / sx;
    F[yz * pitch + x] = make_float2(p ? p[i] : 0.f, q ? q[i] : 0.f);
  }
}

// One component of a pitched pair buffer -> unpitched volume.
__global__ void k_unpack(const float2 *__restrict__ F, float *__restrict__ out, int comp, int sx, int sy, int sz,
                         int pitch) {
  const size_t n = (size_t)sx * sy * sz;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t x = i % sx, yz = i / sx;
    const float2 v = F[yz * pitch + x];
    out[i] = comp ? v.y : v.x;
  }
}

// Coefficient k of the device block -> unpitched volume.
__global__ void k_unpack_coef(const float *__restrict__ coef, float *__restrict__ out, int k, int sx, int sy, int sz,
                              int pitch) {
  const size_t n = (size_t)sx * sy * sz;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const size_t x = i % sx, y = (i / sx) % sy, z = i / ((size_t)sx * sy);
    out[i] = coef[((z * kNumCoef + k) * sy + y) * pitch + x];
  }
}

// Test aid: writes v into the pitch padding (columns sx .. pitch-1) of
// `rows` rows of `width` floats per cell.
__global__ void k_poison_pad(float *buf, int width, int sx, int pitch, long rows, float v) {
  const long pad = (long)(pitch - sx) * width;
  const long n = rows * pad;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const long r = i / pad, c = i % pad;
    buf[r * (long)pitch * width + (long)sx * width + c] = v;
  }
}

// Adds val to both fields of one cell (source outside the fused path).
__global__ void k_add_source(float2 *F, size_t idx, float val) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    float2 v = F[idx];
    v.x = v.x + val;
    v.y = v.y + val;
    F[idx] = v;
  }
}

// ---- helpers -------------------------------------------------------------------

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

int encode(CUtensorMap *m, CUtensorMapDataType dt, int rank, void *base, const cuuint64_t *dims,
           const cuuint64_t *strides, const cuuint32_t *box) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return fail(FLETCHER_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  cuuint32_t es[5] = {1, 1, 1, 1, 1};
  CUresult r = fn(m, dt, (cuuint32_t)rank, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(FLETCHER_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return FLETCHER_OK;
}

int grid_for(size_t n) {
  size_t b = (n + 255) / 256;
  const size_t cap = (size_t)(g.num_sms > 0 ? g.num_sms : 148) * 16;
  return (int)(b < cap ? (b ? b : 1) : cap);
}

// Chooses the number of z-chunks: balances the persistent CTAs' last round
// against the 8 warm-up planes each chunk re-reads.
// Work split of one shot among `ctas` persistent CTAs, as segments {x0, y0,
// z0, z1} (a z range of one tile column) listed CTA by CTA.  The tiles
// (x fastest) are cut into z-chunks; the chunk-major items fill whole rounds
// of `ctas` (CTA b takes items b, b + ctas, ...: CTAs side by side work on
// neighbouring tiles at the same depth and share their halo rows through
// L2).  With `spread`, each item of the last, partial round is then cut into
// equal z pieces of at least kMinPiece planes, as many as lets every CTA
// take at most one piece; without it the partial round stays round-robin.
// The plan (chunk count 1..16 or `req`, spread or not) minimises the busiest
// CTA's cost: its planes plus kHaloCost a segment for the 8 halo planes,
// shared-out pieces counting 3/2 (measured on GB300 at 280^3, 328^3 and
// 576^3: the pieces of neighbouring tiles run at different depths and lose
// their L2 halo sharing); a spread plan must beat the best round-robin one
// by 3%.
constexpr int kMinPiece = 8;
constexpr int kHaloCost = 4;

struct Split {
  std::vector<int4> seg;
  std::vector<int> first;
  long max_cost = 0, total_cost = 0;
  bool spread = false;  // false: uniform chunks of `len` planes, all round-robin
  int len = 0;
};

Split split_work(int ctas, int ntx, int nty, int TY, int zlo, int depth, int nchunk, bool spread = true) {
  const int ntiles = ntx * nty;
  const int len = (depth + nchunk - 1) / nchunk;
  const int cc = (depth + len - 1) / len;
  const long items = (long)ntiles * cc;
  const long full = spread ? items / ctas * ctas : items;
  auto tile_x0 = [&](long t) { return kRadius + (int)(t % ntx) * kTileX; };
  auto tile_y0 = [&](long t) { return kRadius + (int)(t / ntx) * TY; };
  auto item_z = [&](long i, int *z0, int *z1) {
    const int ch = (int)(i / ntiles);
    *z0 = ch * len;
    *z1 = std::min(depth, *z0 + len);
  };
  std::vector<std::vector<int4>> per(ctas);
  std::vector<long> cost(ctas, 0);
  for (long i = 0; i < full; ++i) {
    int z0, z1;
    item_z(i, &z0, &z1);
    const long t = i % ntiles;
    per[i % ctas].push_back(make_int4(tile_x0(t), tile_y0(t), zlo + z0, zlo + z1));
    cost[i % ctas] += 2 * ((z1 - z0) + kHaloCost);  // costs in half planes
  }
  // The partial round: each of its items cut into p equal z pieces (at
  // least kMinPiece planes, p * items <= ctas), one piece per CTA.
  const long rem = items - full;
  if (rem > 0) {
    const long p = std::max(1L, std::min((long)ctas / rem, (long)len / kMinPiece));
    long b = 0;
    for (long i = full; i < items; ++i) {
      int z0, z1;
      item_z(i, &z0, &z1);
      const long t = i % ntiles, n = z1 - z0;
      for (long j = 0; j < p; ++j, ++b) {
        const int a0 = z0 + (int)(n * j / p), a1 = z0 + (int)(n * (j + 1) / p);
        if (a1 <= a0) continue;
        per[b % ctas].push_back(make_int4(tile_x0(t), tile_y0(t), zlo + a0, zlo + a1));
        cost[b % ctas] += 3 * ((a1 - a0) + kHaloCost);
      }
    }
  }
  Split sp;
  sp.spread = full < items;
  sp.len = len;
  sp.first.push_back(0);
  for (int b = 0; b < ctas; ++b) {
    sp.seg.insert(sp.seg.end(), per[b].begin(), per[b].end());
    sp.first.push_back((int)sp.seg.size());
    sp.max_cost = std::max(sp.max_cost, cost[b] / 2);
    sp.total_cost += cost[b] / 2;
  }
  return sp;
}

Split plan_segments(int ctas, int ntx, int nty, int TY, int zlo, int depth, int req) {
  if (req > 0) return split_work(ctas, ntx, nty, TY, zlo, depth, std::min(req, depth));
  if (req < 0) return split_work(ctas, ntx, nty, TY, zlo, depth, std::min(-req, depth), false);
  Split best[2];  // round-robin, spread
  for (int c = 1; c <= 16 && c <= depth; ++c)
    for (int spread = 0; spread < 2; ++spread) {
      Split sp = split_work(ctas, ntx, nty, TY, zlo, depth, c, spread != 0);
      Split &b = best[spread];
      if (b.first.empty() || sp.max_cost < b.max_cost || (sp.max_cost == b.max_cost && sp.total_cost < b.total_cost))
        b = std::move(sp);
    }
  // Round-robin keeps neighbouring tiles in step for L2 and measured faster
  // at 504^3 than a spread plan the model rates 1% cheaper: spread only when
  // it saves more than 3%.
  return best[1].max_cost * 100 < best[0].max_cost * 97 ? best[1] : best[0];
}

int check_dims(int sx, int sy, int sz) {
  if (!g.init) return fail(FLETCHER_ERR_ARGS, "DRIVER_Initialize has not been called");
  if (sx != g.sx || sy != g.sy || sz != g.sz)
    return fail(FLETCHER_ERR_ARGS, "grid %dx%dx%d differs from the initialised %dx%dx%d", sx, sy, sz, g.sx, g.sy,
                g.sz);
  return FLETCHER_OK;
}

size_t pitched_index(long idx) {
  const long x = idx % g.sx, yz = idx / g.sx;
  return (size_t)yz * g.pitch + x;
}

bool in_update_region(long idx) {
  const long x = idx % g.sx, y = (idx / g.sx) % g.sy, z = idx / ((long)g.sx * g.sy);
  return x >= g.bord && x < g.sx - g.bord && y >= g.bord && y < g.sy - g.bord && z >= g.bord && z < g.sz - g.bord;
}

bool half_form() { return g.form == FLETCHER_FORM_FP16 || g.form == FLETCHER_FORM_FP16X; }

int check_err_word() {
  const unsigned w = g.err_host ? *(volatile unsigned *)g.err_host : 0u;
  if (w & 3u)
    return fail(FLETCHER_ERR_TIMEOUT, "a propagate kernel gave up waiting for its data (error word 0x%x)", w);
  if (w & 4u) return fail(FLETCHER_ERR_RANGE, "a stored value exceeded FP16's range (error word 0x%x)", w);
  return FLETCHER_OK;
}

void free_state() {
  tune.active = false;
  abc_release_resident();
  snapshot_release();
  if (g.F[0]) cudaFree(g.F[0]);
  if (g.F[1]) cudaFree(g.F[1]);
  if (g.coef) cudaFree(g.coef);
  if (g.scratch) cudaFree(g.scratch);
  for (int b = 0; b < 2; ++b) {
    if (g.Hh[b]) cudaFree(g.Hh[b]);
    if (g.Hl[b]) cudaFree(g.Hl[b]);
  }
  if (g.E) cudaFree(g.E);
  if (g.Mx) cudaFree(g.Mx);
  if (g.seg) cudaFree(g.seg);
  if (g.cta_first) cudaFree(g.cta_first);
  if (g.err_host) cudaFreeHost(g.err_host);
  if (g.ids) cudaFree(g.ids);
  if (g.mtab) cudaFree(g.mtab);
  if (g.mwork) cudaFree(g.mwork);
  g = State();
}

// Page-locks caller arrays for the duration of copies between them and the
// device: from or to pageable memory the driver stages a copy through its
// own buffers at a fraction of the link's speed (on GB300 about 10 GB/s,
// against a few ms per GB to lock and unlock).  An array that cannot be
// locked (already locked, or not lockable) is copied as it is.  Unlocked,
// after the stream's copies, when the object goes out of scope.
struct HostPins {
  void *p[10] = {};
  int n = 0;
  // `dest`: the device writes the array (read-back); otherwise it only reads it.
  void add(const void *a, size_t bytes, bool dest = false) {
    if (!a || !bytes || n == 10) return;
    void *q = const_cast<void *>(a);
    if (dest || cudaHostRegister(q, bytes, cudaHostRegisterReadOnly) != cudaSuccess) {
      cudaGetLastError();
      if (cudaHostRegister(q, bytes, cudaHostRegisterDefault) != cudaSuccess) {
        cudaGetLastError();
        return;
      }
    }
    p[n++] = q;
  }
  ~HostPins() {
    if (n && g_stream) cudaStreamSynchronize(g_stream);
    for (int k = 0; k < n; ++k) cudaHostUnregister(p[k]);
    cudaGetLastError();
  }
};

int ensure_stream() {
  if (!g_stream) {
    CK(cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking));
    g_own_stream = true;
  }
  return FLETCHER_OK;
}

}  // namespace

namespace flt {

// The six TMA descriptors of one shot: both field buffers with the halo box
// and the point box, and the coefficient block with the 3- and 7-coefficient
// boxes.
int build_maps(ShotMaps *m, float2 *const F[2], float *coef, int sx, int sy, int sz, int pitch, int TY) {
  const cuuint64_t dims[3] = {(cuuint64_t)sx, (cuuint64_t)sy, (cuuint64_t)sz};
  const cuuint64_t str[2] = {(cuuint64_t)pitch * 8, (cuuint64_t)pitch * sy * 8};
  const cuuint32_t hbox[3] = {(cuuint32_t)(kTileX + 2 * kRadius), (cuuint32_t)(TY + 2 * kRadius), 1};
  const cuuint32_t pbox[3] = {(cuuint32_t)kTileX, (cuuint32_t)TY, 1};
  for (int b = 0; b < 2 && F[b]; ++b) {
    if (encode(&m->halo[b], CU_TENSOR_MAP_DATA_TYPE_INT64, 3, F[b], dims, str, hbox)) return g_last_err;
    if (encode(&m->pt[b], CU_TENSOR_MAP_DATA_TYPE_INT64, 3, F[b], dims, str, pbox)) return g_last_err;
  }
  const cuuint64_t cdims[4] = {(cuuint64_t)sx, (cuuint64_t)sy, (cuuint64_t)kNumCoef, (cuuint64_t)sz};
  const cuuint64_t cstr[3] = {(cuuint64_t)pitch * 4, (cuuint64_t)pitch * sy * 4,
                              (cuuint64_t)pitch * sy * kNumCoef * 4};
  const cuuint32_t abox[4] = {(cuuint32_t)kTileX, (cuuint32_t)TY, (cuuint32_t)kArrivalCoef, 1};
  const cuuint32_t ubox[4] = {(cuuint32_t)kTileX, (cuuint32_t)TY, (cuuint32_t)kUpdateCoef, 1};
  if (encode(&m->arr, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, coef, cdims, cstr, abox)) return g_last_err;
  if (encode(&m->upd, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, coef, cdims, cstr, ubox)) return g_last_err;
  return FLETCHER_OK;
}

// TMA descriptors of the 16-bit forms: for each choice of current buffer c,
// the current field's halo boxes and the previous field's point boxes, plus
// the coefficient boxes.
int build_half_maps(HalfMaps hm[2], unsigned *const Hh[2], unsigned short *const Hl[2], const ShotMaps &fm, int sx,
                    int sy, int sz, int pitch, int TY) {
  const cuuint64_t dims[3] = {(cuuint64_t)sx, (cuuint64_t)sy, (cuuint64_t)sz};
  const cuuint64_t sh[2] = {(cuuint64_t)pitch * 4, (cuuint64_t)pitch * sy * 4};
  const cuuint64_t sl[2] = {(cuuint64_t)pitch * 2, (cuuint64_t)pitch * sy * 2};
  const cuuint32_t hbox[3] = {(cuuint32_t)(kTileX + 2 * kRadius), (cuuint32_t)(TY + 2 * kRadius), 1};
  const cuuint32_t pbox[3] = {(cuuint32_t)kTileX, (cuuint32_t)TY, 1};
  const cuuint32_t lbox[3] = {(cuuint32_t)(kTileX + 2 * kRadius), (cuuint32_t)TY, 1};
  for (int c = 0; c < 2; ++c) {
    const int p = 1 - c;
    HalfMaps &m = hm[c];
    memset(&m, 0, sizeof(m));
    if (encode(&m.cur_hi, CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, Hh[c], dims, sh, hbox)) return g_last_err;
    if (encode(&m.prev_hi, CU_TENSOR_MAP_DATA_TYPE_UINT32, 3, Hh[p], dims, sh, pbox)) return g_last_err;
    if (Hl[c]) {
      if (encode(&m.cur_lo, CU_TENSOR_MAP_DATA_TYPE_UINT16, 3, Hl[c], dims, sl, hbox)) return g_last_err;
      if (encode(&m.prev_lo, CU_TENSOR_MAP_DATA_TYPE_UINT16, 3, Hl[p], dims, sl, lbox)) return g_last_err;
    }
    m.arr = fm.arr;
    m.upd = fm.upd;
  }
  return FLETCHER_OK;
}

// Work items of one shot, chunk-major then rows then columns, so CTAs that
// run at the same time work on neighbouring tiles of the same z range.
void fill_items(int4 *items, int shot, int ntx, int nty, int nchunk, int TY) {
  int n = 0;
  for (int c = 0; c < nchunk; ++c)
    for (int ty = 0; ty < nty; ++ty)
      for (int tx = 0; tx < ntx; ++tx) items[n++] = make_int4(shot, kRadius + tx * kTileX, kRadius + ty * TY, c);
}

}  // namespace flt

namespace {

// Tensor maps, work items and the shot descriptor for a tile shape (at
// initialisation, or between steps: results do not depend on the shape).
int setup_tiles(int rows, int stages) {
  const int TY = rows, sx = g.sx, sy = g.sy, sz = g.sz, bord = g.bord;
  if (g.media && !propagate_fp32_media_supported(rows, stages))
    return fail(FLETCHER_ERR_ARGS, "tile shape (%d rows, %d stages) is not built for the media-table layout", rows,
                stages);
  if (build_maps(&g.maps, g.F, g.coef, sx, sy, sz, g.pitch, TY)) return g_last_err;
  if (g.media) {
    const cuuint64_t idims[3] = {(cuuint64_t)(sx + kIdShift), (cuuint64_t)sy, (cuuint64_t)sz};
    const cuuint64_t istr[2] = {(cuuint64_t)g.ipitch, (cuuint64_t)g.ipitch * sy};
    const cuuint32_t ibox[3] = {(cuuint32_t)kTileX, (cuuint32_t)TY, 1};
    if (encode(&g.mids, CU_TENSOR_MAP_DATA_TYPE_UINT8, 3, g.ids, idims, istr, ibox)) return g_last_err;
    const cuuint64_t cdims[4] = {(cuuint64_t)sx, (cuuint64_t)sy, (cuuint64_t)kNumCoef, (cuuint64_t)sz};
    const cuuint64_t cstr[3] = {(cuuint64_t)g.pitch * 4, (cuuint64_t)g.pitch * sy * 4,
                                (cuuint64_t)g.pitch * sy * kNumCoef * 4};
    const cuuint32_t vbox[4] = {(cuuint32_t)kTileX, (cuuint32_t)TY, (cuuint32_t)kVelCoef, 1};
    if (encode(&g.mvel, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, g.coef, cdims, cstr, vbox)) return g_last_err;
  }
  if (half_form() && build_half_maps(g.hm, g.Hh, g.Hl, g.maps, sx, sy, sz, g.pitch, TY)) return g_last_err;
  g.tile_rows = rows;
  g.stages = stages;
  g.ntx = (sx - bord - kRadius + kTileX - 1) / kTileX;
  g.nty = (sy - bord - kRadius + TY - 1) / TY;
  const int per_sm = half_form() ? propagate_half_ctas_per_sm(TY, stages, g.form == FLETCHER_FORM_FP16X, false)
                                  : propagate_fp32_ctas_per_sm(TY);
  if (per_sm < 1) return fail(FLETCHER_ERR_CUDA, "tile shape (%d rows, %d stages) fits no CTA on an SM", TY, stages);
  const int ctas = g.num_sms * per_sm;
  const Split sp = plan_segments(ctas, g.ntx, g.nty, TY, bord, sz - 2 * bord, g.zchunks);
  if (g.seg) cudaFree(g.seg);
  if (g.cta_first) cudaFree(g.cta_first);
  g.seg = nullptr;
  g.cta_first = nullptr;
  CK(dev_malloc(&g.seg, sp.seg.size() * sizeof(int4)));
  CK(dev_malloc(&g.cta_first, sp.first.size() * sizeof(int)));
  CK(cudaMemcpy(g.seg, sp.seg.data(), sp.seg.size() * sizeof(int4), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(g.cta_first, sp.first.data(), sp.first.size() * sizeof(int), cudaMemcpyHostToDevice));
  // CTAs past the last one with work are not launched.
  int grid = ctas;
  while (grid > 1 && sp.first[grid - 1] == sp.first[grid]) --grid;
  g.seg_grid = grid;
  g.nseg = (int)sp.seg.size();
  g.spread = sp.spread;
  if (sp.spread) {
    g.nitems = g.nseg;
    g.grid = grid;
    g.chunk = 0;
  } else {
    // A round-robin plan: the FP32 kernel decodes its items arithmetically
    // (tiles x chunks of `len` planes, chunk-major), no list lookups.
    g.chunk = sp.len;
    g.nitems = g.ntx * g.nty * ((sz - 2 * bord + sp.len - 1) / sp.len);
    g.grid = std::min(g.nitems, ctas);
  }
  memset(&g.desc, 0, sizeof(g.desc));
  g.desc.F[0] = g.F[0];
  g.desc.F[1] = g.F[1];
  g.desc.sx = sx; g.desc.sy = sy; g.desc.sz = sz; g.desc.pitch = g.pitch; g.desc.bord = bord;
  g.desc.ntx = g.ntx; g.desc.nty = g.nty; g.desc.chunk = g.chunk;
  g.desc.src_x = g.desc.src_y = g.desc.src_z = -1000;
  g.desc.cor_x = g.desc.cor_y = g.desc.cor_z = -1000;
  return FLETCHER_OK;
}

int initialize(int sx, int sy, int sz, int bord, float dx, float dy, float dz, float dt, const float *vpz,
               const float *vsv, const float *epsilon, const float *delta, const float *phi, const float *theta,
               const float *pp, const float *pc, const float *qp, const float *qc) {
  if (g.init) free_state();
  if (bord < kRadius) return fail(FLETCHER_ERR_ARGS, "bord (%d) must be at least the stencil radius %d", bord, kRadius);
  if (sx <= 2 * bord || sy <= 2 * bord || sz <= 2 * bord)
    return fail(FLETCHER_ERR_ARGS, "grid %dx%dx%d has no interior for bord %d", sx, sy, sz, bord);
  if (!(dx > 0.f) || !(dy > 0.f) || !(dz > 0.f)) return fail(FLETCHER_ERR_ARGS, "grid spacing must be positive");
  if (!vpz || !vsv || !epsilon || !delta || !phi || !theta)
    return fail(FLETCHER_ERR_ARGS, "model arrays must not be NULL");
  if (g_form < FLETCHER_FORM_FP32 || g_form > FLETCHER_FORM_FP16X)
    return fail(FLETCHER_ERR_ARGS, "unknown storage form %d", g_form);
  const bool half = g_form != FLETCHER_FORM_FP32;
  const bool ext = g_form == FLETCHER_FORM_FP16X;
  // Default shapes (measured at 504^3): 16 rows; 5 stages for FP32 (2.20 ms
  // per step against 2.40 for 12 x 5) and FP16X (3.45 against 3.68 for 16 x 4),
  // 4 for FP16 (3.02 against 3.18 for 16 x 5).
  if (g_numerics == FLETCHER_NUMERICS_D1D1 && g_form != FLETCHER_FORM_FP32)
    return fail(FLETCHER_ERR_ARGS, "the Der1-Der1 numerics need the FP32 form");
  const bool d1d1 = g_numerics == FLETCHER_NUMERICS_D1D1;
  if (d1d1 && (g_req_rows || g_req_stages) && (g_req_rows != kD1D1Rows || g_req_stages != kD1D1Stages))
    return fail(FLETCHER_ERR_ARGS, "the Der1-Der1 numerics run %d x %d tiles only", kD1D1Rows, kD1D1Stages);
  if (g_coef_layout == FLETCHER_COEF_MEDIA && (half || d1d1))
    return fail(FLETCHER_ERR_ARGS, "the media-table layout needs the FP32 form and the default numerics");
  int rows = d1d1 ? kD1D1Rows : (g_req_rows ? g_req_rows : 16);
  int stages = d1d1 ? kD1D1Stages : (g_req_stages ? g_req_stages : (g_form == FLETCHER_FORM_FP16 ? 4 : 5));
  // The media-table layout, where the form and the tile shape allow it (its
  // default shape: 16 rows, kMediaStages stages).
  const int mrows = g_req_rows ? g_req_rows : 16, mstages = g_req_stages ? g_req_stages : kMediaStages;
  const bool want_media = !half && !d1d1 && g_coef_layout != FLETCHER_COEF_PLANES &&
                          propagate_fp32_media_supported(mrows, mstages);
  if (g_coef_layout == FLETCHER_COEF_MEDIA && !want_media)
    return fail(FLETCHER_ERR_ARGS, "tile shape (%d rows, %d stages) is not built for the media-table layout", mrows,
                mstages);
  if (!(half ? propagate_half_supported(rows, stages) : propagate_fp32_supported(rows, stages) || want_media))
    return fail(FLETCHER_ERR_ARGS, "tile shape (%d rows, %d stages) is not built for form %d", rows, stages, g_form);
  if (half) {
    // The 16-bit forms rescale every plane each step, so the cells that are
    // never written must hold zero.
    const float *f4[4] = {pp, pc, qp, qc};
    for (int a = 0; a < 4; ++a) {
      if (!f4[a]) continue;
      for (long z = 0; z < sz; ++z)
        for (long y = 0; y < sy; ++y) {
          const bool inner = z >= bord && z < sz - bord && y >= bord && y < sy - bord;
          for (long x = 0; x < sx; x = (inner && x == bord - 1) ? sx - bord : x + 1)
            if (f4[a][(z * sy + y) * sx + x] != 0.0f)
              return fail(FLETCHER_ERR_ARGS,
                          "16-bit forms need zero initial fields outside the updated region (cell %ld)",
                          (z * sy + y) * sx + x);
        }
    }
  }
  if (ensure_stream()) return g_last_err;

  int dev = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&g.num_sms, cudaDevAttrMultiProcessorCount, dev));
  g.sx = sx; g.sy = sy; g.sz = sz; g.bord = bord;
  g.dx = dx; g.dy = dy; g.dz = dz; g.dt = dt;
  g.pitch = (sx + 31) / 32 * 32;
  g.n = (size_t)sx * sy * sz;
  g.npitch = (size_t)g.pitch * sy * sz;
  g.tile_rows = rows;
  g.stages = stages;
  g.zchunks = g_req_chunks;

  cudaStream_t s = g_stream;

  g.form = g_form;
  g.numerics = g_numerics;
  if (half) {
    for (int b = 0; b < 2; ++b) {
      CK(dev_malloc(&g.Hh[b], g.npitch * sizeof(unsigned)));
      CK(cudaMemsetAsync(g.Hh[b], 0, g.npitch * sizeof(unsigned), s));
      if (ext) {
        CK(dev_malloc(&g.Hl[b], g.npitch * sizeof(unsigned short)));
        CK(cudaMemsetAsync(g.Hl[b], 0, g.npitch * sizeof(unsigned short), s));
      }
    }
    CK(dev_malloc(&g.E, 3 * sz * sizeof(int)));
    CK(dev_malloc(&g.Mx, 2 * sz * sizeof(unsigned)));
    CK(cudaMemsetAsync(g.E, 0, 3 * sz * sizeof(int), s));
    CK(cudaMemsetAsync(g.Mx, 0, 2 * sz * sizeof(unsigned), s));
    g.dev_bytes = 2 * g.npitch * (sizeof(unsigned) + (ext ? sizeof(unsigned short) : 0)) + 5 * sz * sizeof(int);
  } else {
    CK(dev_malloc(&g.F[0], g.npitch * sizeof(float2)));
    CK(dev_malloc(&g.F[1], g.npitch * sizeof(float2)));
    CK(cudaMemsetAsync(g.F[0], 0, g.npitch * sizeof(float2), s));
    CK(cudaMemsetAsync(g.F[1], 0, g.npitch * sizeof(float2), s));
    g.dev_bytes = 2 * g.npitch * sizeof(float2);
  }
  CK(dev_malloc(&g.coef, g.npitch * kNumCoef * sizeof(float)));
  CK(dev_malloc(&g.scratch, g.n * sizeof(float)));
  CK(cudaHostAlloc(&g.err_host, sizeof(unsigned), cudaHostAllocMapped));
  *g.err_host = 0;
  CK(cudaHostGetDevicePointer((void **)&g.err_dev, g.err_host, 0));
  g.dev_bytes += g.npitch * kNumCoef * sizeof(float) + g.n * sizeof(float);
  CK(cudaMemsetAsync(g.coef, 0, g.npitch * kNumCoef * sizeof(float), s));
  g_init_mark[1] = now_s();

  // Raw model arrays -> coefficients.  On systems whose GPU reads pageable
  // host memory (Grace over NVLink-C2C) the kernels read the caller's arrays
  // in place; elsewhere they go through a temporary 6-volume device buffer.
  int pma = 0;
  CK(cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, dev));
  g.hostmem = pma && g_host_access == 1;
  float *raw = nullptr;
  const float *src6[6] = {vpz, vsv, epsilon, delta, phi, theta};
  Raw6 r6;
  HostPins pins;
  if (g.hostmem) {
    for (int k = 0; k < 6; ++k) r6.a[k] = src6[k];
  } else {
    CK(dev_malloc(&raw, 6 * g.n * sizeof(float)));
    // Each array is locked while the copies before it run.
    for (int k = 0; k < 6; ++k) {
      pins.add(src6[k], g.n * sizeof(float));
      CK(cudaMemcpyAsync(raw + k * g.n, src6[k], g.n * sizeof(float), cudaMemcpyHostToDevice, s));
      r6.a[k] = raw + k * g.n;
    }
    for (const float *f : {pp, pc, qp, qc}) pins.add(f, g.n * sizeof(float));
  }
  g_init_mark[2] = now_s();
  const unsigned long long all_finite = ~0ull;
  CK(cudaMemcpyToSymbolAsync(g_bad_model, &all_finite, sizeof(all_finite), 0, cudaMemcpyHostToDevice, s));
  k_precompute<<<grid_for(g.n), 256, 0, s>>>(r6, g.coef, sx, sy, sz, g.pitch);
  CK(cudaGetLastError());
  // Media table: ids from the raw angles, then the table from the planes.
  unsigned long long *&mwork = g.mwork;
  if (want_media) {
    g.ipitch = (sx + kIdShift + 15) / 16 * 16;
    const size_t ibytes = (size_t)g.ipitch * sy * sz;
    CK(dev_malloc(&g.ids, ibytes));
    CK(dev_malloc(&g.mtab, kAngleCoef * kMediaMax * sizeof(float)));
    CK(dev_malloc(&mwork, (2 * kMediaMax + 1) * sizeof(unsigned long long)));
    g.dev_bytes += ibytes + kAngleCoef * kMediaMax * sizeof(float);
    CK(cudaMemsetAsync(g.ids, 0, ibytes, s));
    CK(cudaMemsetAsync(mwork, 0xff, kMediaMax * sizeof(unsigned long long), s));
    CK(cudaMemsetAsync(mwork + 2 * kMediaMax, 0, sizeof(unsigned long long), s));
    k_media_ids<<<grid_for(g.n), 256, 0, s>>>(r6.a[4], r6.a[5], g.ids, mwork, mwork + kMediaMax,
                                               reinterpret_cast<unsigned *>(mwork + 2 * kMediaMax), sx, sy, sz,
                                               g.ipitch);
    CK(cudaGetLastError());
    k_media_table<<<1, kMediaMax, 0, s>>>(mwork, mwork + kMediaMax, g.coef, g.mtab, sx, sy, g.pitch);
    CK(cudaGetLastError());
  }
  // Initial fields (the reference's OpenMP back-end works on the caller's
  // arrays, so their contents are the initial state).
  g.cur = 0;
  g.ecur = 0;
  const float *fp[2][2] = {{pc, qc}, {pp, qp}};
  for (int b = 0; b < 2; ++b) {
    const float *p = fp[b][0], *q = fp[b][1];
    if (!g.hostmem) {
      // The coefficient kernel has finished with `raw` before these copies
      // (same stream).
      if (p) CK(cudaMemcpyAsync(raw, p, g.n * sizeof(float), cudaMemcpyHostToDevice, s));
      if (q) CK(cudaMemcpyAsync(raw + g.n, q, g.n * sizeof(float), cudaMemcpyHostToDevice, s));
      p = p ? raw : nullptr;
      q = q ? raw + g.n : nullptr;
    }
    if (half) {
      // Buffer 0 holds the current field (exponent slot 0), buffer 1 the
      // previous one (slot 2).
      CK(half_encode(p, q, g.Hh[b], g.Hl[b], g.E + (b ? 2 : 0) * sz, g.Mx + b * sz, sx, sy, sz, g.pitch, ext, s));
    } else {
      k_pack<<<grid_for(g.n), 256, 0, s>>>(p, q, g.F[b], sx, sy, sz, g.pitch);
      CK(cudaGetLastError());
    }
  }
  CK(cudaStreamSynchronize(s));
  g_init_mark[3] = now_s();
  if (raw) CK(cudaFree(raw));
  unsigned long long bad = 0;
  CK(cudaMemcpyFromSymbol(&bad, g_bad_model, sizeof(bad)));
  if (bad != ~0ull) {
    return fail(FLETCHER_ERR_ARGS, "model array %s holds a value that is not finite at cell %llu", kModelNames[bad % 8],
                bad / 8);
  }
  if (want_media) {
    unsigned long long over = 0;
    CK(cudaMemcpy(&over, mwork + 2 * kMediaMax, sizeof(over), cudaMemcpyDeviceToHost));
    cudaFree(mwork);
    mwork = nullptr;
    if (over && g_coef_layout == FLETCHER_COEF_MEDIA)
      return fail(FLETCHER_ERR_ARGS, "the model has more than %d distinct (phi, theta) pairs: no media table",
                  kMediaMax);
    if (over && !propagate_fp32_supported(rows, stages))
      return fail(FLETCHER_ERR_ARGS,
                  "tile shape (%d rows, %d stages) is built for the media-table layout only, which this model "
                  "(more than %d distinct (phi, theta) pairs) cannot use",
                  rows, stages, kMediaMax);
    if (over) {
      // More pairs than slots: the plane layout.
      cudaFree(g.ids);
      cudaFree(g.mtab);
      g.ids = nullptr;
      g.mtab = nullptr;
      g.dev_bytes -= (size_t)g.ipitch * sy * sz + kAngleCoef * kMediaMax * sizeof(float);
    } else {
      g.media = true;
      rows = mrows;
      stages = mstages;
    }
  }

  if (setup_tiles(rows, stages)) return g_last_err;
  g.launches = 0;
  g.pending = Source();
  g.owed = Source();
  g.init = true;
  g_init_mark[4] = now_s();
  return FLETCHER_OK;
}

const char *form_name(int form) {
  return form == FLETCHER_FORM_FP16    ? "fp16"
         : form == FLETCHER_FORM_FP16X ? "fp16x"
         : form == FLETCHER_TUNE_FP32_MEDIA ? "fp32-media"
                                       : "fp32";
}

// The tuning-file key of the current state: its storage form, or the FP32
// form in the media-table layout.
int tune_key() { return g.media ? FLETCHER_TUNE_FP32_MEDIA : g.form; }

int tune_before_step() {
  if (tune.left == 0) {
    if (setup_tiles(tune.rows[tune.idx], tune.stages[tune.idx])) return g_last_err;
    tune.left = tune.per_shape + 1;
  }
  if (tune.left == tune.per_shape) CK(cudaEventRecord(tune.e0, g_stream));
  return FLETCHER_OK;
}

int tune_after_step() {
  if (--tune.left > 0) return FLETCHER_OK;
  CK(cudaEventRecord(tune.e1, g_stream));
  CK(cudaEventSynchronize(tune.e1));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, tune.e0, tune.e1));
  tune.ms.push_back(ms / tune.per_shape);
  if (++tune.idx < tune.rows.size()) return FLETCHER_OK;
  size_t best = 0;
  for (size_t i = 1; i < tune.ms.size(); ++i)
    if (tune.ms[i] < tune.ms[best]) best = i;
  tune.active = false;
  if (setup_tiles(tune.rows[best], tune.stages[best])) return g_last_err;
  cudaDeviceProp prop;
  int dev = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaGetDeviceProperties(&prop, dev));
  return FLETCHER_TuneConfigStore(tune.path, prop.name, g.sx, tune_key(), tune.rows[best], tune.stages[best]);
}

// One step: source `pending` (if any) fused, then rotation.
int step() {
  if (tune.active && tune_before_step()) return g_last_err;
  PropLaunch L;
  const int c = g.cur, p = 1 - g.cur;
  L.tile_rows = g.tile_rows;
  L.stages = g.stages;
  L.grid = g.grid;
  L.batch = false;
  L.d1d1 = g.numerics == FLETCHER_NUMERICS_D1D1;
  L.media = g.media;
  L.m.cur_halo = g.maps.halo[c];
  L.m.prev_pt = g.maps.pt[p];
  L.m.arr = g.maps.arr;
  L.m.upd = g.maps.upd;
  if (g.media) {
    L.m.ids = g.mids;
    L.m.vel = g.mvel;
  }
  PropParams &P = L.p;
  P.media = g.mtab;
  P.shots = nullptr;
  P.maps = nullptr;
  P.items = nullptr;
  P.seg = g.spread ? g.seg : nullptr;
  P.cta_first = g.cta_first;
  P.nitems = g.nitems;
  P.parity = c;
  P.inv_dx = 1.0f / g.dx;
  P.inv_dy = 1.0f / g.dy;
  P.inv_dz = 1.0f / g.dz;
  P.inv_dxx = 1.0f / (g.dx * g.dx);
  P.inv_dyy = 1.0f / (g.dy * g.dy);
  P.inv_dzz = 1.0f / (g.dz * g.dz);
  P.inv_dxy = 1.0f / (g.dx * g.dy);
  P.inv_dxz = 1.0f / (g.dx * g.dz);
  P.inv_dyz = 1.0f / (g.dy * g.dz);
  // On an isotropic grid every derivative carries the same 1/h^2, applied
  // once with the time step; otherwise each derivative is scaled.
  P.iso = (g.dx == g.dy && g.dx == g.dz) ? 1 : 0;
  P.dt2 = P.iso ? (g.dt * g.dt) * P.inv_dxx : g.dt * g.dt;
  P.dt = g.dt;
  P.err = g.err_dev;
  // Every wait is bounded (2 s); an injected stall (tests) uses its own limit
  // and applies to this one launch.
  P.wait_ns = g_fault_stall >= 0 && g_fault_wait_ns ? g_fault_wait_ns : kWaitLimitNs;
  P.stall_step = g_fault_stall;
  g_fault_stall = -1;
  ShotDesc &want = P.one;
  want = g.desc;
  want.src_x = want.src_y = want.src_z = -1000;
  want.cor_x = want.cor_y = want.cor_z = -1000;
  P.src = 0.f;
  P.cor = 0.f;
  bool fused = false;
  if (g.pending.on) {
    if (in_update_region(g.pending.idx)) {
      const long i = g.pending.idx;
      want.src_x = (int)(i % g.sx);
      want.src_y = (int)((i / g.sx) % g.sy);
      want.src_z = (int)(i / ((long)g.sx * g.sy));
      P.src = g.pending.val;
      fused = true;
    } else {
      k_add_source<<<1, 32, 0, g_stream>>>(g.F[c], pitched_index(g.pending.idx), g.pending.val);
      CK(cudaGetLastError());
    }
  }
  if (g.owed.on) {
    const long i = g.owed.idx;
    want.cor_x = (int)(i % g.sx);
    want.cor_y = (int)((i / g.sx) % g.sy);
    want.cor_z = (int)(i / ((long)g.sx * g.sy));
    P.cor = g.owed.val;
  }
  if (half_form()) {
    const int enew = (g.ecur + 1) % 3, eprev = (g.ecur + 2) % 3;
    const int sz = g.sz;
    int sz_src = -1000;
    if (fused) sz_src = want.src_z;
    else if (g.owed.on) sz_src = want.cor_z;
    const float sabs = fabsf(P.src) + fabsf(P.cor);
    CK(half_scales(g.Mx + c * sz, g.Mx + p * sz, g.E + enew * sz, sz, sz_src, sabs, g_stream));
    HalfLaunch HL;
    memset(&HL, 0, sizeof(HL));
    HL.batch = false;
    HL.h.p = P;
    HL.h.p.seg = g.seg;  // the 16-bit kernel always walks the segment list
    HL.h.p.nitems = g.nseg;
    HL.h.out_hi = g.Hh[p];
    HL.h.out_lo = g.Hl[p];
    HL.h.e_cur = g.E + g.ecur * sz;
    HL.h.e_prev = g.E + eprev * sz;
    HL.h.e_new = g.E + enew * sz;
    HL.h.m_new = g.Mx + p * sz;
    HL.m = g.hm[c];
    HL.tile_rows = g.tile_rows;
    HL.stages = g.stages;
    HL.grid = g.seg_grid;
    CK(propagate_half_launch(HL, g.form == FLETCHER_FORM_FP16X, g_stream));
    g.ecur = enew;
  } else {
    const bool abc = abc_active();
    CK(propagate_fp32_launch(L, g_stream));
    if (abc) CK(abc_after_step(resident_view()));
  }
  ++g.launches;
  if (tune.active && tune_after_step()) return g_last_err;
  // The buffer that was current becomes the previous field; it lacks the
  // fused source, which the next step adds when it reads that cell.
  g.owed = fused ? g.pending : Source();
  g.pending = Source();
  g.cur = p;
  return FLETCHER_OK;
}

// Component comp of buffer buf (which holds the current field when buf ==
// g.cur) -> host.
int read_component(int buf, int comp, float *host) {
  // Where the GPU writes host memory directly, the kernel writes the
  // caller's array; otherwise it goes through `scratch` and a copy.
  float *out = g.hostmem ? host : g.scratch;
  HostPins pin;
  if (!g.hostmem) pin.add(host, g.n * sizeof(float), true);
  if (half_form()) {
    const int slot = buf == g.cur ? g.ecur : (g.ecur + 2) % 3;
    CK(half_decode(g.Hh[buf], g.Hl[buf], g.E + slot * g.sz, out, comp, g.sx, g.sy, g.sz, g.pitch,
                   g.form == FLETCHER_FORM_FP16X, grid_for(g.n), g_stream));
  } else {
    k_unpack<<<grid_for(g.n), 256, 0, g_stream>>>(g.F[buf], out, comp, g.sx, g.sy, g.sz, g.pitch);
    CK(cudaGetLastError());
  }
  if (!g.hostmem) CK(cudaMemcpyAsync(host, g.scratch, g.n * sizeof(float), cudaMemcpyDeviceToHost, g_stream));
  CK(cudaStreamSynchronize(g_stream));
  return check_err_word();
}

}  // namespace

// ===== Part 1 ====================================================================

namespace flt {
int resident_field_to_device(int which, float *dev_out, long *fix_idx, float *fix_val) {
  if (!g.init) return fail(FLETCHER_ERR_ARGS, "no resident state");
  if (which < 0 || which > 3) return fail(FLETCHER_ERR_ARGS, "bad field selector %d", which);
  const int buf = which < 2 ? g.cur : 1 - g.cur, comp = which & 1;
  if (half_form()) {
    const int slot = buf == g.cur ? g.ecur : (g.ecur + 2) % 3;
    CK(half_decode(g.Hh[buf], g.Hl[buf], g.E + slot * g.sz, dev_out, comp, g.sx, g.sy, g.sz, g.pitch,
                   g.form == FLETCHER_FORM_FP16X, grid_for(g.n), g_stream));
  } else {
    k_unpack<<<grid_for(g.n), 256, 0, g_stream>>>(g.F[buf], dev_out, comp, g.sx, g.sy, g.sz, g.pitch);
    CK(cudaGetLastError());
  }
  const Source &fix = which < 2 ? g.pending : g.owed;
  *fix_idx = fix.on ? fix.idx : -1;
  *fix_val = fix.on ? fix.val : 0.f;
  return FLETCHER_OK;
}
size_t resident_cells() { return g.init ? g.n : 0; }
bool resident_dims(int *sx, int *sy, int *sz) {
  if (!g.init) return false;
  *sx = g.sx;
  *sy = g.sy;
  *sz = g.sz;
  return true;
}
cudaStream_t resident_stream() { return g_stream; }
}  // namespace flt

extern "C" void DRIVER_Initialize(const int sx, const int sy, const int sz, const int bord, float dx, float dy,
                                  float dz, float dt, float *vpz, float *vsv, float *epsilon, float *delta,
                                  float *phi, float *theta, float *pp, float *pc, float *qp, float *qc) {
  for (double &m : g_init_mark) m = 0.0;
  g_init_mark[0] = now_s();
  if (initialize(sx, sy, sz, bord, dx, dy, dz, dt, vpz, vsv, epsilon, delta, phi, theta, pp, pc, qp, qc) !=
      FLETCHER_OK)
    free_state();
  g_init_mark[5] = now_s();
}

extern "C" int FLETCHER_InitPhases(double *out) {
  if (!out) return fail(FLETCHER_ERR_ARGS, "FLETCHER_InitPhases: NULL output");
  for (int k = 0; k < 5; ++k)
    out[k] = g_init_mark[k + 1] > 0.0 && g_init_mark[k] > 0.0 ? g_init_mark[k + 1] - g_init_mark[k] : 0.0;
  return FLETCHER_OK;
}

extern "C" void DRIVER_Finalize(void) {
  if (g.init && g_stream) cudaStreamSynchronize(g_stream);
  free_state();
  if (g_own_stream && g_stream) {
    cudaStreamDestroy(g_stream);
    g_stream = nullptr;
    g_own_stream = false;
  }
}

extern "C" void DRIVER_Propagate(const int sx, const int sy, const int sz, const int bord, const float dx,
                                 const float dy, const float dz, const float dt, const int it, float *pp, float *pc,
                                 float *qp, float *qc) {
  (void)bord; (void)dx; (void)dy; (void)dz; (void)dt; (void)it; (void)pp; (void)pc; (void)qp; (void)qc;
  if (check_dims(sx, sy, sz)) return;
  if (step()) return;
  cudaError_t e = cudaStreamSynchronize(g_stream);
  if (e != cudaSuccess) {
    fail(FLETCHER_ERR_CUDA, "propagate step failed: %s", cudaGetErrorString(e));
    return;
  }
  check_err_word();
}

extern "C" void DRIVER_Update_pointers(const int sx, const int sy, const int sz, float *pc) {
  if (check_dims(sx, sy, sz) || !pc) return;
  if (read_component(g.cur, 0, pc)) return;
  if (g.pending.on) pc[g.pending.idx] = pc[g.pending.idx] + g.pending.val;
}

extern "C" void DRIVER_InsertSource(float dt, int it, int iSource, float *p, float *q, float src) {
  (void)dt; (void)it; (void)p; (void)q;
  if (!g.init) {
    fail(FLETCHER_ERR_ARGS, "DRIVER_InsertSource before DRIVER_Initialize");
    return;
  }
  if (iSource < 0 || (size_t)iSource >= g.n) {
    fail(FLETCHER_ERR_ARGS, "source index %d outside the grid", iSource);
    return;
  }
  if (half_form() && !in_update_region(iSource)) {
    fail(FLETCHER_ERR_ARGS, "16-bit forms need the source inside the updated region");
    return;
  }
  if (g.pending.on) {
    if (half_form()) {
      fail(FLETCHER_ERR_ARGS, "16-bit forms take one source per step");
      return;
    }
    // A second source before the next step: store the first one now.
    k_add_source<<<1, 32, 0, g_stream>>>(g.F[g.cur], pitched_index(g.pending.idx), g.pending.val);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      fail(FLETCHER_ERR_CUDA, "source kernel: %s", cudaGetErrorString(e));
      return;
    }
  }
  g.pending.on = true;
  g.pending.idx = iSource;
  g.pending.val = src;
}

// ===== Part 2 ====================================================================

extern "C" void FLETCHER_SetErrorMode(int mode) { g_errmode = mode; }
extern "C" int FLETCHER_GetLastError(void) { return g_last_err; }
extern "C" const char *FLETCHER_GetLastErrorString(void) { return g_errmsg; }
extern "C" void FLETCHER_ClearError(void) {
  g_last_err = FLETCHER_OK;
  g_errmsg[0] = 0;
  if (g.err_host) *g.err_host = 0;
}

extern "C" int FLETCHER_SetStream(void *s) {
  if (g_own_stream && g_stream) {
    cudaStreamSynchronize(g_stream);
    cudaStreamDestroy(g_stream);
  }
  g_stream = static_cast<cudaStream_t>(s);
  g_own_stream = false;
  return FLETCHER_OK;
}
extern "C" void *FLETCHER_GetStream(void) { return g_stream; }

extern "C" int FLETCHER_SetHostAccess(int mode) {
  if (mode != 1 && mode != 0) return fail(FLETCHER_ERR_ARGS, "FLETCHER_SetHostAccess: mode must be 0 or 1");
  g_host_access = mode;
  return FLETCHER_OK;
}

extern "C" int FLETCHER_HostAccess(void) { return g.init && g.hostmem ? 1 : 0; }

extern "C" int FLETCHER_SetForm(int form) {
  if (form < FLETCHER_FORM_FP32 || form > FLETCHER_FORM_FP16X)
    return fail(FLETCHER_ERR_ARGS, "unknown storage form %d", form);
  g_form = form;
  return FLETCHER_OK;
}

extern "C" int FLETCHER_DebugPoisonPadding(float v) {
  if (!g.init) return fail(FLETCHER_ERR_ARGS, "FLETCHER_DebugPoisonPadding before DRIVER_Initialize");
  if (half_form()) return fail(FLETCHER_ERR_ARGS, "FLETCHER_DebugPoisonPadding: FP32 form only");
  if (g.pitch == g.sx) return FLETCHER_OK;  // no padding
  const long rows = (long)g.sy * g.sz;
  for (int b = 0; b < 2; ++b) {
    k_poison_pad<<<grid_for((size_t)rows * (g.pitch - g.sx) * 2), 256, 0, g_stream>>>(
        reinterpret_cast<float *>(g.F[b]), 2, g.sx, g.pitch, rows, v);
    CK(cudaGetLastError());
  }
  k_poison_pad<<<grid_for((size_t)rows * kNumCoef * (g.pitch - g.sx)), 256, 0, g_stream>>>(
      g.coef, 1, g.sx, g.pitch, rows * kNumCoef, v);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(g_stream));
  return FLETCHER_OK;
}

extern "C" int FLETCHER_SetCoefLayout(int layout) {
  if (layout != FLETCHER_COEF_AUTO && layout != FLETCHER_COEF_PLANES && layout != FLETCHER_COEF_MEDIA)
    return fail(FLETCHER_ERR_ARGS, "unknown coefficient layout %d", layout);
  g_coef_layout = layout;
  return FLETCHER_OK;
}

extern "C" int FLETCHER_CoefLayout(void) {
  if (!g.init) return -fail(FLETCHER_ERR_ARGS, "FLETCHER_CoefLayout before DRIVER_Initialize");
  return g.media ? FLETCHER_COEF_MEDIA : FLETCHER_COEF_PLANES;
}

extern "C" int FLETCHER_SetNumerics(int mode) {
  if (mode != FLETCHER_NUMERICS_FAST && mode != FLETCHER_NUMERICS_D1D1)
    return fail(FLETCHER_ERR_ARGS, "unknown numerics mode %d", mode);
  g_numerics = mode;
  return FLETCHER_OK;
}

extern "C" int FLETCHER_InjectFault(int kind, int arg, int wait_us) {
  switch (kind) {
    case FLETCHER_FAULT_NONE:
      g_fault_alloc = -1;
      g_fault_stall = -1;
      g_fault_wait_ns = 0;
      return FLETCHER_OK;
    case FLETCHER_FAULT_ALLOC:
      if (arg < 0) return fail(FLETCHER_ERR_ARGS, "FLETCHER_InjectFault: allocation index must be >= 0");
      g_fault_alloc = arg;
      return FLETCHER_OK;
    case FLETCHER_FAULT_STALL:
      if (arg < 0 || wait_us < 1000 || wait_us > 2000000)
        return fail(FLETCHER_ERR_ARGS, "FLETCHER_InjectFault: stall step must be >= 0 and the wait 1 ms .. 2 s");
      g_fault_stall = arg;
      g_fault_wait_ns = (unsigned long long)wait_us * 1000ull;
      return FLETCHER_OK;
    default:
      return fail(FLETCHER_ERR_ARGS, "FLETCHER_InjectFault: unknown kind %d", kind);
  }
}

extern "C" int FLETCHER_PlanSegments(int ctas, int ntx, int nty, int tile_rows, int zlo, int depth, int zchunks,
                                     int *seg_out, int cap, int *first_out, long *max_cost) {
  if (ctas < 1 || ntx < 1 || nty < 1 || tile_rows < 1 || depth < 1 || cap < 0 || !first_out)
    return -fail(FLETCHER_ERR_ARGS, "FLETCHER_PlanSegments: bad arguments");
  const Split sp = plan_segments(ctas, ntx, nty, tile_rows, zlo, depth, zchunks);
  const int n = (int)sp.seg.size();
  if (seg_out && n <= cap) memcpy(seg_out, sp.seg.data(), sizeof(int4) * n);
  memcpy(first_out, sp.first.data(), sizeof(int) * (ctas + 1));
  if (max_cost) *max_cost = sp.max_cost;
  return n;
}

extern "C" int FLETCHER_SetTileConfig(int rows, int stages, int zchunks) {
  const int r = rows ? rows : 16, s = stages ? stages : 5;
  if (!propagate_fp32_supported(r, s) && !propagate_half_supported(r, s) && !propagate_fp32_media_supported(r, s))
    return fail(FLETCHER_ERR_ARGS, "tile shape (%d, %d) is not built", r, s);
  g_req_rows = rows;
  g_req_stages = stages;
  g_req_chunks = zchunks;
  return FLETCHER_OK;
}

extern "C" int FLETCHER_Run(int nsteps, long iSource, const float *src) {
  if (!g.init) return fail(FLETCHER_ERR_ARGS, "FLETCHER_Run before DRIVER_Initialize");
  if (iSource >= 0 && ((size_t)iSource >= g.n || !src)) return fail(FLETCHER_ERR_ARGS, "bad source");
  if (half_form() && iSource >= 0 && (!in_update_region(iSource) || g.pending.on))
    return fail(FLETCHER_ERR_ARGS, "16-bit forms take one source per step inside the updated region");
  for (int s = 0; s < nsteps; ++s) {
    if (iSource >= 0) {
      if (g.pending.on) {
        k_add_source<<<1, 32, 0, g_stream>>>(g.F[g.cur], pitched_index(g.pending.idx), g.pending.val);
        CK(cudaGetLastError());
      }
      g.pending.on = true;
      g.pending.idx = iSource;
      g.pending.val = src[s];
    }
    if (step()) return g_last_err;
  }
  return FLETCHER_OK;
}

extern "C" int FLETCHER_Synchronize(void) {
  if (!g_stream) return FLETCHER_OK;
  CK(cudaStreamSynchronize(g_stream));
  return check_err_word();
}

extern "C" int FLETCHER_GetField(int which, float *host) {
  if (!g.init) return fail(FLETCHER_ERR_ARGS, "FLETCHER_GetField before DRIVER_Initialize");
  if (which < 0 || which > 3 || !host) return fail(FLETCHER_ERR_ARGS, "bad field selector %d", which);
  const int buf = which < 2 ? g.cur : 1 - g.cur;
  if (read_component(buf, which & 1, host)) return g_last_err;
  const Source &fix = which < 2 ? g.pending : g.owed;
  if (fix.on) host[fix.idx] = host[fix.idx] + fix.val;
  return FLETCHER_OK;
}

extern "C" int FLETCHER_GetCoefficients(float *host) {
  if (!g.init) return fail(FLETCHER_ERR_ARGS, "FLETCHER_GetCoefficients before DRIVER_Initialize");
  // Reference declaration order: ch1dxx ch1dyy ch1dzz ch1dxy ch1dyz ch1dxz v2px v2pz v2sz v2pn.
  const int order[kNumCoef] = {DC_XX, DC_YY, DC_ZZ, DC_XY, DC_YZ, DC_XZ, DC_V2PX, DC_V2PZ, DC_V2SZ, DC_V2PN};
  for (int k = 0; k < kNumCoef; ++k) {
    k_unpack_coef<<<grid_for(g.n), 256, 0, g_stream>>>(g.coef, g.scratch, order[k], g.sx, g.sy, g.sz, g.pitch);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(host + k * g.n, g.scratch, g.n * sizeof(float), cudaMemcpyDeviceToHost, g_stream));
  }
  CK(cudaStreamSynchronize(g_stream));
  return FLETCHER_OK;
}

extern "C" long FLETCHER_KernelLaunches(void) { return g.launches; }
extern "C" size_t FLETCHER_DeviceBytes(void) { return g.dev_bytes; }
extern "C" double FLETCHER_BytesPerCell(void) {
  // current (p,q) + previous (p,q) + next (p,q) + ten FP32 coefficients (40 B):
  // 8 B per field pair in FP32, 4 B in FP16, 6 B in FP16X.  The media-table
  // layout reads four coefficients (16 B) and a one-byte id instead.
  const int form = g.init ? g.form : g_form;
  const double pair = form == FLETCHER_FORM_FP16 ? 4.0 : (form == FLETCHER_FORM_FP16X ? 6.0 : 8.0);
  const bool media = g.init && g.media;
  return 3.0 * pair + (media ? 4.0 * kVelCoef + 1.0 : 4.0 * kNumCoef);
}

// ---- tile-shape tuning with a configuration file --------------------------------

extern "C" int FLETCHER_TuneConfigLookup(const char *path, const char *gpu, int sx, int form, int *rows,
                                         int *stages) {
  if (!path || !gpu || !rows || !stages) return fail(FLETCHER_ERR_ARGS, "TuneConfigLookup: bad arguments");
  FILE *f = fopen(path, "r");
  if (!f) return 0;
  char line[512];
  int found = 0;
  while (fgets(line, sizeof(line), f)) {
    char name[128], fname[16];
    int ssx, bx, by, st;
    // The reference's four fields first (original_singleGPU_PDP/model.c:81), then ours.
    if (sscanf(line, "%127[^|] | %d | %d | %d | %d | %15s", name, &ssx, &bx, &by, &st, fname) != 6) continue;
    size_t L = strlen(name);
    while (L && (name[L - 1] == ' ' || name[L - 1] == '\t')) name[--L] = 0;
    if (strcmp(name, gpu) || ssx != sx || bx != kTileX || strcmp(fname, form_name(form))) continue;
    const bool ok = form == FLETCHER_FORM_FP32         ? propagate_fp32_supported(by, st)
                    : form == FLETCHER_TUNE_FP32_MEDIA ? propagate_fp32_media_supported(by, st)
                                                       : propagate_half_supported(by, st);
    if (!ok) continue;
    *rows = by;
    *stages = st;
    found = 1;  // the last matching line wins
  }
  fclose(f);
  return found;
}

extern "C" int FLETCHER_TuneConfigStore(const char *path, const char *gpu, int sx, int form, int rows, int stages) {
  if (!path || !gpu) return fail(FLETCHER_ERR_ARGS, "TuneConfigStore: bad arguments");
  FILE *f = fopen(path, "a");
  if (!f) return fail(FLETCHER_ERR_ARGS, "TuneConfigStore: cannot open %s", path);
  fprintf(f, "%s | %d | %d | %d | %d | %s\n", gpu, sx, kTileX, rows, stages, form_name(form));
  fclose(f);
  return FLETCHER_OK;
}

extern "C" int FLETCHER_Autotune(const char *path, int steps_per_shape) {
  if (!g.init) return fail(FLETCHER_ERR_ARGS, "FLETCHER_Autotune before DRIVER_Initialize");
  if (g.numerics == FLETCHER_NUMERICS_D1D1)
    return fail(FLETCHER_ERR_ARGS, "FLETCHER_Autotune: the Der1-Der1 numerics have one tile shape");
  if (!path || strlen(path) >= sizeof(tune.path) || steps_per_shape < 1)
    return fail(FLETCHER_ERR_ARGS, "FLETCHER_Autotune: bad arguments");
  cudaDeviceProp prop;
  int dev = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaGetDeviceProperties(&prop, dev));
  int rows = 0, stages = 0;
  const int found = FLETCHER_TuneConfigLookup(path, prop.name, g.sx, tune_key(), &rows, &stages);
  if (found < 0) return g_last_err;
  if (found) {
    tune.active = false;
    if (setup_tiles(rows, stages)) return g_last_err;
    return 1;
  }
  tune = Tuner();
  strcpy(tune.path, path);
  tune.per_shape = steps_per_shape;
  static const int cand[][2] = {{12, 4}, {12, 5}, {12, 6}, {16, 5}, {16, 6}, {16, 7}, {8, 5}, {8, 6}};
  for (const auto &c : cand) {
    const bool ok = g.media       ? propagate_fp32_media_supported(c[0], c[1])
                    : half_form() ? propagate_half_supported(c[0], c[1])
                                  : propagate_fp32_supported(c[0], c[1]);
    if (ok) {
      tune.rows.push_back(c[0]);
      tune.stages.push_back(c[1]);
    }
  }
  CK(cudaEventCreate(&tune.e0));
  CK(cudaEventCreate(&tune.e1));
  tune.active = true;
  return 0;
}

extern "C" int FLETCHER_GetTileConfig(int *rows, int *stages) {
  if (!g.init) return fail(FLETCHER_ERR_ARGS, "FLETCHER_GetTileConfig before DRIVER_Initialize");
  if (rows) *rows = g.tile_rows;
  if (stages) *stages = g.stages;
  return tune.active ? 1 : 0;
}

// ===== Batched shots ==============================================================
//
// Many independent shots of different sizes advance together: one persistent
// launch per time step covers the work items of every shot that is still
// running (16-bit forms: preceded by one launch that sets the new planes'
// scales of every running shot), and the whole time loop is captured in a
// CUDA graph.  Shots are ordered by step count (longest first), so the shots
// still running at any step are a prefix of that order and so are their work
// items.

#include <algorithm>
#include <vector>

namespace {

struct BatchShot {
  int sx = 0, sy = 0, sz = 0, pitch = 0, nsteps = 0;
  long isrc = 0;
  size_t n = 0, npitch = 0;
  float2 *F[2] = {nullptr, nullptr};  // FP32 form
  // 16-bit forms: the two field buffers (half2 per cell, residual bytes),
  // per-plane exponents [3][sz] and maxima [2][sz].
  unsigned *Hh[2] = {nullptr, nullptr};
  unsigned short *Hl[2] = {nullptr, nullptr};
  int *E = nullptr;
  unsigned *Mx = nullptr;
  float *coef = nullptr;
  int ntx = 0, nty = 0, chunk = 0, nchunk = 0;
};

struct Batch {
  bool open = false;
  int form = FLETCHER_FORM_FP32;  // storage form of every shot (fixed at creation)
  int bord = 4;
  float dx = 0, dy = 0, dz = 0, dt = 0;
  std::vector<BatchShot> shots;
  std::vector<int> order;      // shot indices, longest run first
  std::vector<int> items_upto; // items of order[0..i]
  int sealed_rows = 0;
  ShotDesc *d_desc = nullptr;
  ShotMaps *d_maps = nullptr;
  int4 *d_items = nullptr;          // 16-bit forms: {shot, x0, y0, chunk} items
  // FP32: for r running shots (the first r of `order`), their single-shot
  // plans stacked per CTA at d_plan + plan_off[r-1] ({x0 + (shot << 16), y0,
  // z0, z1}), each CTA's first segment at d_first + (r-1) * (plan_ctas + 1).
  int4 *d_plan = nullptr;
  int *d_first = nullptr;
  std::vector<long> plan_off;
  std::vector<int> plan_grid;
  int plan_ctas = 0;
  HalfShot *d_hshots = nullptr;     // 16-bit forms
  HalfShotMaps *d_hmaps = nullptr;
  int *d_order = nullptr;
  float *scratch = nullptr;
  size_t max_n = 0;
  int rows = 12, stages = 5;
  int ctas = 0;  // persistent CTAs of a launch (resident ones, for the sealed shape)
  long launches = 0;
  size_t dev_bytes = 0;
  int num_sms = 0;
  unsigned *err_host = nullptr, *err_dev = nullptr;
  std::vector<float> src;      // source values of the last run
  // Chain schedule (FP32, chains > 0, FLETCHER_BatchSetChains): every step
  // of a shot is a single-shot launch; the shots are dealt over `chains`
  // concurrent streams, each running its shots one after another.  Per
  // shot: its descriptor with the single-shot plan's chunk, its tensor
  // maps, and its plan (tile items, or a segment list in d_sseg / d_sfirst).
  int chains = -1;  // -1: chosen at the run (batch_auto_chains)
  int last_chains = 0;  // the schedule of the last run
  std::vector<ShotDesc> h_desc;
  std::vector<ShotMaps> h_maps;
  std::vector<HalfShot> h_hshots;   // 16-bit forms
  std::vector<HalfShotMaps> h_hmaps;
  std::vector<ShotDesc> s_desc;
  std::vector<int> s_nitems, s_grid;
  std::vector<long> s_seg_off, s_first_off;  // s_seg_off < 0: tile items
  int4 *d_sseg = nullptr;
  int *d_sfirst = nullptr;
  int splan_ctas = 0;
  cudaStream_t chain_s[kMaxChains] = {};
  cudaEvent_t fork = nullptr, join[kMaxChains] = {};
};
Batch B;

void batch_free_tables() {
  if (B.d_plan) cudaFree(B.d_plan);
  if (B.d_first) cudaFree(B.d_first);
  B.d_plan = nullptr;
  B.d_first = nullptr;
  B.plan_ctas = 0;
  if (B.d_sseg) cudaFree(B.d_sseg);
  if (B.d_sfirst) cudaFree(B.d_sfirst);
  B.d_sseg = nullptr;
  B.d_sfirst = nullptr;
  B.splan_ctas = 0;
  if (B.d_desc) cudaFree(B.d_desc);
  if (B.d_maps) cudaFree(B.d_maps);
  if (B.d_items) cudaFree(B.d_items);
  if (B.d_hshots) cudaFree(B.d_hshots);
  if (B.d_hmaps) cudaFree(B.d_hmaps);
  if (B.d_order) cudaFree(B.d_order);
  B.d_desc = nullptr;
  B.d_maps = nullptr;
  B.d_items = nullptr;
  B.d_hshots = nullptr;
  B.d_hmaps = nullptr;
  B.d_order = nullptr;
  B.sealed_rows = 0;
}

void batch_free() {
  batch_free_tables();
  for (auto &s : B.shots) {
    for (int b = 0; b < 2; ++b) {
      if (s.F[b]) cudaFree(s.F[b]);
      if (s.Hh[b]) cudaFree(s.Hh[b]);
      if (s.Hl[b]) cudaFree(s.Hl[b]);
    }
    if (s.E) cudaFree(s.E);
    if (s.Mx) cudaFree(s.Mx);
    if (s.coef) cudaFree(s.coef);
  }
  if (B.scratch) cudaFree(B.scratch);
  if (B.err_host) cudaFreeHost(B.err_host);
  for (int c = 0; c < kMaxChains; ++c) {
    if (B.chain_s[c]) cudaStreamDestroy(B.chain_s[c]);
    if (B.join[c]) cudaEventDestroy(B.join[c]);
  }
  if (B.fork) cudaEventDestroy(B.fork);
  B = Batch();
}

// Work list, descriptors and TMA descriptors for tile height `rows`.
bool batch_half() { return B.form != FLETCHER_FORM_FP32; }

bool batch_shape_built(int rows, int stages) {
  return batch_half() ? propagate_half_supported(rows, stages) : propagate_fp32_supported(rows, stages);
}

int batch_seal(int rows, int stages) {
  if (!batch_shape_built(rows, stages))
    return fail(FLETCHER_ERR_ARGS, "tile shape (%d rows, %d stages) is not built for form %d", rows, stages, B.form);
  if (B.sealed_rows == rows) {
    B.stages = stages;
    return FLETCHER_OK;
  }
  batch_free_tables();
  const int ns = (int)B.shots.size();
  std::vector<ShotDesc> desc(ns);
  std::vector<ShotMaps> maps(ns);
  std::vector<HalfShot> hshots(ns);
  std::vector<HalfShotMaps> hmaps(ns);
  std::vector<int4> items;
  B.order.resize(ns);
  for (int i = 0; i < ns; ++i) B.order[i] = i;
  std::stable_sort(B.order.begin(), B.order.end(),
                   [](int a, int b) { return B.shots[a].nsteps > B.shots[b].nsteps; });
  B.items_upto.assign(ns, 0);
  for (int oi = 0; oi < ns; ++oi) {
    const int i = B.order[oi];
    BatchShot &s = B.shots[i];
    const int depth = s.sz - 2 * B.bord;
    s.ntx = (s.sx - B.bord - kRadius + kTileX - 1) / kTileX;
    s.nty = (s.sy - B.bord - kRadius + rows - 1) / rows;
    s.nchunk = (depth + 127) / 128;
    s.chunk = (depth + s.nchunk - 1) / s.nchunk;
    s.nchunk = (depth + s.chunk - 1) / s.chunk;
    if (build_maps(&maps[i], s.F, s.coef, s.sx, s.sy, s.sz, s.pitch, rows)) return g_last_err;
    if (batch_half()) {
      if (build_half_maps(hmaps[i].m, s.Hh, s.Hl, maps[i], s.sx, s.sy, s.sz, s.pitch, rows)) return g_last_err;
      HalfShot &h = hshots[i];
      for (int b = 0; b < 2; ++b) {
        h.hi[b] = s.Hh[b];
        h.lo[b] = s.Hl[b];
      }
      h.E = s.E;
      h.Mx = s.Mx;
    }
    ShotDesc &d = desc[i];
    memset(&d, 0, sizeof(d));
    d.F[0] = s.F[0];
    d.F[1] = s.F[1];
    d.sx = s.sx; d.sy = s.sy; d.sz = s.sz; d.pitch = s.pitch; d.bord = B.bord;
    d.ntx = s.ntx; d.nty = s.nty; d.chunk = s.chunk;
    d.src_x = (int)(s.isrc % s.sx);
    d.src_y = (int)((s.isrc / s.sx) % s.sy);
    d.src_z = (int)(s.isrc / ((long)s.sx * s.sy));
    d.cor_x = d.src_x; d.cor_y = d.src_y; d.cor_z = d.src_z;
    const size_t base = items.size();
    items.resize(base + (size_t)s.ntx * s.nty * s.nchunk);
    fill_items(items.data() + base, i, s.ntx, s.nty, s.nchunk, rows);
    B.items_upto[oi] = (int)items.size();
  }
  CK(dev_malloc(&B.d_desc, sizeof(ShotDesc) * ns));
  CK(dev_malloc(&B.d_maps, sizeof(ShotMaps) * ns));
  CK(dev_malloc(&B.d_items, sizeof(int4) * items.size()));
  CK(cudaMemcpy(B.d_desc, desc.data(), sizeof(ShotDesc) * ns, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(B.d_maps, maps.data(), sizeof(ShotMaps) * ns, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(B.d_items, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice));
  B.h_desc = desc;
  B.h_maps = maps;
  B.h_hshots = hshots;
  B.h_hmaps = hmaps;
  if (batch_half()) {
    CK(dev_malloc(&B.d_hshots, sizeof(HalfShot) * ns));
    CK(dev_malloc(&B.d_hmaps, sizeof(HalfShotMaps) * ns));
    CK(dev_malloc(&B.d_order, sizeof(int) * ns));
    CK(cudaMemcpy(B.d_hshots, hshots.data(), sizeof(HalfShot) * ns, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.d_hmaps, hmaps.data(), sizeof(HalfShotMaps) * ns, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.d_order, B.order.data(), sizeof(int) * ns, cudaMemcpyHostToDevice));
  }
  B.sealed_rows = rows;
  B.stages = stages;
  return FLETCHER_OK;
}

// The FP32 batch's work split for `ctas` persistent CTAs: each shot's own
// single-shot plan (plan_segments, the balanced split the shot would get
// alone), and for every number r of running shots those of the first r
// shots of `order` stacked per CTA -- CTA b runs its segments of
// order[0], then of order[1], ...  So neighbouring CTAs work on
// neighbouring tiles of the same shot, and every CTA's load is balanced
// shot by shot.
int batch_plan(int ctas) {
  if (B.d_plan && B.plan_ctas == ctas) return FLETCHER_OK;
  if (B.d_plan) cudaFree(B.d_plan);
  if (B.d_first) cudaFree(B.d_first);
  B.d_plan = nullptr;
  B.d_first = nullptr;
  const int ns = (int)B.shots.size();
  if (ns >= 32768) return fail(FLETCHER_ERR_ARGS, "a batch holds at most 32767 shots");
  std::vector<Split> per(ns);
  for (int oi = 0; oi < ns; ++oi) {
    const BatchShot &s = B.shots[B.order[oi]];
    if (s.sx >= 65536) return fail(FLETCHER_ERR_ARGS, "batched shots need sx < 65536");
    per[oi] = plan_segments(ctas, s.ntx, s.nty, B.sealed_rows, B.bord, s.sz - 2 * B.bord, 0);
  }
  std::vector<int4> plan;
  std::vector<int> first((size_t)ns * (ctas + 1));
  B.plan_off.assign(ns, 0);
  B.plan_grid.assign(ns, 1);
  for (int r = 1; r <= ns; ++r) {
    const size_t base = plan.size();
    B.plan_off[r - 1] = (long)base;
    int *f = first.data() + (size_t)(r - 1) * (ctas + 1);
    for (int b = 0; b < ctas; ++b) {
      f[b] = (int)(plan.size() - base);
      for (int oi = 0; oi < r; ++oi) {
        const Split &sp = per[oi];
        const int shot = B.order[oi];
        for (int k = sp.first[b]; k < sp.first[b + 1]; ++k) {
          const int4 w = sp.seg[k];
          plan.push_back(make_int4(w.x | (shot << 16), w.y, w.z, w.w));
        }
      }
    }
    f[ctas] = (int)(plan.size() - base);
    int grid = ctas;  // CTAs past the last one with work are not launched
    while (grid > 1 && f[grid - 1] == f[grid]) --grid;
    B.plan_grid[r - 1] = grid;
  }
  CK(dev_malloc(&B.d_plan, sizeof(int4) * plan.size()));
  CK(dev_malloc(&B.d_first, sizeof(int) * first.size()));
  CK(cudaMemcpy(B.d_plan, plan.data(), sizeof(int4) * plan.size(), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(B.d_first, first.data(), sizeof(int) * first.size(), cudaMemcpyHostToDevice));
  B.plan_ctas = ctas;
  return FLETCHER_OK;
}

// The chain schedule's per-shot plans for `ctas` persistent CTAs: each
// shot's own single-shot plan, as DRIVER_Initialize would make it (the
// 16-bit kernel always walks a segment list).
int batch_single_plans(int ctas) {
  if (B.splan_ctas == ctas && !B.s_desc.empty()) return FLETCHER_OK;
  if (B.d_sseg) cudaFree(B.d_sseg);
  if (B.d_sfirst) cudaFree(B.d_sfirst);
  B.d_sseg = nullptr;
  B.d_sfirst = nullptr;
  const int ns = (int)B.shots.size();
  B.s_desc.assign(ns, ShotDesc());
  B.s_nitems.assign(ns, 0);
  B.s_grid.assign(ns, 1);
  B.s_seg_off.assign(ns, -1);
  B.s_first_off.assign(ns, -1);
  std::vector<int4> segs;
  std::vector<int> firsts;
  for (int i = 0; i < ns; ++i) {
    const BatchShot &s = B.shots[i];
    const int depth = s.sz - 2 * B.bord;
    const Split sp = plan_segments(ctas, s.ntx, s.nty, B.sealed_rows, B.bord, depth, 0);
    ShotDesc d = B.h_desc[i];
    if (sp.spread || batch_half()) {
      B.s_seg_off[i] = (long)segs.size();
      B.s_first_off[i] = (long)firsts.size();
      segs.insert(segs.end(), sp.seg.begin(), sp.seg.end());
      firsts.insert(firsts.end(), sp.first.begin(), sp.first.end());
      int grid = ctas;
      while (grid > 1 && sp.first[grid - 1] == sp.first[grid]) --grid;
      B.s_grid[i] = grid;
      B.s_nitems[i] = (int)sp.seg.size();
      d.chunk = 0;
    } else {
      d.chunk = sp.len;
      B.s_nitems[i] = s.ntx * s.nty * ((depth + sp.len - 1) / sp.len);
      B.s_grid[i] = std::min(B.s_nitems[i], ctas);
    }
    B.s_desc[i] = d;
  }
  if (!segs.empty()) {
    CK(dev_malloc(&B.d_sseg, sizeof(int4) * segs.size()));
    CK(dev_malloc(&B.d_sfirst, sizeof(int) * firsts.size()));
    CK(cudaMemcpy(B.d_sseg, segs.data(), sizeof(int4) * segs.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(B.d_sfirst, firsts.data(), sizeof(int) * firsts.size(), cudaMemcpyHostToDevice));
  }
  B.splan_ctas = ctas;
  return FLETCHER_OK;
}

// The schedule of an FP32 batch left to the library: one chain when most of
// its work (updated cells x steps) is in shots that fill the GPU on their
// own, else the persistent multi-shot launch.
int batch_auto_chains(int steps) {
  double fill = 0.0, total = 0.0;
  for (const BatchShot &s : B.shots) {
    const double cells = (double)(s.sx - 2 * B.bord) * (s.sy - 2 * B.bord) * (s.sz - 2 * B.bord);
    const double work = cells * std::min(s.nsteps, steps);
    total += work;
    if (cells >= kChainFillCells) fill += work;
  }
  return 2.0 * fill >= total ? 1 : 0;
}

int batch_max_steps() {
  int m = 0;
  for (auto &s : B.shots) m = std::max(m, s.nsteps);
  return m;
}

// Issues steps [it0, it1) of the time loop on the stream (no synchronisation).
int batch_issue(int it0, int it1, const float *src) {
  const int ns = (int)B.shots.size();
  PropLaunch L;
  memset(&L, 0, sizeof(L));
  L.batch = true;
  L.p.wait_ns = kWaitLimitNs;
  L.p.stall_step = -1;
  L.tile_rows = B.sealed_rows;
  L.stages = B.stages;
  PropParams &P = L.p;
  P.shots = B.d_desc;
  P.maps = B.d_maps;
  P.items = B.d_items;
  P.inv_dx = 1.0f / B.dx;
  P.inv_dy = 1.0f / B.dy;
  P.inv_dz = 1.0f / B.dz;
  P.inv_dxx = 1.0f / (B.dx * B.dx);
  P.inv_dyy = 1.0f / (B.dy * B.dy);
  P.inv_dzz = 1.0f / (B.dz * B.dz);
  P.inv_dxy = 1.0f / (B.dx * B.dy);
  P.inv_dxz = 1.0f / (B.dx * B.dz);
  P.inv_dyz = 1.0f / (B.dy * B.dz);
  P.iso = (B.dx == B.dy && B.dx == B.dz) ? 1 : 0;
  P.dt2 = P.iso ? (B.dt * B.dt) * P.inv_dxx : B.dt * B.dt;
  P.dt = B.dt;
  P.err = B.err_dev;
  const int ctas = B.ctas;
  int active = ns;  // shots still running, a prefix of B.order
  for (int it = it0; it < it1; ++it) {
    while (active > 0 && B.shots[B.order[active - 1]].nsteps <= it) --active;
    if (active == 0) break;
    P.nitems = B.items_upto[active - 1];
    P.parity = it & 1;
    P.src = src[it];
    P.cor = it > 0 ? src[it - 1] : 0.0f;
    L.grid = P.nitems < ctas ? P.nitems : ctas;
    if (batch_half()) {
      // The new field's plane exponents (every running shot, one launch),
      // then the step; the current field uses exponent slot it % 3.
      const int ecur = it % 3;
      CK(half_scales_batch(B.d_hshots, B.d_desc, B.d_order, active, P.parity, ecur, fabsf(P.src) + fabsf(P.cor),
                           g_stream));
      HalfLaunch HL;
      memset(&HL, 0, sizeof(HL));
      HL.h.p = P;
      HL.h.hshots = B.d_hshots;
      HL.h.hmaps = B.d_hmaps;
      HL.h.ecur = ecur;
      HL.tile_rows = L.tile_rows;
      HL.stages = L.stages;
      HL.grid = L.grid;
      HL.batch = true;
      CK(propagate_half_launch(HL, B.form == FLETCHER_FORM_FP16X, g_stream));
      B.launches += 2;
      continue;
    }
    P.seg = B.d_plan + B.plan_off[active - 1];
    P.cta_first = B.d_first + (size_t)(active - 1) * (B.plan_ctas + 1);
    L.grid = B.plan_grid[active - 1];
    CK(propagate_fp32_launch(L, g_stream));
    ++B.launches;
  }
  return FLETCHER_OK;
}

// The chain schedule: steps [0, steps) of every shot as single-shot
// launches, the shots dealt (longest run first, each to the chain with the
// least work so far) over B.chains streams forked from and joined back into
// the library's
// stream, so the whole run is one graph when captured.  A launch waits on
// no other kernel, so kernels of different chains may share the GPU.
int batch_issue_chains(int chains, int steps, const float *src) {
  const int ns = (int)B.shots.size();
  const int nc = std::max(1, std::min(std::min(chains, kMaxChains), ns));
  if (!B.fork) CK(cudaEventCreateWithFlags(&B.fork, cudaEventDisableTiming));
  for (int c = 0; c < nc; ++c) {
    if (!B.chain_s[c]) CK(cudaStreamCreateWithFlags(&B.chain_s[c], cudaStreamNonBlocking));
    if (!B.join[c]) CK(cudaEventCreateWithFlags(&B.join[c], cudaEventDisableTiming));
  }
  std::vector<std::vector<int>> chain(nc);
  std::vector<double> load(nc, 0.0);
  for (int oi = 0; oi < ns; ++oi) {
    const int i = B.order[oi];
    const BatchShot &s = B.shots[i];
    const double work = (double)(s.sx - 2 * B.bord) * (s.sy - 2 * B.bord) * (s.sz - 2 * B.bord) *
                        std::min(s.nsteps, steps);
    const int c = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    chain[c].push_back(i);
    load[c] += work;
  }
  PropLaunch L;
  memset(&L, 0, sizeof(L));
  L.batch = false;
  L.tile_rows = B.sealed_rows;
  L.stages = B.stages;
  PropParams &P = L.p;
  P.wait_ns = kWaitLimitNs;
  P.stall_step = -1;
  P.inv_dx = 1.0f / B.dx;
  P.inv_dy = 1.0f / B.dy;
  P.inv_dz = 1.0f / B.dz;
  P.inv_dxx = 1.0f / (B.dx * B.dx);
  P.inv_dyy = 1.0f / (B.dy * B.dy);
  P.inv_dzz = 1.0f / (B.dz * B.dz);
  P.inv_dxy = 1.0f / (B.dx * B.dy);
  P.inv_dxz = 1.0f / (B.dx * B.dz);
  P.inv_dyz = 1.0f / (B.dy * B.dz);
  P.iso = (B.dx == B.dy && B.dx == B.dz) ? 1 : 0;
  P.dt2 = P.iso ? (B.dt * B.dt) * P.inv_dxx : B.dt * B.dt;
  P.dt = B.dt;
  P.err = B.err_dev;
  const bool half = batch_half(), ext = B.form == FLETCHER_FORM_FP16X;
  CK(cudaEventRecord(B.fork, g_stream));
  for (int c = 0; c < nc; ++c) {
    cudaStream_t cs = B.chain_s[c];
    CK(cudaStreamWaitEvent(cs, B.fork, 0));
    for (const int i : chain[c]) {
      if (half) {
        // The single-shot 16-bit step: the new planes' scales, then the
        // step (buffer it & 1 current, exponent slot it % 3, as the
        // persistent launch keeps them).
        const HalfShot &h = B.h_hshots[i];
        const int sz = B.shots[i].sz;
        HalfLaunch HL;
        memset(&HL, 0, sizeof(HL));
        HL.batch = false;
        HL.h.p = P;
        HL.h.p.one = B.s_desc[i];
        HL.h.p.nitems = B.s_nitems[i];
        HL.h.p.seg = B.d_sseg + B.s_seg_off[i];
        HL.h.p.cta_first = B.d_sfirst + B.s_first_off[i];
        HL.tile_rows = B.sealed_rows;
        HL.stages = B.stages;
        HL.grid = B.s_grid[i];
        const int n = std::min(B.shots[i].nsteps, steps);
        for (int it = 0; it < n; ++it) {
          const int cur = it & 1, prv = cur ^ 1;
          const int ecur = it % 3, enew = (it + 1) % 3, eprev = (it + 2) % 3;
          HL.h.p.parity = cur;
          HL.h.p.src = src[it];
          HL.h.p.cor = it > 0 ? src[it - 1] : 0.0f;
          CK(half_scales(h.Mx + cur * sz, h.Mx + prv * sz, h.E + enew * sz, sz, HL.h.p.one.src_z,
                         fabsf(HL.h.p.src) + fabsf(HL.h.p.cor), cs));
          HL.h.out_hi = h.hi[prv];
          HL.h.out_lo = h.lo[prv];
          HL.h.e_cur = h.E + ecur * sz;
          HL.h.e_prev = h.E + eprev * sz;
          HL.h.e_new = h.E + enew * sz;
          HL.h.m_new = h.Mx + prv * sz;
          HL.m = B.h_hmaps[i].m[cur];
          CK(propagate_half_launch(HL, ext, cs));
          B.launches += 2;
        }
        continue;
      }
      const ShotMaps &m = B.h_maps[i];
      P.one = B.s_desc[i];
      P.nitems = B.s_nitems[i];
      P.seg = B.s_seg_off[i] < 0 ? nullptr : B.d_sseg + B.s_seg_off[i];
      P.cta_first = B.s_seg_off[i] < 0 ? nullptr : B.d_sfirst + B.s_first_off[i];
      L.grid = B.s_grid[i];
      L.m.arr = m.arr;
      L.m.upd = m.upd;
      const int n = std::min(B.shots[i].nsteps, steps);
      for (int it = 0; it < n; ++it) {
        P.parity = it & 1;
        P.src = src[it];
        P.cor = it > 0 ? src[it - 1] : 0.0f;
        L.m.cur_halo = m.halo[P.parity];
        L.m.prev_pt = m.pt[P.parity ^ 1];
        CK(propagate_fp32_launch(L, cs));
        ++B.launches;
      }
    }
    CK(cudaEventRecord(B.join[c], cs));
    CK(cudaStreamWaitEvent(g_stream, B.join[c], 0));
  }
  return FLETCHER_OK;
}

}  // namespace

extern "C" int FLETCHER_BatchSetChains(int chains) {
  if (chains < -1 || chains > kMaxChains)
    return fail(FLETCHER_ERR_ARGS, "FLETCHER_BatchSetChains: chains must be -1 .. %d (got %d)", kMaxChains, chains);
  if (!B.open) return fail(FLETCHER_ERR_ARGS, "FLETCHER_BatchSetChains before FLETCHER_BatchCreate");
  B.chains = chains;
  return FLETCHER_OK;
}

extern "C" int FLETCHER_BatchCreate(int bord, float dx, float dy, float dz, float dt) {
  batch_free();
  if (bord < kRadius) return fail(FLETCHER_ERR_ARGS, "bord (%d) must be at least %d", bord, kRadius);
  if (!(dx > 0.f) || !(dy > 0.f) || !(dz > 0.f)) return fail(FLETCHER_ERR_ARGS, "grid spacing must be positive");
  if (ensure_stream()) return g_last_err;
  int dev = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&B.num_sms, cudaDevAttrMultiProcessorCount, dev));
  CK(cudaHostAlloc(&B.err_host, sizeof(unsigned), cudaHostAllocMapped));
  *B.err_host = 0;
  CK(cudaHostGetDevicePointer((void **)&B.err_dev, B.err_host, 0));
  B.open = true;
  B.bord = bord;
  B.dx = dx; B.dy = dy; B.dz = dz; B.dt = dt;
  B.form = g_form;
  B.rows = g_req_rows ? g_req_rows : 16;
  B.stages = g_req_stages ? g_req_stages : (B.form == FLETCHER_FORM_FP16 ? 4 : 5);
  return FLETCHER_OK;
}

extern "C" int FLETCHER_BatchAddShot(int sx, int sy, int sz, const float *model, long iSource, int nsteps) {
  if (!B.open) return -fail(FLETCHER_ERR_ARGS, "FLETCHER_BatchAddShot before FLETCHER_BatchCreate");
  const int b = B.bord;
  if (sx <= 2 * b || sy <= 2 * b || sz <= 2 * b || !model || nsteps < 0)
    return -fail(FLETCHER_ERR_ARGS, "bad shot %dx%dx%d", sx, sy, sz);
  BatchShot s;
  s.sx = sx; s.sy = sy; s.sz = sz; s.nsteps = nsteps; s.isrc = iSource;
  s.pitch = (sx + 31) / 32 * 32;
  s.n = (size_t)sx * sy * sz;
  s.npitch = (size_t)s.pitch * sy * sz;
  const long x = iSource % sx, y = (iSource / sx) % sy, z = iSource / ((long)sx * sy);
  if (iSource < 0 || (size_t)iSource >= s.n || x < b || x >= sx - b || y < b || y >= sy - b || z < b ||
      z >= sz - b)
    return -fail(FLETCHER_ERR_ARGS, "batched source %ld must lie in the updated region", iSource);
  cudaStream_t st = g_stream;
  const bool half = batch_half(), ext = B.form == FLETCHER_FORM_FP16X;
  // Field buffers of the shot's form (zeroed below), the coefficients and a
  // temporary for the raw model; everything is released on failure.
  const size_t fbytes = half ? s.npitch * sizeof(unsigned) : s.npitch * sizeof(float2);
  bool ok = true;
  for (int b = 0; b < 2; ++b) {
    if (half) {
      ok = ok && dev_malloc(&s.Hh[b], fbytes) == cudaSuccess;
      if (ext) ok = ok && dev_malloc(&s.Hl[b], s.npitch * sizeof(unsigned short)) == cudaSuccess;
    } else {
      ok = ok && dev_malloc(&s.F[b], fbytes) == cudaSuccess;
    }
  }
  if (half) {
    ok = ok && dev_malloc(&s.E, 3 * sz * sizeof(int)) == cudaSuccess;
    ok = ok && dev_malloc(&s.Mx, 2 * sz * sizeof(unsigned)) == cudaSuccess;
  }
  ok = ok && dev_malloc(&s.coef, s.npitch * kNumCoef * sizeof(float)) == cudaSuccess;
  float *raw = nullptr;
  ok = ok && dev_malloc(&raw, 6 * s.n * sizeof(float)) == cudaSuccess;
  auto release = [&]() {
    for (int b = 0; b < 2; ++b) {
      if (s.F[b]) cudaFree(s.F[b]);
      if (s.Hh[b]) cudaFree(s.Hh[b]);
      if (s.Hl[b]) cudaFree(s.Hl[b]);
    }
    if (s.E) cudaFree(s.E);
    if (s.Mx) cudaFree(s.Mx);
    if (s.coef) cudaFree(s.coef);
    if (raw) cudaFree(raw);
  };
  if (!ok) {
    release();
    cudaGetLastError();
    return -fail(FLETCHER_ERR_NOMEM, "device allocation for shot %zu failed", B.shots.size());
  }
  HostPins pin;
  pin.add(model, 6 * s.n * sizeof(float));
  cudaError_t e = cudaMemcpyAsync(raw, model, 6 * s.n * sizeof(float), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(s.coef, 0, s.npitch * kNumCoef * sizeof(float), st);
  const unsigned long long all_finite = ~0ull;
  if (e == cudaSuccess)
    e = cudaMemcpyToSymbolAsync(g_bad_model, &all_finite, sizeof(all_finite), 0, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) {
    Raw6 r6;
    for (int k = 0; k < 6; ++k) r6.a[k] = raw + k * s.n;
    k_precompute<<<grid_for(s.n), 256, 0, st>>>(r6, s.coef, sx, sy, sz, s.pitch);
    e = cudaGetLastError();
  }
  for (int b = 0; b < 2; ++b) {
    if (e == cudaSuccess) e = cudaMemsetAsync(half ? (void *)s.Hh[b] : (void *)s.F[b], 0, fbytes, st);
    if (e == cudaSuccess && s.Hl[b]) e = cudaMemsetAsync(s.Hl[b], 0, s.npitch * sizeof(unsigned short), st);
  }
  if (e == cudaSuccess && half) e = cudaMemsetAsync(s.E, 0, 3 * sz * sizeof(int), st);
  if (e == cudaSuccess && half) e = cudaMemsetAsync(s.Mx, 0, 2 * sz * sizeof(unsigned), st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(raw);
  raw = nullptr;
  if (e != cudaSuccess) {
    release();
    return -fail(FLETCHER_ERR_CUDA, "shot set-up: %s", cudaGetErrorString(e));
  }
  unsigned long long bad = 0;
  e = cudaMemcpyFromSymbol(&bad, g_bad_model, sizeof(bad));
  if (e != cudaSuccess || bad != ~0ull) {
    release();
    if (e != cudaSuccess) return -fail(FLETCHER_ERR_CUDA, "shot set-up: %s", cudaGetErrorString(e));
    return -fail(FLETCHER_ERR_ARGS, "shot %zu: model array %s holds a value that is not finite at cell %llu",
                 B.shots.size(), kModelNames[bad % 8], bad / 8);
  }
  B.dev_bytes += 2 * fbytes + s.npitch * kNumCoef * sizeof(float);
  if (half) B.dev_bytes += (ext ? 2 * s.npitch * sizeof(unsigned short) : 0) + 5 * sz * sizeof(int);
  if (s.n > B.max_n) {
    if (B.scratch) cudaFree(B.scratch);
    B.scratch = nullptr;
    if (dev_malloc(&B.scratch, s.n * sizeof(float)) != cudaSuccess) {
      cudaGetLastError();
      return -fail(FLETCHER_ERR_NOMEM, "read-back buffer allocation failed");
    }
    B.max_n = s.n;
  }
  B.shots.push_back(s);
  batch_free_tables();
  return (int)B.shots.size() - 1;
}

extern "C" int FLETCHER_BatchReset(void) {
  if (!B.open) return fail(FLETCHER_ERR_ARGS, "no batch");
  for (auto &s : B.shots) {
    for (int b = 0; b < 2; ++b) {
      if (s.F[b]) CK(cudaMemsetAsync(s.F[b], 0, s.npitch * sizeof(float2), g_stream));
      if (s.Hh[b]) CK(cudaMemsetAsync(s.Hh[b], 0, s.npitch * sizeof(unsigned), g_stream));
      if (s.Hl[b]) CK(cudaMemsetAsync(s.Hl[b], 0, s.npitch * sizeof(unsigned short), g_stream));
    }
    if (s.E) CK(cudaMemsetAsync(s.E, 0, 3 * s.sz * sizeof(int), g_stream));
    if (s.Mx) CK(cudaMemsetAsync(s.Mx, 0, 2 * s.sz * sizeof(unsigned), g_stream));
  }
  CK(cudaStreamSynchronize(g_stream));
  return FLETCHER_OK;
}

extern "C" int FLETCHER_BatchRun(const float *src, int max_steps, int use_graph, float *elapsed_ms) {
  if (!B.open || B.shots.empty()) return fail(FLETCHER_ERR_ARGS, "empty batch");
  if (!src) return fail(FLETCHER_ERR_ARGS, "source values missing");
  if (batch_seal(B.rows, B.stages)) return g_last_err;
  int steps = batch_max_steps();
  if (max_steps > 0 && max_steps < steps) steps = max_steps;
  B.src.assign(src, src + steps);
  // Kernel attributes are set outside any capture.
  const cudaError_t pe = batch_half()
                            ? propagate_half_prepare(B.sealed_rows, B.stages, B.form == FLETCHER_FORM_FP16X, true)
                            : propagate_fp32_prepare(B.sealed_rows, B.stages);
  if (pe != cudaSuccess) return fail(FLETCHER_ERR_CUDA, "kernel attribute set-up failed");
  const int per_sm = batch_half() ? propagate_half_ctas_per_sm(B.sealed_rows, B.stages,
                                                               B.form == FLETCHER_FORM_FP16X, true)
                                  : propagate_fp32_ctas_per_sm(B.sealed_rows);
  if (per_sm < 1)
    return fail(FLETCHER_ERR_CUDA, "tile shape (%d rows, %d stages) fits no CTA on an SM", B.sealed_rows, B.stages);
  B.ctas = B.num_sms * per_sm;
  const int nchains = B.chains < 0 ? batch_auto_chains(steps) : B.chains;
  B.last_chains = nchains;
  const bool chains = nchains > 0;
  int plan_ctas = B.ctas;
  if (chains && batch_half()) {
    // The single-shot 16-bit kernel: its own attributes and residency.
    const bool ext = B.form == FLETCHER_FORM_FP16X;
    if (propagate_half_prepare(B.sealed_rows, B.stages, ext, false) != cudaSuccess)
      return fail(FLETCHER_ERR_CUDA, "kernel attribute set-up failed");
    plan_ctas = B.num_sms * propagate_half_ctas_per_sm(B.sealed_rows, B.stages, ext, false);
    if (plan_ctas < 1) return fail(FLETCHER_ERR_CUDA, "tile shape fits no single-shot CTA on an SM");
  }
  if (chains ? batch_single_plans(plan_ctas) : (!batch_half() && batch_plan(B.ctas))) return g_last_err;
  auto issue = [&]() { return chains ? batch_issue_chains(nchains, steps, src) : batch_issue(0, steps, src); };
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  cudaGraphExec_t exec = nullptr;
  if (use_graph) {
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(g_stream, cudaStreamCaptureModeThreadLocal));
    const int rc = issue();
    cudaError_t ce = cudaStreamEndCapture(g_stream, &graph);
    if (rc) return rc;
    CK(ce);
    CK(cudaGraphInstantiate(&exec, graph, 0));
    CK(cudaGraphDestroy(graph));
    CK(cudaGraphUpload(exec, g_stream));
  }
  CK(cudaEventRecord(e0, g_stream));
  if (use_graph) {
    CK(cudaGraphLaunch(exec, g_stream));
  } else if (issue()) {
    return g_last_err;
  }
  CK(cudaEventRecord(e1, g_stream));
  CK(cudaStreamSynchronize(g_stream));
  float ms = 0.f;
  CK(cudaEventElapsedTime(&ms, e0, e1));
  if (elapsed_ms) *elapsed_ms = ms;
  if (exec) cudaGraphExecDestroy(exec);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (*(volatile unsigned *)B.err_host)
    return fail(FLETCHER_ERR_TIMEOUT, "a batched propagate kernel gave up waiting (error word 0x%x)",
                *(volatile unsigned *)B.err_host);
  return FLETCHER_OK;
}

extern "C" int FLETCHER_BatchGetField(int shot, int which, float *host) {
  if (!B.open || shot < 0 || shot >= (int)B.shots.size() || which < 0 || which > 3 || !host)
    return fail(FLETCHER_ERR_ARGS, "bad shot %d or field %d", shot, which);
  const BatchShot &s = B.shots[shot];
  // After nsteps steps the current field is in buffer nsteps & 1 (16-bit
  // forms: with exponent slot nsteps % 3, the previous field's two slots on).
  const int buf = which < 2 ? (s.nsteps & 1) : ((s.nsteps + 1) & 1);
  if (batch_half()) {
    const int slot = which < 2 ? s.nsteps % 3 : (s.nsteps + 2) % 3;
    CK(half_decode(s.Hh[buf], s.Hl[buf], s.E + slot * s.sz, B.scratch, which & 1, s.sx, s.sy, s.sz, s.pitch,
                   B.form == FLETCHER_FORM_FP16X, grid_for(s.n), g_stream));
  } else {
    k_unpack<<<grid_for(s.n), 256, 0, g_stream>>>(s.F[buf], B.scratch, which & 1, s.sx, s.sy, s.sz, s.pitch);
    CK(cudaGetLastError());
  }
  HostPins pin;
  pin.add(host, s.n * sizeof(float), true);
  CK(cudaMemcpyAsync(host, B.scratch, s.n * sizeof(float), cudaMemcpyDeviceToHost, g_stream));
  CK(cudaStreamSynchronize(g_stream));
  // The previous-field buffer lacks the last step's source at the source
  // cell (the next step would add it when reading): add it here, as the
  // reference's in-place InsertSource leaves it.
  if (which >= 2 && s.nsteps > 0 && (size_t)s.nsteps <= B.src.size())
    host[s.isrc] = host[s.isrc] + B.src[s.nsteps - 1];
  return FLETCHER_OK;
}

extern "C" int FLETCHER_BatchSetTileConfig(int rows, int stages) {
  if (!B.open) return fail(FLETCHER_ERR_ARGS, "no batch");
  const int r = rows ? rows : 16, s = stages ? stages : (B.form == FLETCHER_FORM_FP16 ? 4 : 5);
  if (!batch_shape_built(r, s))
    return fail(FLETCHER_ERR_ARGS, "tile shape (%d, %d) is not built for form %d", r, s, B.form);
  B.rows = r;
  B.stages = s;
  return FLETCHER_OK;
}

extern "C" int FLETCHER_BatchLastChains(void) { return B.last_chains; }

extern "C" int FLETCHER_BatchInfo(long *nshots, double *cell_steps, long *launches, size_t *device_bytes) {
  if (nshots) *nshots = (long)B.shots.size();
  if (cell_steps) {
    double c = 0.0;
    for (auto &s : B.shots)
      c += (double)(s.sx - 2 * B.bord) * (s.sy - 2 * B.bord) * (s.sz - 2 * B.bord) * s.nsteps;
    *cell_steps = c;
  }
  if (launches) *launches = B.launches;
  if (device_bytes) *device_bytes = B.dev_bytes;
  return FLETCHER_OK;
}

extern "C" void FLETCHER_BatchDestroy(void) {
  if (g_stream) cudaStreamSynchronize(g_stream);
  batch_free();
}
