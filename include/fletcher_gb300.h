/*
 * fletcher_gb300.h -- C ABI of libfletcher_gb300.so, the GB300 (sm_103a)
 * back-end of the Fletcher TTI pseudo-acoustic propagator.
 *
 * Part 1 is the reference's five-function back-end interface, with the
 * same names, argument meaning and ownership rules, so the reference's
 * front-end (main.c, model.c, boundary.c, source.c, utils.c, map.c,
 * walltime.c) links against this library in place of its OpenMP or CUDA
 * back-end objects.  Part 2 holds extension entry points (error status,
 * launch stream, multi-step runs, field read-back); part 3 the host-side
 * model preparation and time loop this library ships for its own
 * front-end.  All pointers are plain host pointers unless stated.
 */
#ifndef FLETCHER_GB300_H
#define FLETCHER_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ===== Part 1: the reference back-end interface ========================= */

/* Replaces original/driver.h:8-12.  Copies the six raw model arrays and the
 * four initial fields (sx*sy*sz floats each, x fastest) to the GPU, computes
 * the ten coefficient fields there in FP64 (original/precomp.h:14-58) and
 * keeps everything resident.  Requires bord >= 4 (the stencil radius).  A
 * model value that is not finite (NaN or infinity) is rejected with
 * FLETCHER_ERR_ARGS, naming the array and the cell. */
void DRIVER_Initialize(const int sx, const int sy, const int sz, const int bord, float dx,
                       float dy, float dz, float dt, float *vpz, float *vsv, float *epsilon,
                       float *delta, float *phi, float *theta, float *pp, float *pc, float *qp,
                       float *qc);

/* Replaces original/driver.h:14.  Frees all device state. */
void DRIVER_Finalize(void);

/* Replaces original/driver.h:16-18.  Advances p and q one time step over
 * the cells [bord, s-bord) of each axis and rotates the device buffers, as
 * original/OpenMP/openmp_propagate.c:9-41 with original/sample.h:32-89 does.
 * A source registered by DRIVER_InsertSource since the last step is applied
 * inside the same kernel.  The host field pointers are not read (the
 * device holds the state, as in original/CUDA/cuda_driver.c:78-88); the call
 * returns after the step has completed. */
void DRIVER_Propagate(const int sx, const int sy, const int sz, const int bord, const float dx,
                      const float dy, const float dz, const float dt, const int it, float *pp,
                      float *pc, float *qp, float *qc);

/* Replaces original/driver.h:20.  Writes the current p field into host pc
 * (sx*sy*sz floats), as original/CUDA/cuda_stuff.cu:195-201 does. */
void DRIVER_Update_pointers(const int sx, const int sy, const int sz, float *pc);

/* Replaces original/driver.h:22.  Adds src to the current p and q at linear
 * index iSource (original/OpenMP/openmp_insertsource.c:7-13); the addition
 * is fused into the next DRIVER_Propagate. */
void DRIVER_InsertSource(float dt, int it, int iSource, float *p, float *q, float src);

/* ===== Part 2: extension entry points (this library only) ================ */

/* Error handling.  The reference's back-ends print and exit(1) on a CUDA
 * error (original/CUDA/cuda_defines.h:14-20); that is the default here
 * (FLETCHER_ERRMODE_EXIT).  FLETCHER_ERRMODE_RETURN prints, records a sticky
 * status and returns instead. */
#define FLETCHER_ERRMODE_EXIT 0
#define FLETCHER_ERRMODE_RETURN 1
#define FLETCHER_OK 0
#define FLETCHER_ERR_ARGS 1      /* invalid sizes, indices or call order */
#define FLETCHER_ERR_CUDA 2      /* a CUDA runtime call failed */
#define FLETCHER_ERR_TIMEOUT 3   /* a kernel's bounded wait gave up */
#define FLETCHER_ERR_NOMEM 4     /* device allocation failed */
#define FLETCHER_ERR_RANGE 5     /* a 16-bit form's stored value left FP16's range */
void FLETCHER_SetErrorMode(int mode);
int FLETCHER_GetLastError(void);
const char *FLETCHER_GetLastErrorString(void);
void FLETCHER_ClearError(void);

/* Stream on which every kernel and copy is issued (a cudaStream_t; NULL =
 * the library's own stream).  Set before DRIVER_Initialize or between
 * steps. */
int FLETCHER_SetStream(void *cuda_stream);
void *FLETCHER_GetStream(void);

/* Host arrays.  By default DRIVER_Initialize copies the caller's model and
 * field arrays to device buffers, and read-backs copy to the caller's
 * arrays.  FLETCHER_SetHostAccess(1), before DRIVER_Initialize, lets the
 * kernels read and write the caller's arrays in place where the GPU
 * accesses pageable host memory (cudaDevAttrPageableMemoryAccess, e.g.
 * Grace over NVLink-C2C); on GB300 that measured slower than the copies.
 * FLETCHER_HostAccess() tells which path the resident state uses. */
int FLETCHER_SetHostAccess(int mode);
int FLETCHER_HostAccess(void);

/* Storage form of the wave fields, chosen before DRIVER_Initialize.
 * FLETCHER_FORM_FP32: p,q in FP32 (the reference's precision).
 * FLETCHER_FORM_FP16: p,q stored as FP16 with one power-of-two scale per
 *   z-plane (set every step from the planes' largest magnitudes); the
 *   arithmetic stays FP32.
 * FLETCHER_FORM_FP16X: FP16 plus one residual byte per value (a 19-bit
 *   significand, 3 bytes per value).
 * The 16-bit forms keep every cell outside the updated region at zero:
 * DRIVER_Initialize rejects initial fields that are not, and a source must
 * lie inside the updated region, one per step. */
#define FLETCHER_FORM_FP32 0
#define FLETCHER_FORM_FP16 1
#define FLETCHER_FORM_FP16X 2
int FLETCHER_SetForm(int form);

/* Numerics of the FP32 step, chosen before DRIVER_Initialize.  The
 * reference ships each formulation as its own source tree; this selects
 * between two of them in one library.
 * FLETCHER_NUMERICS_FAST (default): the update of original/sample.h:32-89
 *   with each DerCross evaluated as a first derivative of a first derivative
 *   (equal in real arithmetic: its weights are products of the Der1
 *   weights) and fused multiply-adds; within 1e-5 relative L2 of both trees
 *   over short runs.
 * FLETCHER_NUMERICS_D1D1: the Der1-Der1 tree's formulation and operation
 *   order (der1der1/sample.h:35-120): first derivatives scaled and kept
 *   (pDx = Der1_x(p)/dx, pDy = Der1_y(p)/dy), mixed derivatives as their
 *   first derivatives (pxy = Der1_y(pDx)/dy, pxz = Der1_z(pDx)/dz,
 *   pyz = Der1_z(pDy)/dz), every operation rounded on its own in the
 *   reference's order -- the floats of that tree built without
 *   floating-point contraction.  FP32 form, single shot, 16 x 4 tiles.
 * Returns a FLETCHER_* status. */
#define FLETCHER_NUMERICS_FAST 0
#define FLETCHER_NUMERICS_D1D1 1
int FLETCHER_SetNumerics(int mode);

/* Device layout of the ten coefficient fields of the FP32 form (original/
 * precomp.h:14-58), chosen before DRIVER_Initialize.  No counterpart in the
 * reference, which streams all ten per cell.
 * FLETCHER_COEF_PLANES (default): ten FP32 planes per z-plane; a step
 *   streams 64 bytes per cell (24 of fields, 40 of coefficients).
 * FLETCHER_COEF_MEDIA: the six angle coefficients depend on a cell's
 *   (phi, theta) only; a model with at most 256 distinct (phi, theta) bit
 *   pairs keeps them in a table, one byte per cell names the pair, and a
 *   step streams 41 bytes per cell (the four velocity coefficients stay per
 *   cell).  The floats used are the same, so results are bit-identical to
 *   FLETCHER_COEF_PLANES.  16-row tiles of 5, 6 or 7 stages (default 7).
 *   On GB300 at 504^3 it streams 36% fewer bytes but runs 3-5% slower than
 *   the planes (the step's limit is its per-plane chain of shared-memory
 *   reads, which the table lengthens, not DRAM); it leaves more HBM
 *   bandwidth to other work on the GPU.
 *   DRIVER_Initialize fails with FLETCHER_ERR_ARGS when the model has more
 *   pairs, or with a 16-bit form or the Der1-Der1 numerics.
 * FLETCHER_COEF_AUTO: FLETCHER_COEF_MEDIA where the form, the numerics,
 *   the requested tile shape and the model allow it, else
 *   FLETCHER_COEF_PLANES.
 * FLETCHER_CoefLayout: the layout of the initialised state (PLANES or
 *   MEDIA), or a negative status before DRIVER_Initialize.
 * Tuning files (FLETCHER_Autotune) keep the media-table layout's shapes
 * under the form key FLETCHER_TUNE_FP32_MEDIA ("fp32-media"). */
#define FLETCHER_COEF_AUTO 0
#define FLETCHER_COEF_PLANES 1
#define FLETCHER_COEF_MEDIA 2
#define FLETCHER_TUNE_FP32_MEDIA 3
int FLETCHER_SetCoefLayout(int layout);
int FLETCHER_CoefLayout(void);

/* Fault injection for tests of the failure paths (no counterpart in the
 * reference, whose back-ends exit on any error).  Nothing here faults or
 * hangs the GPU.
 * FLETCHER_FAULT_ALLOC: the device allocation `arg` allocations from now
 *   (0 = the next one) fails as if memory were exhausted; the call that
 *   makes it reports FLETCHER_ERR_NOMEM and releases what it allocated.
 * FLETCHER_FAULT_STALL: in the next propagate launch (FP32 form, default
 *   16 x 5 tiles and numerics; that launch uses a variant of the kernel
 *   built with the hook, the regular kernels carry none), CTA 0
 *   skips the loads of its step `arg` (counted from 0), and every wait of
 *   that launch gives up after wait_us microseconds (1000 .. 2000000); the
 *   CTA's waits for that stage run out, it drains the loads in flight and
 *   leaves, and the step reports FLETCHER_ERR_TIMEOUT.  The fields of that
 *   step are then undefined; the state stays usable (re-initialise it).
 * FLETCHER_FAULT_NONE: cancels pending injections. */
#define FLETCHER_FAULT_NONE 0
#define FLETCHER_FAULT_ALLOC 1
#define FLETCHER_FAULT_STALL 2
int FLETCHER_InjectFault(int kind, int arg, int wait_us);

/* Kernel shape override for tuning (0 keeps the default): rows per tile,
 * pipeline stages, z-chunks per column (> 0: that many, the last partial
 * round of items shared out over the CTAs; < 0: -zchunks, all items
 * round-robin). */
int FLETCHER_SetTileConfig(int tile_rows, int stages, int zchunks);

/* The work split of a single-shot launch (host only): ntx x nty tiles of
 * 32 x tile_rows cells, planes [zlo, zlo + depth), over `ctas` persistent
 * CTAs.  Whole rounds of z-chunks go round-robin (CTAs side by side on
 * neighbouring tiles); the last partial round is shared out in equal
 * pieces of at least 8 planes.  Writes the segments {x0, y0, z0, z1} CTA by
 * CTA into seg_out (when they fit in `cap`), each CTA's first segment into
 * first_out [ctas + 1], and the busiest CTA's cost (its planes plus 4 a
 * segment for the halo, shared-out pieces counting 3/2) into max_cost;
 * returns the segment count (negative on error).  zchunks as in
 * FLETCHER_SetTileConfig (0: the cheapest plan). */
int FLETCHER_PlanSegments(int ctas, int ntx, int nty, int tile_rows, int zlo, int depth, int zchunks, int *seg_out,
                          int cap, int *first_out, long *max_cost);

/* Tile-shape tuning with a configuration file in the format of the
 * reference's block-size tuner (original_singleGPU_PDP/model.c:51-113,
 * lines "<GPU name> | <sx> | <bsize_x> | <bsize_y>", appended): here
 * "<GPU name> | <sx> | 32 | <tile rows> | <stages> | <form>".  The
 * reference's loader reads these lines as 32 x rows blocks; lines without
 * the last two fields are not ours and are skipped.
 * FLETCHER_Autotune(path, steps_per_shape), after DRIVER_Initialize: when
 * path holds a line for this GPU, sx and storage form, that shape is applied
 * at once (returns 1).  Otherwise (returns 0) the next steps, through any
 * entry point, try each built shape for 1 + steps_per_shape steps -- the
 * simulation advances normally; results do not depend on the shape -- and
 * the fastest is then applied and appended to path.
 * FLETCHER_GetTileConfig: the current shape; returns 1 while tuning. */
int FLETCHER_Autotune(const char *path, int steps_per_shape);
int FLETCHER_GetTileConfig(int *tile_rows, int *stages);
int FLETCHER_TuneConfigLookup(const char *path, const char *gpu_name, int sx, int form, int *tile_rows,
                              int *stages);
int FLETCHER_TuneConfigStore(const char *path, const char *gpu_name, int sx, int form, int tile_rows, int stages);

/* Runs nsteps steps back to back on the stream without host
 * synchronisation: step s adds src[s] at iSource (iSource < 0: no source),
 * then propagates.  Equivalent to nsteps x (DRIVER_InsertSource +
 * DRIVER_Propagate + swap).  Returns a FLETCHER_* status. */
int FLETCHER_Run(int nsteps, long iSource, const float *src);

/* Waits for the stream; returns a FLETCHER_* status (including a kernel's
 * timeout flag). */
int FLETCHER_Synchronize(void);

/* Copies one field to host memory (sx*sy*sz floats): which = 0 current p,
 * 1 current q, 2 previous p, 3 previous q. */
int FLETCHER_GetField(int which, float *host);

/* Copies the ten coefficient fields to host memory (10*sx*sy*sz floats) in
 * the order ch1dxx ch1dyy ch1dzz ch1dxy ch1dyz ch1dxz v2px v2pz v2sz v2pn
 * (original/precomp.h:14-58). */
int FLETCHER_GetCoefficients(float *host);

/* Number of propagate-kernel launches issued since DRIVER_Initialize. */
long FLETCHER_KernelLaunches(void);

/* Test aid, in place of a memory sanitizer: writes v into the pitch padding
 * (columns sx .. pitch-1 of every row) of both field buffers and of the
 * coefficient block of the initialised FP32 state.  Those cells are never
 * read, so NaN there must leave every result unchanged. */
int FLETCHER_DebugPoisonPadding(float v);

/* Wall-clock phases (s) of the last successful DRIVER_Initialize, in out[5]:
 * device allocations; locking the caller's host arrays and issuing their
 * copies; the device work (copies, coefficient precompute, field packing)
 * until it completes; tile planning and tensor maps; unlocking the host
 * arrays.  Zero where the call stopped early. */
int FLETCHER_InitPhases(double *out);

/* Device bytes held by the current state. */
size_t FLETCHER_DeviceBytes(void);

/* Algorithmic HBM bytes one updated cell costs in the current form and
 * coefficient layout (reads of the current and previous fields and the
 * coefficients -- or, in the media-table layout, the four velocity
 * coefficients and the id byte -- and writes of the next field). */
double FLETCHER_BytesPerCell(void);

/* ---- Output path (original/utils.c:7-227, original/model.c:98-107).
 *
 * Snapshots: FLETCHER_SnapshotBegin(which, host) starts copying field
 * `which` (0 current p, 1 current q, 2 previous p, 3 previous q; any storage
 * form, decoded to FP32) of the resident state into `host` (sx*sy*sz
 * floats) and returns at once: the copy is ordered after the steps issued so
 * far and overlaps the steps issued after it.  FLETCHER_SnapshotWait()
 * waits for the snapshots started so far.  A page-locked destination
 * (FLETCHER_PinHost, cudaHostAlloc) is written by the copy engine directly;
 * any other buffer through a page-locked staging buffer.  The destination
 * must not be touched until FLETCHER_SnapshotWait returns. */
int FLETCHER_SnapshotBegin(int which, float *host);
int FLETCHER_SnapshotWait(void);
int FLETCHER_PinHost(void *ptr, size_t bytes);
int FLETCHER_UnpinHost(void *ptr);

/* RSF (Madagascar) files with the reference's names and layout: a text
 * header <fName>.rsf and a binary <fName>.rsf@ of native floats, x fastest.
 * Boxes are inclusive grid indices [ixStart, ixEnd] x ... as in the
 * reference.  DumpFieldToFile writes one box of a host array
 * (original/utils.c:7-52).  A slice file (OpenSliceFile, :66-120) is
 * appended to from a host array (DumpSliceFile, :126-146) or, without
 * blocking, from the resident state (SliceAppend: the box is gathered on
 * the device and written by a host callback after its copy); CloseSliceFile
 * (:152-198) waits for pending appends and writes the header with the
 * frame count.  DumpSliceSummary (:204-224) prints the box's extrema. */
typedef struct FletcherSlice FletcherSlice;
int FLETCHER_DumpFieldToFile(int sx, int sy, int sz, int ixStart, int ixEnd, int iyStart, int iyEnd, int izStart,
                             int izEnd, float d1, float d2, float d3, const float *arr, const char *fName);
FletcherSlice *FLETCHER_OpenSliceFile(int ixStart, int ixEnd, int iyStart, int iyEnd, int izStart, int izEnd,
                                      float dx, float dy, float dz, float dt, const char *fName);
int FLETCHER_DumpSliceFile(int sx, int sy, int sz, const float *arr, FletcherSlice *slice);
int FLETCHER_SliceAppend(FletcherSlice *slice, int which);
int FLETCHER_CloseSliceFile(FletcherSlice *slice);
int FLETCHER_SliceFrames(const FletcherSlice *slice);
int FLETCHER_DumpSliceSummary(int sx, int sy, int sz, const FletcherSlice *slice, float dt, int it,
                              const float *arr, float src);

/* ---- Batched shots (no counterpart in the reference, whose runs are one
 * shot per process).  Independent shots of different sizes share one
 * persistent launch per time step; the time loop runs as one CUDA graph.
 * All shots share bord, spacing and time step; each has its own grid,
 * model, source cell (inside the updated region) and step count.  The
 * single-shot state of part 1 is separate and unaffected. */

/* Starts an empty batch (frees a previous one).  Every shot of the batch
 * is stored in the form FLETCHER_SetForm last selected (FP32, FP16 or
 * FP16X; 16-bit forms take two launches per step: the plane scales of all
 * running shots, then the step). */
int FLETCHER_BatchCreate(int bord, float dx, float dy, float dz, float dt);
/* Adds a shot: grid sx*sy*sz, model = vpz vsv epsilon delta phi theta
 * (sx*sy*sz floats each, consecutive, boundary already applied), source
 * index, number of steps.  Copies the model to the GPU and computes its
 * coefficients in FP64.  Returns the shot index (>= 0) or -status. */
int FLETCHER_BatchAddShot(int sx, int sy, int sz, const float *model, long iSource, int nsteps);
/* Tile shape for the next FLETCHER_BatchRun (0 = default). */
int FLETCHER_BatchSetTileConfig(int tile_rows, int stages);
/* Schedule of a batch's run, after FLETCHER_BatchCreate.
 * chains = -1 (default): one chain when most of the batch's work (updated
 *   cells x steps) is in shots of at least 2.1 M updated cells, which fill
 *   the GPU on their own, else the persistent launch (measured on GB300: 48
 *   shots of 168^3-392^3 ran 7% faster on one chain than on the persistent
 *   launch; 48 shots of 56^3 and 32 of 80^3 ran 6-7% slower).
 * chains = 0: one persistent launch per time step advances every running
 *   shot (FP32: the shots' single-shot plans stacked per CTA; 16-bit forms:
 *   the plane-scale launch of every running shot first).
 * chains = 1 .. 8: every step of a shot is its own single-shot launch; the
 *   shots are dealt, longest run first, each to the stream with the least
 *   work so far, over `chains` concurrent streams,
 *   each running its shots one after another (one graph when captured).
 *   A launch waits on no other kernel, so kernels of different chains
 *   share the GPU where one leaves SMs idle, and each chain works on one
 *   shot's memory at a time.  In the 16-bit forms each step is the
 *   single-shot pair of launches (the new planes' scales, then the step).
 * Results are bit-identical in every schedule. */
int FLETCHER_BatchSetChains(int chains);
/* The schedule of the last FLETCHER_BatchRun: 0 (persistent launch) or the
 * number of chains. */
int FLETCHER_BatchLastChains(void);
/* Runs every shot from its current state for its own step count (or only
 * the first max_steps steps when max_steps > 0, e.g. for tuning; read-back
 * assumes a full run): step it adds src[it] at each running shot's source
 * cell (the reference's InsertSource) then advances.  use_graph != 0
 * captures the loop in a CUDA graph first.  *elapsed_ms (may be NULL) =
 * device time of the loop. */
int FLETCHER_BatchRun(const float *src, int max_steps, int use_graph, float *elapsed_ms);
/* Zeroes every shot's fields (the coefficients stay). */
int FLETCHER_BatchReset(void);
/* Copies one field of a shot after the run: which = 0 current p, 1 current
 * q, 2 previous p, 3 previous q (as the reference leaves them: the previous
 * fields include the last step's source). */
int FLETCHER_BatchGetField(int shot, int which, float *host);
/* Shots, sum over shots of updated cells x steps, kernel launches issued,
 * device bytes held. */
int FLETCHER_BatchInfo(long *nshots, double *cell_steps, long *launches, size_t *device_bytes);
void FLETCHER_BatchDestroy(void);

/* No counterpart in the reference.  Read-back for callers that cannot
 * allocate device memory: codes that reserve the whole GPU for their own
 * wavefield and coefficient volumes up front, or whose time loop must not
 * call cudaMalloc (an allocation there fails once memory is fully reserved,
 * or stalls the stream).  Copies component `comp` (0 = p, 1 = q) of a
 * caller-owned (p, q) pair volume on the current device -- float2 pairs,
 * [sz][sy][pitch], x fastest, pitch (in pairs) >= sx: the layout of the FP32
 * form's field buffers (the 16-bit forms store half2 and are not accepted)
 * -- into host_out (sx*sy*sz floats).  It allocates nothing: it stages
 * through a fixed array of FLETCHER_NOALLOC_MAX_CELLS floats (16 MiB) built
 * into the library, which every GPU that loads the library holds until the
 * process exits; larger grids are rejected with FLETCHER_ERR_ARGS.  The
 * first call on a device (and the first after that device's context was
 * reset) looks up that array's device address, so make it before any
 * stream capture.  All calls share the array: calls that overlap on the GPU
 * (from concurrent host threads, or on different streams) race on it.  Runs
 * on FLETCHER_GetStream(): the caller's writes to dev_pairs must be ordered
 * before the call -- issued on that stream (FLETCHER_SetStream names the
 * caller's stream) or complete before it.  Returns when host_out is filled;
 * returns a FLETCHER_* status. */
#define FLETCHER_NOALLOC_MAX_CELLS (4u * 1024u * 1024u)
int FLETCHER_ReadFieldNoAlloc(const void *dev_pairs, int sx, int sy, int sz, int pitch, int comp,
                              float *host_out);

/* ===== Part 3: host-side model preparation and time loop ================= */

/* Fills the six model arrays (vpz vsv epsilon delta phi theta, n floats
 * each, consecutive in `model`) with one homogeneous medium; angles in
 * radians. */
void FLETCHER_ModelHomogeneous(long n, float vpz, float vsv, float epsilon, float delta,
                               float phi, float theta, float *model);

/* Horizontally layered TTI medium over the whole grid: `nlayers` layers of
 * seeded random thickness that tile the interior depth nz, vpz drawn in
 * [vmin, vmax] and sorted to increase with depth, epsilon ~ U[0, 0.3],
 * delta ~ U[0, epsilon], theta ~ U[0, 45 deg], phi ~ U[0, 90 deg],
 * vsv = vs_ratio * vpz.  Cells above / below the interior take the first /
 * last layer.  The six arrays are consecutive in `model`.  Draws come from
 * a splitmix64 stream seeded by `seed`, so results are identical on every
 * platform.  layer_top (nlayers ints, may be NULL) receives each layer's
 * first interior z index. */
void FLETCHER_ModelLayered(int sx, int sy, int sz, int bord, int absorb, int nlayers,
                           uint64_t seed, float vmin, float vmax, float vs_ratio, float *model,
                           int *layer_top);

/* RandomVelocityBoundary, as original/boundary.c:7-98: random-velocity
 * absorbing zone of width `absorb` and a zero-velocity `bord` shell, drawn
 * with the C library rand() after srand(seed). */
void FLETCHER_RandomVelocityBoundary(int sx, int sy, int sz, int nx, int ny, int nz, int bord,
                                     int absorb, float *vpz, float *vsv, unsigned seed);

/* Ricker source value at time it*dt (original/source.c:7-15) for cut
 * frequency fcut (original/source.h:11 fixes 40); peak frequency fcut/3. */
float FLETCHER_Source(float dt, int it, double fcut);

/* Advisory time step (original/main.c:225-239). */
float FLETCHER_RecommendedDt(long n, const float *vpz, const float *epsilon, float dx, float dy,
                             float dz);

/* The time loop of original/model.c:32-164 through Part 1: coefficient set-up
 * and DRIVER_Initialize, then for it = 1..st DRIVER_InsertSource with the
 * source for time (it-1)*dt, DRIVER_Propagate and the pointer swap (the
 * timed region, as original/model.c:82-88), and DRIVER_Update_pointers of
 * the current p every dt_output seconds of simulated time (dt_output <= 0:
 * never; the snapshots are asynchronous and land in the host array the
 * reference's loop would name pc at that step -- both host p arrays are
 * page-locked for the call).  The final current p and q are copied to pc and qc, and
 * DRIVER_Finalize is called.  Results in stats (may be NULL):
 * stats[0] = propagate wall seconds, stats[1] = MSamples/s by the
 * reference's definition, stats[2] = whole-call wall seconds, stats[3] =
 * host-to-device bytes, stats[4] = device-to-host bytes.  Returns a
 * FLETCHER_* status. */
int FLETCHER_Model(int st, long iSource, double fcut, float dt_output, int sx, int sy, int sz,
                   int bord, float dx, float dy, float dz, float dt, float *pp, float *pc,
                   float *qp, float *qc, float *vpz, float *vsv, float *epsilon, float *delta,
                   float *phi, float *theta, double *stats);
/* Wall seconds of the last FLETCHER_Model call by phase: phases[0] set-up
 * (DRIVER_Initialize, page-locking the snapshot arrays), [1] the time loop,
 * [2] waiting for the last snapshots, [3] final read-back and
 * DRIVER_Finalize. */
void FLETCHER_ModelPhases(double *phases);

/* ===== Part 4: learned absorbing boundary (no counterpart in the reference,
 * whose absorbing zone is the random-velocity shell of original/boundary.c).
 *
 * The grid is interior + a layer of L cells + bord on every side, the medium
 * extended into the layer.  The plain update covers interior and layer; the
 * layer's outer 4 cells (the ghost zone: d = L-3 .. L cells outside the
 * interior, whose stencils reach the zero border) are then overwritten with
 * the box-scheme update of the one-way wave equation along the outward
 * normal, u_g(t+1) = u_i(t) + k (u_g(t) - u_i(t+1)) (g the cell, i its
 * inward neighbour), outward from d = L-3, z faces, then y, then x.
 * FLETCHER_BOUNDARY_ONEWAY takes k = (1 - r) / (1 + r), r = c dt / h, from
 * the medium (c = vpz along z, vpz sqrt(1 + 2 eps) along x and y);
 * FLETCHER_BOUNDARY_LEARNED takes (k_p, k_q) = sigmoid(y) of a per-cell MLP
 * (40 -> 32 -> 32 -> 2, tanh, FP16 weights, FP32 accumulation) evaluated
 * every step.  Inputs: the 9-point outward-normal stencils of p and q at t
 * and t-1 (points beyond the layer read as zero, all divided by their
 * largest magnitude s), vpz / 4000, epsilon, delta, d / L.
 * FLETCHER_ABC_PARAMS master weights (FP32): W1 [32][40], b1 [32],
 * W2 [32][32], b2 [32], W3 [2][32], b3 [2]. */
#define FLETCHER_ABC_PARAMS 2434
#define FLETCHER_BOUNDARY_PLAIN 0
#define FLETCHER_BOUNDARY_LEARNED 1
#define FLETCHER_BOUNDARY_SPONGE 2
#define FLETCHER_BOUNDARY_ONEWAY 3

/* Network weights: random initialisation (Xavier, seeded; output biases
 * start at k ~ 0.7), set, get. */
int FLETCHER_AbcInit(unsigned seed);
int FLETCHER_AbcSetWeights(const float *params);
int FLETCHER_AbcGetWeights(float *params);

/* Training set on the device: AbcReserve(capacity) (re)allocates and
 * empties it; AbcCollect appends samples from the resident FP32 state (its
 * current and previous fields): around the interior box [lo, hi) with a
 * layer of `layer` cells, a random fraction keep_frac of the ghost cells
 * whose stencil magnitude s exceeds min_scale, each with its 40 inputs and
 * targets a = (u_g(t) - u_i(t+1)) / s, b = (u_g(t+1) - u_i(t)) / s for p
 * and q, u(t+1) being the plain update on the resident field.  The box, its
 * layer and 4 more cells must lie in the updated region. */
int FLETCHER_AbcReserve(long capacity);
int FLETCHER_AbcCollect(const int *interior_lo, const int *interior_hi, int layer, float keep_frac, unsigned seed,
                        float min_scale);
long FLETCHER_AbcSamples(void);
/* Samples [start, start + n): features [n][40], targets [n][4] (a_p, a_q,
 * b_p, b_q), and the cell of each ([n][4] ints: x, y, z, face + 8 d; faces
 * 0..5 are z-, z+, y-, y+, x-, x+); any pointer may be NULL. */
int FLETCHER_AbcGetSamples(long start, long n, float *features, float *targets, int *cells);

/* iters Adam steps (cosine-decayed learning rate from lr) on random batches
 * of `batch` samples, the stencil inputs perturbed by noise of standard
 * deviation `noise` (0: none).  loss_out: iters losses. */
int FLETCHER_AbcTrain(int iters, int batch, float lr, unsigned seed, float noise, float *loss_out);

/* One forward and backward pass on n given samples (features [n][40],
 * targets [n][4]): loss = sum_c (sigmoid(y_c) a_c - b_c)^2 / (2 n) and its
 * gradient with respect to the master weights. */
int FLETCHER_AbcGradient(const float *features, const float *targets, int n, float *grad, float *loss);

/* The inference path (tensor cores) on n given feature rows: raw outputs
 * y [n][2] (k = sigmoid(y)). */
int FLETCHER_AbcForward(const float *features, int n, float *out);

/* Boundary of the resident FP32 state, a layer of `layer` cells (>= 5)
 * inside the updated region (interior = updated region shrunk by `layer`).
 * FLETCHER_BOUNDARY_PLAIN: none.  FLETCHER_BOUNDARY_ONEWAY and
 * FLETCHER_BOUNDARY_LEARNED: the ghost-zone update after every step, in one
 * cooperative launch that also evaluates the network on the learned form's
 * evaluation steps (two launches per step in all).
 * damping > 0 also scales every layer cell by exp(-(damping d)^2) after the
 * step; FLETCHER_BOUNDARY_SPONGE is that scaling alone (damping > 0).
 * FLETCHER_AbcLayerCells: ghost cells updated per step (one-way forms). */
int FLETCHER_SetBoundary(int mode, int layer, float damping);
/* The learned form evaluates the network every `steps` steps (default 1)
 * and keeps the last coefficients in between (counted from SetBoundary). */
int FLETCHER_AbcSetInterval(int steps);
long FLETCHER_AbcLayerCells(void);
void FLETCHER_AbcRelease(void);

#ifdef __cplusplus
}
#endif
#endif
