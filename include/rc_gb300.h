/*
 * rc_gb300 — GB300-native w-projection gridding / degridding engine.
 *
 * C ABI of librc_gb300.so.  Two layers:
 *
 *  1. Drop-in symbols of the reference's kernel-binding ABI
 *     (SKA-ScienceDataProcessor/RC, MS5/MS6 DNA/Flow `Flow.Halide`): the same
 *     names, argument order, buffer_t layout and return conventions.  They take
 *     HOST buffers, run on the GPU, and return only when the result is back in
 *     host memory (the reference's semantics).
 *
 *  2. The engine API on DEVICE pointers (gb_*): a visibility plan (FP64 index
 *     math, w-plane assignment, sort/bin by grid tile), the FP32 batched
 *     gridder/degridder written as an exact adjoint pair, the plain FP64
 *     gridder/degridder, and on-GPU w-kernel (GCF) generation.  Every launch
 *     goes on the caller's stream and can be captured in a CUDA graph.
 *
 * Return value of every int function: 0 on success, negative on error;
 * gb_last_error() gives the message of the calling thread's last error.
 */
#ifndef RC_GB300_H
#define RC_GB300_H

#include <stdbool.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ buffer_t
 * Legacy Halide buffer descriptor, 72 bytes, byte-for-byte the layout the
 * reference's Haskell marshaller writes (MS6/kernel/common/halide_buf.h:17-27;
 * offsets 8/16/32/48/64/68 in MS6/dna/flow/Flow/Halide/BufferT.hs:26-99).
 * `dev` is ignored (the reference never sets a device pointer,
 * BufferT.hs:60-78); `host` is the data, `min` the coordinate of its first
 * element in each dimension.  elem_size must be 8 (double). */
#ifndef BUFFER_T_DEFINED
#define BUFFER_T_DEFINED
typedef struct buffer_t {
  uint64_t dev;
  uint8_t *host;
  int32_t extent[4];
  int32_t stride[4];
  int32_t min[4];
  int32_t elem_size;
  bool host_dirty;
  bool dev_dirty;
  uint8_t _padding[10 - sizeof(void *)];
} buffer_t;
#endif

/* ------------------------------------------------------------------ errors */
#define GB_OK 0
/* legacy "unsupported GCF size" codes of the reference dispatchers */
#define GB_ERR_SCATTER_SIZE (-444)     /* MS6/kernel/cpu/gridding/scatter1.cpp:19 */
#define GB_ERR_DEGRID_SIZE (-555)      /* MS6/kernel/cpu/gridding/degrid1.cpp:18 */
#define GB_ERR_SCATTER_GPU_SIZE (-222) /* MS6/kernel/gpu/gridding/kern_scatter_gpu1.cpp:31 */
#define GB_ERR_DEGRID_GPU_SIZE (-333)  /* MS6/kernel/gpu/gridding/kern_degrid_gpu1.cpp:71 */
#define GB_ERR_ARG (-1001)      /* malformed buffer / argument */
#define GB_ERR_CUDA (-1002)     /* CUDA runtime or cuFFT error */
#define GB_ERR_TIMEOUT (-1003)  /* a bounded device-side wait ran out */
#define GB_ERR_NOMEM (-1004)    /* device or host allocation failed */
#define GB_ERR_CAPACITY (-1005) /* a size exceeds a documented limit */

const char *gb_last_error(void);
const char *gb_version(void);

/* ------------------------------------------------------------------ layer 1: reference ABI
 * Gridder type (Haskell, MS6/programs/Kernel/Gridder.hs:65-71):
 *   HalideBind Double (HalideBind Int32 (HalideBind Int32
 *     (HalideFun '[VisRepr, GCFsRepr] UVGMarginRepr)))
 * vis: dims (5, N) stride (1, 5), fields u, v, w (wavelengths), re, im.
 * gcf: dims (2, S, S, 64) strides (1, 2, 2S, 2S^2), phase index ou + 8*ov.
 * uvg: dims (2, W, H) strides (1, 2, stride2), min (0, u0, v0): accumulated
 *      in place (+=), never overwritten.
 * The reference dispatchers accept S in {8, 16, 32, 64} and return the legacy
 * code otherwise; these do the same (the engine below accepts any S). */

/* Precision of the gridders (kern_scatter_gpu1, kern_scatter, nvGridder):
 * the taps are summed per 32 x 32 grid block in shared memory in the
 * degridders' double-float arithmetic (below), and each block's sums are
 * added into the grid with FP64 atomics, in an order that varies between
 * runs.  Inputs holding an Inf, a NaN or a subnormal take FP64 products with
 * FP64 atomics instead.
 * replaces MS6/kernel/gpu/gridding/kern_scatter_gpu1.cpp:21-40 */
int kern_scatter_gpu1(double scale, int32_t grid_size, int32_t margin_size,
                      buffer_t *vis, buffer_t *gcf, buffer_t *uvg);
#ifndef GB_MS5_ABI /* the MS5 variant binds its own kern_scatter (rc_gb300_ms5.h) */
/* replaces MS6/kernel/cpu/gridding/scatter1.cpp:9-20 (the CPU slot; runs on the GPU) */
int kern_scatter(double scale, int32_t grid_size, int32_t margin_size,
                 buffer_t *vis, buffer_t *gcf, buffer_t *uvg);
#endif
/* replaces MS6/kernel/nvidia/gridder/halide_api.cu:4-29, in the form the
 * Haskell side binds it (MS6/programs/Kernel/Gridder.hs:70: three scalars,
 * margin included); same semantics as kern_scatter_gpu1. */
int nvGridder(double scale, int32_t grid_size, int32_t margin_size,
              buffer_t *vis, buffer_t *gcf, buffer_t *uvg);

/* Degridder type (MS6/programs/Kernel/Degrid.hs:146-147): vis_out = vis
 * minus sum(grid * gcf) for in-bound visibilities (no conjugate), u,v,w
 * copied; uvg is the full grid, min 0.
 *
 * Precision of both degridders: the products and sums run in double-float
 * arithmetic on the FP32 pipe (each double split into two floats after a
 * power-of-two scaling of its array), a 48-bit significand rather than FP64's
 * 53: a sum errs by about 2^-48 of the sum of its terms' magnitudes (within
 * 1e-12 relative of FP64 on every tested input).  Grid and GCF values below
 * 2^-74 of their array's largest magnitude lose their low part, and those
 * below 2^-126 of it count as zero.  Inputs holding an Inf, a NaN or a
 * subnormal take a native FP64 loop instead.  The index math (pixel, phase,
 * bounds) is FP64 and exact.
 * replaces MS6/kernel/gpu/gridding/kern_degrid_gpu1.cpp:61-81 */
int kern_degrid_gpu1(double scale, int32_t grid_size, int32_t margin_size,
                     buffer_t *gcf, buffer_t *uvg, buffer_t *vis, buffer_t *vis_out);
/* replaces MS6/kernel/cpu/gridding/degrid1.cpp:9-19 */
int kern_degrid(double scale, int32_t grid_size, int32_t margin_size,
                buffer_t *gcf, buffer_t *uvg, buffer_t *vis, buffer_t *vis_out);

/* replaces MS6/kernel/cpu/gridding/init.cpp:8-15 (zero a complex grid buffer) */
int kern_init(buffer_t *uvg);
/* replaces MS6/kernel/cpu/gridding/psf_vis.cpp:16-27 (vis_out = vis with re=1, im=0) */
int kern_psf_vis(buffer_t *vis, buffer_t *vis_out);

/* ------------------------------------------------------------------ layer 2: engine API */

typedef struct gb_plan gb_plan;

/* Geometry of one grid and its w-planes.  The grid is the full grid
 * (min 0): ext_x * ext_y pixels, row pitch `pitch` complex elements.
 * grid_size (the reference's centring parameter), scale (FoV in radians,
 * the reference's `scale`), and margin (the reference's margin_size; pass the
 * largest support to reproduce the MS6 bounds) follow the reference meaning.
 * supports[p] is plane p's GCF support S_p (>= 1, <= GB_MAX_SUPPORT);
 * gcf_offsets[p] is the offset, in complex elements, of plane p's GCF
 * ([64][S_p][S_p], phase ou + 8*ov, row sy, column sx) inside the GCF array
 * passed to the execute calls.  Planes are assigned per visibility by the
 * reference's w-binning rule over [w_low, w_high] (Binning.hs:85-89), or
 * taken from an explicit per-visibility plane array. */
#define GB_MAX_SUPPORT 256
#define GB_MAX_PLANES 4096
typedef struct gb_geometry {
  double scale;
  int32_t grid_size;
  int32_t margin;
  int32_t ext_x, ext_y;
  int64_t pitch;
  int32_t n_planes;
  int32_t tile;            /* grid tile edge of the FP32 kernels (8..128): 0 = 24 */
  int32_t threads;         /* threads per CTA of the FP32 kernels (128, 256, 512): 0 = 256 */
  int32_t period_cap;      /* largest footprint piece edge (8..64, cap^2 <= 8 threads):
                              0 = 40 (32 with 128 threads) */
  int32_t bundles_per_cta; /* work granularity: target bundles per resident CTA (1..64): 0 = 4 */
  const int32_t *supports; /* host, n_planes */
  const int64_t *gcf_offsets; /* host, n_planes */
  double w_low, w_high;    /* w-binning range (ignored with an explicit plane array) */
} gb_geometry;

/* Build a plan for n_vis visibilities.  d_uvw: device, u v w doubles of
 * visibility t at d_uvw[t*uvw_stride + {0,1,2}].  d_plane: optional device
 * int32 plane index per visibility (negative = skip), else NULL.  The plan
 * keeps d_uvw's address (for the plain FP64 path) but none of the visibility
 * values; keep d_uvw alive while the plan is used.  Runs on `stream`
 * (cudaStream_t) and synchronises it once. */
int gb_plan_create(const gb_geometry *geo, int64_t n_vis, const double *d_uvw,
                   int64_t uvw_stride, const int32_t *d_plane, void *stream,
                   gb_plan **out);
int gb_plan_destroy(gb_plan *plan);

/* Statistics of a plan: [0] visibilities kept, [1] sum over kept visibilities
 * of S_v^2 (taps), [2] work items, [3] grid tiles with work, [4] tile edge,
 * [5] largest support, [6] threads per CTA. */
int gb_plan_stats(const gb_plan *plan, int64_t *stats7);

/* How FP32 degridding stages each tile's grid region in shared memory:
 *   GB_STAGE_SPLIT: per-thread asynchronous copies into rows split into their
 *     even and then their odd pixels, so the two taps of a pair are read by
 *     two loads contiguous across the lanes (best when most taps are paired:
 *     even supports, a 16-byte aligned GCF);
 *   GB_STAGE_TMA: one 2-D TMA copy per region, rows as in the grid (single
 *     grid, even tile edge, even row pitch, 16-byte aligned grid);
 *   GB_STAGE_ROWS: per-thread asynchronous copies, rows as in the grid.
 * GB_STAGE_AUTO (the default) takes SPLIT when at least half of the plan's
 * taps are paired and the GCF is 16-byte aligned, otherwise TMA where it
 * applies, otherwise ROWS.  A forced TMA falls back to ROWS where TMA does
 * not apply. */
#define GB_STAGE_AUTO (-1)
#define GB_STAGE_SPLIT 0
#define GB_STAGE_TMA 1
#define GB_STAGE_ROWS 2
int gb_plan_set_stage(gb_plan *plan, int32_t stage);

/* 1 when the reference-ABI calls on the current device reach host buffers
 * directly from their kernels (pageable memory through the host's page
 * tables, e.g. Grace with NVLink-C2C): gridding and degridding then move only
 * the 32 x 32-pixel grid blocks their visibilities touch, and kern_detile runs
 * in place on the GPU.  0 when they copy
 * whole buffers instead (no such access, or RC_GB300_HOST_DIRECT=0 in the
 * environment when the first call was made); buffers not 16-byte aligned are
 * always copied.  No counterpart in the reference. */
int gb_host_direct(void);

/* Test hook (host-side fault injection): let the next `after` device
 * allocations of the library succeed and fail the `count` after them with
 * GB_ERR_NOMEM, as a cudaMalloc out of memory would.  (0, 0) turns it off.
 * Every entry point then returns its error and leaves no partial object. */
int gb_debug_fail_allocs(int32_t after, int32_t count);

/* Bounds-checked build (compiled with -DGB_CHECKED: rc_gb300.build(checked=True),
 * librc_gb300_checked.so): the FP32 tiled kernels test every shared-memory,
 * GCF, record and visibility index against its array, count violations in a
 * device word and redirect the access to element 0.  gb_checked_violations
 * returns the count since its last call and clears it (-1 in the normal
 * build); gb_checked_selftest counts two out-of-range indices without touching
 * memory (GB_ERR_ARG in the normal build). */
int gb_checked_violations(int64_t *out);
int gb_checked_selftest(void);

/* Device-side status of a plan's degridding, read synchronously on `stream`:
 * out2[0] = 1 when a TMA stage of a degridding launch did not complete within
 * its bounded wait since the last call (that launch's predictions are then
 * invalid; the word is cleared by this call), out2[1] = the GB_STAGE_* form
 * the last degridding launch used.  Returns GB_ERR_TIMEOUT when out2[0] is
 * set. */
int gb_plan_device_status(gb_plan *plan, int32_t *out2, void *stream);

/* Per-visibility index record (x0, y0, phase ou+8*ov, plane, kept) as the
 * plan computed it, 5 int32 per visibility, into device memory. */
int gb_plan_export_index(const gb_plan *plan, int32_t *d_out5, void *stream);

/* FP32 batched adjoint pair (complex64, interleaved re/im floats).
 *   G (gridding):   grid[pix] += sum_v vis[v] * gcf_v[pix - corner_v]
 *   D (degridding): pred[v]    = sum_pix grid[pix] * conj(gcf_v[pix - corner_v])
 * D is the exact adjoint of G: <D x, y> = <x, G y>.  mode 1 of the degridder
 * gives the reference's kern_degrid product instead: pred = -sum grid * gcf.
 * Visibilities the plan skipped get pred = 0.  Gridding sums each tile's
 * taps in shared memory (float2 per pixel) and adds them into the grid with
 * float2 atomics; degridding adds each lane's products to a compensated sum.
 * Against FP64: rel-L2 about 1e-7 to 2e-7 on the benchmark workloads. */
int gb_grid_f32(gb_plan *plan, const float *d_vis, const float *d_gcf, float *d_grid,
                void *stream);
int gb_degrid_f32(gb_plan *plan, const float *d_gcf, const float *d_grid, float *d_pred,
                  int32_t mode, void *stream);
/* Forward / backward names of the pair, for callers that differentiate
 * through it (a least-squares imaging gradient; no counterpart in the
 * reference, whose degridder is not an adjoint of its gridder).  Both
 * operators are complex-linear, so a backward (vector-Jacobian product in the
 * conjugate convention torch uses for complex tensors) is the adjoint:
 *   gb_grid_forward:    grid += G vis                 (as gb_grid_f32)
 *   gb_grid_backward:   vis_grad = G^H grid_grad = D grid_grad
 *                       (as gb_degrid_f32 mode 0; overwrites vis_grad)
 *   gb_degrid_forward:  pred = D grid                 (as gb_degrid_f32 mode 0)
 *   gb_degrid_backward: grid_grad += D^H pred_grad = G pred_grad
 *                       (as gb_grid_f32; accumulates into grid_grad)
 * Arguments: plan, GCFs, the input, the output, stream. */
int gb_grid_forward(gb_plan *plan, const float *d_gcf, const float *d_vis, float *d_grid,
                    void *stream);
int gb_grid_backward(gb_plan *plan, const float *d_gcf, const float *d_grid_grad,
                     float *d_vis_grad, void *stream);
int gb_degrid_forward(gb_plan *plan, const float *d_gcf, const float *d_grid,
                      float *d_pred, void *stream);
int gb_degrid_backward(gb_plan *plan, const float *d_gcf, const float *d_pred_grad,
                       float *d_grid_grad, void *stream);

/* Plain FP64 path (complex128): no tiling, no sorting; one warp per
 * visibility, FP64 atomics into the grid.  Same operators as above.
 * Degridding computes in double-float (every double held as two floats, to
 * 2^-48; sums to about 2^-48 of the running sum) and takes the native FP64
 * loop when the grid or the GCF holds an Inf, a NaN or a subnormal.  Its
 * first call on a plan allocates the plan's scratch (16 bytes per grid cell
 * of ext_x x ext_y and per GCF element): make it before any stream capture. */
int gb_grid_f64(gb_plan *plan, const double *d_vis, const double *d_gcf, double *d_grid,
                void *stream);
int gb_degrid_f64(gb_plan *plan, const double *d_gcf, const double *d_grid,
                  double *d_pred, int32_t mode, void *stream);
/* The FP64 pair under the forward / backward names (meanings as for
 * gb_grid_forward and the rest above). */
int gb_grid_forward_f64(gb_plan *plan, const double *d_gcf, const double *d_vis,
                        double *d_grid, void *stream);
int gb_grid_backward_f64(gb_plan *plan, const double *d_gcf, const double *d_grid_grad,
                         double *d_vis_grad, void *stream);
int gb_degrid_forward_f64(gb_plan *plan, const double *d_gcf, const double *d_grid,
                          double *d_pred, void *stream);
int gb_degrid_backward_f64(gb_plan *plan, const double *d_gcf, const double *d_pred_grad,
                           double *d_grid_grad, void *stream);

/* On-GPU w-kernel generation (MS4/kernel/cpu/gcf/GCF.cpp semantics): for
 * each plane p, the FP64 phase screen exp(-2 pi i w_p (1 - sqrt(1-l^2-m^2)))
 * times taper(l) taper(m) on a max_support^2 patch (l, m = k * t2 /
 * (max_support/2)), centred in an (8 max_support)^2 arena, centred inverse
 * FFT (cuFFT, FP64), per-phase normalisation by the sum of real parts, and
 * extraction of the centred S_p x S_p taps per phase.  Writes complex128
 * (d_gcf64, may be NULL) and complex64 (d_gcf32, may be NULL) GCF arrays laid
 * out by gcf_offsets.  d_taper: device, max_support doubles, or NULL for none.
 * Allocates its FFT workspace per call. */
int gb_gcf_generate(int32_t n_planes, const double *w_planes, const int32_t *supports,
                    const int64_t *gcf_offsets, int32_t max_support, double t2,
                    const double *d_taper, double *d_gcf64, float *d_gcf32, void *stream);

/* Hogbom CLEAN minor loop on the GPU (engine form, FP32), replacing the
 * reference's kern_hogbom_* minor cycles (MS6/kernel/cpu/gridding/hogbom.cpp)
 * and the MS4 GPU peak-find / PSF-subtract kernels (MS4/kernel/gpu/hogbom/
 * hogbom.cu:31-53).  n_iter iterations of: peak = residual pixel of largest
 * |value| (lowest row-major index on ties); stop when |peak| < threshold;
 * residual -= (gain * peak / psf[ppy][ppx]) * psf shifted so that its peak
 * (psf_peak_x, psf_peak_y) lands on the residual peak (zero outside the PSF);
 * model[peak] += gain * peak.  Images are row-major nx * ny floats; the PSF
 * pnx * pny.  d_work: gb_hogbom_work_bytes() bytes of device scratch.  One
 * launch per iteration, no synchronisation: the sequence can be captured in
 * a CUDA graph.  gb_hogbom_iterations reads back how many iterations
 * subtracted a component (synchronises). */
int gb_hogbom_work_bytes(int32_t nx, int32_t ny, int64_t *bytes);
int gb_hogbom_f32(float *d_residual, int32_t nx, int32_t ny, const float *d_psf, int32_t pnx,
                  int32_t pny, int32_t psf_peak_x, int32_t psf_peak_y, float gain,
                  float threshold, int32_t n_iter, float *d_model, void *d_work,
                  int64_t work_bytes, void *stream);
int gb_hogbom_iterations(const void *d_work, int32_t *iterations, void *stream);

/* The reference's CLEAN kernels (host FP64 images, synchronous), with the
 * reference's own rules: 12 cycles, the "PSF peak" taken as the argmax of
 * |res| over the PSF's extent, the absolute peak value used for subtraction
 * and model, clamped PSF shift; kern_hogbom_model accumulates into `model`,
 * kern_hogbom_residual writes the residual of the cycle that first fell under
 * the threshold (or of the last cycle).
 * replace MS6/kernel/cpu/gridding/hogbom.cpp:128-129, bound at
 * MS6/programs/Kernel/Cleaning.hs:22-44 */
int kern_hogbom_model(double gain, double threshold, buffer_t *psf, buffer_t *res,
                      buffer_t *model);
int kern_hogbom_residual(double gain, double threshold, buffer_t *psf, buffer_t *res,
                         buffer_t *residual);

/* De-tiling and facet rotation, the steps either side of tiled / faceted
 * gridding strategies.
 * kern_detile: out(c,x,y) += in(c,x,y) over the overlap of the two buffers'
 *   (min, extent) regions; replaces MS6/kernel/cpu/gridding/detile.cpp:10-39
 *   (bound at MS6/programs/Kernel/Gridder.hs:81-85).
 * kern_rotate: facet phase rotation vis * exp(2 pi i ((0,0,1) - R (0,0,1)) . uvw)
 *   and, with uvproj != 0, uvw reprojection, R = xyz2uvw(out) * uvw2xyz(in),
 *   out_lon = out_lon0 + out->min[2] * out_lon_incr (lat likewise, min[3]);
 *   replaces MS6/kernel/cpu/gridding/rotate.cpp:11-84 (bound at
 *   MS6/programs/Kernel/Facet.hs:25-54).
 * gb_detile_f32 / gb_rotate_f64: the same on device buffers (complex64 grids
 * with row pitches; 5-double visibility records). */
int kern_detile(buffer_t *in_grid, buffer_t *out_grid);
int kern_rotate(double in_lon, double in_lat, double out_lon0, double out_lat0,
                double out_lon_incr, double out_lat_incr, int32_t uvproj, buffer_t *vis,
                buffer_t *out);
int gb_detile_f32(const float *d_tile, int64_t tile_pitch, int32_t tile_min_x,
                  int32_t tile_min_y, int32_t tile_w, int32_t tile_h, float *d_grid,
                  int64_t grid_pitch, int32_t grid_min_x, int32_t grid_min_y, int32_t grid_w,
                  int32_t grid_h, void *stream);
int gb_rotate_f64(double in_lon, double in_lat, double out_lon, double out_lat, int32_t uvproj,
                  int64_t n, const double *d_vis5, double *d_out5, void *stream);

/* Batched FP32 gridding / degridding: up to GB_MAX_BATCH grids (channels,
 * facets, data sets; any sizes and w-plane sets) in ONE persistent launch fed
 * by one device work queue, longest work first.  The reference runs such units
 * as separate actors, one kernel call per (tile, w-bin) region
 * (MS6/programs/continuum.hs:134-193).  Every member is planned like
 * gb_plan_create (all members must use the same tile and threads); the GCF
 * array is shared (each member's gcf_offsets index into it).  The execute
 * calls take host arrays of n_members device pointers and capture into a CUDA
 * graph. */
#define GB_MAX_BATCH 96
typedef struct gb_batch gb_batch;
typedef struct gb_batch_member {
  gb_geometry geo;
  int64_t n_vis;
  const double *d_uvw;
  int64_t uvw_stride;
  const int32_t *d_plane; /* optional, as for gb_plan_create */
} gb_batch_member;
int gb_batch_create(int32_t n_members, const gb_batch_member *members, void *stream,
                    gb_batch **out);
int gb_batch_destroy(gb_batch *batch);
/* [0] visibilities kept, [1] taps, [2] items, [3] bundles, [4] tile, [5] members, [6] threads */
int gb_batch_stats(const gb_batch *batch, int64_t *stats7);
int gb_batch_grid_f32(gb_batch *batch, const float *const *d_vis, const float *d_gcf,
                      float *const *d_grids, void *stream);
int gb_batch_degrid_f32(gb_batch *batch, const float *d_gcf, const float *const *d_grids,
                        float *const *d_preds, int32_t mode, void *stream);
/* The plain FP64 path over the members (one launch per member, complex128).
 * Degridding as gb_degrid_f64, with one scratch for the batch, grown to the
 * largest member on the first call. */
int gb_batch_grid_f64(gb_batch *batch, const double *const *d_vis, const double *d_gcf,
                      double *const *d_grids, void *stream);
int gb_batch_degrid_f64(gb_batch *batch, const double *d_gcf, const double *const *d_grids,
                        double *const *d_preds, int32_t mode, void *stream);

/* Allocation-free gridding.  No counterpart in the reference.
 *
 * For callers that cannot call cudaMalloc: code running inside a host
 * framework that owns all device memory (a pipeline runtime with a fixed
 * budget or pool, a plugin of another GPU application), or real-time paths
 * where an allocation's latency or failure is not acceptable.  It does what
 * gb_plan_create + gb_grid_f32 + gb_plan_destroy do together (grid += G vis,
 * same FP32 tiled kernel, same tolerance) for one batch of visibilities, and
 * calls no cudaMalloc, cudaFree or allocating library routine: its working
 * memory is one static device array of GB_NOALLOC_SCRATCH_BYTES (8 MiB),
 * which every GPU that loads this library holds until the process exits.
 * The caller passes inputs and the output grid (device pointers, as for
 * gb_plan_create / gb_grid_f32).
 *
 * Limits: at most GB_NOALLOC_MAX_VIS visibilities, GB_NOALLOC_MAX_PLANES
 * planes, n_vis * k^2 <= GB_NOALLOC_MAX_PIECES footprint pieces (k = pieces
 * per axis of the largest support, ceil(S / period_cap)), and at most
 * GB_NOALLOC_MAX_BINS (grid tile, thread-group class) bins; larger requests
 * return GB_ERR_CAPACITY before any GPU work.  A grid more than 32767 tiles
 * wide or high returns GB_ERR_ARG, as gb_plan_create does.
 *
 * The call synchronises `stream` once (to size the kernel launch), so it
 * cannot be captured into a CUDA graph.  The first call on a device looks up
 * the array's device address (cudaGetSymbolAddress) and keeps it for the
 * process: after cudaDeviceReset on a device, do not call this entry point
 * there again.
 * Every call on a device shares the array and leaves its contents behind; each
 * call clears what must start at zero.  Calls whose GPU work overlaps (other
 * streams, other host threads) race on the array: serialise them. */
#define GB_NOALLOC_MAX_VIS (1 << 17)
#define GB_NOALLOC_MAX_PIECES (1 << 18)
#define GB_NOALLOC_MAX_BINS (1 << 16)
#define GB_NOALLOC_MAX_PLANES 256
#define GB_NOALLOC_SCRATCH_BYTES (8 << 20)
int gb_grid_f32_noalloc(const gb_geometry *geo, int64_t n_vis, const double *d_uvw,
                        int64_t uvw_stride, const int32_t *d_plane, const float *d_vis,
                        const float *d_gcf, float *d_grid, void *stream);

/* Image <-> grid transforms either side of the gridder (grid correction and
 * centred FFT), replacing the reference's kern_fft / kern_ifft
 * (MS6/kernel/cpu/gridding/fft1.cpp:29-57) and its GPU cuFFT + fftshift step
 * (MS4/kernel/gpu/fft/cufftshift.cu:9-73).  For an even n x n real image x and
 * a separable taper t (n values, NULL = none):
 *   image_to_grid: grid = fftshift(FFT(ifftshift(x / (t_y t_x))))   (exp(-2 pi i))
 *   grid_to_image: x    = Re[fftshift(IFFT(ifftshift(grid))) / (t_y t_x)]
 * with IFFT unnormalised (exp(+2 pi i)), so grid_to_image is the exact adjoint
 * of image_to_grid.  d_work: n*n complex scratch (not aliasing d_grid). */
int gb_image_to_grid_f32(const float *d_image, const float *d_taper, int32_t n, float *d_grid,
                         void *stream);
int gb_grid_to_image_f32(const float *d_grid, const float *d_taper, int32_t n, float *d_work,
                         float *d_image, void *stream);
int gb_image_to_grid_f64(const double *d_image, const double *d_taper, int32_t n,
                         double *d_grid, void *stream);
int gb_grid_to_image_f64(const double *d_grid, const double *d_taper, int32_t n, double *d_work,
                         double *d_image, void *stream);

/* The reference's FFT kernels on host buffers, same symbols and arguments:
 * kern_fft(image (n,n) doubles, grid (2,n,n) doubles) and kern_ifft(grid,
 * image), n in {1024, 2048, 3072, 4096, 6144, 8192}.  replaces
 * MS6/kernel/cpu/gridding/fft1.cpp:29-57 (dispatch, size check) and the Halide
 * pipelines of fft.cpp:546-677; the exact transforms are stated in
 * rc_gb300/csrc/gb_imaging.cu.  Returns GB_ERR_FFT_SIZE for mismatched or
 * unsupported sizes, GB_ERR_ARG for a malformed buffer.  Synchronous. */
#define GB_ERR_FFT_SIZE (-666) /* MS6/kernel/cpu/gridding/fft1.cpp:38,52 */
#ifndef GB_MS5_ABI /* the MS5 variant binds its own kern_fft (rc_gb300_ms5.h) */
int kern_fft(buffer_t *image, buffer_t *uvg_herm);
#endif
int kern_ifft(buffer_t *uvg, buffer_t *img_shifted);

/* GCF choice for a w-region [w0, w1] among precomputed GCFs of nominal w
 * w_files[i]: the largest w_files[i] <= max(|w0|, |w1|) (the last of equal
 * ones), and whether to conjugate it (w0 < -w1: a mostly negative-w region).
 * replaces gcfGet (MS6/programs/Kernel/Config.hs:128-132) and the conjugation
 * of gcfKernel (MS6/programs/Kernel/IO.hs:97-115).  Host logic, no GPU. */
int gb_gcf_select(int32_t n_files, const double *w_files, double w0, double w1, int32_t *index,
                  int32_t *conjugate);
/* Conjugate a device GCF array in place (negate the imaginary parts). */
int gb_gcf_conjugate_f32(float *d_gcf, int64_t n_complex, void *stream);
int gb_gcf_conjugate_f64(double *d_gcf, int64_t n_complex, void *stream);

/* Zero `n_complex` complex64 grid elements (device). */
int gb_grid_zero_f32(float *d_grid, int64_t n_complex, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* RC_GB300_H */
