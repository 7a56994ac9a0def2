/*
 * ORACLE — test infrastructure only.
 *
 * CPU FP64 restatement of the reference's convolutional gridding and
 * degridding, used by tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline leg as the checker and as the timed CPU baseline.  Nothing in
 * the rc_gb300 product path links or calls this file.
 *
 * Semantics restated (SKA-ScienceDataProcessor/RC):
 *   index math      MS6/kernel/cpu/gridding/scatter.cpp:56-76, degrid.cpp:46-67
 *   gridding        MS6/kernel/cpu/gridding/scatter.cpp:89-111
 *   degridding      MS6/kernel/cpu/gridding/degrid.cpp:78-98
 *   complex product MS6/kernel/cpu/gridding/utils.h:25-30
 *   w-binning       MS6/programs/Kernel/Binning.hs:60-90
 *
 * The reference kernels are Halide generators; Halide is a third-party
 * dependency that is not vendored (unpinned; the legacy buffer_t API dates it
 * to 2015-16 Halide).  Its `round` is taken as round-half-to-even (nearbyint
 * under FE_TONEAREST), `floor`/`clamp` are the usual, integer division of
 * non-negative values truncates.  A cast<int> of a value outside the int32
 * range (or NaN) yields INT_MIN on x86, which lands out of bounds, so such a
 * visibility is skipped; the restatement encodes exactly that.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OVER 8

/* cast<int>(x) for an integral-valued double x, with the x86 out-of-range
 * result (INT_MIN) for |x| >= 2^31 or NaN. */
static inline int32_t cast_int(double x) {
  if (!(x > -2147483649.0 && x < 2147483648.0)) return INT32_MIN;
  return (int32_t)x;
}

/* scatter.cpp:69-71: uvs = uv*scale; overc = clamp(round(8*(uvs-floor(uvs))),0,7);
 * uv = cast<int>(round(uvs) + grid_size/2 - S/2). */
static inline void index1(double uv, double scale, int32_t grid_size, int32_t S,
                          int32_t *corner, int32_t *over) {
  double s = uv * scale;
  double fr = s - floor(s);
  double o = nearbyint((double)OVER * fr);
  int32_t oi = cast_int(o);
  if (oi < 0) oi = 0;
  if (oi > OVER - 1) oi = OVER - 1;
  *over = oi;
  *corner = cast_int(nearbyint(s) + (double)(grid_size / 2) - (double)(S / 2));
}

/* scatter.cpp:58-62 / degrid.cpp:46-50: accepted range of the GCF corner. */
static inline void bounds(int32_t margin, int32_t S, int32_t min_x, int32_t min_y,
                          int32_t ext_x, int32_t ext_y,
                          int32_t *lo_x, int32_t *hi_x, int32_t *lo_y, int32_t *hi_y) {
  int32_t gm = (margin - S) / 2;
  if (margin - S < 0) gm = 0; /* max(0, floor((margin-S)/2)) */
  *lo_x = min_x + gm;
  *hi_x = min_x + ext_x - S - 1 - gm;
  *lo_y = min_y + gm;
  *hi_y = min_y + ext_y - S - 1 - gm;
}

/*
 * Per-visibility index record: x0, y0 (GCF corner pixel, absolute grid
 * coordinates), ou, ov (oversample phase), inb (1 if the visibility is
 * gridded).  out has 5 int32 per visibility.
 */
void orc_index(int64_t n, const double *vis, int64_t vis_stride, double scale,
               int32_t grid_size, int32_t S, int32_t margin, int32_t min_x,
               int32_t min_y, int32_t ext_x, int32_t ext_y, int32_t *out) {
  int32_t lo_x, hi_x, lo_y, hi_y;
  bounds(margin, S, min_x, min_y, ext_x, ext_y, &lo_x, &hi_x, &lo_y, &hi_y);
  for (int64_t t = 0; t < n; t++) {
    const double *r = vis + t * vis_stride;
    int32_t x0, y0, ou, ov;
    index1(r[0], scale, grid_size, S, &x0, &ou);
    index1(r[1], scale, grid_size, S, &y0, &ov);
    int32_t *o = out + 5 * t;
    o[0] = x0; o[1] = y0; o[2] = ou; o[3] = ov;
    o[4] = (x0 >= lo_x && x0 <= hi_x && y0 >= lo_y && y0 <= hi_y) ? 1 : 0;
  }
}

/*
 * kern_scatter semantics (scatter.cpp:89-111).  vis: n records of 5 doubles
 * (u, v, w, re, im) with record stride vis_stride; gcf: [64][S][S][2] doubles
 * with phase index ou + 8*ov; grid: complex doubles, row pitch `pitch`
 * complex elements, covering x in [min_x, min_x+ext_x), y in [min_y, min_y+ext_y).
 * Loop nest as in the reference RDom: gcfy outermost, then visibility, then
 * gcfx, then the complex component.
 */
void orc_scatter(double scale, int32_t grid_size, int32_t margin, int32_t S,
                 int64_t n, const double *vis, int64_t vis_stride,
                 const double *gcf, double *grid, int32_t min_x, int32_t min_y,
                 int32_t ext_x, int32_t ext_y, int64_t pitch) {
  int32_t *idx = (int32_t *)malloc(sizeof(int32_t) * 5 * (n > 0 ? n : 1));
  orc_index(n, vis, vis_stride, scale, grid_size, S, margin, min_x, min_y, ext_x,
            ext_y, idx);
  for (int32_t j = 0; j < S; j++) {
    for (int64_t t = 0; t < n; t++) {
      const int32_t *o = idx + 5 * t;
      if (!o[4]) continue;
      const double vr = vis[t * vis_stride + 3], vi = vis[t * vis_stride + 4];
      const double *g = gcf + 2 * ((int64_t)(o[2] + OVER * o[3]) * S * S + (int64_t)j * S);
      double *row = grid + 2 * ((int64_t)(o[1] + j - min_y) * pitch + (o[0] - min_x));
      for (int32_t i = 0; i < S; i++) {
        const double gr = g[2 * i], gi = g[2 * i + 1];
        row[2 * i + 0] += vr * gr - vi * gi;
        row[2 * i + 1] += vr * gi + vi * gr;
      }
    }
  }
  free(idx);
}

/*
 * kern_degrid semantics (degrid.cpp:78-98): vis_out = vis, then for in-bound
 * visibilities vis_out[re,im] -= sum_{j,i} grid[y0+j][x0+i] * gcf[...][j][i]
 * (no conjugate), gcfy outer, gcfx inner.  Out-of-bound visibilities pass
 * through unchanged.
 */
void orc_degrid(double scale, int32_t grid_size, int32_t margin, int32_t S,
                int64_t n, const double *vis, int64_t vis_stride,
                const double *gcf, const double *grid, int32_t min_x,
                int32_t min_y, int32_t ext_x, int32_t ext_y, int64_t pitch,
                double *vis_out, int64_t out_stride) {
  int32_t lo_x, hi_x, lo_y, hi_y;
  bounds(margin, S, min_x, min_y, ext_x, ext_y, &lo_x, &hi_x, &lo_y, &hi_y);
  for (int64_t t = 0; t < n; t++) {
    const double *r = vis + t * vis_stride;
    double *o = vis_out + t * out_stride;
    for (int k = 0; k < 5; k++) o[k] = r[k];
    int32_t x0, y0, ou, ov;
    index1(r[0], scale, grid_size, S, &x0, &ou);
    index1(r[1], scale, grid_size, S, &y0, &ov);
    if (!(x0 >= lo_x && x0 <= hi_x && y0 >= lo_y && y0 <= hi_y)) continue;
    const double *g0 = gcf + 2 * ((int64_t)(ou + OVER * ov) * S * S);
    double accr = o[3], acci = o[4];
    for (int32_t j = 0; j < S; j++) {
      const double *row = grid + 2 * ((int64_t)(y0 + j - min_y) * pitch + (x0 - min_x));
      const double *g = g0 + 2 * (int64_t)j * S;
      for (int32_t i = 0; i < S; i++) {
        const double ur = row[2 * i], ui = row[2 * i + 1];
        const double gr = g[2 * i], gi = g[2 * i + 1];
        accr -= ur * gr - ui * gi;
        acci -= ur * gi + ui * gr;
      }
    }
    o[3] = accr;
    o[4] = acci;
  }
}

/*
 * Multi-plane forms (the batched engine's semantics): visibility t uses the
 * GCF of plane[t] with support supp[plane[t]], stored at complex offset
 * gcf_off[plane[t]] in `gcf` ([64][S][S] complex per plane).  The grid is the
 * full grid (min 0) of ext_x x ext_y pixels with row pitch `pitch`.  Each
 * visibility follows the single-GCF index/bounds rules above with its own S.
 * Visibility values are complex (re, im) pairs, uvw separate (stride
 * uvw_stride doubles).  plane[t] < 0 skips the visibility.
 *
 * mode for degridding: 0 = exact adjoint of gridding,
 * pred = sum grid * conj(gcf); 1 = the reference's kern_degrid form,
 * pred = -sum grid * gcf (no conjugate, subtracted).
 */
static void scatter_planes_range(double scale, int32_t grid_size, int32_t margin,
                                 int64_t t0, int64_t t1, const double *uvw,
                                 int64_t uvw_stride, const double *vis,
                                 const int32_t *plane, const int32_t *supp,
                                 const int64_t *gcf_off, const double *gcf,
                                 double *grid, int32_t ext_x, int32_t ext_y,
                                 int64_t pitch) {
  for (int64_t t = t0; t < t1; t++) {
    const int32_t p = plane[t];
    if (p < 0) continue;
    const int32_t S = supp[p];
    int32_t lo_x, hi_x, lo_y, hi_y, x0, y0, ou, ov;
    bounds(margin, S, 0, 0, ext_x, ext_y, &lo_x, &hi_x, &lo_y, &hi_y);
    index1(uvw[t * uvw_stride + 0], scale, grid_size, S, &x0, &ou);
    index1(uvw[t * uvw_stride + 1], scale, grid_size, S, &y0, &ov);
    if (!(x0 >= lo_x && x0 <= hi_x && y0 >= lo_y && y0 <= hi_y)) continue;
    const double vr = vis[2 * t], vi = vis[2 * t + 1];
    const double *g0 = gcf + 2 * (gcf_off[p] + (int64_t)(ou + OVER * ov) * S * S);
    for (int32_t j = 0; j < S; j++) {
      double *row = grid + 2 * ((int64_t)(y0 + j) * pitch + x0);
      const double *g = g0 + 2 * (int64_t)j * S;
      for (int32_t i = 0; i < S; i++) {
        const double gr = g[2 * i], gi = g[2 * i + 1];
        row[2 * i + 0] += vr * gr - vi * gi;
        row[2 * i + 1] += vr * gi + vi * gr;
      }
    }
  }
}

void orc_scatter_planes(double scale, int32_t grid_size, int32_t margin, int64_t n,
                        const double *uvw, int64_t uvw_stride, const double *vis,
                        const int32_t *plane, const int32_t *supp,
                        const int64_t *gcf_off, const double *gcf, double *grid,
                        int32_t ext_x, int32_t ext_y, int64_t pitch) {
  scatter_planes_range(scale, grid_size, margin, 0, n, uvw, uvw_stride, vis, plane,
                       supp, gcf_off, gcf, grid, ext_x, ext_y, pitch);
}

/* All-core variant of the above: per-thread private grids and a final sum, as
 * the reference's OpenMP gridder does (MS4 scatter_gridder_w_dependent_dyn_1p.cpp:
 * 210-230, addGrids :24-43).  Returns the number of threads used. */
int orc_scatter_planes_omp(double scale, int32_t grid_size, int32_t margin, int64_t n,
                           const double *uvw, int64_t uvw_stride, const double *vis,
                           const int32_t *plane, const int32_t *supp,
                           const int64_t *gcf_off, const double *gcf, double *grid,
                           int32_t ext_x, int32_t ext_y, int64_t pitch, int nthreads) {
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  if (nthreads == 1) {
    scatter_planes_range(scale, grid_size, margin, 0, n, uvw, uvw_stride, vis, plane,
                         supp, gcf_off, gcf, grid, ext_x, ext_y, pitch);
    return 1;
  }
  const int64_t cells = 2 * (int64_t)ext_y * pitch;
  double *priv = (double *)calloc((size_t)cells * (size_t)(nthreads - 1), sizeof(double));
  if (!priv) return -1;
#pragma omp parallel num_threads(nthreads)
  {
    const int tid = omp_get_thread_num();
    const int nt = omp_get_num_threads();
    double *mine = tid == 0 ? grid : priv + (int64_t)(tid - 1) * cells;
    const int64_t t0 = n * tid / nt, t1 = n * (tid + 1) / nt;
    scatter_planes_range(scale, grid_size, margin, t0, t1, uvw, uvw_stride, vis, plane,
                         supp, gcf_off, gcf, mine, ext_x, ext_y, pitch);
#pragma omp barrier
#pragma omp for schedule(static)
    for (int64_t c = 0; c < cells; c++) {
      double s = 0.0;
      for (int k = 0; k < nt - 1; k++) s += priv[(int64_t)k * cells + c];
      grid[c] += s;
    }
  }
  free(priv);
  return nthreads;
#else
  (void)nthreads;
  scatter_planes_range(scale, grid_size, margin, 0, n, uvw, uvw_stride, vis, plane,
                       supp, gcf_off, gcf, grid, ext_x, ext_y, pitch);
  return 1;
#endif
}

void orc_degrid_planes(double scale, int32_t grid_size, int32_t margin, int64_t n,
                       const double *uvw, int64_t uvw_stride, const int32_t *plane,
                       const int32_t *supp, const int64_t *gcf_off, const double *gcf,
                       const double *grid, int32_t ext_x, int32_t ext_y, int64_t pitch,
                       int32_t mode, double *pred, int nthreads) {
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads)
#else
  (void)nthreads;
#endif
  for (int64_t t = 0; t < n; t++) {
    pred[2 * t] = 0.0;
    pred[2 * t + 1] = 0.0;
    const int32_t p = plane[t];
    if (p < 0) continue;
    const int32_t S = supp[p];
    int32_t lo_x, hi_x, lo_y, hi_y, x0, y0, ou, ov;
    bounds(margin, S, 0, 0, ext_x, ext_y, &lo_x, &hi_x, &lo_y, &hi_y);
    index1(uvw[t * uvw_stride + 0], scale, grid_size, S, &x0, &ou);
    index1(uvw[t * uvw_stride + 1], scale, grid_size, S, &y0, &ov);
    if (!(x0 >= lo_x && x0 <= hi_x && y0 >= lo_y && y0 <= hi_y)) continue;
    const double *g0 = gcf + 2 * (gcf_off[p] + (int64_t)(ou + OVER * ov) * S * S);
    const double sgn = mode == 1 ? -1.0 : 1.0;
    const double cj = mode == 1 ? 1.0 : -1.0; /* sign applied to the GCF imaginary part */
    double ar = 0.0, ai = 0.0;
    for (int32_t j = 0; j < S; j++) {
      const double *row = grid + 2 * ((int64_t)(y0 + j) * pitch + x0);
      const double *g = g0 + 2 * (int64_t)j * S;
      for (int32_t i = 0; i < S; i++) {
        const double ur = row[2 * i], ui = row[2 * i + 1];
        const double gr = g[2 * i], gi = cj * g[2 * i + 1];
        ar += ur * gr - ui * gi;
        ai += ur * gi + ui * gr;
      }
    }
    pred[2 * t] = sgn * ar;
    pred[2 * t + 1] = sgn * ai;
  }
}

/* Binning.hs:88-89: bin = clamp(floor((w-low)/(high-low)*bins), 0, bins-1);
 * visibilities outside [low, high] get -1 (Binning.hs:85). */
void orc_wbin(int64_t n, const double *uvw, int64_t uvw_stride, double low, double high,
              int32_t bins, int32_t *out) {
  for (int64_t t = 0; t < n; t++) {
    const double w = uvw[t * uvw_stride + 2];
    if (!(w >= low && w <= high)) { out[t] = -1; continue; }
    if (bins <= 1 || !(high > low)) { out[t] = 0; continue; } /* degenerate range */
    double b = floor((w - low) / (high - low) * (double)bins);
    int32_t bi = !(b >= 0) ? 0 : (b > bins - 1 ? bins - 1 : (int32_t)b); /* NaN -> 0 */
    out[t] = bi;
  }
}
