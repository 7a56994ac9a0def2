// Plain FP64 gridder / degridder (complex128) and the reference-ABI entry
// points built on them.
//
// "Plain" = no sorting, no tiling, no shared memory: one warp per
// visibility, lanes over the S*S taps, FP64 atomics into the grid (gridding)
// or a warp-shuffle reduction (degridding).  It is the FP64 GPU comparison
// path of the engine and the implementation behind kern_scatter_gpu1 /
// kern_degrid_gpu1 / nvGridder / kern_scatter / kern_degrid, whose semantics
// are the reference's (MS6/kernel/cpu/gridding/scatter.cpp:56-111,
// degrid.cpp:41-98) on Halide buffer_t host buffers.
#include <stdio.h>
#include <string.h>

#include "gb_common.cuh"
#include "gb_plan.cuh"
#include "gb_runtime.cuh"
#include "rc_gb300_ms5.h"

namespace gb {

// Tap walk of a warp over an S x S footprint, lane-strided: tap k = lane +
// 32 m, (i, j) = (k mod S, k div S), advanced incrementally.
struct TapWalk {
  int i, j, di, dj, S;
  __device__ __forceinline__ TapWalk(int S_, int lane) : S(S_) {
    j = lane / S_;
    i = lane - j * S_;
    dj = 32 / S_;
    di = 32 - dj * S_;
  }
  __device__ __forceinline__ void next() {
    i += di;
    j += dj;
    if (i >= S) {
      i -= S;
      j++;
    }
  }
};

// grid[y0+j][x0+i] += vis * gcf[j][i] for the S*S taps of one visibility.
__device__ __forceinline__ void warp_scatter64(double2* __restrict__ base, int64_t pitch,
                                               const double2* __restrict__ g, int S,
                                               double vr, double vi, int lane) {
  TapWalk w(S, lane);
  for (; w.j < S; w.next()) {
    const double2 c = __ldg(g + w.j * S + w.i);
    double2* p = base + (int64_t)w.j * pitch + w.i;
    atomicAdd(&p->x, vr * c.x - vi * c.y);
    atomicAdd(&p->y, vr * c.y + vi * c.x);
  }
}

// sum over taps of grid * gcf (conj_g: grid * conj(gcf)), reduced over the warp.
__device__ __forceinline__ double2 warp_gather64(const double2* __restrict__ base, int64_t pitch,
                                                 const double2* __restrict__ g, int S,
                                                 bool conj_g, int lane) {
  double ar = 0.0, ai = 0.0;
  const double sg = conj_g ? -1.0 : 1.0;
  TapWalk w(S, lane);
  for (; w.j < S; w.next()) {
    const double2 c = __ldg(g + w.j * S + w.i);
    const double2 u = base[(int64_t)w.j * pitch + w.i];
    const double ci = sg * c.y;
    ar += u.x * c.x - u.y * ci;
    ai += u.x * ci + u.y * c.x;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ar += __shfl_xor_sync(0xffffffffu, ar, o);
    ai += __shfl_xor_sync(0xffffffffu, ai, o);
  }
  return make_double2(ar, ai);
}

// ---------------------------------------------------------------- single GCF (ABI form)
struct SingleGeo {
  double scale;
  int32_t grid_size, margin, S;
  int32_t min_x, min_y, ext_x, ext_y;
  int64_t pitch;  // complex elements per grid row
};

__global__ void k_scatter_single64(int64_t n, const double* __restrict__ vis5,
                                   const double2* __restrict__ gcf, double2* __restrict__ grid,
                                   SingleGeo geo) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t t = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); t < n;
       t += warps) {
    const double* r = vis5 + 5 * t;
    const VisIndex ix = vis_index(r[0], r[1], geo.scale, geo.grid_size, geo.S, geo.margin,
                                  geo.min_x, geo.min_y, geo.ext_x, geo.ext_y);
    if (!ix.keep) continue;
    double2* base = grid + (int64_t)(ix.y0 - geo.min_y) * geo.pitch + (ix.x0 - geo.min_x);
    warp_scatter64(base, geo.pitch, gcf + (int64_t)ix.phase * geo.S * geo.S, geo.S, r[3], r[4],
                   lane);
  }
}

// vis_out = vis; in-bound: vis_out.re/im -= sum grid * gcf (degrid.cpp:78-98).
__global__ void k_degrid_single64(int64_t n, const double* __restrict__ vis5,
                                  const double2* __restrict__ gcf,
                                  const double2* __restrict__ grid, double* __restrict__ out5,
                                  SingleGeo geo) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t t = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); t < n;
       t += warps) {
    const double* r = vis5 + 5 * t;
    double* o = out5 + 5 * t;
    const VisIndex ix = vis_index(r[0], r[1], geo.scale, geo.grid_size, geo.S, geo.margin,
                                  geo.min_x, geo.min_y, geo.ext_x, geo.ext_y);
    double2 acc = make_double2(0.0, 0.0);
    if (ix.keep) {
      const double2* base =
          grid + (int64_t)(ix.y0 - geo.min_y) * geo.pitch + (ix.x0 - geo.min_x);
      acc = warp_gather64(base, geo.pitch, gcf + (int64_t)ix.phase * geo.S * geo.S, geo.S,
                          false, lane);
    }
    if (lane < 5) {
      double val = r[lane];
      if (lane == 3) val -= acc.x;
      if (lane == 4) val -= acc.y;
      o[lane] = val;
    }
  }
}

// ---------------------------------------------------------------- multi-plane (engine form)
__global__ void k_grid_plain64(PlanDev P, const double2* __restrict__ vis,
                               const double2* __restrict__ gcf, double2* __restrict__ grid) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t t = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); t < P.n_vis;
       t += warps) {
    const int32_t p = P.plane[t];
    if (p < 0) continue;
    const int32_t S = P.supports[p];
    const double* r = P.uvw + t * P.uvw_stride;
    const VisIndex ix =
        vis_index(r[0], r[1], P.scale, P.grid_size, S, P.margin, 0, 0, P.ext_x, P.ext_y);
    if (!ix.keep) continue;
    const double2 v = vis[t];
    warp_scatter64(grid + (int64_t)ix.y0 * P.pitch + ix.x0, P.pitch,
                   gcf + P.gcf_offsets[p] + (int64_t)ix.phase * S * S, S, v.x, v.y, lane);
  }
}

__global__ void k_degrid_plain64(PlanDev P, const double2* __restrict__ gcf,
                                 const double2* __restrict__ grid, double2* __restrict__ pred,
                                 int mode) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t t = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); t < P.n_vis;
       t += warps) {
    const int32_t p = P.plane[t];
    double2 acc = make_double2(0.0, 0.0);
    if (p >= 0) {
      const int32_t S = P.supports[p];
      const double* r = P.uvw + t * P.uvw_stride;
      const VisIndex ix =
          vis_index(r[0], r[1], P.scale, P.grid_size, S, P.margin, 0, 0, P.ext_x, P.ext_y);
      if (ix.keep) {
        acc = warp_gather64(grid + (int64_t)ix.y0 * P.pitch + ix.x0, P.pitch,
                            gcf + P.gcf_offsets[p] + (int64_t)ix.phase * S * S, S, mode == 0,
                            lane);
        if (mode == 1) {
          acc.x = -acc.x;
          acc.y = -acc.y;
        }
      }
    }
    if (lane == 0) pred[t] = acc;
  }
}

static int plain_grid_dims(int64_t n, int* blocks) {
  const int64_t warps_needed = n;
  int64_t b = (warps_needed + 7) / 8;
  const int64_t cap = (int64_t)sm_count() * 16;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  *blocks = (int)b;
  return 256;
}

int launch_grid_plain64(const gb_plan* plan, const double* vis, const double* gcf, double* grid,
                        cudaStream_t s) {
  int blocks;
  const int threads = plain_grid_dims(plan->dev.n_vis, &blocks);
  k_grid_plain64<<<blocks, threads, 0, s>>>(plan->dev, (const double2*)vis, (const double2*)gcf,
                                            (double2*)grid);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

int launch_degrid_plain64(const gb_plan* plan, const double* gcf, const double* grid,
                          double* pred, int mode, cudaStream_t s) {
  int blocks;
  const int threads = plain_grid_dims(plan->dev.n_vis, &blocks);
  k_degrid_plain64<<<blocks, threads, 0, s>>>(plan->dev, (const double2*)gcf,
                                              (const double2*)grid, (double2*)pred, mode);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

// ---------------------------------------------------------------- buffer_t validation
// GCF size as the reference dispatchers read it (gcf_common.h:8-14).
static int32_t check_size(const buffer_t* gcf) {
  const int32_t size = gcf->extent[1];
  if (gcf->extent[0] == 2 && gcf->extent[2] == size) return size;
  return -1;
}

static bool legacy_size(int32_t S) { return S == 8 || S == 16 || S == 32 || S == 64; }

// GCF constraints of the generated kernels (scatter.cpp:36-41).
static int check_gcf(const buffer_t* g, int32_t S, const char* who) {
  if (!g->host || g->elem_size != 8 || g->stride[0] != 1 || g->stride[1] != 2 ||
      g->stride[2] != 2 * S || g->stride[3] != 2 * S * S || g->extent[3] != GB_PHASES ||
      g->min[0] != 0 || g->min[1] != 0 || g->min[2] != 0 || g->min[3] != 0) {
    gb_set_error(GB_ERR_ARG, "%s: gcf buffer must be dense (2,%d,%d,64) doubles", who, S, S);
    return GB_ERR_ARG;
  }
  return GB_OK;
}

// Visibility buffer: (5, N) doubles, strides (1, 5), min(0) = 0 (scatter.cpp:30-32).
static int check_vis(const buffer_t* v, const char* who, const char* name) {
  if (v->elem_size != 8 || v->extent[0] != 5 || v->stride[0] != 1 || v->min[0] != 0 ||
      v->extent[1] < 0 || (v->extent[1] > 1 && v->stride[1] != 5) ||
      (v->extent[1] > 0 && !v->host)) {
    gb_set_error(GB_ERR_ARG, "%s: %s buffer must be (5,N) doubles with strides (1,5)", who,
                 name);
    return GB_ERR_ARG;
  }
  return GB_OK;
}

// Complex grid buffer: (2, W, H) doubles, strides (1, 2, stride2), stride2 even
// and >= 2W (scatter.cpp:52-54).
static int check_grid(const buffer_t* u, const char* who) {
  if (!u->host || u->elem_size != 8 || u->extent[0] != 2 || u->stride[0] != 1 ||
      u->stride[1] != 2 || u->extent[1] <= 0 || u->extent[2] <= 0 ||
      (u->extent[2] > 1 && (u->stride[2] < 2 * u->extent[1] || (u->stride[2] & 1)))) {
    gb_set_error(GB_ERR_ARG, "%s: grid buffer must be (2,W,H) doubles, strides (1,2,>=2W)", who);
    return GB_ERR_ARG;
  }
  return GB_OK;
}

static int64_t grid_row_doubles(const buffer_t* u) {
  return u->extent[2] > 1 ? (int64_t)u->stride[2] : 2 * (int64_t)u->extent[1];
}

// Synchronous single-GCF gridding on host buffers.
static int compat_scatter(const char* who, int size_err, double scale, int32_t grid_size,
                          int32_t margin, buffer_t* vis, buffer_t* gcf, buffer_t* uvg) {
  if (!vis || !gcf || !uvg) {
    gb_set_error(GB_ERR_ARG, "%s: NULL buffer", who);
    return GB_ERR_ARG;
  }
  const int32_t S = check_size(gcf);
  if (!legacy_size(S)) return size_err;
  int rc;
  if ((rc = check_gcf(gcf, S, who)) || (rc = check_vis(vis, who, "vis")) ||
      (rc = check_grid(uvg, who)))
    return rc;
  const int64_t n = vis->extent[1];
  const int32_t W = uvg->extent[1], H = uvg->extent[2];
  const int64_t row = grid_row_doubles(uvg);
  cudaStream_t s;
  if ((rc = stage_stream(&s))) return rc;
  void *d_vis, *d_gcf, *d_grid;
  const size_t gcf_bytes = (size_t)GB_PHASES * S * S * 16;
  const size_t grid_bytes = (size_t)W * H * 16;
  if ((rc = stage_buffer(0, (size_t)n * 40, &d_vis)) || (rc = stage_buffer(1, gcf_bytes, &d_gcf)) ||
      (rc = stage_buffer(2, grid_bytes, &d_grid)))
    return rc;
  if (n > 0) GB_CUDA_TRY(cudaMemcpyAsync(d_vis, vis->host, (size_t)n * 40, cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemcpyAsync(d_gcf, gcf->host, gcf_bytes, cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemcpy2DAsync(d_grid, (size_t)W * 16, uvg->host, (size_t)row * 8, (size_t)W * 16,
                                H, cudaMemcpyHostToDevice, s));
  if (n > 0) {
    SingleGeo geo{scale, grid_size, margin, S, uvg->min[1], uvg->min[2], W, H, (int64_t)W};
    int blocks;
    const int threads = plain_grid_dims(n, &blocks);
    k_scatter_single64<<<blocks, threads, 0, s>>>(n, (const double*)d_vis, (const double2*)d_gcf,
                                                  (double2*)d_grid, geo);
    GB_CUDA_TRY(cudaGetLastError());
  }
  GB_CUDA_TRY(cudaMemcpy2DAsync(uvg->host, (size_t)row * 8, d_grid, (size_t)W * 16, (size_t)W * 16,
                                H, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GB_OK;
}

// Synchronous single-GCF degridding on host buffers.
static int compat_degrid(const char* who, int size_err, double scale, int32_t grid_size,
                         int32_t margin, buffer_t* gcf, buffer_t* uvg, buffer_t* vis,
                         buffer_t* vis_out) {
  if (!vis || !gcf || !uvg || !vis_out) {
    gb_set_error(GB_ERR_ARG, "%s: NULL buffer", who);
    return GB_ERR_ARG;
  }
  const int32_t S = check_size(gcf);
  if (!legacy_size(S)) return size_err;
  int rc;
  if ((rc = check_gcf(gcf, S, who)) || (rc = check_vis(vis, who, "vis")) ||
      (rc = check_vis(vis_out, who, "vis_out")) || (rc = check_grid(uvg, who)))
    return rc;
  // vis_out(f, t) = vis(f, t) over vis_out's region: vis must cover it
  // (degrid.cpp:80-82).
  const int64_t n = vis_out->extent[1];
  const int64_t first = (int64_t)vis_out->min[1] - vis->min[1];
  if (n > 0 && (first < 0 || first + n > vis->extent[1])) {
    gb_set_error(GB_ERR_ARG, "%s: vis does not cover the vis_out region", who);
    return GB_ERR_ARG;
  }
  const int32_t W = uvg->extent[1], H = uvg->extent[2];
  const int64_t row = grid_row_doubles(uvg);
  cudaStream_t s;
  if ((rc = stage_stream(&s))) return rc;
  void *d_vis, *d_gcf, *d_grid, *d_out;
  const size_t gcf_bytes = (size_t)GB_PHASES * S * S * 16;
  const size_t grid_bytes = (size_t)W * H * 16;
  if ((rc = stage_buffer(0, (size_t)n * 40, &d_vis)) || (rc = stage_buffer(1, gcf_bytes, &d_gcf)) ||
      (rc = stage_buffer(2, grid_bytes, &d_grid)) || (rc = stage_buffer(3, (size_t)n * 40, &d_out)))
    return rc;
  if (n == 0) return GB_OK;
  GB_CUDA_TRY(cudaMemcpyAsync(d_vis, (const double*)vis->host + 5 * first, (size_t)n * 40,
                              cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemcpyAsync(d_gcf, gcf->host, gcf_bytes, cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemcpy2DAsync(d_grid, (size_t)W * 16, uvg->host, (size_t)row * 8, (size_t)W * 16,
                                H, cudaMemcpyHostToDevice, s));
  SingleGeo geo{scale, grid_size, margin, S, uvg->min[1], uvg->min[2], W, H, (int64_t)W};
  int blocks;
  const int threads = plain_grid_dims(n, &blocks);
  k_degrid_single64<<<blocks, threads, 0, s>>>(n, (const double*)d_vis, (const double2*)d_gcf,
                                               (const double2*)d_grid, (double*)d_out, geo);
  GB_CUDA_TRY(cudaGetLastError());
  GB_CUDA_TRY(cudaMemcpyAsync(vis_out->host, d_out, (size_t)n * 40, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GB_OK;
}

}  // namespace gb

using namespace gb;

extern "C" int kern_scatter_gpu1(double scale, int32_t grid_size, int32_t margin_size,
                                 buffer_t* vis, buffer_t* gcf, buffer_t* uvg) {
  return compat_scatter("kern_scatter_gpu1", GB_ERR_SCATTER_GPU_SIZE, scale, grid_size,
                        margin_size, vis, gcf, uvg);
}

#ifdef GB_MS5_ABI
// MS5's gridder binding (MS5/programs/Kernel/Gridder.hs:28-35; the kernel is
// generated by MS5/kernel/cpu/gridding/scatter.cpp:10-121): no margin argument
// and the GCF size fixed at 16.  Its bounds, min .. min + extent - 16 - 1, are
// the MS6 rule with the margin equal to the support.
extern "C" int kern_scatter(double scale, int32_t grid_size, buffer_t* vis, buffer_t* gcf,
                            buffer_t* uvg) {
  if (gcf && check_size(gcf) != 16) {
    gb_set_error(GB_ERR_ARG, "kern_scatter: the GCF must be (2,16,16,64) (MS5/scatter.cpp:36-41)");
    return GB_ERR_ARG;
  }
  return compat_scatter("kern_scatter", GB_ERR_ARG, scale, grid_size, 16, vis, gcf, uvg);
}
#else
extern "C" int kern_scatter(double scale, int32_t grid_size, int32_t margin_size, buffer_t* vis,
                            buffer_t* gcf, buffer_t* uvg) {
  return compat_scatter("kern_scatter", GB_ERR_SCATTER_SIZE, scale, grid_size, margin_size, vis,
                        gcf, uvg);
}
#endif

extern "C" int nvGridder(double scale, int32_t grid_size, int32_t margin_size, buffer_t* vis,
                         buffer_t* gcf, buffer_t* uvg) {
  return compat_scatter("nvGridder", GB_ERR_SCATTER_GPU_SIZE, scale, grid_size, margin_size, vis,
                        gcf, uvg);
}

extern "C" int kern_degrid_gpu1(double scale, int32_t grid_size, int32_t margin_size,
                                buffer_t* gcf, buffer_t* uvg, buffer_t* vis, buffer_t* vis_out) {
  return compat_degrid("kern_degrid_gpu1", GB_ERR_DEGRID_GPU_SIZE, scale, grid_size, margin_size,
                       gcf, uvg, vis, vis_out);
}

extern "C" int kern_degrid(double scale, int32_t grid_size, int32_t margin_size, buffer_t* gcf,
                           buffer_t* uvg, buffer_t* vis, buffer_t* vis_out) {
  return compat_degrid("kern_degrid", GB_ERR_DEGRID_SIZE, scale, grid_size, margin_size, gcf, uvg,
                       vis, vis_out);
}

// kern_init (init.cpp:8-15): zero the complex grid region described by uvg.
// The buffer is host memory and the reference's result is wanted there, so
// this is a host memset of the region (no device round trip).
extern "C" int kern_init(buffer_t* uvg) {
  if (!uvg) {
    gb_set_error(GB_ERR_ARG, "kern_init: NULL buffer");
    return GB_ERR_ARG;
  }
  int rc = check_grid(uvg, "kern_init");
  if (rc) return rc;
  const int64_t row = grid_row_doubles(uvg);
  double* p = (double*)uvg->host;
  for (int32_t y = 0; y < uvg->extent[2]; y++)
    memset(p + (int64_t)y * row, 0, (size_t)uvg->extent[1] * 16);
  return GB_OK;
}

// kern_psf_vis (psf_vis.cpp:16-27): out = vis with re = 1, im = 0, over
// out's region.  Host buffers, host loop (a 40-byte record copy).
extern "C" int kern_psf_vis(buffer_t* vis, buffer_t* out) {
  if (!vis || !out) {
    gb_set_error(GB_ERR_ARG, "kern_psf_vis: NULL buffer");
    return GB_ERR_ARG;
  }
  int rc;
  if ((rc = check_vis(vis, "kern_psf_vis", "vis")) || (rc = check_vis(out, "kern_psf_vis", "out")))
    return rc;
  const int64_t n = out->extent[1];
  const int64_t first = (int64_t)out->min[1] - vis->min[1];
  if (n > 0 && (first < 0 || first + n > vis->extent[1])) {
    gb_set_error(GB_ERR_ARG, "kern_psf_vis: vis does not cover the output region");
    return GB_ERR_ARG;
  }
  const double* src = (const double*)vis->host + 5 * first;
  double* dst = (double*)out->host;
  for (int64_t t = 0; t < n; t++) {
    dst[5 * t + 0] = src[5 * t + 0];
    dst[5 * t + 1] = src[5 * t + 1];
    dst[5 * t + 2] = src[5 * t + 2];
    dst[5 * t + 3] = 1.0;
    dst[5 * t + 4] = 0.0;
  }
  return GB_OK;
}
