// Tiling and facetting steps either side of the gridder: de-tiling (adding a
// margin-padded grid tile into the full grid) and facet rotation (phase
// rotation of visibilities to a facet centre, optional uvw reprojection).
//
//   kern_detile  replaces MS6/kernel/cpu/gridding/detile.cpp:10-39:
//     out(c, x, y) += in(c, x, y) over the overlap of both buffers' (min,
//     extent) regions (tiles with margins stick out of the field).
//   kern_rotate  replaces MS6/kernel/cpu/gridding/rotate.cpp:11-84 (matrix
//     helpers utils.h:119-163):
//     out_lon = out_lon0 + min(2) * out_lon_incr, out_lat likewise with min(3)
//     R   = xyz2uvw(out_lon, out_lat) * uvw2xyz(in_lon, in_lat)
//     M   = uvproj ? R^T * (inv2x2(R)^T * R) : I
//     uvw' = M uvw;  vis' = vis * exp(2 pi i ((0,0,1) - R (0,0,1)) . uvw)
// The 3x3 matrices are formed on the host in FP64 and the per-visibility work
// runs on the GPU in FP64.
#include <math.h>
#include <string.h>

#include <algorithm>

#include "gb_common.cuh"
#include "gb_runtime.cuh"

namespace gb {

struct Mat3 {
  double a[9];
};

static Mat3 mul(const Mat3& x, const Mat3& y) {
  Mat3 r;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double s = 0;
      for (int k = 0; k < 3; k++) s += x.a[3 * i + k] * y.a[3 * k + j];
      r.a[3 * i + j] = s;
    }
  return r;
}
static Mat3 transpose(const Mat3& x) {
  Mat3 r;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) r.a[3 * i + j] = x.a[3 * j + i];
  return r;
}
// the upper-left 2x2 inverted, third row/column identity (utils.h:121-126)
static Mat3 inverse2x2(const Mat3& x) {
  const double det = x.a[0] * x.a[4] - x.a[1] * x.a[3];
  return Mat3{{x.a[4] / det, -x.a[1] / det, 0, -x.a[3] / det, x.a[0] / det, 0, 0, 0, 1}};
}
static Mat3 rot_x(double p) {
  const double s = sin(p), c = cos(p);
  return Mat3{{1, 0, 0, 0, c, -s, 0, s, c}};
}
static Mat3 rot_z(double p) {
  const double s = sin(p), c = cos(p);
  return Mat3{{c, -s, 0, s, c, 0, 0, 0, 1}};
}
static const double kPi = 3.141592653589793238462643383279502884;
static Mat3 xyz2uvw(double lon, double lat) { return mul(rot_x(-(kPi / 2) + lat), rot_z(-(kPi / 2) - lon)); }
static Mat3 uvw2xyz(double lon, double lat) { return mul(rot_z((kPi / 2) + lon), rot_x((kPi / 2) - lat)); }

struct RotateArgs {
  Mat3 M;
  double dx, dy, dz;  // (0,0,1) - R (0,0,1)
};

__global__ void k_rotate64(int64_t n, const double* __restrict__ in, double* __restrict__ out,
                           RotateArgs r) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const double* v = in + 5 * t;
    const double u = v[0], vv = v[1], w = v[2];
    double* o = out + 5 * t;
    o[0] = r.M.a[0] * u + r.M.a[1] * vv + r.M.a[2] * w;
    o[1] = r.M.a[3] * u + r.M.a[4] * vv + r.M.a[5] * w;
    o[2] = r.M.a[6] * u + r.M.a[7] * vv + r.M.a[8] * w;
    const double path = r.dx * u + r.dy * vv + r.dz * w;
    double s, c;
    sincos(2.0 * 3.141592653589793238462643383279502884 * path, &s, &c);
    const double re = v[3], im = v[4];
    o[3] = c * re - s * im;
    o[4] = c * im + s * re;
  }
}

// out[(y - oy) * out_pitch + (x - ox)] += in[(y - iy) * in_pitch + (x - ix)] over the overlap
template <class C>
__global__ void k_detile(const C* __restrict__ in, int64_t in_pitch, int ix, int iy, C* out,
                         int64_t out_pitch, int ox, int oy, int x0, int y0, int w, int h) {
  const int64_t n = (int64_t)w * h;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int x = x0 + (int)(e % w), y = y0 + (int)(e / w);
    const C a = in[(int64_t)(y - iy) * in_pitch + (x - ix)];
    C& b = out[(int64_t)(y - oy) * out_pitch + (x - ox)];
    b.x += a.x;
    b.y += a.y;
  }
}

static int blocks_of(int64_t n) {
  const int64_t b = (n + 255) / 256, cap = (int64_t)sm_count() * 16;
  return (int)std::max<int64_t>(1, std::min(b, cap));
}

static RotateArgs rotate_args(double in_lon, double in_lat, double out_lon, double out_lat,
                              int uvproj) {
  const Mat3 R = mul(xyz2uvw(out_lon, out_lat), uvw2xyz(in_lon, in_lat));
  RotateArgs a;
  if (uvproj) {
    const Mat3 P = transpose(inverse2x2(R));
    a.M = mul(transpose(R), mul(P, R));
  } else {
    a.M = Mat3{{1, 0, 0, 0, 1, 0, 0, 0, 1}};
  }
  a.dx = 0.0 - R.a[2];
  a.dy = 0.0 - R.a[5];
  a.dz = 1.0 - R.a[8];
  return a;
}

static int check_grid3(const buffer_t* b, const char* who) {
  if (!b || !b->host || b->elem_size != 8 || b->extent[0] != 2 || b->stride[0] != 1 ||
      b->stride[1] != 2 || b->extent[1] < 1 || b->extent[2] < 1 ||
      (b->extent[2] > 1 && (b->stride[2] < 2 * b->extent[1] || (b->stride[2] & 1)))) {
    gb_set_error(GB_ERR_ARG, "%s: grid buffers must be (2,W,H) doubles, strides (1,2,>=2W)", who);
    return GB_ERR_ARG;
  }
  return GB_OK;
}

}  // namespace gb

using namespace gb;

// ---------------------------------------------------------------- device entries
extern "C" int gb_rotate_f64(double in_lon, double in_lat, double out_lon, double out_lat,
                             int32_t uvproj, int64_t n, const double* d_vis5, double* d_out5,
                             void* stream) {
  if (n < 0 || (n > 0 && (!d_vis5 || !d_out5))) {
    gb_set_error(GB_ERR_ARG, "gb_rotate_f64: bad arguments");
    return GB_ERR_ARG;
  }
  if (n == 0) return GB_OK;
  const RotateArgs a = rotate_args(in_lon, in_lat, out_lon, out_lat, uvproj);
  k_rotate64<<<blocks_of(n), 256, 0, (cudaStream_t)stream>>>(n, d_vis5, d_out5, a);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

extern "C" int gb_detile_f32(const float* d_tile, int64_t tile_pitch, int32_t tile_min_x,
                             int32_t tile_min_y, int32_t tile_w, int32_t tile_h, float* d_grid,
                             int64_t grid_pitch, int32_t grid_min_x, int32_t grid_min_y,
                             int32_t grid_w, int32_t grid_h, void* stream) {
  if (!d_tile || !d_grid || tile_pitch < tile_w || grid_pitch < grid_w) {
    gb_set_error(GB_ERR_ARG, "gb_detile_f32: bad arguments");
    return GB_ERR_ARG;
  }
  const int x0 = std::max(tile_min_x, grid_min_x), x1 = std::min(tile_min_x + tile_w, grid_min_x + grid_w);
  const int y0 = std::max(tile_min_y, grid_min_y), y1 = std::min(tile_min_y + tile_h, grid_min_y + grid_h);
  if (x1 <= x0 || y1 <= y0) return GB_OK;
  k_detile<float2><<<blocks_of((int64_t)(x1 - x0) * (y1 - y0)), 256, 0, (cudaStream_t)stream>>>(
      (const float2*)d_tile, tile_pitch, tile_min_x, tile_min_y, (float2*)d_grid, grid_pitch,
      grid_min_x, grid_min_y, x0, y0, x1 - x0, y1 - y0);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

// ---------------------------------------------------------------- reference ABI
extern "C" int kern_detile(buffer_t* in_grid, buffer_t* out_grid) {
  int rc;
  if ((rc = check_grid3(in_grid, "kern_detile")) || (rc = check_grid3(out_grid, "kern_detile")))
    return rc;
  const int iw = in_grid->extent[1], ih = in_grid->extent[2];
  const int ow = out_grid->extent[1], oh = out_grid->extent[2];
  const int64_t ip = in_grid->extent[2] > 1 ? in_grid->stride[2] / 2 : iw;
  const int64_t op = out_grid->extent[2] > 1 ? out_grid->stride[2] / 2 : ow;
  const int x0 = std::max(in_grid->min[1], out_grid->min[1]);
  const int x1 = std::min(in_grid->min[1] + iw, out_grid->min[1] + ow);
  const int y0 = std::max(in_grid->min[2], out_grid->min[2]);
  const int y1 = std::min(in_grid->min[2] + ih, out_grid->min[2] + oh);
  if (x1 <= x0 || y1 <= y0) return GB_OK;
  cudaStream_t s;
  if ((rc = stage_stream(&s))) return rc;
  if (host_direct(in_grid->host, 2 * ip) && host_direct(out_grid->host, 2 * op)) {
    // the GPU adds in place over the overlap, loads and stores over the link
    k_detile<double2><<<blocks_of((int64_t)(x1 - x0) * (y1 - y0)), 256, 0, s>>>(
        (const double2*)in_grid->host, ip, in_grid->min[1], in_grid->min[2],
        (double2*)out_grid->host, op, out_grid->min[1], out_grid->min[2], x0, y0, x1 - x0,
        y1 - y0);
    GB_CUDA_TRY(cudaGetLastError());
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    return GB_OK;
  }
  void *d_in, *d_out;
  if ((rc = stage_buffer(0, (size_t)iw * ih * 16, &d_in)) ||
      (rc = stage_buffer(1, (size_t)ow * oh * 16, &d_out)))
    return rc;
  GB_CUDA_TRY(cudaMemcpy2DAsync(d_in, (size_t)iw * 16, in_grid->host, (size_t)ip * 16,
                                (size_t)iw * 16, ih, cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemcpy2DAsync(d_out, (size_t)ow * 16, out_grid->host, (size_t)op * 16,
                                (size_t)ow * 16, oh, cudaMemcpyHostToDevice, s));
  k_detile<double2><<<blocks_of((int64_t)(x1 - x0) * (y1 - y0)), 256, 0, s>>>(
      (const double2*)d_in, iw, in_grid->min[1], in_grid->min[2], (double2*)d_out, ow,
      out_grid->min[1], out_grid->min[2], x0, y0, x1 - x0, y1 - y0);
  GB_CUDA_TRY(cudaGetLastError());
  GB_CUDA_TRY(cudaMemcpy2DAsync(out_grid->host, (size_t)op * 16, d_out, (size_t)ow * 16,
                                (size_t)ow * 16, oh, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GB_OK;
}

extern "C" int kern_rotate(double in_lon, double in_lat, double out_lon0, double out_lat0,
                           double out_lon_incr, double out_lat_incr, int32_t uvproj, buffer_t* vis,
                           buffer_t* out) {
  if (!vis || !out || !vis->host || !out->host || vis->elem_size != 8 || out->elem_size != 8 ||
      vis->extent[0] != 5 || out->extent[0] != 5 || vis->stride[0] != 1 || out->stride[0] != 1 ||
      (vis->extent[1] > 1 && vis->stride[1] != 5) || (out->extent[1] > 1 && out->stride[1] != 5)) {
    gb_set_error(GB_ERR_ARG, "kern_rotate: vis and out must be (5,N) doubles, strides (1,5)");
    return GB_ERR_ARG;
  }
  // out(f, t) is computed over out's region from vis(f, t)
  const int64_t n = out->extent[1];
  const int64_t first = (int64_t)out->min[1] - vis->min[1];
  if (n > 0 && (first < 0 || first + n > vis->extent[1])) {
    gb_set_error(GB_ERR_ARG, "kern_rotate: vis does not cover the output region");
    return GB_ERR_ARG;
  }
  if (n == 0) return GB_OK;
  const double out_lon = out_lon0 + out->min[2] * out_lon_incr;
  const double out_lat = out_lat0 + out->min[3] * out_lat_incr;
  int rc;
  cudaStream_t s;
  if ((rc = stage_stream(&s))) return rc;
  void *d_in, *d_out;
  if ((rc = stage_buffer(0, (size_t)n * 40, &d_in)) || (rc = stage_buffer(1, (size_t)n * 40, &d_out)))
    return rc;
  GB_CUDA_TRY(cudaMemcpyAsync(d_in, (const double*)vis->host + 5 * first, (size_t)n * 40,
                              cudaMemcpyHostToDevice, s));
  rc = gb_rotate_f64(in_lon, in_lat, out_lon, out_lat, uvproj, n, (const double*)d_in,
                     (double*)d_out, s);
  if (rc) return rc;
  GB_CUDA_TRY(cudaMemcpyAsync(out->host, d_out, (size_t)n * 40, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GB_OK;
}
