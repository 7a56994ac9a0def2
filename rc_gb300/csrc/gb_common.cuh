// Shared device/host definitions of the GB300 gridding engine.
//
// Index math is the reference's, restated (SKA-ScienceDataProcessor/RC,
// MS6/kernel/cpu/gridding/scatter.cpp:56-76 and degrid.cpp:46-67):
//   us   = u * scale
//   ou   = clamp(int(round(8 * (us - floor(us)))), 0, 7)
//   x0   = int(round(us) + grid_size/2 - S/2)
//   keep = lo_x <= x0 <= hi_x (and the same in y), with
//   gm   = max(0, (margin - S)/2), lo_x = min_x + gm, hi_x = min_x + ext_x - S - 1 - gm
// `round` is round-half-to-even (rint), and an out-of-int32-range or NaN
// coordinate is treated as x86's cast<int> result INT_MIN, i.e. out of bounds.
// All of it is evaluated in FP64, on the GPU, for every precision of the
// gridder.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/rc_gb300.h"

#define GB_OVER 8
#define GB_PHASES (GB_OVER * GB_OVER)

namespace gb {

struct VisIndex {
  int32_t x0, y0;   // GCF corner pixel (absolute grid coordinates)
  int32_t phase;    // ou + 8 * ov
  bool keep;        // gridded / degridded at all
};

__host__ __device__ __forceinline__ int32_t cast_int(double x) {
  if (!(x > -2147483649.0 && x < 2147483648.0)) return INT32_MIN;
  return (int32_t)x;
}

__host__ __device__ __forceinline__ void index1(double uv, double scale, int32_t half_off,
                                                int32_t* corner, int32_t* over) {
  const double s = uv * scale;
  const double fr = s - floor(s);
  int32_t oi = cast_int(rint((double)GB_OVER * fr));
  oi = oi < 0 ? 0 : (oi > GB_OVER - 1 ? GB_OVER - 1 : oi);
  *over = oi;
  *corner = cast_int(rint(s) + (double)half_off);
}

// half_off = grid_size/2 - S/2 (both C integer divisions of non-negative values)
__host__ __device__ __forceinline__ VisIndex vis_index(double u, double v, double scale,
                                                      int32_t grid_size, int32_t S,
                                                      int32_t margin, int32_t min_x,
                                                      int32_t min_y, int32_t ext_x,
                                                      int32_t ext_y) {
  VisIndex r;
  int32_t ou, ov;
  const int32_t half_off = grid_size / 2 - S / 2;
  index1(u, scale, half_off, &r.x0, &ou);
  index1(v, scale, half_off, &r.y0, &ov);
  r.phase = ou + GB_OVER * ov;
  const int32_t gm = margin - S < 0 ? 0 : (margin - S) / 2;
  const int32_t lo_x = min_x + gm, hi_x = min_x + ext_x - S - 1 - gm;
  const int32_t lo_y = min_y + gm, hi_y = min_y + ext_y - S - 1 - gm;
  r.keep = r.x0 >= lo_x && r.x0 <= hi_x && r.y0 >= lo_y && r.y0 <= hi_y;
  return r;
}

// MS6/programs/Kernel/Binning.hs:85-89: w outside [low, high] is not binned;
// bin = clamp(floor((w - low) / (high - low) * bins), 0, bins - 1).
__host__ __device__ __forceinline__ int32_t w_plane(double w, double low, double high,
                                                   int32_t bins) {
  if (!(w >= low && w <= high)) return -1;
  if (bins <= 1 || !(high > low)) return 0;
  const double b = floor((w - low) / (high - low) * (double)bins);
  if (!(b >= 0.0)) return 0;  // also an infinite range (NaN)
  return b > (double)(bins - 1) ? bins - 1 : (int32_t)b;
}

}  // namespace gb

// Error reporting shared by every translation unit of the library.
void gb_set_error(int code, const char* fmt, ...);

#define GB_CUDA_TRY(expr)                                                        \
  do {                                                                           \
    cudaError_t _e = (expr);                                                     \
    if (_e != cudaSuccess) {                                                     \
      gb_set_error(GB_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #expr,       \
                   cudaGetErrorString(_e));                                      \
      return GB_ERR_CUDA;                                                        \
    }                                                                            \
  } while (0)
