// Hogbom CLEAN on the GPU: the minor loop of the imaging major cycle.
//
// Engine form, gb_hogbom_f32 (FP32 residual/model/PSF): per iteration
//   peak   = residual pixel of largest |value| (ties: lowest row-major index)
//   stop   if |peak| < threshold (every later iteration is a no-op)
//   residual -= (gain * peak / psf_peak) * psf shifted so its peak sits on
//               the residual peak (zero outside the PSF)
//   model[peak] += gain * peak
// One launch per iteration (the caller captures the sequence in a CUDA graph).
// The image is cut into 64x64 tiles whose maxima are cached: an iteration
// touches only the tiles the shifted PSF overlaps, refreshes their maxima,
// and the last CTA to finish (threadfence + counter, no waiting) reduces the
// tile maxima to the next peak, written to the other slot of a ping-pong
// buffer.  Arithmetic is unfused (__fmul_rn / __fsub_rn) so a numpy float32
// loop reproduces it bit for bit.
//
// Reference form, kern_hogbom_model / kern_hogbom_residual: the reference's
// Halide CLEAN (MS6/kernel/cpu/gridding/hogbom.cpp:10-109) restated on the GPU
// in FP64 with its own rules: 12 cycles; the "PSF peak" is the argmax of
// |residual| over the PSF's domain (hogbom.cpp:58); the peak value is the
// absolute value (hogbom.cpp:85-90); the PSF shift is clamped (:99-100); the
// model gets gain*|peak| (:108); the residual returned is the one of the cycle
// at which the threshold was first crossed, else the last (:68-74).
#include <math.h>
#include <stddef.h>

#include <algorithm>

#include "gb_common.cuh"
#include "gb_runtime.cuh"

namespace gb {

constexpr int kCleanTile = 64;

struct Peak {
  float val;    // signed value
  float absv;   // |value|
  int64_t idx;  // row-major pixel index
};

__device__ __forceinline__ bool better(float a, int64_t ia, float b, int64_t ib) {
  return a > b || (a == b && ia < ib);
}

struct CleanState {
  Peak peak[2];        // ping-pong: iteration i reads peak[i & 1]
  uint32_t retire;     // CTAs finished in the current launch
  int32_t done;        // set once |peak| < threshold
  int32_t iterations;  // iterations that subtracted a component
  int32_t pad;
};

// tile maxima (abs value + index) of the tiles in [t0, t1), then the last CTA
// reduces all tile maxima into st->peak[slot]
__device__ void tiles_and_reduce(float* __restrict__ res, int nx, int ny,
                                 const float* __restrict__ psf, int pnx, int pny, int dx, int dy,
                                 float s, bool subtract, float* __restrict__ tmax,
                                 int64_t* __restrict__ tidx, int ntx, int nty, CleanState* st,
                                 int slot) {
  __shared__ float s_v[256];
  __shared__ int64_t s_i[256];
  __shared__ bool s_last;
  const int ntiles = ntx * nty;
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int tx = t % ntx, ty = t / ntx;
    const int x0 = tx * kCleanTile, y0 = ty * kCleanTile;
    // does the shifted PSF (covering [dx, dx + pnx) x [dy, dy + pny)) touch this tile?
    const bool touched = subtract && x0 < dx + pnx && dx < x0 + kCleanTile && y0 < dy + pny &&
                         dy < y0 + kCleanTile;
    if (subtract && !touched) continue;  // its cached maximum still holds
    float best = -1.f;
    int64_t bi = INT64_MAX;
    for (int e = threadIdx.x; e < kCleanTile * kCleanTile; e += blockDim.x) {
      const int x = x0 + (e % kCleanTile), y = y0 + (e / kCleanTile);
      if (x >= nx || y >= ny) continue;
      const int64_t i = (int64_t)y * nx + x;
      float v = res[i];
      if (touched) {
        const int px = x - dx, py = y - dy;
        if (px >= 0 && px < pnx && py >= 0 && py < pny) {
          v = __fsub_rn(v, __fmul_rn(s, psf[(int64_t)py * pnx + px]));
          res[i] = v;
        }
      }
      const float a = fabsf(v);
      if (better(a, i, best, bi)) {
        best = a;
        bi = i;
      }
    }
    s_v[threadIdx.x] = best;
    s_i[threadIdx.x] = bi;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
      if ((int)threadIdx.x < o &&
          better(s_v[threadIdx.x + o], s_i[threadIdx.x + o], s_v[threadIdx.x], s_i[threadIdx.x])) {
        s_v[threadIdx.x] = s_v[threadIdx.x + o];
        s_i[threadIdx.x] = s_i[threadIdx.x + o];
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      tmax[t] = s_v[0];
      tidx[t] = s_i[0];
    }
    __syncthreads();
  }
  // last CTA reduces the tile maxima
  __threadfence();
  if (threadIdx.x == 0) s_last = atomicAdd(&st->retire, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  float best = -1.f;
  int64_t bi = INT64_MAX;
  for (int t = threadIdx.x; t < ntiles; t += blockDim.x) {
    const float a = ((volatile float*)tmax)[t];
    const int64_t i = ((volatile int64_t*)tidx)[t];
    if (better(a, i, best, bi)) {
      best = a;
      bi = i;
    }
  }
  s_v[threadIdx.x] = best;
  s_i[threadIdx.x] = bi;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o &&
        better(s_v[threadIdx.x + o], s_i[threadIdx.x + o], s_v[threadIdx.x], s_i[threadIdx.x])) {
      s_v[threadIdx.x] = s_v[threadIdx.x + o];
      s_i[threadIdx.x] = s_i[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    Peak p;
    p.idx = s_i[0];
    p.absv = s_v[0];
    p.val = p.idx < (int64_t)nx * ny ? ((volatile float*)res)[p.idx] : 0.f;
    st->peak[slot] = p;
    st->retire = 0;
  }
}

__global__ void __launch_bounds__(256) k_clean_init(float* res, int nx, int ny, float* tmax,
                                                    int64_t* tidx, int ntx, int nty,
                                                    CleanState* st) {
  tiles_and_reduce(res, nx, ny, nullptr, 0, 0, 0, 0, 0.f, false, tmax, tidx, ntx, nty, st, 0);
}

__global__ void __launch_bounds__(256) k_clean_iter(float* res, int nx, int ny,
                                                    const float* __restrict__ psf, int pnx,
                                                    int pny, int ppx, int ppy,
                                                    float gain, float threshold,
                                                    float* __restrict__ model, float* tmax,
                                                    int64_t* tidx, int ntx, int nty,
                                                    CleanState* st, int it) {
  if (st->done) return;  // uniform: written only by the previous launch
  const Peak p = st->peak[it & 1];
  const float psf_peak = psf[(int64_t)ppy * pnx + ppx];
  if (p.absv < threshold || p.idx >= (int64_t)nx * ny || psf_peak == 0.f) {
    if (blockIdx.x == 0 && threadIdx.x == 0) st->done = 1;
    return;
  }
  const int px = (int)(p.idx % nx), py = (int)(p.idx / nx);
  const float s = __fdiv_rn(__fmul_rn(gain, p.val), psf_peak);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    model[p.idx] = __fadd_rn(model[p.idx], __fmul_rn(gain, p.val));
    st->iterations += 1;
  }
  tiles_and_reduce(res, nx, ny, psf, pnx, pny, px - ppx, py - ppy, s, true, tmax, tidx, ntx, nty,
                   st, (it + 1) & 1);
}

// ---------------------------------------------------------------- reference form (FP64)
struct RefPeak {
  double absv;
  int64_t idx;
};

// argmax of |res| over x < wx, y < wy (row-major index into a buffer of row
// length nx), first index on ties: one block, written to *out
__global__ void __launch_bounds__(1024) k_ref_argmax(const double* __restrict__ res, int nx,
                                                     int wx, int wy, RefPeak* out) {
  __shared__ double s_v[1024];
  __shared__ int64_t s_i[1024];
  double best = -1.0;
  int64_t bi = INT64_MAX;
  for (int64_t e = threadIdx.x; e < (int64_t)wx * wy; e += blockDim.x) {
    const int x = (int)(e % wx), y = (int)(e / wx);
    const int64_t i = (int64_t)y * nx + x;
    const double a = fabs(res[i]);
    if (a > best || (a == best && i < bi)) {
      best = a;
      bi = i;
    }
  }
  s_v[threadIdx.x] = best;
  s_i[threadIdx.x] = bi;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      const double a = s_v[threadIdx.x + o];
      const int64_t i = s_i[threadIdx.x + o];
      if (a > s_v[threadIdx.x] || (a == s_v[threadIdx.x] && i < s_i[threadIdx.x])) {
        s_v[threadIdx.x] = a;
        s_i[threadIdx.x] = i;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = RefPeak{s_v[0], s_i[0]};
}

// one reference cycle's update; peaks[0] = the "PSF peak", peaks[1 + c] = cycle c's peak
__global__ void k_ref_cycle(double* __restrict__ res, int nx, int ny,
                            const double* __restrict__ psf, int pnx, int pny,
                            const RefPeak* __restrict__ peaks, int c, double gain,
                            double threshold, double* __restrict__ model, int32_t* under) {
  if (*under) return;
  const RefPeak pk = peaks[1 + c], pp = peaks[0];
  if (pk.absv < threshold) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *under = 1;
    return;
  }
  const int peakX = (int)(pk.idx % nx), peakY = (int)(pk.idx / nx);
  const int ppx = (int)(pp.idx % nx), ppy = (int)(pp.idx / nx);
  const int dx = min(max(peakX - ppx, -pnx), nx), dy = min(max(peakY - ppy, -pny), ny);
  const double s = gain * pk.absv / pp.absv;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)nx * ny;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(e % nx), y = (int)(e / nx);
    const int qx = x - dx, qy = y - dy;
    const double pv = (qx >= 0 && qx < pnx && qy >= 0 && qy < pny) ? psf[(int64_t)qy * pnx + qx]
                                                                    : 0.0;
    res[e] = res[e] - s * pv;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const int cx = min(max(peakX, 0), nx - 1), cy = min(max(peakY, 0), ny - 1);
    model[(int64_t)cy * nx + cx] += gain * pk.absv;
  }
}

}  // namespace gb

using namespace gb;

extern "C" int gb_hogbom_f32(float* d_residual, int32_t nx, int32_t ny, const float* d_psf,
                             int32_t pnx, int32_t pny, int32_t psf_peak_x, int32_t psf_peak_y,
                             float gain, float threshold, int32_t n_iter, float* d_model,
                             void* d_work, int64_t work_bytes, void* stream) {
  const int ntx = (nx + kCleanTile - 1) / kCleanTile, nty = (ny + kCleanTile - 1) / kCleanTile;
  const int64_t need = (int64_t)sizeof(CleanState) + (int64_t)ntx * nty * 12 + 16;
  if (!d_residual || !d_psf || !d_model || !d_work || nx < 1 || ny < 1 || pnx < 1 || pny < 1 ||
      psf_peak_x < 0 || psf_peak_x >= pnx || psf_peak_y < 0 || psf_peak_y >= pny || n_iter < 0 ||
      work_bytes < need) {
    gb_set_error(GB_ERR_ARG, "gb_hogbom_f32: bad arguments (work needs %lld bytes)",
                 (long long)need);
    return GB_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  unsigned char* w = (unsigned char*)d_work;
  CleanState* st = (CleanState*)w;
  int64_t* tidx = (int64_t*)(w + ((sizeof(CleanState) + 15) & ~(size_t)15));
  float* tmax = (float*)(tidx + (int64_t)ntx * nty);
  GB_CUDA_TRY(cudaMemsetAsync(st, 0, sizeof(CleanState), s));
  const int blocks = std::min(ntx * nty, sm_count() * 8);
  k_clean_init<<<blocks, 256, 0, s>>>(d_residual, nx, ny, tmax, tidx, ntx, nty, st);
  GB_CUDA_TRY(cudaGetLastError());
  for (int it = 0; it < n_iter; it++) {
    k_clean_iter<<<blocks, 256, 0, s>>>(d_residual, nx, ny, d_psf, pnx, pny, psf_peak_x,
                                        psf_peak_y, gain, threshold, d_model, tmax, tidx, ntx, nty,
                                        st, it);
    GB_CUDA_TRY(cudaGetLastError());
  }
  return GB_OK;
}

extern "C" int gb_hogbom_work_bytes(int32_t nx, int32_t ny, int64_t* out) {
  if (!out || nx < 1 || ny < 1) {
    gb_set_error(GB_ERR_ARG, "gb_hogbom_work_bytes: bad arguments");
    return GB_ERR_ARG;
  }
  const int64_t ntx = (nx + kCleanTile - 1) / kCleanTile, nty = (ny + kCleanTile - 1) / kCleanTile;
  *out = (int64_t)sizeof(CleanState) + ntx * nty * 12 + 16;
  return GB_OK;
}

extern "C" int gb_hogbom_iterations(const void* d_work, int32_t* out, void* stream) {
  if (!d_work || !out) {
    gb_set_error(GB_ERR_ARG, "gb_hogbom_iterations: NULL argument");
    return GB_ERR_ARG;
  }
  GB_CUDA_TRY(cudaMemcpyAsync(out, (const unsigned char*)d_work + offsetof(CleanState, iterations),
                              sizeof(int32_t), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  GB_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  return GB_OK;
}

// ---------------------------------------------------------------- reference ABI
namespace {
constexpr int kRefCycles = 12;  // MS6/kernel/cpu/gridding/hogbom.cpp:4

int check_img(const buffer_t* b, const char* who, const char* name) {
  if (!b || !b->host || b->elem_size != 8 || b->extent[0] < 1 || b->extent[1] < 1 ||
      b->stride[0] != 1 || (b->extent[1] > 1 && b->stride[1] != b->extent[0])) {
    gb_set_error(GB_ERR_ARG, "%s: %s must be a dense 2-D double image", who, name);
    return GB_ERR_ARG;
  }
  return GB_OK;
}

// shared body: runs the 12 cycles on device copies; returns the model and the
// residual of the threshold cycle (or the last)
int ref_clean(double gain, double threshold, buffer_t* psf, buffer_t* res, buffer_t* model,
              buffer_t* res_out, const char* who) {
  int rc;
  if ((rc = check_img(psf, who, "psf")) || (rc = check_img(res, who, "res"))) return rc;
  buffer_t* out = model ? model : res_out;
  if ((rc = check_img(out, who, "output"))) return rc;
  const int nx = res->extent[0], ny = res->extent[1];
  const int pnx = psf->extent[0], pny = psf->extent[1];
  if (out->extent[0] != nx || out->extent[1] != ny) {
    gb_set_error(GB_ERR_ARG, "%s: output must match the residual's extent", who);
    return GB_ERR_ARG;
  }
  cudaStream_t s;
  if ((rc = stage_stream(&s))) return rc;
  void *d_res, *d_psf, *d_model, *d_aux;
  const size_t nres = (size_t)nx * ny * 8, npsf = (size_t)pnx * pny * 8;
  if ((rc = stage_buffer(0, nres, &d_res)) || (rc = stage_buffer(1, npsf, &d_psf)) ||
      (rc = stage_buffer(2, nres, &d_model)) ||
      (rc = stage_buffer(3, sizeof(RefPeak) * (kRefCycles + 1) + 16, &d_aux)))
    return rc;
  RefPeak* peaks = (RefPeak*)d_aux;
  int32_t* under = (int32_t*)(peaks + kRefCycles + 1);
  GB_CUDA_TRY(cudaMemcpyAsync(d_res, res->host, nres, cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemcpyAsync(d_psf, psf->host, npsf, cudaMemcpyHostToDevice, s));
  if (model)
    GB_CUDA_TRY(cudaMemcpyAsync(d_model, model->host, nres, cudaMemcpyHostToDevice, s));
  else
    GB_CUDA_TRY(cudaMemsetAsync(d_model, 0, nres, s));
  GB_CUDA_TRY(cudaMemsetAsync(under, 0, sizeof(int32_t), s));
  // "PSF peak": argmax |res| over the PSF's domain (hogbom.cpp:57-61)
  k_ref_argmax<<<1, 1024, 0, s>>>((const double*)d_res, nx, std::min(pnx, nx), std::min(pny, ny),
                                  peaks);
  GB_CUDA_TRY(cudaGetLastError());
  const int blocks = (int)std::min<int64_t>(((int64_t)nx * ny + 255) / 256, sm_count() * 8);
  // Once a cycle's peak is under the threshold it neither subtracts nor adds
  // to the model and sets `under`, which makes every later cycle a no-op: the
  // residual left is the one of the crossing cycle (hogbom.cpp:68-74).
  for (int c = 0; c < kRefCycles; c++) {
    k_ref_argmax<<<1, 1024, 0, s>>>((const double*)d_res, nx, nx, ny, peaks + 1 + c);
    GB_CUDA_TRY(cudaGetLastError());
    k_ref_cycle<<<blocks, 256, 0, s>>>((double*)d_res, nx, ny, (const double*)d_psf, pnx, pny,
                                       peaks, c, gain, threshold, (double*)d_model, under);
    GB_CUDA_TRY(cudaGetLastError());
  }
  if (model)
    GB_CUDA_TRY(cudaMemcpyAsync(model->host, d_model, nres, cudaMemcpyDeviceToHost, s));
  else
    GB_CUDA_TRY(cudaMemcpyAsync(res_out->host, d_res, nres, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GB_OK;
}
}  // namespace

// replaces kern_hogbom_model (MS6/kernel/cpu/gridding/hogbom.cpp:128,
// bound at MS6/programs/Kernel/Cleaning.hs:22-32): model accumulates in place
extern "C" int kern_hogbom_model(double gain, double threshold, buffer_t* psf, buffer_t* res,
                                 buffer_t* model) {
  return ref_clean(gain, threshold, psf, res, model, nullptr, "kern_hogbom_model");
}

// replaces kern_hogbom_residual (hogbom.cpp:129, Cleaning.hs:35-44)
extern "C" int kern_hogbom_residual(double gain, double threshold, buffer_t* psf, buffer_t* res,
                                    buffer_t* residual) {
  return ref_clean(gain, threshold, psf, res, nullptr, residual, "kern_hogbom_residual");
}
