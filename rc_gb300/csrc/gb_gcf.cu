// On-GPU w-kernel (GCF) generation, FP64.
//
// Semantics: the reference's GCF generator, MS4/kernel/cpu/gcf/GCF.cpp
// (screen :58-97, per-phase normalisation and extraction :16-52) with its
// centred backward FFT (MS4/kernel/cpu/fft/fft_dyn_padded.cpp:76-103:
// fftshift, unnormalised exp(+2 pi i) transform, fftshift), and the MS4 GPU
// kernels' split into screen / FFT / extract steps (MS4/kernel/gpu/gcf/
// GCF.cu:9-128).  The output layout is the MS6 one the gridders read:
// [ou + 8 ov][sy][sx].
//
// Per batch of planes:
//   k_gcf_screen   screen(l, m) = taper(l) taper(m) (cos 2 pi ph, -sin 2 pi ph),
//                  ph = w (1 - sqrt(1 - l^2 - m^2)), written straight into the
//                  fftshift-ed position of a zeroed (8 Smax)^2 arena;
//   cufftExecZ2Z   CUFFT_INVERSE (exp(+2 pi i), unnormalised), batched;
//   k_gcf_sums     per (plane, phase) sum of real parts over the whole arena
//                  (the output's fftshift is an index map, applied on read);
//   k_gcf_extract  centred S_p x S_p taps per phase, divided by the phase
//                  sum, written as complex128 and/or complex64.
#include <cufft.h>

#include <algorithm>
#include <vector>

#include "gb_common.cuh"
#include "gb_runtime.cuh"

namespace gb {

struct GcfPlaneDev {
  double w;
  int32_t S;
  int64_t off;
};

// arena index of the fftshift-ed array for even N: (k + N/2) mod N
__device__ __forceinline__ int shift_idx(int k, int N) {
  const int h = N / 2;
  return k + h < N ? k + h : k + h - N;
}

__global__ void k_gcf_screen(const GcfPlaneDev* __restrict__ planes, int p0, int smax, int N,
                             double t2, const double* __restrict__ taper,
                             double2* __restrict__ arena) {
  const int b = blockIdx.z;
  const double w = planes[p0 + b].w;
  const int r = smax / 2;
  const double normer = t2 / (double)r;
  const int a0 = N / 2 - r;
  for (int ii = blockIdx.y * blockDim.y + threadIdx.y; ii < smax; ii += gridDim.y * blockDim.y)
    for (int jj = blockIdx.x * blockDim.x + threadIdx.x; jj < smax;
         jj += gridDim.x * blockDim.x) {
      const double x = (double)(ii - r) * normer;
      const double y = (double)(jj - r) * normer;
      const double ph = w * (1.0 - sqrt(1.0 - x * x - y * y));
      double s, c;
      sincos(2.0 * 3.141592653589793238462643383279502884 * ph, &s, &c);
      double tw = 1.0;
      if (taper) tw = taper[ii] * taper[jj];
      const int row = shift_idx(a0 + ii, N), col = shift_idx(a0 + jj, N);
      arena[(int64_t)b * N * N + (int64_t)row * N + col] = make_double2(c * tw, -s * tw);
    }
}

// one block per (plane in batch, phase): sum of real parts of the final
// (fftshift-ed) arena at rows == ou (mod 8), columns == ov (mod 8).
__global__ void k_gcf_sums(const double2* __restrict__ arena, int N, double* __restrict__ sums) {
  const int b = blockIdx.y;
  const int ph = blockIdx.x;  // ou * 8 + ov
  const int ou = ph / GB_OVER, ov = ph % GB_OVER;
  const int n8 = N / GB_OVER;
  double acc = 0.0;
  for (int64_t e = threadIdx.x; e < (int64_t)n8 * n8; e += blockDim.x) {
    const int rf = (int)(e / n8) * GB_OVER + ou;
    const int cf = (int)(e % n8) * GB_OVER + ov;
    acc += arena[(int64_t)b * N * N + (int64_t)shift_idx(rf, N) * N + shift_idx(cf, N)].x;
  }
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[b * GB_PHASES + ph] = red[0];
}

// dst[off + (ou + 8 ov) S^2 + sy S + sx] =
//   final[(c + sx) 8 + ou][(c + sy) 8 + ov] / sums[ou][ov],  c = smax/2 - S/2
__global__ void k_gcf_extract(const GcfPlaneDev* __restrict__ planes, int p0, int smax, int N,
                              const double2* __restrict__ arena, const double* __restrict__ sums,
                              double2* __restrict__ out64, float2* __restrict__ out32) {
  const int b = blockIdx.y;
  const GcfPlaneDev pl = planes[p0 + b];
  const int S = pl.S;
  const int c = smax / 2 - S / 2;
  const int64_t n = (int64_t)GB_PHASES * S * S;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int phase = (int)(e / ((int64_t)S * S));
    const int rem = (int)(e - (int64_t)phase * S * S);
    const int sy = rem / S, sx = rem - sy * S;
    const int ou = phase % GB_OVER, ov = phase / GB_OVER;
    const int rf = (c + sx) * GB_OVER + ou, cf = (c + sy) * GB_OVER + ov;
    const double2 v = arena[(int64_t)b * N * N + (int64_t)shift_idx(rf, N) * N + shift_idx(cf, N)];
    const double d = sums[b * GB_PHASES + ou * GB_OVER + ov];
    const double2 q = make_double2(v.x / d, v.y / d);
    if (out64) out64[pl.off + e] = q;
    if (out32) out32[pl.off + e] = make_float2((float)q.x, (float)q.y);
  }
}

}  // namespace gb

using namespace gb;

#define GB_CUFFT_TRY(expr)                                                           \
  do {                                                                               \
    cufftResult _r = (expr);                                                         \
    if (_r != CUFFT_SUCCESS) {                                                       \
      gb_set_error(GB_ERR_CUDA, "%s:%d %s: cuFFT error %d", __FILE__, __LINE__, #expr, \
                   (int)_r);                                                         \
      rc = GB_ERR_CUDA;                                                              \
      goto done;                                                                     \
    }                                                                                \
  } while (0)

#define GB_CUDA_GOTO(expr)                                                           \
  do {                                                                               \
    cudaError_t _e = (expr);                                                         \
    if (_e != cudaSuccess) {                                                         \
      gb_set_error(GB_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #expr,             \
                   cudaGetErrorString(_e));                                          \
      rc = GB_ERR_CUDA;                                                              \
      goto done;                                                                     \
    }                                                                                \
  } while (0)

extern "C" int gb_gcf_generate(int32_t n_planes, const double* w_planes, const int32_t* supports,
                               const int64_t* gcf_offsets, int32_t max_support, double t2,
                               const double* d_taper, double* d_gcf64, float* d_gcf32,
                               void* stream) {
  if (n_planes < 1 || n_planes > GB_MAX_PLANES || !w_planes || !supports || !gcf_offsets ||
      max_support < 2 || max_support > GB_MAX_SUPPORT || (max_support & 1) || !(t2 > 0.0) ||
      (!d_gcf64 && !d_gcf32)) {
    gb_set_error(GB_ERR_ARG, "gb_gcf_generate: bad arguments (max_support must be even, 2..%d)",
                 GB_MAX_SUPPORT);
    return GB_ERR_ARG;
  }
  for (int p = 0; p < n_planes; p++) {
    if (supports[p] < 1 || supports[p] > max_support || gcf_offsets[p] < 0) {
      gb_set_error(GB_ERR_ARG, "gb_gcf_generate: plane %d support %d out of range", p, supports[p]);
      return GB_ERR_ARG;
    }
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int N = GB_OVER * max_support;
  const size_t arena_bytes = (size_t)N * N * sizeof(double2);
  // batch so that the FFT arenas stay within ~1 GiB
  int batch = (int)std::max<size_t>(1, ((size_t)1 << 30) / arena_bytes);
  batch = std::min(batch, n_planes);
  std::vector<GcfPlaneDev> hp(n_planes);
  for (int p = 0; p < n_planes; p++) hp[p] = GcfPlaneDev{w_planes[p], supports[p], gcf_offsets[p]};
  int rc = GB_OK;
  GcfPlaneDev* d_planes = nullptr;
  double2* arena = nullptr;
  double* sums = nullptr;
  cufftHandle plan = 0;
  bool have_plan = false;
  int nfft[2] = {N, N};
  if ((rc = dev_alloc((void**)&d_planes, sizeof(GcfPlaneDev) * n_planes, "GCF generation")) ||
      (rc = dev_alloc((void**)&arena, arena_bytes * batch, "GCF generation")) ||
      (rc = dev_alloc((void**)&sums, sizeof(double) * GB_PHASES * batch, "GCF generation")))
    goto done;
  GB_CUDA_GOTO(cudaMemcpyAsync(d_planes, hp.data(), sizeof(GcfPlaneDev) * n_planes,
                               cudaMemcpyHostToDevice, s));
  GB_CUFFT_TRY(cufftPlanMany(&plan, 2, nfft, nullptr, 1, N * N, nullptr, 1, N * N, CUFFT_Z2Z, batch));
  have_plan = true;
  GB_CUFFT_TRY(cufftSetStream(plan, s));
  for (int p0 = 0; p0 < n_planes; p0 += batch) {
    const int nb = std::min(batch, n_planes - p0);
    GB_CUDA_GOTO(cudaMemsetAsync(arena, 0, arena_bytes * batch, s));
    dim3 blk(32, 8), grd((max_support + 31) / 32, (max_support + 7) / 8, nb);
    k_gcf_screen<<<grd, blk, 0, s>>>(d_planes, p0, max_support, N, t2, d_taper, arena);
    GB_CUDA_GOTO(cudaGetLastError());
    // unused batch slots hold zeros: transforming them is harmless
    GB_CUFFT_TRY(cufftExecZ2Z(plan, (cufftDoubleComplex*)arena, (cufftDoubleComplex*)arena,
                              CUFFT_INVERSE));
    k_gcf_sums<<<dim3(GB_PHASES, nb), 256, 0, s>>>(arena, N, sums);
    GB_CUDA_GOTO(cudaGetLastError());
    k_gcf_extract<<<dim3(64, nb), 256, 0, s>>>(d_planes, p0, max_support, N, arena, sums,
                                              (double2*)d_gcf64, (float2*)d_gcf32);
    GB_CUDA_GOTO(cudaGetLastError());
  }
  GB_CUDA_GOTO(cudaStreamSynchronize(s));
done:
  if (have_plan) cufftDestroy(plan);
  cudaFree(d_planes);
  cudaFree(arena);
  cudaFree(sums);
  return rc;
}

// ---------------------------------------------------------------- GCF choice per w-region
// MS6/programs/Kernel/Config.hs:128-132: the GCF file with the largest w not
// above max(|w0|, |w1|) (maximumBy keeps the last of equal maxima); and
// MS6/programs/Kernel/IO.hs:110-113: conjugate when the region lies mostly at
// negative w (low < -high).
extern "C" int gb_gcf_select(int32_t n_files, const double* w_files, double w0, double w1,
                             int32_t* index, int32_t* conjugate) {
  if (n_files < 1 || !w_files || !index || !conjugate) {
    gb_set_error(GB_ERR_ARG, "gb_gcf_select: bad arguments");
    return GB_ERR_ARG;
  }
  const double w = fabs(w0) > fabs(w1) ? fabs(w0) : fabs(w1);
  int best = -1;
  for (int i = 0; i < n_files; i++)
    if (w_files[i] <= w && (best < 0 || w_files[i] >= w_files[best])) best = i;
  if (best < 0) {
    gb_set_error(GB_ERR_ARG, "gb_gcf_select: no GCF with w <= %g", w);
    return GB_ERR_ARG;
  }
  *index = best;
  *conjugate = w0 < -w1 ? 1 : 0;
  return GB_OK;
}

namespace gb {
template <class C>
__global__ void k_conjugate(C* __restrict__ g, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    g[i].y = -g[i].y;
}
}  // namespace gb

extern "C" int gb_gcf_conjugate_f32(float* d_gcf, int64_t n_complex, void* stream) {
  if (!d_gcf || n_complex < 0) {
    gb_set_error(GB_ERR_ARG, "gb_gcf_conjugate_f32: bad arguments");
    return GB_ERR_ARG;
  }
  if (!n_complex) return GB_OK;
  const int b = (int)std::min<int64_t>((n_complex + 255) / 256, 4096);
  k_conjugate<float2><<<b, 256, 0, (cudaStream_t)stream>>>((float2*)d_gcf, n_complex);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

extern "C" int gb_gcf_conjugate_f64(double* d_gcf, int64_t n_complex, void* stream) {
  if (!d_gcf || n_complex < 0) {
    gb_set_error(GB_ERR_ARG, "gb_gcf_conjugate_f64: bad arguments");
    return GB_ERR_ARG;
  }
  if (!n_complex) return GB_OK;
  const int b = (int)std::min<int64_t>((n_complex + 255) / 256, 4096);
  k_conjugate<double2><<<b, 256, 0, (cudaStream_t)stream>>>((double2*)d_gcf, n_complex);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}
