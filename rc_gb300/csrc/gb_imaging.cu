// Image <-> grid transforms either side of the gridder: grid correction,
// centred 2-D FFT, and the exact adjoint.
//
// The reference does this with its Halide FFT (MS6/kernel/cpu/gridding/
// fft.cpp:603-677, fft1.cpp:29-57: fftshift, FFT, Hermitian handling) and,
// on the GPU, with cuFFT plus its fftshift kernels (MS4/kernel/gpu/fft/
// cufftshift.cu:9-73, MS4/dna-programs/Kernel/GPU/FFT.hs:37).  Here, for an
// even N x N real image x and a separable image-domain taper t (the
// gridding kernel's transform, so dividing by it is the grid correction):
//
//   A x   = fftshift( FFT( ifftshift( x / (t_y t_x) ) ) )          (image -> grid)
//   A^H y = Re[ (1/(t_y t_x)) * fftshift( IFFT_unnorm( ifftshift( y ) ) ) ]
//
// FFT is exp(-2 pi i) (cuFFT forward), IFFT_unnorm exp(+2 pi i) without the
// 1/N^2, so A^H is the adjoint of A for the real inner product on images.
// For even N, fftshift and ifftshift are the same permutation.
#include <cufft.h>

#include <map>
#include <mutex>
#include <tuple>

#include "gb_common.cuh"
#include "gb_runtime.cuh"

namespace gb {

template <class R>
struct Cx;
template <>
struct Cx<float> {
  typedef float2 T;
};
template <>
struct Cx<double> {
  typedef double2 T;
};

__device__ __forceinline__ int half_shift(int k, int n) {
  const int h = n / 2;
  return k + h < n ? k + h : k + h - n;
}

// grid[shift(i)][shift(j)] = x[i][j] / (t[i] t[j])   (real -> complex)
template <class R>
__global__ void k_image_in(const R* __restrict__ x, const R* __restrict__ t, int n,
                           typename Cx<R>::T* __restrict__ g) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nn;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e - (int64_t)i * n);
    R v = x[e];
    if (t) v = v / (t[i] * t[j]);
    typename Cx<R>::T c;
    c.x = v;
    c.y = (R)0;
    g[(int64_t)half_shift(i, n) * n + half_shift(j, n)] = c;
  }
}

// in-place quadrant swap (fftshift for even n): (i, j) <-> (i + n/2, j + n/2)
template <class C>
__global__ void k_quadrant_swap(C* __restrict__ g, int n) {
  const int h = n / 2;
  const int64_t half = (int64_t)h * n;  // rows [0, h) against rows [h, n)
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < half;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e - (int64_t)i * n);
    const int64_t a = (int64_t)i * n + j;
    const int64_t b = (int64_t)(i + h) * n + half_shift(j, n);
    const C va = g[a], vb = g[b];
    g[a] = vb;
    g[b] = va;
  }
}

// copy with the output shift: w[shift(i)][shift(j)] = y[i][j]
template <class C>
__global__ void k_shift_copy(const C* __restrict__ y, int n, C* __restrict__ w) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nn;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e - (int64_t)i * n);
    w[(int64_t)half_shift(i, n) * n + half_shift(j, n)] = y[e];
  }
}

// x[i][j] = Re(w[shift(i)][shift(j)]) / (t[i] t[j])
template <class R>
__global__ void k_image_out(const typename Cx<R>::T* __restrict__ w, const R* __restrict__ t,
                            int n, R* __restrict__ x) {
  const int64_t nn = (int64_t)n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nn;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(e / n), j = (int)(e - (int64_t)i * n);
    R v = w[(int64_t)half_shift(i, n) * n + half_shift(j, n)].x;
    if (t) v = v / (t[i] * t[j]);
    x[e] = v;
  }
}

// cuFFT plans, one per (device, n, precision), created on first use.
static int fft_plan(int n, bool dbl, cufftHandle* out) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, int>, cufftHandle> plans;
  int dev = 0;
  GB_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  auto key = std::make_tuple(dev, n, dbl ? 1 : 0);
  auto it = plans.find(key);
  if (it != plans.end()) {
    *out = it->second;
    return GB_OK;
  }
  cufftHandle h;
  const cufftResult r = cufftPlan2d(&h, n, n, dbl ? CUFFT_Z2Z : CUFFT_C2C);
  if (r != CUFFT_SUCCESS) {
    gb_set_error(GB_ERR_CUDA, "cufftPlan2d(%d): error %d", n, (int)r);
    return GB_ERR_CUDA;
  }
  plans[key] = h;
  *out = h;
  return GB_OK;
}

static std::mutex g_exec_mu;  // a plan is shared: serialise set-stream + enqueue

template <class R>
static int exec_fft(typename Cx<R>::T* buf, int n, int dir, cudaStream_t s) {
  cufftHandle h;
  int rc = fft_plan(n, sizeof(R) == 8, &h);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(g_exec_mu);
  cufftResult r = cufftSetStream(h, s);
  if (r == CUFFT_SUCCESS) {
    if (sizeof(R) == 8)
      r = cufftExecZ2Z(h, (cufftDoubleComplex*)buf, (cufftDoubleComplex*)buf, dir);
    else
      r = cufftExecC2C(h, (cufftComplex*)buf, (cufftComplex*)buf, dir);
  }
  if (r != CUFFT_SUCCESS) {
    gb_set_error(GB_ERR_CUDA, "cuFFT exec (n=%d): error %d", n, (int)r);
    return GB_ERR_CUDA;
  }
  return GB_OK;
}

static int blocks_nn(int64_t nn) {
  int64_t b = (nn + 255) / 256;
  const int64_t cap = (int64_t)sm_count() * 16;
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

template <class R>
static int image_to_grid(const R* x, const R* t, int n, typename Cx<R>::T* g, cudaStream_t s) {
  if (!x || !g || n < 2 || (n & 1)) {
    gb_set_error(GB_ERR_ARG, "image_to_grid: NULL buffer or odd/too small n=%d", n);
    return GB_ERR_ARG;
  }
  const int64_t nn = (int64_t)n * n;
  k_image_in<R><<<blocks_nn(nn), 256, 0, s>>>(x, t, n, g);
  GB_CUDA_TRY(cudaGetLastError());
  int rc = exec_fft<R>(g, n, CUFFT_FORWARD, s);
  if (rc) return rc;
  k_quadrant_swap<<<blocks_nn(nn / 2), 256, 0, s>>>(g, n);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

template <class R>
static int grid_to_image(const typename Cx<R>::T* g, const R* t, int n, typename Cx<R>::T* w,
                         R* x, cudaStream_t s) {
  if (!x || !g || !w || n < 2 || (n & 1) || (const void*)w == (const void*)g) {
    gb_set_error(GB_ERR_ARG, "grid_to_image: NULL/aliased buffer or odd/too small n=%d", n);
    return GB_ERR_ARG;
  }
  const int64_t nn = (int64_t)n * n;
  k_shift_copy<<<blocks_nn(nn), 256, 0, s>>>(g, n, w);
  GB_CUDA_TRY(cudaGetLastError());
  int rc = exec_fft<R>(w, n, CUFFT_INVERSE, s);
  if (rc) return rc;
  k_image_out<R><<<blocks_nn(nn), 256, 0, s>>>(w, t, n, x);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

}  // namespace gb

using namespace gb;

extern "C" int gb_image_to_grid_f32(const float* d_image, const float* d_taper, int32_t n,
                                    float* d_grid, void* stream) {
  return image_to_grid<float>(d_image, d_taper, n, (float2*)d_grid, (cudaStream_t)stream);
}

extern "C" int gb_grid_to_image_f32(const float* d_grid, const float* d_taper, int32_t n,
                                    float* d_work, float* d_image, void* stream) {
  return grid_to_image<float>((const float2*)d_grid, d_taper, n, (float2*)d_work, d_image,
                              (cudaStream_t)stream);
}

extern "C" int gb_image_to_grid_f64(const double* d_image, const double* d_taper, int32_t n,
                                    double* d_grid, void* stream) {
  return image_to_grid<double>(d_image, d_taper, n, (double2*)d_grid, (cudaStream_t)stream);
}

extern "C" int gb_grid_to_image_f64(const double* d_grid, const double* d_taper, int32_t n,
                                    double* d_work, double* d_image, void* stream) {
  return grid_to_image<double>((const double2*)d_grid, d_taper, n, (double2*)d_work, d_image,
                               (cudaStream_t)stream);
}
