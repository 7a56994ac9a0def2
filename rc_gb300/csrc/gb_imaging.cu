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
#include "rc_gb300_ms5.h"
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

// ---------------------------------------------------------------- kern_fft / kern_ifft
// The reference's Halide FFT kernels on host buffers (MS6/kernel/cpu/gridding/
// fft.cpp:546-677, bound by fft1.cpp:29-57), restated on cuFFT in FP64.  For an
// n x n grid g (complex) and image x (real), n in {1024, 2048, 3072, 4096,
// 6144, 8192}, indices taken mod n, h = n / 2:
//
// kern_ifft (fft.cpp:546-589):
//   H(u,v)  = (g(u,v) + conj(g(n-1-u, n-1-v))) / 2          the "hermitised" grid
//   S(u,v)  = H(u+h, v+h)
//   D(x,v)  = sum_u S(u,v) e^{+2 pi i u x/n}                  rows v = 0..h only
//   X(x,v)  = D(x,v) for v < h, conj(D(x, n-v)) for v >= h    (fft2d_c2r, :430-509)
//   T_x(y)  = sum_v X(x,v) e^{+2 pi i v y/n}
//   I(x,y)  = Re T_x(y) - Im T_{x+h}(y)  (x < h),  Im T_{x-h}(y) + Re T_x(y)  (x >= h)
//             (two real columns packed into one complex transform; where X's rows 0
//             and h are not real, the imaginary parts cross between the two columns)
//   out(x,y) = I(x+h, y+h) / n
// kern_fft (fft.cpp:607-662):
//   F(u,v)  = sum_{x,y} x(x-h, y-h) e^{-2 pi i (u x + v y)/n}, kept for rows v <= h
//             (fft2d_r2c's half spectrum, zero elsewhere): B
//   out(u,v) = (B(u-h, v-h) + conj(B(h-u-1, h-v-1))) / n
// The reference builds its twiddle angles from float(2 pi) and float(sqrt(2)/2),
// so it sits about 1e-8 (relative) from these exact transforms.
constexpr int kFftSizeError = -666;  // fft1.cpp:38, 52

__global__ void k_ifft_prep(const double2* __restrict__ g, int n, double herm_scale,
                            double2* __restrict__ a) {
  const int h = n / 2;
  const int64_t total = (int64_t)(h + 1) * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int v = (int)(i / n), u = (int)(i - (int64_t)v * n);
    const int ua = half_shift(u, n), vb = half_shift(v, n);
    const double2 p = g[(int64_t)vb * n + ua];
    const double2 m = g[(int64_t)(n - 1 - vb) * n + (n - 1 - ua)];
    a[i] = make_double2((p.x + m.x) * herm_scale, (p.y - m.y) * herm_scale);
  }
}

__global__ void k_ifft_complete(const double2* __restrict__ a, int n, double2* __restrict__ b) {
  const int h = n / 2;
  const int64_t total = (int64_t)n * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int v = (int)(i / n), x = (int)(i - (int64_t)v * n);
    if (v < h) {
      b[i] = a[i];
    } else {
      const double2 d = a[(int64_t)(n - v) * n + x];
      b[i] = make_double2(d.x, -d.y);
    }
  }
}

__global__ void k_ifft_out(const double2* __restrict__ t, int n, double rn,
                           double* __restrict__ out) {
  const int h = n / 2;
  const int64_t total = (int64_t)n * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / n), x = (int)(i - (int64_t)y * n);
    const int sx = half_shift(x, n), sy = half_shift(y, n);
    const double2* row = t + (int64_t)sy * n;
    const double val = sx < h ? row[sx].x - row[sx + h].y : row[sx - h].y + row[sx].x;
    out[i] = val * rn;
  }
}

__global__ void k_fft_prep(const double* __restrict__ img, int n, double2* __restrict__ z) {
  const int64_t total = (int64_t)n * n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int v = (int)(i / n), u = (int)(i - (int64_t)v * n);
    z[i] = make_double2(img[(int64_t)half_shift(v, n) * n + half_shift(u, n)], 0.0);
  }
}

__global__ void k_fft_out(const double2* __restrict__ f, int n, double2* __restrict__ out) {
  const int h = n / 2;
  const int64_t total = (int64_t)n * n;
  const double rn = 1.0 / n;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int v = (int)(i / n), u = (int)(i - (int64_t)v * n);
    const int a1 = half_shift(u, n), b1 = half_shift(v, n);  // u - h, v - h (mod n)
    const int a2 = h - 1 - u < 0 ? h - 1 - u + n : h - 1 - u;
    const int b2 = h - 1 - v < 0 ? h - 1 - v + n : h - 1 - v;
    const double2 t1 = b1 <= h ? f[(int64_t)b1 * n + a1] : make_double2(0.0, 0.0);
    const double2 t2 = b2 <= h ? f[(int64_t)b2 * n + a2] : make_double2(0.0, 0.0);
    out[i] = make_double2((t1.x + t2.x) * rn, (t1.y - t2.y) * rn);
  }
}

// Batched 1-D double-complex plans (rows: stride 1, dist n; columns: stride n,
// dist 1), one per (device, n, batch, layout), created on first use.
static int plan_1d(int n, int batch, bool columns, cufftHandle* out) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, int, int>, cufftHandle> plans;
  int dev = 0;
  GB_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  auto key = std::make_tuple(dev, n, batch, columns ? 1 : 0);
  auto it = plans.find(key);
  if (it != plans.end()) {
    *out = it->second;
    return GB_OK;
  }
  cufftHandle hdl;
  int len = n, emb = n;
  const int stride = columns ? n : 1, dist = columns ? 1 : n;
  const cufftResult r = cufftPlanMany(&hdl, 1, &len, &emb, stride, dist, &emb, stride, dist,
                                      CUFFT_Z2Z, batch);
  if (r != CUFFT_SUCCESS) {
    gb_set_error(GB_ERR_CUDA, "cufftPlanMany(%d x %d): error %d", n, batch, (int)r);
    return GB_ERR_CUDA;
  }
  plans[key] = hdl;
  *out = hdl;
  return GB_OK;
}

static int exec_1d(double2* buf, int n, int batch, bool columns, cudaStream_t s) {
  cufftHandle hdl;
  int rc = plan_1d(n, batch, columns, &hdl);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(g_exec_mu);
  cufftResult r = cufftSetStream(hdl, s);
  if (r == CUFFT_SUCCESS)
    r = cufftExecZ2Z(hdl, (cufftDoubleComplex*)buf, (cufftDoubleComplex*)buf, CUFFT_INVERSE);
  if (r != CUFFT_SUCCESS) {
    gb_set_error(GB_ERR_CUDA, "cuFFT exec 1-D (n=%d): error %d", n, (int)r);
    return GB_ERR_CUDA;
  }
  return GB_OK;
}

// fft1.cpp:3-11 (checkSize) plus the layouts the Halide pipelines require:
// image (n, n) doubles with unit stride, grid (2, n, n) doubles with strides
// (1, 2, >= 2n), all mins 0.  Returns n, kFftSizeError for a size the
// reference does not provide, or GB_ERR_ARG for a malformed buffer.
static int fft_size(const buffer_t* img, const buffer_t* uvg, const char* who) {
  if (!img || !uvg || !img->host || !uvg->host || img->elem_size != 8 || uvg->elem_size != 8 ||
      img->stride[0] != 1 || uvg->extent[0] != 2 || uvg->stride[0] != 1 || uvg->stride[1] != 2 ||
      img->min[0] || img->min[1] || uvg->min[0] || uvg->min[1] || uvg->min[2]) {
    gb_set_error(GB_ERR_ARG, "%s: image must be (n,n) doubles with unit stride and the grid "
                             "(2,n,n) doubles with strides (1,2,>=2n), mins 0", who);
    return GB_ERR_ARG;
  }
  const int n = img->extent[0];
  if (img->extent[1] != n || uvg->extent[1] != n || uvg->extent[2] != n) {
    gb_set_error(kFftSizeError, "%s: image and grid must both be n x n", who);
    return kFftSizeError;
  }
  if (n != 1024 && n != 2048 && n != 3072 && n != 4096 && n != 6144 && n != 8192) {
    gb_set_error(kFftSizeError, "%s: n = %d is not one of the reference's sizes", who, n);
    return kFftSizeError;
  }
  if (img->stride[1] < n || uvg->stride[2] < 2 * n || (uvg->stride[2] & 1)) {
    gb_set_error(GB_ERR_ARG, "%s: row strides too small", who);
    return GB_ERR_ARG;
  }
  return n;
}

}  // namespace gb

using namespace gb;

// The inverse pipeline with its two scale factors: MS6's kern_ifft hermitises
// with 1/2 and divides the image by n; MS5's kern_fft does neither.
static int ifft_host(buffer_t* uvg, buffer_t* img, const char* who, double herm_scale,
                     bool scale_by_n, int only_size) {
  const int n = fft_size(img, uvg, who);
  if (n < 0) return n;
  if (only_size && n != only_size) {
    gb_set_error(GB_ERR_ARG, "%s: the grid must be %d x %d", who, only_size, only_size);
    return GB_ERR_ARG;
  }
  int rc;
  cudaStream_t s;
  if ((rc = stage_stream(&s))) return rc;
  const size_t cells = (size_t)n * n;
  void *d0, *d1;
  if ((rc = stage_buffer(0, cells * 16, &d0)) || (rc = stage_buffer(1, cells * 16, &d1)))
    return rc;
  double2* g = (double2*)d0;
  double2* a = (double2*)d1;
  GB_CUDA_TRY(cudaMemcpy2DAsync(g, (size_t)n * 16, uvg->host, (size_t)uvg->stride[2] * 8,
                                (size_t)n * 16, n, cudaMemcpyHostToDevice, s));
  k_ifft_prep<<<blocks_nn((int64_t)(n / 2 + 1) * n), 256, 0, s>>>(g, n, herm_scale, a);
  GB_CUDA_TRY(cudaGetLastError());
  if ((rc = exec_1d(a, n, n / 2 + 1, false, s))) return rc;
  k_ifft_complete<<<blocks_nn((int64_t)cells), 256, 0, s>>>(a, n, g);
  GB_CUDA_TRY(cudaGetLastError());
  if ((rc = exec_1d(g, n, n, true, s))) return rc;
  double* out = (double*)d1;
  k_ifft_out<<<blocks_nn((int64_t)cells), 256, 0, s>>>(g, n, scale_by_n ? 1.0 / n : 1.0, out);
  GB_CUDA_TRY(cudaGetLastError());
  GB_CUDA_TRY(cudaMemcpy2DAsync(img->host, (size_t)img->stride[1] * 8, out, (size_t)n * 8,
                                (size_t)n * 8, n, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GB_OK;
}

extern "C" int kern_ifft(buffer_t* uvg, buffer_t* img) {
  return ifft_host(uvg, img, "kern_ifft", 0.5, true, 0);
}

#ifdef GB_MS5_ABI
// MS5's kern_fft (MS5/programs/Kernel/FFT.hs:15-16, generated by
// MS5/kernel/cpu/gridding/fft.cpp:540-605): grid -> image, 2048 x 2048 only,
// the grid hermitised without the 1/2 and the image not divided by n, i.e.
// 2 n times MS6's kern_ifft.
extern "C" int kern_fft(buffer_t* uvg, buffer_t* img) {
  return ifft_host(uvg, img, "kern_fft", 1.0, false, 2048);
}
#else
extern "C" int kern_fft(buffer_t* img, buffer_t* uvg) {
  const int n = fft_size(img, uvg, "kern_fft");
  if (n < 0) return n;
  int rc;
  cudaStream_t s;
  if ((rc = stage_stream(&s))) return rc;
  const size_t cells = (size_t)n * n;
  void *d0, *d1;
  if ((rc = stage_buffer(0, cells * 16, &d0)) || (rc = stage_buffer(1, cells * 16, &d1)))
    return rc;
  double* x = (double*)d1;
  double2* z = (double2*)d0;
  GB_CUDA_TRY(cudaMemcpy2DAsync(x, (size_t)n * 8, img->host, (size_t)img->stride[1] * 8,
                                (size_t)n * 8, n, cudaMemcpyHostToDevice, s));
  k_fft_prep<<<blocks_nn((int64_t)cells), 256, 0, s>>>(x, n, z);
  GB_CUDA_TRY(cudaGetLastError());
  if ((rc = exec_fft<double>(z, n, CUFFT_FORWARD, s))) return rc;
  double2* out = (double2*)d1;
  k_fft_out<<<blocks_nn((int64_t)cells), 256, 0, s>>>(z, n, out);
  GB_CUDA_TRY(cudaGetLastError());
  GB_CUDA_TRY(cudaMemcpy2DAsync(uvg->host, (size_t)uvg->stride[2] * 8, out, (size_t)n * 16,
                                (size_t)n * 16, n, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GB_OK;
}
#endif  // GB_MS5_ABI

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
