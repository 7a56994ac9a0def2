// FP32 tiled gridder / degridder: the engine's adjoint pair.
//
// Work decomposition (built by the plan, gb_plan.cu): every visibility
// footprint is cut into pieces of at most P x P taps; pieces are binned by
// the grid tile (T x T pixels) holding their corner and sorted by period P.
// An item is a run of pieces of one tile; a bundle is up to G items that one
// CTA runs side by side, one thread group of L threads per item.  CTAs are
// persistent and pull bundles, longest first, from a device work queue (one
// atomic counter; no device-side waits).
//
// Gridding (G): each group owns an A x A accumulator in shared memory
// (A = T + Pmax - 1, the tile plus the footprint overhang).  Within a run of
// equal period P, thread r of the group owns the residue class
// (a, b) = (r mod P, r div P) of pixel coordinates mod P: piece tap (i, j)
// lands on pixel (x0 + i, y0 + j) with i = (a - x0) mod P, so no two threads
// ever touch the same pixel and the accumulation is a plain read-modify-write
// with an error-free transformation (TwoSum) carrying the rounding error of
// every addition in a second accumulator.  At the end the group adds sum +
// compensation into the global grid with float2 atomics, skipping pixels no
// piece touched; atomics are needed only because neighbouring tiles'
// overhangs and other items of the same tile overlap.
//
// Degridding (D = G^H): each group stages its A x A grid region in shared
// memory with coalesced loads, then each warp takes pieces, gathers the taps
// from shared memory, multiplies by conj(GCF), sums with per-lane TwoSum and
// a warp-shuffle reduction.  A visibility whose footprint was cut into
// several pieces accumulates them with float2 atomics; otherwise a plain store.
#include <algorithm>
#include <mutex>

#include "gb_common.cuh"
#include "gb_plan.cuh"
#include "gb_runtime.cuh"

namespace gb {

struct TiledArgs {
  const Bundle* bundles;
  const Item* items;
  const Rec* recs;
  int32_t* queue;
  ClassInfo cls[kMaxClasses];
  int32_t n_bundles;
  int32_t T, ext_x, ext_y;
  int64_t pitch;
};

__device__ __forceinline__ void group_sync(int id, int n, bool whole_cta) {
  if (whole_cta)
    __syncthreads();
  else
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}

// s + x with the rounding error accumulated into c (Knuth's TwoSum).
__device__ __forceinline__ void two_sum(float& s, float& c, float x) {
  const float t = __fadd_rn(s, x);
  const float bp = __fsub_rn(t, s);
  const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(x, bp));
  s = t;
  c = __fadd_rn(c, e);
}

constexpr int kInvalidResidue = 1 << 14;

// Class table lookup without dynamic indexing of the kernel parameter block
// (which would copy it to local memory).
__device__ __forceinline__ ClassInfo class_of(const TiledArgs& a, int c) {
  static_assert(kMaxClasses == 4, "class_of covers 4 classes");
  return c == 0 ? a.cls[0] : c == 1 ? a.cls[1] : c == 2 ? a.cls[2] : a.cls[3];
}

template <int R, int U>
__device__ __forceinline__ void grid_item(const TiledArgs& a, const Item& it, int lt, int L,
                                          int bar, bool whole, int A, float2* __restrict__ sum,
                                          float2* __restrict__ cmp, Rec* __restrict__ srec,
                                          float2* __restrict__ svis,
                                          const float2* __restrict__ vis,
                                          const float2* __restrict__ gcf,
                                          float2* __restrict__ grid) {
  const int AA = A * A;
  for (int q = lt; q < AA; q += L) {
    sum[q] = make_float2(0.f, 0.f);
    cmp[q] = make_float2(0.f, 0.f);
  }
  int curP = -1;
  int ra[R], rb[R];
  const int end = it.start + it.count;
  for (int base = it.start; base < end; base += L) {
    const int nb = min(L, end - base);
    group_sync(bar, L, whole);  // zeroing done / previous batch consumed
    if (lt < nb) {
      const Rec r = a.recs[base + lt];
      srec[lt] = r;
      svis[lt] = __ldg(vis + r.vis);
    }
    group_sync(bar, L, whole);
    int k = 0;
    while (k < nb) {
      const int pm1 = srec[k].pm1;
      const int P = pm1 + 1;
      if (P != curP) {
        // the residue map changes: finish every read-modify-write of the old one
        group_sync(bar, L, whole);
        curP = P;
#pragma unroll
        for (int m = 0; m < R; m++) {
          const int rr = lt + m * L;
          if (rr < P * P) {
            rb[m] = rr / P;
            ra[m] = rr - rb[m] * P;
          } else {
            ra[m] = kInvalidResidue;
            rb[m] = kInvalidResidue;
          }
        }
      }
      int e = k + 1;
      while (e < nb && srec[e].pm1 == pm1) e++;
      // U pieces at a time: all GCF loads first, then the ordered RMWs
      for (; k + U <= e; k += U) {
        float2 c[U][R];
        int qi[U][R];
        float2 v[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
          const Rec r = srec[k + u];
          v[u] = svis[k + u];
          const float2* gp = gcf + r.gcf;
          const int pitch = r.sm1 + 1;
#pragma unroll
          for (int m = 0; m < R; m++) {
            int i = ra[m] - r.xm;
            i += i < 0 ? P : 0;
            int j = rb[m] - r.ym;
            j += j < 0 ? P : 0;
            if (i < r.wx && j < r.wy) {
              c[u][m] = __ldg(gp + j * pitch + i);
              qi[u][m] = (r.yl + j) * A + r.xl + i;
            } else {
              c[u][m] = make_float2(0.f, 0.f);
              qi[u][m] = -1;
            }
          }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
#pragma unroll
          for (int m = 0; m < R; m++) {
            const int q = qi[u][m];
            if (q >= 0) {
              const float tr = v[u].x * c[u][m].x - v[u].y * c[u][m].y;
              const float ti = v[u].x * c[u][m].y + v[u].y * c[u][m].x;
              float2 s = sum[q], cc = cmp[q];
              two_sum(s.x, cc.x, tr);
              two_sum(s.y, cc.y, ti);
              sum[q] = s;
              cmp[q] = cc;
            }
          }
        }
      }
      for (; k < e; k++) {
        const Rec r = srec[k];
        const float2 vv = svis[k];
        const float2* gp = gcf + r.gcf;
        const int pitch = r.sm1 + 1;
#pragma unroll
        for (int m = 0; m < R; m++) {
          int i = ra[m] - r.xm;
          i += i < 0 ? P : 0;
          int j = rb[m] - r.ym;
          j += j < 0 ? P : 0;
          if (i < r.wx && j < r.wy) {
            const float2 c = __ldg(gp + j * pitch + i);
            const int q = (r.yl + j) * A + r.xl + i;
            const float tr = vv.x * c.x - vv.y * c.y;
            const float ti = vv.x * c.y + vv.y * c.x;
            float2 s = sum[q], cc = cmp[q];
            two_sum(s.x, cc.x, tr);
            two_sum(s.y, cc.y, ti);
            sum[q] = s;
            cmp[q] = cc;
          }
        }
      }
    }
  }
  group_sync(bar, L, whole);
  const int x0 = it.tile_x * a.T, y0 = it.tile_y * a.T;
  for (int q = lt; q < AA; q += L) {
    const float2 s = sum[q], c = cmp[q];
    if (s.x != 0.f || s.y != 0.f || c.x != 0.f || c.y != 0.f) {
      const int py = q / A, px = q - py * A;
      const int gx = x0 + px, gy = y0 + py;
      if (gx < a.ext_x && gy < a.ext_y)
        atomicAdd(grid + (int64_t)gy * a.pitch + gx, make_float2(s.x + c.x, s.y + c.y));
    }
  }
}

template <int NT, int R, int U>
__global__ void __launch_bounds__(NT) k_grid_tiled(TiledArgs a, const float2* __restrict__ vis,
                                                   const float2* __restrict__ gcf,
                                                   float2* __restrict__ grid) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_b;
  const int tid = threadIdx.x;
  for (;;) {
    if (tid == 0) s_b = atomicAdd(a.queue, 1);
    __syncthreads();
    const int b = s_b;
    if (b >= a.n_bundles) break;
    const Bundle bd = a.bundles[b];
    const ClassInfo ci = class_of(a, bd.cls);
    const int g = tid / ci.L;
    if (g < bd.n_items) {
      const int lt = tid - g * ci.L;
      const int AA = ci.A * ci.A;
      unsigned char* base = smem + (size_t)g * (16 * (size_t)AA + 24 * (size_t)ci.L);
      float2* sum = (float2*)base;
      float2* cmp = sum + AA;
      Rec* srec = (Rec*)(base + 16 * (size_t)AA);
      float2* svis = (float2*)(base + 16 * (size_t)AA + 16 * (size_t)ci.L);
      grid_item<R, U>(a, a.items[bd.first_item + g], lt, ci.L, 1 + g, ci.L == NT, ci.A, sum, cmp,
                      srec, svis, vis, gcf, grid);
    }
    __syncthreads();
  }
}

template <int MODE>
__device__ __forceinline__ void degrid_item(const TiledArgs& a, const Item& it, int lt, int L,
                                            int bar, bool whole, int A, float2* __restrict__ sg,
                                            const float2* __restrict__ gcf,
                                            const float2* __restrict__ grid,
                                            float2* __restrict__ pred) {
  const int AA = A * A;
  const int x0 = it.tile_x * a.T, y0 = it.tile_y * a.T;
  for (int q = lt; q < AA; q += L) {
    const int py = q / A, px = q - py * A;
    const int gx = x0 + px, gy = y0 + py;
    sg[q] = (gx < a.ext_x && gy < a.ext_y) ? grid[(int64_t)gy * a.pitch + gx]
                                           : make_float2(0.f, 0.f);
  }
  group_sync(bar, L, whole);
  const int nw = L >> 5, w = lt >> 5, lane = lt & 31;
  const int end = it.start + it.count;
  for (int k = it.start + w; k < end; k += nw) {
    const Rec r = a.recs[k];
    const int wx = r.wx, wy = r.wy, pitch = r.sm1 + 1;
    const float2* gp = gcf + r.gcf;
    const float2* sp = sg + r.yl * A + r.xl;
    float ar = 0.f, ai = 0.f, cr = 0.f, ci = 0.f;
    int j = lane / wx;
    int i = lane - j * wx;
    const int dj = 32 / wx, di = 32 - dj * wx;
#pragma unroll 4
    for (; j < wy;) {
      const float2 c = __ldg(gp + j * pitch + i);
      const float2 x = sp[j * A + i];
      float pr, pi;
      if (MODE == 0) {  // x * conj(c)
        pr = x.x * c.x + x.y * c.y;
        pi = x.y * c.x - x.x * c.y;
      } else {  // -(x * c)
        pr = -(x.x * c.x - x.y * c.y);
        pi = -(x.x * c.y + x.y * c.x);
      }
      two_sum(ar, cr, pr);
      two_sum(ai, ci, pi);
      i += di;
      j += dj;
      if (i >= wx) {
        i -= wx;
        j++;
      }
    }
    ar += cr;
    ai += ci;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      ar += __shfl_xor_sync(0xffffffffu, ar, o);
      ai += __shfl_xor_sync(0xffffffffu, ai, o);
    }
    if (lane == 0) {
      if (r.sm1 > r.pm1)
        atomicAdd(pred + r.vis, make_float2(ar, ai));
      else
        pred[r.vis] = make_float2(ar, ai);
    }
  }
}

template <int NT, int MODE>
__global__ void __launch_bounds__(NT) k_degrid_tiled(TiledArgs a, const float2* __restrict__ gcf,
                                                     const float2* __restrict__ grid,
                                                     float2* __restrict__ pred) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int s_b;
  const int tid = threadIdx.x;
  for (;;) {
    if (tid == 0) s_b = atomicAdd(a.queue + 1, 1);
    __syncthreads();
    const int b = s_b;
    if (b >= a.n_bundles) break;
    const Bundle bd = a.bundles[b];
    const ClassInfo ci = class_of(a, bd.cls);
    const int g = tid / ci.L;
    if (g < bd.n_items) {
      const int lt = tid - g * ci.L;
      float2* sg = (float2*)(smem + (size_t)g * 8 * (size_t)ci.A * ci.A);
      degrid_item<MODE>(a, a.items[bd.first_item + g], lt, ci.L, 1 + g, ci.L == NT, ci.A, sg, gcf,
                        grid, pred);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- host side
size_t tiled_smem_grid(const ClassInfo* cls, int n, int) {
  size_t m = 0;
  for (int c = 0; c < n; c++)
    m = std::max(m, (size_t)cls[c].G * (16 * (size_t)cls[c].A * cls[c].A + 24 * (size_t)cls[c].L));
  return m;
}

size_t tiled_smem_degrid(const ClassInfo* cls, int n, int) {
  size_t m = 0;
  for (int c = 0; c < n; c++) m = std::max(m, (size_t)cls[c].G * 8 * (size_t)cls[c].A * cls[c].A);
  return m;
}

int tiled_max_smem() {
  static int cached = 0;
  static std::once_flag once;
  std::call_once(once, [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cached = v > 1024 ? v - 1024 : 48 * 1024;
  });
  return cached;
}

static int residues_needed(const gb_plan* P) {
  int R = 1;
  for (int c = 0; c < P->n_classes; c++) {
    const int pm = P->cls[c].pmax;
    R = std::max(R, (pm * pm + P->cls[c].L - 1) / P->cls[c].L);
  }
  return R <= 1 ? 1 : R <= 2 ? 2 : R <= 4 ? 4 : 8;
}

typedef void (*GridFn)(TiledArgs, const float2*, const float2*, float2*);
typedef void (*DegridFn)(TiledArgs, const float2*, const float2*, float2*);

template <int NT>
static GridFn grid_fn_nt(int R) {
  switch (R) {
    case 1: return k_grid_tiled<NT, 1, 4>;
    case 2: return k_grid_tiled<NT, 2, 4>;
    case 4: return k_grid_tiled<NT, 4, 2>;
    default: return k_grid_tiled<NT, 8, 1>;
  }
}

static GridFn grid_fn(int NT, int R) {
  return NT == 128 ? grid_fn_nt<128>(R) : NT == 256 ? grid_fn_nt<256>(R) : grid_fn_nt<512>(R);
}

static DegridFn degrid_fn(int NT, int mode) {
  if (NT == 128) return mode ? k_degrid_tiled<128, 1> : k_degrid_tiled<128, 0>;
  if (NT == 256) return mode ? k_degrid_tiled<256, 1> : k_degrid_tiled<256, 0>;
  return mode ? k_degrid_tiled<512, 1> : k_degrid_tiled<512, 0>;
}

static int set_smem_attr(const void* fn) {
  GB_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   tiled_max_smem()));
  return GB_OK;
}

int tiled_ctas_per_sm(const gb_plan* P, bool grid) {
  const void* fn = grid ? (const void*)grid_fn(P->NT, residues_needed(P))
                        : (const void*)degrid_fn(P->NT, 0);
  if (set_smem_attr(fn)) return 1;
  if (!grid) set_smem_attr((const void*)degrid_fn(P->NT, 1));
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, P->NT,
                                                grid ? P->smem_grid : P->smem_degrid);
  return n > 0 ? n : 1;
}

static TiledArgs make_args(const gb_plan* P) {
  TiledArgs a;
  a.bundles = P->d_bundles;
  a.items = P->d_items;
  a.recs = P->d_recs;
  a.queue = P->d_queue;
  for (int c = 0; c < kMaxClasses; c++) a.cls[c] = P->cls[c];
  a.n_bundles = P->n_bundles;
  a.T = P->T;
  a.ext_x = P->dev.ext_x;
  a.ext_y = P->dev.ext_y;
  a.pitch = P->dev.pitch;
  return a;
}

int launch_grid_tiled(gb_plan* P, const float* vis, const float* gcf, float* grid,
                      cudaStream_t s) {
  if (P->n_bundles == 0) return GB_OK;
  GB_CUDA_TRY(cudaMemsetAsync(P->d_queue, 0, sizeof(int32_t), s));
  const int blocks = std::min(P->n_bundles, sm_count() * P->ctas_per_sm_grid);
  GridFn fn = grid_fn(P->NT, residues_needed(P));
  fn<<<blocks, P->NT, P->smem_grid, s>>>(make_args(P), (const float2*)vis, (const float2*)gcf,
                                         (float2*)grid);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

int launch_degrid_tiled(gb_plan* P, const float* gcf, const float* grid, float* pred, int mode,
                        cudaStream_t s) {
  GB_CUDA_TRY(cudaMemsetAsync(pred, 0, sizeof(float2) * (size_t)P->dev.n_vis, s));
  if (P->n_bundles == 0) return GB_OK;
  GB_CUDA_TRY(cudaMemsetAsync(P->d_queue + 1, 0, sizeof(int32_t), s));
  const int blocks = std::min(P->n_bundles, sm_count() * P->ctas_per_sm_degrid);
  DegridFn fn = degrid_fn(P->NT, mode);
  fn<<<blocks, P->NT, P->smem_degrid, s>>>(make_args(P), (const float2*)gcf, (const float2*)grid,
                                           (float2*)pred);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

// Launch of the tiled gridding kernel on caller-supplied work tables (used by
// the allocation-free entry point, whose tables live in a static device
// array rather than in a plan).
int launch_grid_tiled_tables(const Bundle* bundles, int n_bundles, const Item* items,
                             const Rec* recs, int32_t* queue, const ClassInfo* cls, int n_classes,
                             int NT, int T, int ext_x, int ext_y, int64_t pitch, size_t smem,
                             const float* vis, const float* gcf, float* grid, cudaStream_t s) {
  if (n_bundles <= 0) return GB_OK;
  int R = 1;
  for (int c = 0; c < n_classes; c++)
    R = std::max(R, (cls[c].pmax * cls[c].pmax + cls[c].L - 1) / cls[c].L);
  R = R <= 1 ? 1 : R <= 2 ? 2 : R <= 4 ? 4 : 8;
  GridFn fn = grid_fn(NT, R);
  int rc = set_smem_attr((const void*)fn);
  if (rc) return rc;
  int per_sm = 0;
  GB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, NT, smem));
  const int blocks = std::min(n_bundles, sm_count() * std::max(1, per_sm));
  TiledArgs a;
  a.bundles = bundles;
  a.items = items;
  a.recs = recs;
  a.queue = queue;
  for (int c = 0; c < kMaxClasses; c++) a.cls[c] = c < n_classes ? cls[c] : ClassInfo{64, 1, 1, 1};
  a.n_bundles = n_bundles;
  a.T = T;
  a.ext_x = ext_x;
  a.ext_y = ext_y;
  a.pitch = pitch;
  GB_CUDA_TRY(cudaMemsetAsync(queue, 0, sizeof(int32_t), s));
  fn<<<blocks, NT, smem, s>>>(a, (const float2*)vis, (const float2*)gcf, (float2*)grid);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

}  // namespace gb

using namespace gb;

extern "C" int gb_grid_f32(gb_plan* P, const float* d_vis, const float* d_gcf, float* d_grid,
                           void* stream) {
  if (!P || !d_grid || (P->n_recs && (!d_vis || !d_gcf))) {
    gb_set_error(GB_ERR_ARG, "gb_grid_f32: NULL argument");
    return GB_ERR_ARG;
  }
  return launch_grid_tiled(P, d_vis, d_gcf, d_grid, (cudaStream_t)stream);
}

extern "C" int gb_degrid_f32(gb_plan* P, const float* d_gcf, const float* d_grid, float* d_pred,
                             int32_t mode, void* stream) {
  if (!P || (P->dev.n_vis && !d_pred) || (P->n_recs && (!d_gcf || !d_grid)) ||
      (mode != 0 && mode != 1)) {
    gb_set_error(GB_ERR_ARG, "gb_degrid_f32: bad argument");
    return GB_ERR_ARG;
  }
  if (P->dev.n_vis == 0) return GB_OK;
  return launch_degrid_tiled(P, d_gcf, d_grid, d_pred, mode, (cudaStream_t)stream);
}

extern "C" int gb_degrid_forward(gb_plan* P, const float* d_gcf, const float* d_grid,
                                 float* d_pred, void* stream) {
  return gb_degrid_f32(P, d_gcf, d_grid, d_pred, 0, stream);
}

extern "C" int gb_degrid_backward(gb_plan* P, const float* d_gcf, const float* d_pred_grad,
                                  float* d_grid_grad, void* stream) {
  return gb_grid_f32(P, d_pred_grad, d_gcf, d_grid_grad, stream);
}
