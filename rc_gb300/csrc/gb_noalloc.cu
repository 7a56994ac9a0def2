// Allocation-free one-shot FP32 gridding: gb_grid_f32_noalloc.
//
// Some callers cannot call cudaMalloc: code that runs inside a host
// framework owning all device memory (a pipeline runtime with a fixed memory
// budget or pool, a plugin of another GPU application), real-time paths where
// an allocation's latency or failure is not acceptable, or callers that must
// not touch the allocator for other reasons.  This entry point serves them:
// it grids up to GB_NOALLOC_MAX_VIS visibilities into the caller's grid with
// the same tiled FP32 kernel as gb_grid_f32, but keeps every piece of its
// working memory (plane table, per-visibility planes, histogram, offsets,
// records, work items, bundles, queue counter) in one file-scope device array
// of GB_NOALLOC_SCRATCH_BYTES instead of a plan.  It calls no cudaMalloc,
// cudaFree or allocating library routine.
//
// The array is a `static __device__` variable: every GPU that loads this
// library holds it until the process exits.  Its host-side name is only a
// stand-in, so the first call on each device looks up its device address with
// cudaGetSymbolAddress (once per device, with that device current) and passes
// that address to the kernels.  Every call on a device shares the array and
// finds it as the previous call left it: the counters, histogram and cursors
// that must start at zero are cleared by each call, and calls whose GPU work
// overlaps (on different streams, or from different host threads) race on the
// array and must be serialised by the caller.  The cached address belongs to
// the device's current context: after cudaDeviceReset on a device this entry
// point is not valid there for the rest of the process.
//
// Unlike a plan, the records of a (thread-group class, tile) bin are placed by
// an atomic cursor, so pieces of different periods within a bin are not kept
// in period order.  The tiled kernel stays correct (a run ends at each change
// of period, with a group barrier), but a mixed bin splits into more, shorter
// runs than a plan's would, and the FP32 summation order can change from call
// to call (results agree to FP32 rounding, not bit for bit).
#include <algorithm>
#include <mutex>

#include "gb_common.cuh"
#include "gb_plan.cuh"
#include "gb_runtime.cuh"

namespace gb {
namespace {

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

constexpr int kMaxVis = GB_NOALLOC_MAX_VIS;
constexpr int kMaxPieces = GB_NOALLOC_MAX_PIECES;
constexpr int kMaxBins = GB_NOALLOC_MAX_BINS;
constexpr int kMaxPlanes = GB_NOALLOC_MAX_PLANES;

// byte layout of the scratch array
constexpr size_t kOffCounters = 0;  // int32[16]: pieces, items, bundles, queue, overflow
constexpr size_t kOffPlanes = 256;  // PlaneInfo[kMaxPlanes]
constexpr size_t kOffPlaneOf = align256(kOffPlanes + sizeof(PlaneInfo) * kMaxPlanes);
constexpr size_t kOffHist = align256(kOffPlaneOf + 4 * (size_t)kMaxVis);
constexpr size_t kOffOffs = align256(kOffHist + 4 * (size_t)kMaxBins);
constexpr size_t kOffCursor = align256(kOffOffs + 4 * ((size_t)kMaxBins + 1));
constexpr size_t kOffRecs = align256(kOffCursor + 4 * (size_t)kMaxBins);
constexpr size_t kOffItems = align256(kOffRecs + sizeof(Rec) * (size_t)kMaxPieces);
constexpr size_t kOffBundles = align256(kOffItems + sizeof(Item) * (size_t)kMaxBins);
constexpr size_t kScratchBytes = align256(kOffBundles + sizeof(Bundle) * (size_t)kMaxBins);
static_assert(kScratchBytes <= (size_t)GB_NOALLOC_SCRATCH_BYTES,
              "scratch layout exceeds the documented size");

enum { kCntPieces = 0, kCntItems = 1, kCntBundles = 2, kCntQueue = 3, kCntOverflow = 4 };

struct NaClasses {
  int32_t n, ntiles, ntx;
  int32_t G[kMaxClasses], pmax[kMaxClasses];
};

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[GB_NOALLOC_SCRATCH_BYTES];

// per visibility: plane, index, then a histogram of pieces per (class, tile)
__global__ void k_na_count(PlanDev P, const PlaneInfo* __restrict__ pl,
                           const int32_t* __restrict__ plane_in, int32_t* __restrict__ plane_out,
                           int32_t n_planes, double w_lo, double w_hi, int32_t T, NaClasses nc,
                           int32_t* __restrict__ hist) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < P.n_vis;
       t += (int64_t)gridDim.x * blockDim.x) {
    const double* r = P.uvw + t * P.uvw_stride;
    int32_t p = plane_in ? plane_in[t] : w_plane(r[2], w_lo, w_hi, n_planes);
    if (p >= n_planes) p = -1;
    plane_out[t] = p;
    if (p < 0) continue;
    const PlaneInfo q = pl[p];
    const VisIndex ix =
        vis_index(r[0], r[1], P.scale, P.grid_size, q.S, P.margin, 0, 0, P.ext_x, P.ext_y);
    if (!ix.keep) continue;
    for (int oy = 0; oy < q.S; oy += q.P)
      for (int ox = 0; ox < q.S; ox += q.P) {
        const int tile = ((ix.y0 + oy) / T) * nc.ntx + (ix.x0 + ox) / T;
        atomicAdd(&hist[q.rank * nc.ntiles + tile], 1);
      }
  }
}

// one block: offsets (exclusive scan of the histogram), one work item per
// non-empty (class, tile) bin, and bundles of up to G items of one class
__global__ void __launch_bounds__(1024) k_na_tables(const int32_t* __restrict__ hist,
                                                    int32_t nkeys, NaClasses nc,
                                                    int32_t* __restrict__ offs,
                                                    Item* __restrict__ items,
                                                    Bundle* __restrict__ bundles,
                                                    int32_t* __restrict__ counters) {
  __shared__ int s_r[1024], s_i[1024];
  __shared__ int cls_first[kMaxClasses + 1];
  const int tid = threadIdx.x;
  const int chunk = (nkeys + 1023) / 1024;
  const int k0 = min(nkeys, tid * chunk), k1 = min(nkeys, k0 + chunk);
  int rsum = 0, isum = 0;
  for (int k = k0; k < k1; k++) {
    const int h = hist[k];
    rsum += h;
    isum += h > 0;
  }
  s_r[tid] = rsum;
  s_i[tid] = isum;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    const int a = tid >= off ? s_r[tid - off] : 0;
    const int b = tid >= off ? s_i[tid - off] : 0;
    __syncthreads();
    s_r[tid] += a;
    s_i[tid] += b;
    __syncthreads();
  }
  int rpre = s_r[tid] - rsum, ipre = s_i[tid] - isum;
  for (int k = k0; k < k1; k++) {
    if (k % nc.ntiles == 0) cls_first[k / nc.ntiles] = ipre;
    const int h = hist[k];
    offs[k] = rpre;
    if (h > 0) {
      const int c = k / nc.ntiles, tile = k - c * nc.ntiles;
      Item it;
      it.start = rpre;
      it.count = h;
      it.tile_x = (int16_t)(tile % nc.ntx);
      it.tile_y = (int16_t)(tile / nc.ntx);
      it.pmax = (int16_t)nc.pmax[c];
      it.cls = (int16_t)c;
      items[ipre++] = it;
    }
    rpre += h;
  }
  if (tid == 1023) {
    offs[nkeys] = s_r[1023];
    counters[kCntPieces] = s_r[1023];
    counters[kCntItems] = s_i[1023];
    cls_first[nc.n] = s_i[1023];
  }
  __syncthreads();
  int nb[kMaxClasses], bs[kMaxClasses + 1];
  bs[0] = 0;
  for (int c = 0; c < nc.n; c++) {
    const int n_c = cls_first[c + 1] - cls_first[c];
    nb[c] = (n_c + nc.G[c] - 1) / nc.G[c];
    bs[c + 1] = bs[c] + nb[c];
  }
  const int total = bs[nc.n];
  for (int b = tid; b < total; b += 1024) {
    int c = 0;
    while (b >= bs[c + 1]) c++;
    const int j = b - bs[c];
    const int n_c = cls_first[c + 1] - cls_first[c];
    Bundle B;
    B.first_item = cls_first[c] + j * nc.G[c];
    B.n_items = (int16_t)min(nc.G[c], n_c - j * nc.G[c]);
    B.cls = (int16_t)c;
    B.grid = 0;
    B.pad = 0;
    bundles[b] = B;
  }
  if (tid == 0) counters[kCntBundles] = total;
}

__global__ void k_na_fill(PlanDev P, const PlaneInfo* __restrict__ pl, int32_t T, NaClasses nc,
                          const int32_t* __restrict__ offs, int32_t* __restrict__ cursor,
                          Rec* __restrict__ recs, int32_t* __restrict__ counters) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < P.n_vis;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int32_t p = P.plane[t];
    if (p < 0) continue;
    const PlaneInfo q = pl[p];
    const double* r = P.uvw + t * P.uvw_stride;
    const VisIndex ix =
        vis_index(r[0], r[1], P.scale, P.grid_size, q.S, P.margin, 0, 0, P.ext_x, P.ext_y);
    if (!ix.keep) continue;
    const int64_t gbase = q.gcf_off + (int64_t)ix.phase * q.S * q.S;
    for (int oy = 0; oy < q.S; oy += q.P) {
      const int Y0 = ix.y0 + oy, wy = min(q.P, q.S - oy);
      for (int ox = 0; ox < q.S; ox += q.P) {
        const int X0 = ix.x0 + ox, wx = min(q.P, q.S - ox);
        const int tx = X0 / T, ty = Y0 / T;
        const int key = q.rank * nc.ntiles + ty * nc.ntx + tx;
        const int32_t pos = offs[key] + atomicAdd(&cursor[key], 1);
        if (pos >= kMaxPieces) {  // cannot happen under the host-side bound; never write past
          atomicExch(&counters[kCntOverflow], 1);
          continue;
        }
        Rec rc;
        rc.vis = (int32_t)t;
        rc.gcf = (uint32_t)(gbase + (int64_t)oy * q.S + ox);
        rc.xl = (uint8_t)(X0 - tx * T);
        rc.yl = (uint8_t)(Y0 - ty * T);
        rc.wx = (uint8_t)wx;
        rc.wy = (uint8_t)wy;
        rc.xm = (uint8_t)(X0 % q.P);
        rc.ym = (uint8_t)(Y0 % q.P);
        rc.pm1 = (uint8_t)(q.P - 1);
        rc.sm1 = (uint8_t)(q.S - 1);
        recs[pos] = rc;
      }
    }
  }
}

// Device address of the scratch array, looked up once per device.
static int scratch_base(unsigned char** out) {
  static std::mutex mu;
  static void* base[64] = {};
  int dev = 0;
  GB_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    gb_set_error(GB_ERR_CAPACITY, "gb_grid_f32_noalloc: device ordinal %d >= 64", dev);
    return GB_ERR_CAPACITY;
  }
  std::lock_guard<std::mutex> lk(mu);
  if (!base[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      gb_set_error(GB_ERR_CUDA, "cudaGetSymbolAddress(g_noalloc_scratch): %s",
                   cudaGetErrorString(e));
      return GB_ERR_CUDA;
    }
    base[dev] = p;
  }
  *out = (unsigned char*)base[dev];
  return GB_OK;
}

static int class_width_na(int P, int NT) {
  for (int L = 64; L <= NT; L *= 2)
    if (P * P <= 2 * L) return L;
  return NT;
}

}  // namespace gb

using namespace gb;

extern "C" int gb_grid_f32_noalloc(const gb_geometry* geo, int64_t n_vis, const double* d_uvw,
                                   int64_t uvw_stride, const int32_t* d_plane, const float* d_vis,
                                   const float* d_gcf, float* d_grid, void* stream) {
  if (!geo || n_vis < 0 || (n_vis > 0 && (!d_uvw || !d_vis || !d_gcf)) || !d_grid ||
      uvw_stride < 3 || geo->n_planes < 1 || !geo->supports || !geo->gcf_offsets ||
      geo->ext_x <= 0 || geo->ext_y <= 0 || geo->pitch < geo->ext_x ||
      !(geo->scale == geo->scale)) {
    gb_set_error(GB_ERR_ARG, "gb_grid_f32_noalloc: bad geometry or arguments");
    return GB_ERR_ARG;
  }
  if (n_vis > kMaxVis || geo->n_planes > kMaxPlanes) {
    gb_set_error(GB_ERR_CAPACITY,
                 "gb_grid_f32_noalloc: %lld visibilities / %d planes exceed the allocation-free "
                 "limits (%d visibilities, %d planes); use gb_plan_create + gb_grid_f32",
                 (long long)n_vis, geo->n_planes, kMaxVis, kMaxPlanes);
    return GB_ERR_CAPACITY;
  }
  const int T = geo->tile ? geo->tile : 32;
  const int NT = geo->threads ? geo->threads : 256;
  const int cap = geo->period_cap ? geo->period_cap : 32;
  if (T < 8 || T > 128 || (NT != 128 && NT != 256 && NT != 512) || cap < 8 || cap > 64 ||
      cap * cap > 8 * NT) {
    gb_set_error(GB_ERR_ARG, "gb_grid_f32_noalloc: unsupported tuning tile=%d threads=%d cap=%d",
                 T, NT, cap);
    return GB_ERR_ARG;
  }
  // work items hold tile indices as int16 (the rule of gb_plan_create): a grid
  // more than 32767 tiles wide or high is rejected before any GPU work
  if (geo->ext_x > 32767 * (int64_t)T || geo->ext_y > 32767 * (int64_t)T) {
    gb_set_error(GB_ERR_ARG,
                 "gb_grid_f32_noalloc: grid extent %d x %d exceeds 32767 tiles of %d pixels",
                 geo->ext_x, geo->ext_y, T);
    return GB_ERR_ARG;
  }
  // planes -> pieces, periods, classes (the rules of gb_plan_create)
  thread_local PlaneInfo pl[kMaxPlanes];
  int widths[kMaxClasses], nwidth = 0, kmax = 1;
  int64_t gcf_len = 0;
  for (int p = 0; p < geo->n_planes; p++) {
    const int S = geo->supports[p];
    if (S < 1 || S > GB_MAX_SUPPORT || geo->gcf_offsets[p] < 0 ||
        geo->gcf_offsets[p] + (int64_t)GB_PHASES * S * S > (int64_t)UINT32_MAX) {
      gb_set_error(GB_ERR_ARG, "gb_grid_f32_noalloc: plane %d support %d / offset out of range",
                   p, S);
      return GB_ERR_ARG;
    }
    PlaneInfo& q = pl[p];
    q.S = S;
    q.k = (S + cap - 1) / cap;
    q.P = (S + q.k - 1) / q.k;
    if (q.k > 1 && !(S & 1) && (q.P & 1) && q.P < cap) q.P++;  // even-width pieces
    q.gcf_off = geo->gcf_offsets[p];
    gcf_len = std::max<int64_t>(gcf_len, q.gcf_off + (int64_t)GB_PHASES * S * S);
    kmax = q.k > kmax ? q.k : kmax;
    const int L = class_width_na(q.P, NT);
    int c = 0;
    while (c < nwidth && widths[c] != L) c++;
    if (c == nwidth) {
      if (nwidth == kMaxClasses) {
        gb_set_error(GB_ERR_CAPACITY, "gb_grid_f32_noalloc: too many thread-group classes");
        return GB_ERR_CAPACITY;
      }
      widths[nwidth++] = L;
    }
  }
  // classes in ascending width, each plane's class index kept in `rank`
  for (int a = 0; a < nwidth; a++)
    for (int b = a + 1; b < nwidth; b++)
      if (widths[b] < widths[a]) {
        const int t = widths[a];
        widths[a] = widths[b];
        widths[b] = t;
      }
  ClassInfo cls[kMaxClasses];
  NaClasses nc{};
  nc.n = nwidth;
  const int smem_cap = tiled_max_smem();
  size_t smem = 0;
  for (int c = 0; c < nwidth; c++) {
    cls[c].L = widths[c];
    cls[c].pmax = 0;
  }
  for (int p = 0; p < geo->n_planes; p++) {
    int c = 0;
    while (widths[c] != class_width_na(pl[p].P, NT)) c++;
    pl[p].rank = c;
    if (pl[p].P > cls[c].pmax) cls[c].pmax = pl[p].P;
  }
  for (int c = 0; c < nwidth; c++) {
    cls[c].A = T + cls[c].pmax - 1;
    const size_t per_group = grid_group_bytes(cls[c].A, cls[c].L);
    int G = NT / cls[c].L;
    while (G > 0 && (size_t)G * per_group > (size_t)smem_cap) G--;
    if (G == 0) {
      gb_set_error(GB_ERR_CAPACITY, "gb_grid_f32_noalloc: tile %d / period %d exceed shared memory",
                   T, cls[c].pmax);
      return GB_ERR_CAPACITY;
    }
    cls[c].G = G;
    nc.G[c] = G;
    nc.pmax[c] = cls[c].pmax;
    if ((size_t)G * per_group > smem) smem = (size_t)G * per_group;
  }
  nc.ntx = (geo->ext_x + T - 1) / T;
  const int nty = (geo->ext_y + T - 1) / T;
  const int64_t ntiles = (int64_t)nc.ntx * nty;
  const int64_t nkeys = ntiles * nwidth;
  if (n_vis * (int64_t)kmax * kmax > kMaxPieces || nkeys > kMaxBins) {
    gb_set_error(GB_ERR_CAPACITY,
                 "gb_grid_f32_noalloc: up to %lld footprint pieces / %lld tile bins exceed the "
                 "allocation-free limits (%d pieces, %d bins)",
                 (long long)(n_vis * kmax * kmax), (long long)nkeys, kMaxPieces, kMaxBins);
    return GB_ERR_CAPACITY;
  }
  nc.ntiles = (int32_t)ntiles;

  unsigned char* base = nullptr;
  int rc = scratch_base(&base);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  int32_t* counters = (int32_t*)(base + kOffCounters);
  PlaneInfo* d_pl = (PlaneInfo*)(base + kOffPlanes);
  int32_t* plane_of = (int32_t*)(base + kOffPlaneOf);
  int32_t* hist = (int32_t*)(base + kOffHist);
  int32_t* offs = (int32_t*)(base + kOffOffs);
  int32_t* cursor = (int32_t*)(base + kOffCursor);
  Rec* recs = (Rec*)(base + kOffRecs);
  Item* items = (Item*)(base + kOffItems);
  Bundle* bundles = (Bundle*)(base + kOffBundles);

  GB_CUDA_TRY(cudaMemcpyAsync(d_pl, pl, sizeof(PlaneInfo) * geo->n_planes,
                              cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemsetAsync(counters, 0, 64, s));
  GB_CUDA_TRY(cudaMemsetAsync(hist, 0, sizeof(int32_t) * nkeys, s));
  GB_CUDA_TRY(cudaMemsetAsync(cursor, 0, sizeof(int32_t) * nkeys, s));
  PlanDev D;
  D.n_vis = n_vis;
  D.uvw = d_uvw;
  D.uvw_stride = uvw_stride;
  D.plane = plane_of;
  D.order = nullptr;
  D.supports = nullptr;
  D.gcf_offsets = nullptr;
  D.scale = geo->scale;
  D.grid_size = geo->grid_size;
  D.margin = geo->margin;
  D.ext_x = geo->ext_x;
  D.ext_y = geo->ext_y;
  D.pitch = geo->pitch;
  const int blocks = (int)std::min<int64_t>((n_vis + 255) / 256 + 1, (int64_t)sm_count() * 8);
  if (n_vis > 0) {
    k_na_count<<<blocks, 256, 0, s>>>(D, d_pl, d_plane, plane_of, geo->n_planes, geo->w_low,
                                      geo->w_high, T, nc, hist);
    GB_CUDA_TRY(cudaGetLastError());
  }
  k_na_tables<<<1, 1024, 0, s>>>(hist, (int32_t)nkeys, nc, offs, items, bundles, counters);
  GB_CUDA_TRY(cudaGetLastError());
  if (n_vis > 0) {
    k_na_fill<<<blocks, 256, 0, s>>>(D, d_pl, T, nc, offs, cursor, recs, counters);
    GB_CUDA_TRY(cudaGetLastError());
  }
  int32_t hc[8] = {0};
  GB_CUDA_TRY(cudaMemcpyAsync(hc, counters, sizeof(hc), cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  if (hc[kCntOverflow]) {
    gb_set_error(GB_ERR_CAPACITY, "gb_grid_f32_noalloc: footprint pieces overflowed the scratch");
    return GB_ERR_CAPACITY;
  }
  return launch_grid_tiled_tables(bundles, hc[kCntBundles], items, recs, counters + kCntQueue, cls,
                                  nwidth, NT, T, geo->ext_x, geo->ext_y, geo->pitch, smem, d_vis,
                                  d_gcf, d_grid, TiledBounds{hc[kCntPieces], gcf_len, n_vis}, s);
}
