// Visibility plan: w-plane assignment, FP64 index math, and the sort / bin of
// footprint pieces by (grid tile, period) that feeds the FP32 tiled kernels.
//
// It replaces the reference's host-side binning (MS6/programs/Kernel/
// Binning.hs:34-181, a scalar Haskell pass per visibility) and the NVIDIA
// gridder's host std::sort (MS6/kernel/nvidia/gridder/binsort.cpp:6-35) with
// a counting sort on the GPU:
//   1. k_plan_count: per visibility, plane + index math (FP64), then a
//      histogram of pieces per (tile, period rank);
//   2. host: exclusive scan of the histogram, work items (record ranges of
//      one tile and one thread-group class, cut by a cost model), bundles of
//      items for the persistent kernels, longest first;
//   3. k_plan_fill: recompute the index, scatter 16-byte records into their
//      bins.
#include <algorithm>
#include <thread>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>

#include "gb_common.cuh"
#include "gb_plan.cuh"
#include "gb_runtime.cuh"

namespace gb {

__global__ void k_plan_count(PlanDev P, const PlaneInfo* __restrict__ pl,
                             const int32_t* __restrict__ plane_in, int32_t* __restrict__ plane_out,
                             int32_t n_planes, double w_lo, double w_hi, int32_t T, int32_t ntx,
                             int32_t nper, int32_t* __restrict__ hist,
                             int32_t* __restrict__ vis_hist,
                             unsigned long long* __restrict__ counters) {
  __shared__ unsigned long long s_kept, s_taps, s_recs, s_paired;
  if (threadIdx.x == 0) s_kept = s_taps = s_recs = s_paired = 0ull;
  __syncthreads();
  unsigned long long kept = 0, taps = 0, recs = 0, paired = 0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < P.n_vis;
       t += (int64_t)gridDim.x * blockDim.x) {
    const double* r = P.uvw + t * P.uvw_stride;
    int32_t p = plane_in ? plane_in[t] : w_plane(r[2], w_lo, w_hi, n_planes);
    if (p >= n_planes) p = -1;
    plane_out[t] = p;
    const int64_t ntiles = (int64_t)ntx * ((P.ext_y + T - 1) / T);
    if (p < 0) {
      atomicAdd(&vis_hist[ntiles], 1);  // skipped visibilities go last
      continue;
    }
    const PlaneInfo q = pl[p];
    const VisIndex ix =
        vis_index(r[0], r[1], P.scale, P.grid_size, q.S, P.margin, 0, 0, P.ext_x, P.ext_y);
    if (!ix.keep) {
      atomicAdd(&vis_hist[ntiles], 1);
      continue;
    }
    atomicAdd(&vis_hist[(int64_t)(ix.y0 / T) * ntx + ix.x0 / T], 1);
    kept++;
    taps += (unsigned long long)q.S * q.S;
    for (int ky = 0; ky < q.k; ky++) {
      const int Y0 = ix.y0 + ky * q.P;
      if (ky * q.P >= q.S) break;
      for (int kx = 0; kx < q.k; kx++) {
        if (kx * q.P >= q.S) break;
        const int X0 = ix.x0 + kx * q.P;
        const int64_t tile = (int64_t)(Y0 / T) * ntx + (X0 / T);
        atomicAdd(&hist[tile * nper + q.rank], 1);
        recs++;
        // degridding pairs the taps of a piece whose rows, GCF rows and GCF
        // offset are all even (the same rule the kernels apply per record)
        const int wx = min(q.P, q.S - kx * q.P), wy = min(q.P, q.S - ky * q.P);
        if (((wx | q.S | (int)((q.gcf_off + kx * q.P) & 1)) & 1) == 0)
          paired += (unsigned long long)wx * wy;
      }
    }
  }
  atomicAdd(&s_kept, kept);
  atomicAdd(&s_taps, taps);
  atomicAdd(&s_recs, recs);
  atomicAdd(&s_paired, paired);
  __syncthreads();
  if (threadIdx.x == 0) {
    atomicAdd(&counters[0], s_kept);
    atomicAdd(&counters[1], s_taps);
    atomicAdd(&counters[2], s_recs);
    atomicAdd(&counters[3], s_paired);
  }
}

__global__ void k_plan_fill(PlanDev P, const PlaneInfo* __restrict__ pl, int32_t T, int32_t ntx,
                            int32_t nper, const int32_t* __restrict__ offs,
                            int32_t* __restrict__ cursor, Rec* __restrict__ recs,
                            const int32_t* __restrict__ vis_offs,
                            int32_t* __restrict__ vis_cursor, int32_t* __restrict__ order) {
  const int64_t ntiles = (int64_t)ntx * ((P.ext_y + T - 1) / T);
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < P.n_vis;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int32_t p = P.plane[t];
    if (p < 0) {
      order[vis_offs[ntiles] + atomicAdd(&vis_cursor[ntiles], 1)] = (int32_t)t;
      continue;
    }
    const PlaneInfo q = pl[p];
    const double* r = P.uvw + t * P.uvw_stride;
    const VisIndex ix =
        vis_index(r[0], r[1], P.scale, P.grid_size, q.S, P.margin, 0, 0, P.ext_x, P.ext_y);
    const int64_t vt = ix.keep ? (int64_t)(ix.y0 / T) * ntx + ix.x0 / T : ntiles;
    order[vis_offs[vt] + atomicAdd(&vis_cursor[vt], 1)] = (int32_t)t;
    if (!ix.keep) continue;
    const int64_t gbase = q.gcf_off + (int64_t)ix.phase * q.S * q.S;
    for (int ky = 0; ky < q.k; ky++) {
      const int oy = ky * q.P;
      if (oy >= q.S) break;
      const int Y0 = ix.y0 + oy;
      const int wy = min(q.P, q.S - oy);
      for (int kx = 0; kx < q.k; kx++) {
        const int ox = kx * q.P;
        if (ox >= q.S) break;
        const int X0 = ix.x0 + ox;
        const int wx = min(q.P, q.S - ox);
        const int tx = X0 / T, ty = Y0 / T;
        const int64_t key = ((int64_t)ty * ntx + tx) * nper + q.rank;
        // lanes with the same bin take consecutive places in lane order (one
        // atomic per bin and warp): neighbouring samples of a baseline, which
        // a warp holds side by side, stay neighbours in the bin, where the
        // gridder sums the taps that consecutive pieces put on one pixel
        const unsigned act = __activemask();
        const unsigned peers = __match_any_sync(act, key);
        const int lane = threadIdx.x & 31, leader = __ffs(peers) - 1;
        int32_t first = 0;
        if (lane == leader) first = atomicAdd(&cursor[key], __popc(peers));
        first = __shfl_sync(act, first, leader);
        const int32_t pos = offs[key] + first + __popc(peers & ((1u << lane) - 1u));
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

__global__ void k_plan_export(PlanDev P, const int32_t* __restrict__ supports,
                              int32_t* __restrict__ out5) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < P.n_vis;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int32_t p = P.plane[t];
    int32_t* o = out5 + 5 * t;
    if (p < 0) {
      o[0] = o[1] = o[2] = 0;
      o[3] = p;
      o[4] = 0;
      continue;
    }
    const double* r = P.uvw + t * P.uvw_stride;
    const VisIndex ix = vis_index(r[0], r[1], P.scale, P.grid_size, supports[p], P.margin, 0, 0,
                                  P.ext_x, P.ext_y);
    o[0] = ix.x0;
    o[1] = ix.y0;
    o[2] = ix.phase;
    o[3] = p;
    o[4] = ix.keep ? 1 : 0;
  }
}

// Thread-group width for a period: the smallest power of two L >= 64 (and
// <= NT) holding P^2 taps in at most two rounds; NT otherwise.
static int class_width(int P, int NT) {
  for (int L = 64; L <= NT; L *= 2)
    if (P * P <= 2 * L) return L;
  return NT;
}

static int blocks_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  const int64_t cap = (int64_t)sm_count() * 32;
  if (b > cap) b = cap;
  return (int)(b < 1 ? 1 : b);
}

static void free_plan(gb_plan* p) {
  if (!p) return;
  cudaFree(p->d_plane);
  cudaFree(p->d_order);
  cudaFree(p->d_supports);
  cudaFree(p->d_offsets);
  cudaFree(p->d_planes);
  cudaFree(p->d_recs);
  cudaFree(p->d_items);
  cudaFree(p->d_bundles);
  cudaFree(p->d_queue);
  p->df.release();
  delete p;
}

template <class T>
static int dalloc(T** p, size_t n) {
  void* q = nullptr;
  const int rc = dev_alloc(&q, sizeof(T) * (n ? n : 1), "plan");
  *p = (T*)q;
  return rc;
}

// idx[0..n) reordered by cost, largest first, in one counting pass over the
// costs quantised to 4096 levels of the largest (ties keep their order): the
// longest-first heuristic needs no finer order, and a comparison sort of tens
// of thousands of items costs milliseconds of host time per plan.
static void order_by_cost(const std::vector<double>& cost, int32_t* idx, size_t n) {
  if (n < 2) return;
  constexpr int K = 4096;
  double top = 0;
  for (size_t i = 0; i < n; i++) top = std::max(top, cost[idx[i]]);
  const double q = top > 0 ? (K - 1) / top : 0.0;
  std::vector<int32_t> cnt(K + 1, 0), tmp(idx, idx + n);
  auto level = [&](int32_t i) {
    const int l = (int)(cost[i] * q);
    return K - 1 - std::min(std::max(l, 0), K - 1);  // largest first
  };
  for (size_t i = 0; i < n; i++) cnt[level(tmp[i]) + 1]++;
  for (int k = 1; k <= K; k++) cnt[k] += cnt[k - 1];
  for (size_t i = 0; i < n; i++) idx[cnt[level(tmp[i])]++] = tmp[i];
}

void make_bundles(const std::vector<HostItem>& items, const ClassInfo* cls, int n_classes,
                  std::vector<Item>& it_out, std::vector<Bundle>& b_out) {
  // items by (class, grid slot), each bucket in the items' own order: one
  // counting pass (a batch has up to kMaxGrids slots)
  int max_grid = 0;
  for (const auto& h : items) max_grid = std::max(max_grid, h.grid);
  const size_t ng = (size_t)max_grid + 1, nb = (size_t)n_classes * ng;
  std::vector<size_t> first(nb + 1, 0);
  for (const auto& h : items) first[(size_t)item_class(h.it.cls) * ng + h.grid + 1]++;
  for (size_t k = 1; k <= nb; k++) first[k] += first[k - 1];
  std::vector<int32_t> order(items.size());
  {
    std::vector<size_t> next(first.begin(), first.end() - 1);
    for (size_t i = 0; i < items.size(); i++)
      order[next[(size_t)item_class(items[i].it.cls) * ng + items[i].grid]++] = (int32_t)i;
  }
  // within a bucket, longest first; groups of G items form a bundle
  struct HB {
    Bundle b;
    double cost;
  };
  std::vector<HB> bundles;
  bundles.reserve(items.size());
  it_out.clear();
  it_out.reserve(items.size());
  std::vector<double> cost(items.size());
  for (size_t i = 0; i < items.size(); i++) cost[i] = items[i].cost;
  for (int c = 0; c < n_classes; c++) {
    const int G = cls[c].G;
    for (size_t g = 0; g < ng; g++) {
      const size_t k = (size_t)c * ng + g;
      if (first[k] == first[k + 1]) continue;
      order_by_cost(cost, order.data() + first[k], first[k + 1] - first[k]);
      for (size_t i = first[k]; i < first[k + 1]; i += G) {
        HB hb;
        hb.b.first_item = (int32_t)it_out.size();
        hb.b.n_items = (int16_t)std::min<size_t>(G, first[k + 1] - i);
        hb.b.cls = (int16_t)c;
        hb.b.grid = (int32_t)g;
        hb.b.pad = 0;
        hb.cost = items[order[i]].cost;
        for (int m = 0; m < hb.b.n_items; m++) it_out.push_back(items[order[i + m]].it);
        bundles.push_back(hb);
      }
    }
  }
  // all bundles, longest first
  std::vector<int32_t> bo(bundles.size());
  std::vector<double> bcost(bundles.size());
  for (size_t i = 0; i < bo.size(); i++) {
    bo[i] = (int32_t)i;
    bcost[i] = bundles[i].cost;
  }
  order_by_cost(bcost, bo.data(), bo.size());
  b_out.clear();
  b_out.reserve(bundles.size());
  for (int32_t i : bo) b_out.push_back(bundles[i].b);
}

// Modelled shared-memory wavefronts per pair that degridding's split-row stage
// costs a sub-warp of SW lanes reading SW consecutive pairs (row-major, rows
// of w2 pairs) with rows r (mod 16) float2 apart: the largest number of
// addresses on one 8-byte bank pair (of 16), averaged over where the run
// starts in its row, per pair of the run.
static double split_stage_cost(int w2, int r, int SW) {
  double sum = 0;
  for (int t0 = 0; t0 < w2; t0++) {
    int cnt[16] = {0};
    for (int l = 0; l < SW; l++) {
      const int t = t0 + l, j = t / w2, i = t - j * w2;
      cnt[(j * r + i) & 15]++;
    }
    sum += *std::max_element(cnt, cnt + 16);
  }
  return sum / w2 / SW;
}

// Sub-warp width of degridding for a class's largest period (the kernel's rule).
static int degrid_subwarp(int pmax) { return pmax <= 8 ? 8 : pmax <= 16 ? 16 : 32; }

static int build_plan(gb_plan* P, const gb_geometry* geo, int64_t n_vis, const double* d_uvw,
                      int64_t uvw_stride, const int32_t* d_plane_in, cudaStream_t s) {
  int rc;
  const int np = geo->n_planes;
  // ---- per-plane pieces, periods, classes
  P->planes.resize(np);
  std::vector<int> periods;
  for (int p = 0; p < np; p++) {
    PlaneInfo& q = P->planes[p];
    q.S = geo->supports[p];
    q.k = (q.S + P->pcap - 1) / P->pcap;
    q.P = (q.S + q.k - 1) / q.k;
    // an even support is cut into even-width pieces (the last one narrower),
    // so degridding can take every piece's taps in pairs
    if (q.k > 1 && !(q.S & 1) && (q.P & 1) && q.P < P->pcap) q.P++;
    q.gcf_off = geo->gcf_offsets[p];
    P->gcf_len = std::max<int64_t>(P->gcf_len, q.gcf_off + (int64_t)GB_PHASES * q.S * q.S);
    periods.push_back(q.P);
    if (q.gcf_off + (int64_t)GB_PHASES * q.S * q.S > (int64_t)UINT32_MAX) {
      gb_set_error(GB_ERR_CAPACITY, "GCF array exceeds 2^32 complex elements");
      return GB_ERR_CAPACITY;
    }
  }
  std::sort(periods.begin(), periods.end());
  periods.erase(std::unique(periods.begin(), periods.end()), periods.end());
  const int nper = (int)periods.size();
  for (auto& q : P->planes)
    q.rank = (int)(std::lower_bound(periods.begin(), periods.end(), q.P) - periods.begin());
  // classes by group width, ascending
  std::vector<int> widths;
  for (int pp : periods) widths.push_back(class_width(pp, P->NT));
  std::vector<int> cls_w = widths;
  std::sort(cls_w.begin(), cls_w.end());
  cls_w.erase(std::unique(cls_w.begin(), cls_w.end()), cls_w.end());
  P->n_classes = (int)cls_w.size();
  if (P->n_classes > kMaxClasses) {
    gb_set_error(GB_ERR_CAPACITY, "too many thread-group classes");
    return GB_ERR_CAPACITY;
  }
  std::vector<int> rank_cls(nper);
  for (int r = 0; r < nper; r++)
    rank_cls[r] = (int)(std::lower_bound(cls_w.begin(), cls_w.end(), widths[r]) - cls_w.begin());
  const int smem_cap = tiled_max_smem();
  for (int c = 0; c < P->n_classes; c++) {
    ClassInfo& ci = P->cls[c];
    ci.L = cls_w[c];
    ci.pmax = 0;
    for (int r = 0; r < nper; r++)
      if (rank_cls[r] == c) ci.pmax = std::max(ci.pmax, periods[r]);
    ci.A = P->T + ci.pmax - 1;
    const size_t per_group = group_bytes(ci.A, ci.L);
    int G = P->NT / ci.L;
    while (G > 0 && (size_t)G * per_group > (size_t)smem_cap) G--;
    if (G == 0) {
      gb_set_error(GB_ERR_CAPACITY,
                   "tile %d with period %d needs %zu B of shared memory (limit %d)", P->T,
                   ci.pmax, per_group, smem_cap);
      return GB_ERR_CAPACITY;
    }
    ci.G = G;
  }
  P->smem_grid = tiled_smem_grid(P->cls, P->n_classes, P->NT);
  P->smem_degrid = tiled_smem_degrid(P->cls, P->n_classes, P->NT);
  P->ctas_per_sm_grid = tiled_ctas_per_sm(P, true);
  for (int st = 0; st < 3; st++) P->ctas_per_sm_degrid[st] = tiled_ctas_per_sm(P, false, st);

  // ---- device tables
  if ((rc = dalloc(&P->d_plane, n_vis)) || (rc = dalloc(&P->d_order, n_vis)) ||
      (rc = dalloc(&P->d_supports, np)) ||
      (rc = dalloc(&P->d_offsets, np)) || (rc = dalloc(&P->d_planes, np)) ||
      (rc = dalloc(&P->d_queue, 3)))
    return rc;
  // [0], [1]: work-queue heads of the grid and degrid kernels; [2]: device
  // error word (a TMA stage completion not seen in time)
  GB_CUDA_TRY(cudaMemsetAsync(P->d_queue, 0, 3 * sizeof(int32_t), s));
  GB_CUDA_TRY(cudaMemcpyAsync(P->d_supports, geo->supports, sizeof(int32_t) * np,
                              cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemcpyAsync(P->d_offsets, geo->gcf_offsets, sizeof(int64_t) * np,
                              cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemcpyAsync(P->d_planes, P->planes.data(), sizeof(PlaneInfo) * np,
                              cudaMemcpyHostToDevice, s));
  PlanDev& D = P->dev;
  D.n_vis = n_vis;
  D.uvw = d_uvw;
  D.uvw_stride = uvw_stride;
  D.plane = P->d_plane;
  D.order = P->d_order;
  D.supports = P->d_supports;
  D.gcf_offsets = P->d_offsets;
  D.scale = geo->scale;
  D.grid_size = geo->grid_size;
  D.margin = geo->margin;
  D.ext_x = geo->ext_x;
  D.ext_y = geo->ext_y;
  D.pitch = geo->pitch;

  // ---- histogram
  P->ntx = (geo->ext_x + P->T - 1) / P->T;
  P->nty = (geo->ext_y + P->T - 1) / P->T;
  const int64_t nkeys = (int64_t)P->ntx * P->nty * nper;
  if (nkeys >= (int64_t)INT32_MAX) {
    gb_set_error(GB_ERR_CAPACITY, "too many (tile, period) bins");
    return GB_ERR_CAPACITY;
  }
  // per-visibility order: one bucket per tile (the footprint corner's) and a
  // last one for the visibilities no kernel grids
  const int64_t nvkeys = (int64_t)P->ntx * P->nty + 1;
  int32_t *d_hist = nullptr, *d_offs = nullptr, *d_vhist = nullptr, *d_voffs = nullptr;
  unsigned long long* d_cnt = nullptr;
  if ((rc = dalloc(&d_hist, nkeys)) || (rc = dalloc(&d_offs, nkeys + 1)) ||
      (rc = dalloc(&d_vhist, nvkeys)) || (rc = dalloc(&d_voffs, nvkeys)) ||
      (rc = dalloc(&d_cnt, 4))) {
    cudaFree(d_hist);
    cudaFree(d_offs);
    cudaFree(d_vhist);
    cudaFree(d_voffs);
    cudaFree(d_cnt);
    return rc;
  }
  struct Tmp {
    void* p[5];
    ~Tmp() {
      for (void* q : p) cudaFree(q);
    }
  } tmp{{d_hist, d_offs, d_vhist, d_voffs, d_cnt}};
  GB_CUDA_TRY(cudaMemsetAsync(d_hist, 0, sizeof(int32_t) * nkeys, s));
  GB_CUDA_TRY(cudaMemsetAsync(d_vhist, 0, sizeof(int32_t) * nvkeys, s));
  GB_CUDA_TRY(cudaMemsetAsync(d_cnt, 0, sizeof(unsigned long long) * 4, s));
  if (n_vis > 0) {
    k_plan_count<<<blocks_for(n_vis, 256), 256, 0, s>>>(
        D, P->d_planes, d_plane_in, P->d_plane, np, geo->w_low, geo->w_high, P->T, P->ntx, nper,
        d_hist, d_vhist, d_cnt);
    GB_CUDA_TRY(cudaGetLastError());
  }
  std::vector<int32_t> hist(nkeys), vhist(nvkeys);
  unsigned long long cnt[4];
  GB_CUDA_TRY(cudaMemcpyAsync(hist.data(), d_hist, sizeof(int32_t) * nkeys, cudaMemcpyDeviceToHost,
                              s));
  GB_CUDA_TRY(cudaMemcpyAsync(vhist.data(), d_vhist, sizeof(int32_t) * nvkeys,
                              cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaMemcpyAsync(cnt, d_cnt, sizeof(cnt), cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  P->kept = (int64_t)cnt[0];
  P->taps = (int64_t)cnt[1];
  P->n_recs = (int64_t)cnt[2];
  P->taps_paired = (int64_t)cnt[3];
  if (P->n_recs >= (int64_t)INT32_MAX) {
    gb_set_error(GB_ERR_CAPACITY, "more than 2^31 footprint pieces");
    return GB_ERR_CAPACITY;
  }

  // ---- scan + items
  std::vector<int32_t> offs(nkeys + 1);
  int64_t acc = 0;
  for (int64_t k = 0; k < nkeys; k++) {
    offs[k] = (int32_t)acc;
    acc += hist[k];
  }
  offs[nkeys] = (int32_t)acc;

  // cost model, in thread-group steps: a piece of period P costs ceil(P^2/L)
  // tap rounds plus one for its record; an item adds zeroing + flush of its
  // A x A accumulator.
  std::vector<double> rec_cost(nper);
  for (int r = 0; r < nper; r++) {
    const int L = P->cls[rank_cls[r]].L;
    rec_cost[r] = (double)((periods[r] * periods[r] + L - 1) / L + 1);
  }
  auto fixed_cost = [&](int c) {
    const ClassInfo& ci = P->cls[c];
    return (double)(2 * ((ci.A * ci.A + ci.L - 1) / ci.L));
  };
  // the histogram's cost per CTA slot (keys run rank-fastest within a tile)
  std::vector<double> rank_w(nper);
  for (int r = 0; r < nper; r++) rank_w[r] = rec_cost[r] / P->cls[rank_cls[r]].G;
  double total_cta = 0;
  for (int64_t k0 = 0; k0 < nkeys; k0 += nper)
    for (int r = 0; r < nper; r++) total_cta += hist[k0 + r] * rank_w[r];
  const int ctas = std::max(1, sm_count() * std::max(1, P->ctas_per_sm_grid));
  const double tau = total_cta / ((double)P->bpc * ctas);
  // a class's periods are consecutive ranks (group width grows with the period)
  std::vector<int> r_lo(P->n_classes, nper), r_hi(P->n_classes, 0);
  for (int r = 0; r < nper; r++) {
    r_lo[rank_cls[r]] = std::min(r_lo[rank_cls[r]], r);
    r_hi[rank_cls[r]] = std::max(r_hi[rank_cls[r]], r + 1);
  }
  // split-row stride residue per item: the residue that minimises the
  // modelled stage cost of its largest run (pieces of period P pair P / 2 taps
  // per row when P is even; choosing for the largest run alone comes within
  // 1 % of minimising over all of an item's runs on the benchmark workloads)
  std::vector<int> rank_residue(nper, -1);
  for (int r = 0; r < nper; r++) {
    const int Pr = periods[r], SW = degrid_subwarp(P->cls[rank_cls[r]].pmax);
    if (Pr & 1) continue;
    double bc = 0;
    for (int m = 0; m < 16; m++) {
      const double c = split_stage_cost(Pr / 2, m, SW);
      if (rank_residue[r] < 0 || c < bc) {
        rank_residue[r] = m;
        bc = c;
      }
    }
  }
  // items of tiles [t0, t1) in tile order, into out
  auto build_items = [&](int64_t t0, int64_t t1, std::vector<HostItem>& out, int64_t& used) {
    int64_t top_taps = 0;
    int top_rank = -1;
    auto close_item = [&](HostItem& h) {
      h.it.cls = item_cls_with_residue(h.it.cls, top_rank < 0 ? -1 : rank_residue[top_rank]);
      top_taps = 0;
      top_rank = -1;
      out.push_back(h);
    };
    for (int64_t tile = t0; tile < t1; tile++) {
      const int64_t k0 = tile * nper;
      if (offs[k0 + nper] == offs[k0]) continue;
      used++;
      const int16_t tx = (int16_t)(tile % P->ntx), ty = (int16_t)(tile / P->ntx);
      for (int c = 0; c < P->n_classes; c++) {
        if (r_lo[c] >= r_hi[c] || offs[k0 + r_hi[c]] == offs[k0 + r_lo[c]]) continue;
        const double fixed = fixed_cost(c), cmax = std::max(4.0 * fixed, tau);
        HostItem cur{};
        bool open = false;
        for (int r = r_lo[c]; r < r_hi[c]; r++) {
          int32_t pos = offs[k0 + r];
          const int32_t end = offs[k0 + r + 1];
          const double rcst = rec_cost[r];
          while (pos < end) {
            if (!open) {
              cur.it.start = pos;
              cur.it.count = 0;
              cur.it.tile_x = tx;
              cur.it.tile_y = ty;
              cur.it.pmax = 0;
              cur.it.cls = (int16_t)c;
              cur.cost = fixed;
              open = true;
            }
            int64_t room = (int64_t)((cmax - cur.cost) / rcst);
            if (room < 1) room = 1;
            const int32_t take = (int32_t)std::min<int64_t>(room, end - pos);
            cur.it.count += take;
            cur.it.pmax = (int16_t)std::max<int>(cur.it.pmax, periods[r]);
            cur.cost += take * rcst;
            if ((int64_t)take * periods[r] * periods[r] > top_taps) {
              top_taps = (int64_t)take * periods[r] * periods[r];
              top_rank = r;
            }
            pos += take;
            if (cur.cost >= cmax) {
              close_item(cur);
              open = false;
            }
          }
        }
        if (open) close_item(cur);
      }
    }
  };
  // tiles in contiguous chunks on up to eight host threads, concatenated in
  // tile order (the same items as one thread makes)
  const int64_t ntiles = (int64_t)P->ntx * P->nty;
  const int nth = (int)std::clamp<int64_t>(ntiles / 8192, 1,
                                           std::min(8u, std::max(1u, std::thread::hardware_concurrency())));
  std::vector<std::vector<HostItem>> parts(nth);
  std::vector<int64_t> used(nth, 0);
  {
    std::vector<std::thread> pool;
    for (int i = 1; i < nth; i++) {
      try {
        pool.emplace_back(build_items, ntiles * i / nth, ntiles * (i + 1) / nth, std::ref(parts[i]),
                          std::ref(used[i]));
      } catch (...) {  // no thread: this one does that chunk below
        break;
      }
    }
    build_items(0, ntiles / nth, parts[0], used[0]);
    for (auto& t : pool) t.join();
    for (int i = (int)pool.size() + 1; i < nth; i++)
      build_items(ntiles * i / nth, ntiles * (i + 1) / nth, parts[i], used[i]);
  }
  std::vector<HostItem> items;
  int64_t tiles_used = 0;
  {
    size_t total = 0;
    for (auto& v : parts) total += v.size();
    items.reserve(total);
    for (int i = 0; i < nth; i++) {
      items.insert(items.end(), parts[i].begin(), parts[i].end());
      tiles_used += used[i];
    }
  }
  P->tiles_used = tiles_used;
  for (auto& h : items) h.grid = 0;
  std::vector<Item> it_sorted;
  std::vector<Bundle> bvec;
  // a batch member's work goes into the batch's own tables instead
  if (P->own_work) make_bundles(items, P->cls, P->n_classes, it_sorted, bvec);
  P->n_items = (int)it_sorted.size();
  P->n_bundles = (int)bvec.size();
  // the items with their costs (any order), for batched launches
  P->host_items = std::move(items);

  // ---- fill
  if ((rc = dalloc(&P->d_recs, P->n_recs)) || (rc = dalloc(&P->d_items, P->n_items)) ||
      (rc = dalloc(&P->d_bundles, P->n_bundles)))
    return rc;
  GB_CUDA_TRY(cudaMemcpyAsync(d_offs, offs.data(), sizeof(int32_t) * (nkeys + 1),
                              cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemsetAsync(d_hist, 0, sizeof(int32_t) * nkeys, s));  // reused as cursor
  std::vector<int32_t> voffs(nvkeys);
  {
    int64_t a = 0;
    for (int64_t k = 0; k < nvkeys; k++) {
      voffs[k] = (int32_t)a;
      a += vhist[k];
    }
  }
  GB_CUDA_TRY(cudaMemcpyAsync(d_voffs, voffs.data(), sizeof(int32_t) * nvkeys,
                              cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemsetAsync(d_vhist, 0, sizeof(int32_t) * nvkeys, s));  // reused as cursor
  if (P->n_items)
    GB_CUDA_TRY(cudaMemcpyAsync(P->d_items, it_sorted.data(), sizeof(Item) * P->n_items,
                                cudaMemcpyHostToDevice, s));
  if (P->n_bundles)
    GB_CUDA_TRY(cudaMemcpyAsync(P->d_bundles, bvec.data(), sizeof(Bundle) * P->n_bundles,
                                cudaMemcpyHostToDevice, s));
  if (n_vis > 0) {
    k_plan_fill<<<blocks_for(n_vis, 256), 256, 0, s>>>(D, P->d_planes, P->T, P->ntx, nper, d_offs,
                                                       d_hist, P->d_recs, d_voffs, d_vhist,
                                                       P->d_order);
    GB_CUDA_TRY(cudaGetLastError());
  }
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GB_OK;
}

}  // namespace gb

using namespace gb;

extern "C" int gb_plan_create(const gb_geometry* geo, int64_t n_vis, const double* d_uvw,
                              int64_t uvw_stride, const int32_t* d_plane, void* stream,
                              gb_plan** out) {
  return gb::plan_create(geo, n_vis, d_uvw, uvw_stride, d_plane, stream, true, out);
}

int gb::plan_create(const gb_geometry* geo, int64_t n_vis, const double* d_uvw,
                    int64_t uvw_stride, const int32_t* d_plane, void* stream, bool own_work,
                    gb_plan** out) {
  if (!out) {
    gb_set_error(GB_ERR_ARG, "gb_plan_create: NULL out");
    return GB_ERR_ARG;
  }
  *out = nullptr;
  if (!geo || n_vis < 0 || n_vis > (int64_t)INT32_MAX || (n_vis > 0 && !d_uvw) ||
      uvw_stride < 3 || geo->n_planes < 1 || geo->n_planes > GB_MAX_PLANES || !geo->supports ||
      !geo->gcf_offsets || geo->ext_x <= 0 || geo->ext_y <= 0 || geo->pitch < geo->ext_x ||
      !(geo->scale == geo->scale)) {
    gb_set_error(GB_ERR_ARG, "gb_plan_create: bad geometry or arguments");
    return GB_ERR_ARG;
  }
  int smax = 0;
  for (int p = 0; p < geo->n_planes; p++) {
    const int S = geo->supports[p];
    if (S < 1 || S > GB_MAX_SUPPORT || geo->gcf_offsets[p] < 0) {
      gb_set_error(GB_ERR_ARG, "gb_plan_create: plane %d support %d / offset out of range", p, S);
      return GB_ERR_ARG;
    }
    smax = std::max(smax, S);
  }
  // defaults: the measured best on the benchmark workloads (tile 24 with
  // 256 threads; pieces up to 40 x 40, so supports up to 40 stay whole and a
  // CTA's accumulators still let four CTAs share an SM)
  const int T = geo->tile ? geo->tile : 24;
  const int NT = geo->threads ? geo->threads : 256;
  const int cap = geo->period_cap ? geo->period_cap : (40 * 40 <= 8 * NT ? 40 : 32);
  const int bpc = geo->bundles_per_cta ? geo->bundles_per_cta : 4;
  if (T < 8 || T > 128 || (NT != 128 && NT != 256 && NT != 512) || cap < 8 || cap > 64 ||
      cap * cap > 8 * NT || bpc < 1 || bpc > 64 || geo->ext_x > 32767 * T ||
      geo->ext_y > 32767 * T) {
    gb_set_error(GB_ERR_ARG, "gb_plan_create: unsupported tuning tile=%d threads=%d cap=%d", T, NT,
                 cap);
    return GB_ERR_ARG;
  }
  int device = 0;
  GB_CUDA_TRY(cudaGetDevice(&device));
  gb_plan* P = new gb_plan();
  P->own_work = own_work;
  P->device = device;
  P->T = T;
  P->NT = NT;
  P->pcap = cap;
  P->bpc = bpc;
  P->n_planes = geo->n_planes;
  P->max_support = smax;
  P->supports.assign(geo->supports, geo->supports + geo->n_planes);
  P->gcf_offsets.assign(geo->gcf_offsets, geo->gcf_offsets + geo->n_planes);
  const int rc = build_plan(P, geo, n_vis, d_uvw, uvw_stride, d_plane, (cudaStream_t)stream);
  if (rc) {
    free_plan(P);
    return rc;
  }
  *out = P;
  return GB_OK;
}

extern "C" int gb_plan_destroy(gb_plan* plan) {
  free_plan(plan);
  return GB_OK;
}

extern "C" int gb_plan_stats(const gb_plan* P, int64_t* st) {
  if (!P || !st) {
    gb_set_error(GB_ERR_ARG, "gb_plan_stats: NULL argument");
    return GB_ERR_ARG;
  }
  st[0] = P->kept;
  st[1] = P->taps;
  st[2] = P->n_items;
  st[3] = P->tiles_used;
  st[4] = P->T;
  st[5] = P->max_support;
  st[6] = P->NT;
  return GB_OK;
}

extern "C" int gb_plan_set_stage(gb_plan* P, int32_t stage) {
  if (!P || stage < GB_STAGE_AUTO || stage > GB_STAGE_ROWS) {
    gb_set_error(GB_ERR_ARG, "gb_plan_set_stage: bad argument");
    return GB_ERR_ARG;
  }
  P->stage_pref = stage;
  return GB_OK;
}

extern "C" int gb_plan_device_status(gb_plan* P, int32_t* out2, void* stream) {
  if (!P || !out2) {
    gb_set_error(GB_ERR_ARG, "gb_plan_device_status: NULL argument");
    return GB_ERR_ARG;
  }
  int32_t err = 0;
  cudaStream_t s = (cudaStream_t)stream;
  GB_CUDA_TRY(cudaMemcpyAsync(&err, P->d_queue + 2, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaMemsetAsync(P->d_queue + 2, 0, sizeof(int32_t), s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  out2[0] = err;
  out2[1] = P->last_stage;
  if (err) {
    gb_set_error(GB_ERR_TIMEOUT, "degridding: a TMA stage did not complete in time");
    return GB_ERR_TIMEOUT;
  }
  return GB_OK;
}

extern "C" int gb_plan_export_index(const gb_plan* P, int32_t* d_out5, void* stream) {
  if (!P || !d_out5) {
    gb_set_error(GB_ERR_ARG, "gb_plan_export_index: NULL argument");
    return GB_ERR_ARG;
  }
  if (P->dev.n_vis == 0) return GB_OK;
  k_plan_export<<<blocks_for(P->dev.n_vis, 256), 256, 0, (cudaStream_t)stream>>>(
      P->dev, P->d_supports, d_out5);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

extern "C" int gb_grid_f64(gb_plan* P, const double* d_vis, const double* d_gcf, double* d_grid,
                           void* stream) {
  if (!P || (P->dev.n_vis && (!d_vis || !d_gcf)) || !d_grid) {
    gb_set_error(GB_ERR_ARG, "gb_grid_f64: NULL argument");
    return GB_ERR_ARG;
  }
  if (P->dev.n_vis == 0) return GB_OK;
  return launch_grid_plain64(P, d_vis, d_gcf, d_grid, (cudaStream_t)stream);
}

extern "C" int gb_degrid_f64(gb_plan* P, const double* d_gcf, const double* d_grid, double* d_pred,
                             int32_t mode, void* stream) {
  if (!P || (P->dev.n_vis && (!d_pred || !d_gcf || !d_grid)) || (mode != 0 && mode != 1)) {
    gb_set_error(GB_ERR_ARG, "gb_degrid_f64: bad argument");
    return GB_ERR_ARG;
  }
  if (P->dev.n_vis == 0) return GB_OK;
  return launch_degrid_plain64(P, d_gcf, d_grid, d_pred, mode, P->df, (cudaStream_t)stream);
}

// The FP64 pair under its forward / backward names (see gb_grid_forward).
extern "C" int gb_grid_forward_f64(gb_plan* P, const double* d_gcf, const double* d_vis,
                                   double* d_grid, void* stream) {
  return gb_grid_f64(P, d_vis, d_gcf, d_grid, stream);
}

extern "C" int gb_grid_backward_f64(gb_plan* P, const double* d_gcf, const double* d_grid_grad,
                                    double* d_vis_grad, void* stream) {
  return gb_degrid_f64(P, d_gcf, d_grid_grad, d_vis_grad, 0, stream);
}

extern "C" int gb_degrid_forward_f64(gb_plan* P, const double* d_gcf, const double* d_grid,
                                     double* d_pred, void* stream) {
  return gb_degrid_f64(P, d_gcf, d_grid, d_pred, 0, stream);
}

extern "C" int gb_degrid_backward_f64(gb_plan* P, const double* d_gcf,
                                      const double* d_pred_grad, double* d_grid_grad,
                                      void* stream) {
  return gb_grid_f64(P, d_pred_grad, d_gcf, d_grid_grad, stream);
}
