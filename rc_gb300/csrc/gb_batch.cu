// Batched gridding / degridding: several grids (channels, facets, data sets
// of different sizes and w-plane sets) in ONE persistent launch.
//
// The reference runs such units as separate DNA actors, each calling the
// kernel once per (tile, w-bin) region (MS6/programs/continuum.hs:134-193,
// MS6/dna/flow/Flow/Halide.hs:309-322).  Here each member gets its own plan
// (index math, sort/bin, items); the batch then merges them: records are
// concatenated, each item keeps its member's grid slot, the thread-group
// class table is the union (by group width, largest period), and bundles are
// rebuilt over all members and ordered longest first, so big and small grids
// share one device work queue without tail effects.  The per-grid pointers
// and geometry travel in a __grid_constant__ kernel parameter block, so a
// batched call is a memset plus one launch and captures into a CUDA graph.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "gb_common.cuh"
#include "gb_plan.cuh"
#include "gb_runtime.cuh"

struct gb_batch {
  std::vector<gb_plan*> members;
  int T = 32, NT = 256;
  int n_classes = 0;
  gb::ClassInfo cls[gb::kMaxClasses] = {};
  size_t smem_grid = 0, smem_degrid = 0;
  int ctas_grid = 1;
  int ctas_degrid[3] = {1, 1, 1};  // per staging form (split and rows are used)
  gb::Rec* d_recs = nullptr;
  gb::Item* d_items = nullptr;
  gb::Bundle* d_bundles = nullptr;
  int32_t* d_queue = nullptr;
  int64_t n_recs = 0;
  int n_items = 0, n_bundles = 0;
  int64_t kept = 0, taps = 0, taps_paired = 0;
  int64_t gcf_len = 0;
  gb::DfScratch df;  // FP64 degridding scratch, shared by the members' launches
};

using namespace gb;

static void free_batch(gb_batch* B) {
  if (!B) return;
  for (gb_plan* p : B->members) gb_plan_destroy(p);
  cudaFree(B->d_recs);
  cudaFree(B->d_items);
  cudaFree(B->d_bundles);
  cudaFree(B->d_queue);
  B->df.release();
  delete B;
}

// The members' plans, built side by side on host threads (each with its own
// stream, ordered after the work already queued on the caller's stream): a
// plan's host part (bins, items) is most of its time.  Returns the first
// member's error, with its message, on the calling thread.
static int build_members(gb_batch* B, int32_t n, const gb_batch_member* m, cudaStream_t s) {
  int dev = 0;
  GB_CUDA_TRY(cudaGetDevice(&dev));
  cudaEvent_t ready;
  GB_CUDA_TRY(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
  const cudaError_t er = cudaEventRecord(ready, s);
  if (er != cudaSuccess) {
    cudaEventDestroy(ready);
    GB_CUDA_TRY(er);
  }
  std::vector<gb_plan*> plans(n, nullptr);
  std::vector<int> rcs(n, GB_OK);
  std::vector<std::string> errs(n);
  std::atomic<int> next{0};
  auto work = [&]() {
    cudaStream_t ws = nullptr;
    const bool ok = cudaSetDevice(dev) == cudaSuccess &&
                    cudaStreamCreateWithFlags(&ws, cudaStreamNonBlocking) == cudaSuccess &&
                    cudaStreamWaitEvent(ws, ready, 0) == cudaSuccess;
    for (int i; (i = next++) < n;) {
      if (!ok) {
        rcs[i] = GB_ERR_CUDA;
        errs[i] = "gb_batch_create: could not set up a worker stream";
        continue;
      }
      rcs[i] = plan_create(&m[i].geo, m[i].n_vis, m[i].d_uvw, m[i].uvw_stride, m[i].d_plane,
                           (void*)ws, false, &plans[i]);
      if (rcs[i]) errs[i] = gb_last_error();
    }
    if (ws) cudaStreamDestroy(ws);
  };
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const int nthreads = (int)std::min<unsigned>({(unsigned)n, hw, 16u});
  std::vector<std::thread> pool;
  for (int t = 1; t < nthreads; t++) pool.emplace_back(work);
  work();
  for (auto& t : pool) t.join();
  cudaEventDestroy(ready);
  int first = -1;
  for (int i = 0; i < n; i++)
    if (rcs[i] && first < 0) first = i;
  if (first >= 0) {
    for (gb_plan* p : plans)
      if (p) gb_plan_destroy(p);
    // errs holds "[code] message": keep the message
    const std::string& e = errs[first];
    const size_t k = e.find("] ");
    gb_set_error(rcs[first], "%s", k == std::string::npos ? e.c_str() : e.c_str() + k + 2);
    return rcs[first];
  }
  B->members = std::move(plans);
  return GB_OK;
}

static int batch_build(gb_batch* B, int32_t n, const gb_batch_member* m, cudaStream_t s) {
  int rc = build_members(B, n, m, s);
  if (rc) return rc;
  for (gb_plan* p : B->members)
    if (p->T != B->members[0]->T || p->NT != B->members[0]->NT) {
      gb_set_error(GB_ERR_ARG, "gb_batch_create: members need the same tile and threads");
      return GB_ERR_ARG;
    }
  B->T = B->members[0]->T;
  B->NT = B->members[0]->NT;
  // union of the thread-group classes, by group width
  std::vector<int> widths;
  for (gb_plan* p : B->members)
    for (int c = 0; c < p->n_classes; c++) widths.push_back(p->cls[c].L);
  std::sort(widths.begin(), widths.end());
  widths.erase(std::unique(widths.begin(), widths.end()), widths.end());
  if ((int)widths.size() > kMaxClasses) {
    gb_set_error(GB_ERR_CAPACITY, "gb_batch_create: too many thread-group classes");
    return GB_ERR_CAPACITY;
  }
  B->n_classes = (int)widths.size();
  for (int c = 0; c < B->n_classes; c++) {
    B->cls[c].L = widths[c];
    B->cls[c].pmax = 0;
  }
  for (gb_plan* p : B->members)
    for (int c = 0; c < p->n_classes; c++) {
      const int u = (int)(std::lower_bound(widths.begin(), widths.end(), p->cls[c].L) -
                          widths.begin());
      B->cls[u].pmax = std::max(B->cls[u].pmax, p->cls[c].pmax);
    }
  const int smem_cap = tiled_max_smem();
  for (int c = 0; c < B->n_classes; c++) {
    ClassInfo& ci = B->cls[c];
    ci.A = B->T + ci.pmax - 1;
    const size_t per_group = group_bytes(ci.A, ci.L);
    int G = B->NT / ci.L;
    while (G > 0 && (size_t)G * per_group > (size_t)smem_cap) G--;
    if (G == 0) {
      gb_set_error(GB_ERR_CAPACITY, "gb_batch_create: tile/period exceed shared memory");
      return GB_ERR_CAPACITY;
    }
    ci.G = G;
  }
  B->smem_grid = tiled_smem_grid(B->cls, B->n_classes, B->NT);
  B->smem_degrid = tiled_smem_degrid(B->cls, B->n_classes, B->NT);
  B->ctas_grid = tiled_ctas_per_sm_for(B->NT, true, B->smem_grid);
  for (int st : {0, 2}) B->ctas_degrid[st] = tiled_ctas_per_sm_for(B->NT, false, B->smem_degrid, st);

  // merged records and items
  std::vector<HostItem> items;
  int64_t off = 0;
  for (int i = 0; i < n; i++) {
    gb_plan* p = B->members[i];
    for (HostItem h : p->host_items) {
      const int u = (int)(std::lower_bound(widths.begin(), widths.end(),
                                           p->cls[item_class(h.it.cls)].L) -
                          widths.begin());
      h.it.cls = (int16_t)((h.it.cls & ~kItemClassMask) | u);
      h.it.start += (int32_t)off;
      h.grid = i;
      items.push_back(h);
    }
    off += p->n_recs;
    B->kept += p->kept;
    B->taps += p->taps;
    B->taps_paired += p->taps_paired;
    B->gcf_len = std::max(B->gcf_len, p->gcf_len);
  }
  B->n_recs = off;
  if (B->n_recs >= (int64_t)INT32_MAX) {
    gb_set_error(GB_ERR_CAPACITY, "gb_batch_create: more than 2^31 footprint pieces");
    return GB_ERR_CAPACITY;
  }
  std::vector<Item> it_out;
  std::vector<Bundle> b_out;
  make_bundles(items, B->cls, B->n_classes, it_out, b_out);
  B->n_items = (int)it_out.size();
  B->n_bundles = (int)b_out.size();
  if ((rc = dev_alloc((void**)&B->d_recs, sizeof(Rec) * (B->n_recs ? B->n_recs : 1), "batch")) ||
      (rc = dev_alloc((void**)&B->d_items, sizeof(Item) * (B->n_items ? B->n_items : 1),
                      "batch")) ||
      (rc = dev_alloc((void**)&B->d_bundles,
                      sizeof(Bundle) * (B->n_bundles ? B->n_bundles : 1), "batch")) ||
      (rc = dev_alloc((void**)&B->d_queue, sizeof(int32_t) * 2, "batch")))
    return rc;
  off = 0;
  for (gb_plan* p : B->members) {
    if (p->n_recs)
      GB_CUDA_TRY(cudaMemcpyAsync(B->d_recs + off, p->d_recs, sizeof(Rec) * p->n_recs,
                                  cudaMemcpyDeviceToDevice, s));
    off += p->n_recs;
  }
  if (B->n_items)
    GB_CUDA_TRY(cudaMemcpyAsync(B->d_items, it_out.data(), sizeof(Item) * B->n_items,
                                cudaMemcpyHostToDevice, s));
  if (B->n_bundles)
    GB_CUDA_TRY(cudaMemcpyAsync(B->d_bundles, b_out.data(), sizeof(Bundle) * B->n_bundles,
                                cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  // the members' own piece tables are merged now: release them
  for (gb_plan* p : B->members) {
    cudaFree(p->d_recs);
    p->d_recs = nullptr;
    p->n_bundles = 0;  // a member can no longer run on its own FP32 tables
  }
  return GB_OK;
}

extern "C" int gb_batch_create(int32_t n_members, const gb_batch_member* members, void* stream,
                               gb_batch** out) {
  if (!out || !members || n_members < 1 || n_members > kMaxGrids) {
    gb_set_error(GB_ERR_ARG, "gb_batch_create: 1..%d members required", kMaxGrids);
    return GB_ERR_ARG;
  }
  *out = nullptr;
  gb_batch* B = new gb_batch();
  const int rc = batch_build(B, n_members, members, (cudaStream_t)stream);
  if (rc) {
    free_batch(B);
    return rc;
  }
  *out = B;
  return GB_OK;
}

extern "C" int gb_batch_destroy(gb_batch* B) {
  free_batch(B);
  return GB_OK;
}

extern "C" int gb_batch_stats(const gb_batch* B, int64_t* st) {
  if (!B || !st) {
    gb_set_error(GB_ERR_ARG, "gb_batch_stats: NULL argument");
    return GB_ERR_ARG;
  }
  st[0] = B->kept;
  st[1] = B->taps;
  st[2] = B->n_items;
  st[3] = B->n_bundles;
  st[4] = B->T;
  st[5] = (int64_t)B->members.size();
  st[6] = B->NT;
  return GB_OK;
}

static int fill_slots(const gb_batch* B, float* const* grids, float* const* vis, GridPtrs* gp,
                      const char* who) {
  memset(gp, 0, sizeof(*gp));
  for (size_t i = 0; i < B->members.size(); i++) {
    const gb_plan* p = B->members[i];
    if (!grids[i] || (p->dev.n_vis > 0 && !vis[i])) {
      gb_set_error(GB_ERR_ARG, "%s: NULL pointer for member %zu", who, i);
      return GB_ERR_ARG;
    }
    gp->s[i].grid = (float2*)grids[i];
    gp->s[i].vis = (float2*)vis[i];
    gp->s[i].pitch = p->dev.pitch;
    gp->s[i].ext_x = p->dev.ext_x;
    gp->s[i].ext_y = p->dev.ext_y;
#ifdef GB_CHECKED
    gp->s[i].n_vis = p->dev.n_vis;
#endif
  }
  return GB_OK;
}

extern "C" int gb_batch_grid_f32(gb_batch* B, const float* const* d_vis, const float* d_gcf,
                                 float* const* d_grids, void* stream) {
  if (!B || !d_vis || !d_grids || (B->n_recs && !d_gcf)) {
    gb_set_error(GB_ERR_ARG, "gb_batch_grid_f32: NULL argument");
    return GB_ERR_ARG;
  }
  GridPtrs gp;
  int rc = fill_slots(B, d_grids, (float* const*)d_vis, &gp, "gb_batch_grid_f32");
  if (rc) return rc;
  return launch_tiled_batch(true, 0, B->NT, B->smem_grid, B->ctas_grid, B->d_bundles,
                            B->n_bundles, B->d_items, B->d_recs, B->d_queue, B->cls,
                            B->n_classes, B->T, gp, d_gcf, 0,
                            TiledBounds{B->n_recs, B->gcf_len, 0}, (cudaStream_t)stream);
}

extern "C" int gb_batch_degrid_f32(gb_batch* B, const float* d_gcf, const float* const* d_grids,
                                   float* const* d_preds, int32_t mode, void* stream) {
  if (!B || !d_grids || !d_preds || (B->n_recs && !d_gcf) || (mode != 0 && mode != 1)) {
    gb_set_error(GB_ERR_ARG, "gb_batch_degrid_f32: bad argument");
    return GB_ERR_ARG;
  }
  GridPtrs gp;
  int rc = fill_slots(B, (float* const*)d_grids, d_preds, &gp, "gb_batch_degrid_f32");
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  for (size_t i = 0; i < B->members.size(); i++)
    if (B->members[i]->dev.n_vis)
      GB_CUDA_TRY(cudaMemsetAsync(d_preds[i], 0, sizeof(float2) * B->members[i]->dev.n_vis, s));
  // several grids: no TMA; split rows when most taps are paired
  const int stage = degrid_stage_choice(-1, B->taps, B->taps_paired, d_gcf, false);
  return launch_tiled_batch(false, mode, B->NT, B->smem_degrid, B->ctas_degrid[stage], B->d_bundles,
                            B->n_bundles, B->d_items, B->d_recs, B->d_queue, B->cls,
                            B->n_classes, B->T, gp, d_gcf, stage,
                            TiledBounds{B->n_recs, B->gcf_len, 0}, s);
}

// Plain FP64 path over the members (one launch each): the comparison path of
// the batched workload.
extern "C" int gb_batch_grid_f64(gb_batch* B, const double* const* d_vis, const double* d_gcf,
                                 double* const* d_grids, void* stream) {
  if (!B || !d_vis || !d_grids || !d_gcf) {
    gb_set_error(GB_ERR_ARG, "gb_batch_grid_f64: NULL argument");
    return GB_ERR_ARG;
  }
  for (size_t i = 0; i < B->members.size(); i++) {
    if (!B->members[i]->dev.n_vis) continue;
    if (!d_vis[i] || !d_grids[i]) {
      gb_set_error(GB_ERR_ARG, "gb_batch_grid_f64: NULL pointer for member %zu", i);
      return GB_ERR_ARG;
    }
    const int rc = launch_grid_plain64(B->members[i], d_vis[i], d_gcf, d_grids[i],
                                       (cudaStream_t)stream);
    if (rc) return rc;
  }
  return GB_OK;
}

extern "C" int gb_batch_degrid_f64(gb_batch* B, const double* d_gcf, const double* const* d_grids,
                                   double* const* d_preds, int32_t mode, void* stream) {
  if (!B || !d_grids || !d_preds || !d_gcf || (mode != 0 && mode != 1)) {
    gb_set_error(GB_ERR_ARG, "gb_batch_degrid_f64: bad argument");
    return GB_ERR_ARG;
  }
  // the scratch at the largest member's size first: the members' launches
  // then reuse it in stream order without reallocating under a running kernel
  int64_t cells = 0;
  for (const gb_plan* p : B->members) cells = std::max(cells, (int64_t)p->dev.ext_x * p->dev.ext_y);
  int rc0;
  if ((rc0 = df_reserve(B->df, cells, B->gcf_len))) return rc0;
  for (size_t i = 0; i < B->members.size(); i++) {
    if (!B->members[i]->dev.n_vis) continue;
    if (!d_grids[i] || !d_preds[i]) {
      gb_set_error(GB_ERR_ARG, "gb_batch_degrid_f64: NULL pointer for member %zu", i);
      return GB_ERR_ARG;
    }
    const int rc = launch_degrid_plain64(B->members[i], d_gcf, d_grids[i], d_preds[i], mode,
                                         B->df, (cudaStream_t)stream);
    if (rc) return rc;
  }
  return GB_OK;
}
