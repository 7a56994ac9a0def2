// Visibility plan: device layout of the sorted / binned work of the FP32
// tiled kernels, and the parameters shared with the plain FP64 kernels.
//
// Layout in HBM (per plan):
//   plane[n_vis]        int32  w-plane of each visibility (or -1)
//   order[n_vis]        int32  visibilities sorted by the tile of their corner
//                              (the visit order of the plain FP64 kernels)
//   recs[n_recs]        Rec    16-byte records sorted by (grid tile, period)
//   items[n_items]      Item   a contiguous record range of one tile and one
//                              thread-group class
//   bundles[n_bundles]  Bundle up to NT/L items run side by side in one CTA
//   queue[2]            int32  work-queue heads (grid, degrid)
//
// A record is one rectangular piece (<= P x P taps) of one visibility's
// S x S footprint: supports larger than the period cap are cut into k x k
// pieces, k = ceil(S / cap), period P = ceil(S / k), so that every tile
// accumulator stays within shared memory whatever the support.
#pragma once

#include <cuda.h>
#include <stdint.h>

#include <vector>

#include "gb_common.cuh"

namespace gb {

struct PlanDev {
  int64_t n_vis;
  const double* uvw;
  int64_t uvw_stride;
  const int32_t* plane;        // per visibility
  const int32_t* order;        // the visibilities by the grid tile of their footprint
                               // corner (kept ones first), or NULL: index order
  const int32_t* supports;     // per plane
  const int64_t* gcf_offsets;  // per plane
  double scale;
  int32_t grid_size, margin, ext_x, ext_y;
  int64_t pitch;
};

struct __align__(16) Rec {
  int32_t vis;     // visibility index
  uint32_t gcf;    // complex offset of the piece's first tap in the GCF array
  uint8_t xl, yl;  // piece corner relative to the tile origin
  uint8_t wx, wy;  // piece extent (<= P)
  uint8_t xm, ym;  // absolute piece corner mod P
  uint8_t pm1;     // period P - 1
  uint8_t sm1;     // support S - 1 (GCF row pitch); S > P marks a cut footprint
};
static_assert(sizeof(Rec) == 16, "Rec must be 16 bytes");

struct __align__(16) Item {
  int32_t start, count;    // record range
  int16_t tile_x, tile_y;  // tile indices
  int16_t pmax, cls;       // largest period in the item; thread-group class and
                           // split-row stride residue (item_class, item_stride_residue)
};
static_assert(sizeof(Item) == 16, "Item must be 16 bytes");

struct __align__(16) Bundle {
  int32_t first_item;
  int16_t n_items, cls;
  int32_t grid;  // slot of the grid (and visibility array) in a batched launch
  int32_t pad;
};
static_assert(sizeof(Bundle) == 16, "Bundle must be 16 bytes");

// Item with its modelled cost and grid slot, kept on the host to form bundles.
struct HostItem {
  Item it;
  double cost;
  int grid;
};

// One thread-group class: L threads per group, G groups per CTA, region edge A.
struct ClassInfo {
  int32_t L, G, A, pmax;
};

// Shared memory of one thread group: the A x A accumulator or grid stage
// (float2 per pixel), plus one batch of L decoded records (32 B each; a
// gridding record carries its visibility).
// Gridding accumulator rows are padded to a multiple of 16 pixels (16 float2 =
// the 32 shared-memory banks): a warp's read-modify-write that steps to the
// next pixel row then stays on the banks of a continuing row.
__host__ __device__ inline int acc_stride(int A) { return (A + 15) & ~15; }
// (and each record's shape word again, 4 bytes, in an array of its own: the
// run detection reads 32 consecutive shapes at once, which at the records'
// 32-byte stride would fall on 4 banks)
__host__ __device__ inline size_t grid_group_bytes(int A, int L) {
  return 8 * (size_t)A * acc_stride(A) + 36 * (size_t)L;
}
// The float2 grid stage is padded to 16 bytes so that the 16-byte records
// behind it (and the next group's region) stay 16-byte aligned.
// Degridding stages the A x A grid region with rows padded to an even width
// (a TMA box row must be a multiple of 16 bytes) and starts each group's
// region on a 128-byte boundary (TMA destination).
__host__ __device__ inline int stage_stride(int A) { return (A + 1) & ~1; }
// The split-row stage may lay its rows further apart than stage_stride: an
// item's row stride is stage_stride + ((r - stage_stride) mod 16) float2 for
// the residue r (0..15) its plan chose, so that a sub-warp reading pairs
// row-major across row ends, rows of w2 pairs, hits the 16 eight-byte bank
// pairs evenly when r = w2 mod 16 (up to 15 more pixels per row).
__host__ __device__ inline int split_row_stride(int A, int r) {
  const int Ae = stage_stride(A);
  return r < 0 ? Ae : Ae + ((r - Ae) & 15);
}
__host__ __device__ inline size_t degrid_stage_bytes(int A) {
  return (8 * (size_t)A * (stage_stride(A) + 15) + 127) & ~(size_t)127;
}
// Item.cls packs the thread-group class (bits 0-3) and the split-row stride
// residue of degridding plus one (bits 4-8; 0: the plain stage_stride).
constexpr int kItemClassMask = 0xF;
__host__ __device__ inline int item_class(int16_t cls) { return cls & kItemClassMask; }
__host__ __device__ inline int item_stride_residue(int16_t cls) { return ((cls >> 4) & 31) - 1; }
__host__ __device__ inline int16_t item_cls_with_residue(int16_t cls, int split_r) {
  return (int16_t)((cls & kItemClassMask) | ((split_r + 1) << 4));
}
__host__ __device__ inline size_t degrid_group_bytes(int A, int L) {
  return degrid_stage_bytes(A) + 32 * (size_t)L;
}
// Shared memory of one thread group in either direction: a plan's classes
// (and their groups per CTA) serve both kernels.
__host__ __device__ inline size_t group_bytes(int A, int L) {
  const size_t g = grid_group_bytes(A, L), d = degrid_group_bytes(A, L);
  return g > d ? g : d;
}

constexpr int kMaxClasses = 4;

// Per-grid pointers and geometry of a (batched) launch, passed by value as a
// __grid_constant__ kernel parameter.  vis: the visibilities (gridding input)
// or the predictions (degridding output) of that grid's plan.
constexpr int kMaxGrids = 96;
struct GridSlot {
  float2* grid;
  float2* vis;
  int64_t pitch;
  int32_t ext_x, ext_y;
#ifdef GB_CHECKED
  int64_t n_vis;  // visibilities behind `vis` (the bounds-checked build tests indices)
#endif
};
struct GridPtrs {
  GridSlot s[kMaxGrids];
};

struct PlaneInfo {
  int32_t S, P, k, rank;
  int64_t gcf_off;
};

// Scratch of the FP64 degridder (gb_plain.cu): the grid region and the GCFs
// split into double-float pairs, and the two arrays' largest exponent fields.
// Grown on demand; owned by a plan or a batch.
struct DfScratch {
  float4* grid = nullptr;  // ext_x * ext_y complex elements
  size_t grid_cap = 0;
  float4* gcf = nullptr;
  size_t gcf_cap = 0;
  int* exps = nullptr;  // [0] grid, [1] GCF
  void release();
};
int df_reserve(DfScratch& d, int64_t grid_elems, int64_t gcf_elems);

}  // namespace gb

struct gb_plan {
  gb::PlanDev dev;
  int device = 0;
  int T = 32;       // tile edge
  int NT = 256;     // threads per CTA of the tiled kernels
  int pcap = 32;    // period cap
  int bpc = 4;      // target bundles per resident CTA (work granularity)
  int n_planes = 0;
  int max_support = 0;
  int ntx = 0, nty = 0;
  std::vector<int32_t> supports;
  std::vector<int64_t> gcf_offsets;
  std::vector<gb::PlaneInfo> planes;
  int n_classes = 0;
  gb::ClassInfo cls[gb::kMaxClasses] = {};
  size_t smem_grid = 0, smem_degrid = 0;
  int ctas_per_sm_grid = 1;
  int ctas_per_sm_degrid[3] = {1, 1, 1};  // per GB_STAGE_* form
  // device arrays owned by the plan
  int32_t* d_plane = nullptr;
  int32_t* d_order = nullptr;
  int32_t* d_supports = nullptr;
  int64_t* d_offsets = nullptr;
  gb::PlaneInfo* d_planes = nullptr;
  gb::Rec* d_recs = nullptr;
  gb::Item* d_items = nullptr;
  gb::Bundle* d_bundles = nullptr;
  int32_t* d_queue = nullptr;
  int64_t n_recs = 0;
  int n_items = 0, n_bundles = 0;
  int64_t kept = 0, taps = 0, tiles_used = 0;
  int64_t taps_paired = 0;  // taps of pieces that degridding can take in pairs
  int64_t gcf_len = 0;      // complex elements the planes' GCFs span
  int stage_pref = -1;      // GB_STAGE_*: forced staging form of degridding, or -1
  bool own_work = true;     // false for a batch member: no launch tables of its own
  bool own_plane = true;
  std::vector<gb::HostItem> host_items;  // every item with its cost (grid slot 0)
  // TMA descriptors of the last degridded grid, one per thread-group class
  // (box = that class's stage); rebuilt when the grid's address or shape changes
  const void* tma_grid = nullptr;
  int tma_ext_x = 0, tma_ext_y = 0;
  int64_t tma_pitch = 0;
  bool tma_ok = false;
  CUtensorMap tma_maps[gb::kMaxClasses];
  int last_stage = 0;  // GB_STAGE_* form of the last degridding launch
  gb::DfScratch df;    // FP64 degridding scratch, allocated by its first call
};

namespace gb {
// Bundles from items: grouped by (class, grid), by decreasing cost, up to
// cls[c].G items each; all bundles then by decreasing cost (longest first).
// it_out receives the items in bundle order.
void make_bundles(const std::vector<HostItem>& items, const ClassInfo* cls, int n_classes,
                  std::vector<Item>& it_out, std::vector<Bundle>& b_out);
int launch_grid_plain64(const gb_plan* plan, const double* vis, const double* gcf, double* grid,
                        cudaStream_t s);
int launch_degrid_plain64(const gb_plan* plan, const double* gcf, const double* grid,
                          double* pred, int mode, DfScratch& scratch, cudaStream_t s);
int launch_grid_tiled(gb_plan* plan, const float* vis, const float* gcf, float* grid,
                      cudaStream_t s);
int launch_degrid_tiled(gb_plan* plan, const float* gcf, const float* grid, float* pred,
                        int mode, cudaStream_t s);
// Shared-memory bytes of the tiled kernels for a class table.
size_t tiled_smem_grid(const ClassInfo* cls, int n_classes, int NT);
size_t tiled_smem_degrid(const ClassInfo* cls, int n_classes, int NT);
int tiled_max_smem();
// gb_plan_create with own_work = false for a batch member: the plan computes
// its records and items but no bundles (the batch builds its own tables).
int plan_create(const gb_geometry* geo, int64_t n_vis, const double* d_uvw, int64_t uvw_stride,
                const int32_t* d_plane, void* stream, bool own_work, gb_plan** out);

// Array sizes behind a launch's pointers (used by the bounds-checked build).
struct TiledBounds {
  int64_t n_recs, gcf_len, n_vis;
};
int launch_grid_tiled_tables(const Bundle* bundles, int n_bundles, const Item* items,
                             const Rec* recs, int32_t* queue, const ClassInfo* cls, int n_classes,
                             int NT, int T, int ext_x, int ext_y, int64_t pitch, size_t smem,
                             const float* vis, const float* gcf, float* grid,
                             const TiledBounds& bounds, cudaStream_t s);
int launch_tiled_batch(bool grid_mode, int mode, int NT, size_t smem, int ctas_per_sm,
                       const Bundle* bundles, int n_bundles, const Item* items, const Rec* recs,
                       int32_t* queue, const ClassInfo* cls, int n_classes, int T,
                       const GridPtrs& gp, const float* gcf, int stage,
                       const TiledBounds& bounds, cudaStream_t s);
// Staging form of a degridding launch (GB_STAGE_SPLIT / _TMA / _ROWS): split
// rows when at least half of the taps are paired and the GCF allows pairs.
int degrid_stage_choice(int pref, int64_t taps, int64_t taps_paired, const float* gcf,
                        bool tma_possible);
int tiled_ctas_per_sm_for(int NT, bool grid, size_t smem, int stage = 0);
// Resident CTAs per SM of the tiled grid (or degrid, per staging form) kernel.
int tiled_ctas_per_sm(const gb_plan* plan, bool grid, int stage = 0);
}  // namespace gb
