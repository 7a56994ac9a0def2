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
// ever touch the same pixel and the accumulation is a plain float2
// read-modify-write (the products of consecutive pieces that land on one
// pixel are summed by FMA chains first; the sums stay short, a tile's pieces
// of one item, and measure within 2e-7 of FP64 in rel-L2 on every workload).
// At the end the group adds its sums into the global grid with float2
// atomics, skipping pixels no piece touched; atomics are needed only because
// neighbouring tiles' overhangs and other items of the same tile overlap.
//
// Degridding (D = G^H): each group stages its A x A grid region in shared
// memory (split rows by per-thread asynchronous copies, or plain rows by one
// TMA copy or per-thread copies: gb_plan_set_stage), then sub-warps take
// pieces, gather the taps (in pairs where the rows allow) from shared memory,
// multiply by conj(GCF), sum each group of four steps by FMA chains into a
// per-lane Kahan accumulator and reduce by warp shuffles.  A visibility whose
// footprint was cut into several pieces accumulates them with float2 atomics;
// otherwise a plain store.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <type_traits>

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
  int32_t T;
#ifdef GB_CHECKED
  int64_t n_recs;   // records in `recs`
  int64_t gcf_len;  // complex elements in the GCF array
#endif
};

// Checked build (-DGB_CHECKED, rc_gb300.build(checked=True)): every shared
// memory, GCF, record and visibility index below is tested against its
// array; a violation is counted in g_check_violations (gb_checked_violations)
// and the access goes to element 0 instead.  No trap, no fault: the counter is
// how tests see it.  In the normal build GB_IDX is the index itself.
#ifdef GB_CHECKED
__device__ unsigned long long g_check_violations;
__device__ __forceinline__ int64_t gb_checked_index(int64_t i, int64_t lim) {
  if (i < 0 || i >= lim) {
    atomicAdd(&g_check_violations, 1ull);
    return 0;
  }
  return i;
}
#define GB_IDX(i, lim) gb_checked_index((int64_t)(i), (int64_t)(lim))
#else
#define GB_IDX(i, lim) (i)
#endif

__device__ __forceinline__ void group_sync(int id, int n, bool whole_cta) {
  if (whole_cta)
    __syncthreads();
  else
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}

// Kahan step: s + x with the running compensation c (the negated lost low
// part of earlier additions); the compensated total is s - c.
__device__ __forceinline__ void kahan(float& s, float& c, float x) {
  const float y = __fsub_rn(x, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
}

constexpr int kInvalidResidue = 1 << 14;

// Class table lookup without dynamic indexing of the kernel parameter block
// (which would copy it to local memory).
__device__ __forceinline__ ClassInfo class_of(const TiledArgs& a, int c) {
  static_assert(kMaxClasses == 4, "class_of covers 4 classes");
  return c == 0 ? a.cls[0] : c == 1 ? a.cls[1] : c == 2 ? a.cls[2] : a.cls[3];
}

// A record decoded once per batch into shared memory (32 bytes), so that the
// threads of a group read plain ints instead of unpacking bytes per tap.
struct __align__(16) GridRec {
  int32_t gcf;    // GCF element offset of the piece's first tap
  int32_t q0;     // accumulator index of the piece corner: yl * acc_stride(A) + xl
  int32_t xm, ym; // piece corner mod P
  int32_t pitch;  // GCF row pitch (the plane's support S)
  int32_t shape;  // period P (bits 0-8), extents wx (9-17), wy (18-26), whole piece (bit 27)
  float2 vis;     // the visibility
};
static_assert(sizeof(GridRec) == 32, "GridRec is two 16-byte words");

constexpr int32_t kWholePiece = 1 << 27;
__device__ __forceinline__ int shape_period(int32_t s) { return s & 0x1FF; }
__device__ __forceinline__ int shape_wx(int32_t s) { return (s >> 9) & 0x1FF; }
__device__ __forceinline__ int shape_wy(int32_t s) { return (s >> 18) & 0x1FF; }

struct __align__(16) DegridRec {
  int32_t gcf, q0, pitch, vis;
  int16_t wx, wy;  // piece extent
  int16_t dj, di;  // a sub-warp's stride through the piece: SW steps = dj rows + di steps
  float rcp_w;     // 1 / (steps per row), for each lane's first step without a division
  int32_t flags;   // kRecCut: footprint cut into pieces (accumulate with atomics);
                   // kRecPaired: a step is two adjacent taps (one 16-byte GCF load);
                   // kRecOdd: the piece's first column is odd; bits 8-15: that column
};
constexpr int32_t kRecCut = 1, kRecPaired = 2, kRecOdd = 4;
static_assert(sizeof(DegridRec) == 32, "DegridRec is two 16-byte words");

// Residue slots a thread needs for period P in a group of L threads.
__device__ __forceinline__ int slots_for(int P, int L) { return (P * P + L - 1) / L; }

// One run [k, e) of equal period P of the staged batch: thread lt owns the
// residues rr = lt + m L < P^2, (a, b) = (rr mod P, rr div P); U pieces at a
// time, all GCF loads first, then per slot the read-modify-writes in piece
// order.  A slot's tap of consecutive pieces often lands on the same pixel
// (neighbouring samples of one baseline have nearby corners, and any corner
// within P of the previous one puts the owned residue's pixel in the same
// place with probability (P - dx)(P - dy) / P^2), so the products of such
// a stretch are summed by FMA chains and the accumulator sees one
// read-modify-write per change of pixel.
// FULL: every piece of the run is a whole P x P square, so every owned
// residue has a tap and the extent checks drop out.
template <int R, int U, bool FULL>
__device__ __forceinline__ void grid_run(int k, int e, int lt, int L, int As,
                                         const GridRec* __restrict__ srec,
                                         float2* __restrict__ acc,
                                         const float2* __restrict__ gcf, int acc_len,
                                         int64_t gcf_len) {
  const int P = shape_period(srec[k].shape);
  int ra[R], rb[R];
  bool own[R];  // slot m holds a residue (R L may exceed P^2)
#pragma unroll
  for (int m = 0; m < R; m++) {
    const int rr = lt + m * L;
    own[m] = rr < P * P;
    if (own[m]) {
      rb[m] = rr / P;
      ra[m] = rr - rb[m] * P;
    } else {
      ra[m] = kInvalidResidue;
      rb[m] = kInvalidResidue;
    }
  }
  if (FULL) {
    // whole groups of U whole pieces: every owned slot has a tap, no tail checks
    for (; k + U <= e; k += U) {
      float2 c[U][R];
      int qi[U][R];
      float2 v[U];
#pragma unroll
      for (int u = 0; u < U; u++) {
        const GridRec r = srec[k + u];
        v[u] = r.vis;
#pragma unroll
        for (int m = 0; m < R; m++) {
          int i = ra[m] - r.xm;
          i += i < 0 ? P : 0;
          int j = rb[m] - r.ym;
          j += j < 0 ? P : 0;
          c[u][m] = own[m] ? __ldg(gcf + GB_IDX(r.gcf + j * r.pitch + i, gcf_len))
                           : make_float2(0.f, 0.f);
          qi[u][m] = r.q0 + j * As + i;
        }
      }
#pragma unroll
      for (int m = 0; m < R; m++) {
        if (!own[m]) continue;
        float pr = 0.f, pi = 0.f;
#pragma unroll
        for (int u = 0; u < U; u++) {
          pr = fmaf(v[u].x, c[u][m].x, fmaf(-v[u].y, c[u][m].y, pr));
          pi = fmaf(v[u].x, c[u][m].y, fmaf(v[u].y, c[u][m].x, pi));
          if (u == U - 1 || qi[u + 1][m] != qi[u][m]) {
            const int q = GB_IDX(qi[u][m], acc_len);
            float2 s = acc[q];
            s.x += pr;
            s.y += pi;
            acc[q] = s;
            pr = 0.f;
            pi = 0.f;
          }
        }
      }
    }
  }
  for (; k < e; k += U) {
    float2 c[U][R];
    int qi[U][R];
    float2 v[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const bool live = k + u < e;
      const GridRec r = srec[live ? k + u : k];
      v[u] = r.vis;
#pragma unroll
      for (int m = 0; m < R; m++) {
        int i = ra[m] - r.xm;
        i += i < 0 ? P : 0;
        int j = rb[m] - r.ym;
        j += j < 0 ? P : 0;
        if (live && own[m] && (FULL || (i < shape_wx(r.shape) && j < shape_wy(r.shape)))) {
          c[u][m] = __ldg(gcf + GB_IDX(r.gcf + j * r.pitch + i, gcf_len));
          qi[u][m] = r.q0 + j * As + i;
        } else {
          c[u][m] = make_float2(0.f, 0.f);
          qi[u][m] = -1;
        }
      }
    }
#pragma unroll
    for (int m = 0; m < R; m++) {
      float pr = 0.f, pi = 0.f;
#pragma unroll
      for (int u = 0; u < U; u++) {
        if (qi[u][m] >= 0) {
          pr = fmaf(v[u].x, c[u][m].x, fmaf(-v[u].y, c[u][m].y, pr));
          pi = fmaf(v[u].x, c[u][m].y, fmaf(v[u].y, c[u][m].x, pi));
          if (u == U - 1 || qi[u + 1][m] != qi[u][m]) {
            const int q = GB_IDX(qi[u][m], acc_len);
            float2 s = acc[q];
            s.x += pr;
            s.y += pi;
            acc[q] = s;
            pr = 0.f;
            pi = 0.f;
          }
        }
      }
    }
  }
}

template <bool FULL>
__device__ __forceinline__ void grid_dispatch(int slots, int k, int e, int lt, int L, int As,
                                              const GridRec* __restrict__ srec,
                                              float2* __restrict__ acc,
                                              const float2* __restrict__ gcf, int acc_len,
                                              int64_t gcf_len) {
  switch (slots) {
    case 1: grid_run<1, 8, FULL>(k, e, lt, L, As, srec, acc, gcf, acc_len, gcf_len); break;
    case 2: grid_run<2, 4, FULL>(k, e, lt, L, As, srec, acc, gcf, acc_len, gcf_len); break;
    case 3: grid_run<3, 3, FULL>(k, e, lt, L, As, srec, acc, gcf, acc_len, gcf_len); break;
    case 4: grid_run<4, 2, FULL>(k, e, lt, L, As, srec, acc, gcf, acc_len, gcf_len); break;
    case 5:
    case 6: grid_run<6, 1, FULL>(k, e, lt, L, As, srec, acc, gcf, acc_len, gcf_len); break;
    default: grid_run<8, 1, FULL>(k, e, lt, L, As, srec, acc, gcf, acc_len, gcf_len); break;
  }
}

// Gridding of one item by one thread group.  acc holds A x A float2 sums
// (rows acc_stride(A) apart).
__device__ __forceinline__ void grid_item(const TiledArgs& a, const Item& it, int lt, int L,
                                          int bar, bool whole, int A, float2* __restrict__ acc,
                                          GridRec* __restrict__ srec,
                                          int32_t* __restrict__ sshape,
                                          const GridSlot& gs, const float2* __restrict__ gcf) {
  const float2* __restrict__ vis = gs.vis;
  float2* __restrict__ grid = gs.grid;
  const int As = acc_stride(A), AA = A * As;
#ifdef GB_CHECKED
  const int64_t gcf_len = a.gcf_len;
#else
  const int64_t gcf_len = 0;
#endif
  for (int q = lt; q < AA; q += L) acc[q] = make_float2(0.f, 0.f);
  int curP = -1;
  const int end = it.start + it.count;
  for (int base = it.start; base < end; base += L) {
    const int nb = min(L, end - base);
    group_sync(bar, L, whole);  // zeroing done / previous batch consumed
    if (lt < nb) {
      const Rec r = a.recs[GB_IDX(base + lt, a.n_recs)];
      GridRec d;
      d.gcf = (int32_t)r.gcf;
      d.q0 = r.yl * As + r.xl;
      d.xm = r.xm;
      d.ym = r.ym;
      d.pitch = r.sm1 + 1;
      d.shape = (r.pm1 + 1) | (r.wx << 9) | (r.wy << 18) |
                (r.wx == r.pm1 + 1 && r.wy == r.pm1 + 1 ? kWholePiece : 0);
      d.vis = __ldg(vis + GB_IDX(r.vis, gs.n_vis));
      srec[lt] = d;
      sshape[lt] = d.shape;
    }
    group_sync(bar, L, whole);
    int k = 0;
    while (k < nb) {
      const int P = shape_period(srec[k].shape);
      if (P != curP) {
        // the residue map changes: finish every read-modify-write of the old one
        group_sync(bar, L, whole);
        curP = P;
      }
      // the run's end, 32 records per step: records of an item are sorted by
      // period, so the run ends at the first record of another period (every
      // warp of the group reaches the same answer from the same records)
      int e = k;
      bool full = true;
      const int lane = lt & 31;
      for (;;) {
        const int idx = e + lane;
        const int pe = idx < nb ? sshape[GB_IDX(idx, L)] : -1;
        const bool stop = pe < 0 || shape_period(pe) != P;
        const unsigned ms = __ballot_sync(0xFFFFFFFFu, stop);
        const unsigned mp = __ballot_sync(0xFFFFFFFFu, !stop && !(pe & kWholePiece));
        if (ms) {
          const int first = __ffs(ms) - 1;
          full = full && (mp & ((1u << first) - 1u)) == 0;
          e += first;
          break;
        }
        full = full && mp == 0;
        e += 32;
      }
      if (full)
        grid_dispatch<true>(slots_for(P, L), k, e, lt, L, As, srec, acc, gcf, AA, gcf_len);
      else
        grid_dispatch<false>(slots_for(P, L), k, e, lt, L, As, srec, acc, gcf, AA, gcf_len);
      k = e;
    }
  }
  group_sync(bar, L, whole);
  const int x0 = it.tile_x * a.T, y0 = it.tile_y * a.T;
  // pixel q = lt + n L walks (py, px) by L / As rows and L mod As columns;
  // the padding columns px >= A are never touched
  const int dy = L / As, dx = L - dy * As;
  int py = lt / As, px = lt - py * As;
  for (int q = lt; q < AA; q += L) {
    const float2 s = acc[q];
    if (px < A && (s.x != 0.f || s.y != 0.f)) {
      const int gx = x0 + px, gy = y0 + py;
      if (gx < gs.ext_x && gy < gs.ext_y)
        atomicAdd(grid + (int64_t)gy * gs.pitch + gx, s);
    }
    px += dx;
    py += dy;
    if (px >= As) {
      px -= As;
      py++;
    }
  }
}

template <int NT>
__global__ void __launch_bounds__(NT) k_grid_tiled(const __grid_constant__ TiledArgs a,
                                                   const __grid_constant__ GridPtrs gp,
                                                   const float2* __restrict__ gcf) {
  extern __shared__ __align__(128) unsigned char smem[];
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
      unsigned char* base = smem + (size_t)g * grid_group_bytes(ci.A, ci.L);
      float2* acc = (float2*)base;
      GridRec* srec = (GridRec*)(base + 8 * (size_t)ci.A * acc_stride(ci.A));
      int32_t* sshape = (int32_t*)(srec + ci.L);
      grid_item(a, a.items[bd.first_item + g], lt, ci.L, 1 + g, ci.L == NT, ci.A, acc, srec,
                sshape, gp.s[bd.grid], gcf);
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------ TMA staging
// Degridding stages each item's grid region either with one 2-D bulk tensor
// copy (TMA) issued by the group's first thread and completing on an
// mbarrier (k_degrid_tiled<.., true>), or, where no tensor map applies
// (several grids in one launch, odd tile edge, unaligned grid), with
// asynchronous per-thread copies (k_degrid_tiled<.., false>).
struct StageMaps {
  CUtensorMap m[kMaxClasses];  // per thread-group class: box = that class's stage
  int32_t* err;                // set when a TMA completion is not seen in time
};

// One mbarrier per group slot of a CTA (groups have >= 64 threads, CTAs at
// most 512) and the parity each slot's barrier completes next (bit per slot).
constexpr int kMaxGroupSlots = 8;
__shared__ __align__(8) uint64_t g_stage_bar[kMaxGroupSlots];
__shared__ unsigned g_stage_phase;

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile(
      "{\n .reg .b64 st;\n mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}" ::"r"(
          smem_u32(bar)),
      "r"(bytes)
      : "memory");
}

// Bounded wait for the phase with the given parity: each try suspends for at
// most about a microsecond, and about half a million tries give up.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
  const unsigned a = smem_u32(bar);
  for (int n = 0; n < (1 << 19); n++) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(a), "r"(parity), "r"(1000u)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Box at element (x, y) of the tensor map into shared memory; x * 8 bytes is a
// multiple of 16 (even tile edge), y is any row.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ const CUtensorMap* stage_map(const StageMaps& sm, int c) {
  static_assert(kMaxClasses == 4, "stage_map covers 4 classes");
  return c == 0 ? &sm.m[0] : c == 1 ? &sm.m[1] : c == 2 ? &sm.m[2] : &sm.m[3];
}

// One tap of degridding added into the running group sums by two FMAs per
// component: MODE 0 adds x * conj(c) (the adjoint of gridding); MODE 1 adds
// x * c, negated once at the end (the reference's -sum grid * gcf).
template <int MODE>
__device__ __forceinline__ void tap_fma(float& br, float& bi, float2 x, float cr, float ci) {
  if (MODE == 0) {
    br = fmaf(x.x, cr, br);
    br = fmaf(x.y, ci, br);
    bi = fmaf(x.y, cr, bi);
    bi = fmaf(-x.x, ci, bi);
  } else {
    br = fmaf(x.x, cr, br);
    br = fmaf(-x.y, ci, br);
    bi = fmaf(x.x, ci, bi);
    bi = fmaf(x.y, cr, bi);
  }
}

// Degridding of one item: stage the A x A grid region, then batches of L
// decoded records; sub-warps of SW lanes take one piece each (32/SW pieces
// per warp at a time), lanes stride the piece's taps by SW in groups of four
// steps; a group's products are summed by FMA chains and the group sum is
// added to the lane's Kahan accumulator (so the compensated error bound does
// not grow with the number of taps); shuffle reduction within the sub-warp.
// Staging forms (the GB_STAGE_* values of the C API).
constexpr int kStageSplit = 0, kStageTma = 1, kStageRows = 2;

template <int MODE, int SW, int STAGE>
__device__ __forceinline__ void degrid_item(const TiledArgs& a, const Item& it, int lt, int L,
                                            int bar, bool whole, int A, float2* __restrict__ sg,
                                            DegridRec* __restrict__ srec, const GridSlot& gs,
                                            const float2* __restrict__ gcf,
                                            const StageMaps& sm, int cls, int slot) {
  const float2* __restrict__ grid = gs.grid;
  float2* __restrict__ pred = gs.vis;
  constexpr bool TMA = STAGE == kStageTma, SPLIT = STAGE == kStageSplit;
  const int Ae = stage_stride(A);  // pixels staged per row (even)
  // TMA and ROWS stage rows as they lie in the grid, Ae apart.  SPLIT stores
  // each row as its even pixels, then its odd pixels (He = Ae / 2 each), so
  // the two taps of a pair are read by two loads that are each contiguous
  // across the lanes, whatever the parity of the piece's first column; its
  // rows are Rs apart, Rs chosen by the plan for the item's piece widths
  // (split_row_stride) so that row-major pair runs spread over the banks.
  const int He = Ae >> 1;
  const int Rs = SPLIT ? split_row_stride(A, item_stride_residue(it.cls)) : Ae;
  const int x0 = it.tile_x * a.T, y0 = it.tile_y * a.T;
  // array sizes for the bounds-checked build (unused otherwise)
  const int stage_len = A * Rs;
#ifdef GB_CHECKED
  const int64_t gcf_len = a.gcf_len;
#else
  const int64_t gcf_len = 0;
#endif
  const int64_t gcf_pairs = gcf_len / 2;
  (void)stage_len;
  (void)gcf_pairs;
  if constexpr (TMA) {
    if (lt == 0) {
      // the stage's earlier reads (generic proxy) come before the copy's writes
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_expect_tx(&g_stage_bar[slot], (unsigned)(A * Ae * 8));
      tma_load_2d(sg, stage_map(sm, cls), &g_stage_bar[slot], x0, y0);
    }
  } else {
    // asynchronous copies straight into shared memory (no register round
    // trip), all in flight at once; pixels outside the grid are zero-filled
    const int AA = A * Ae;
    const int dy = L / Ae, dx = L - dy * Ae;  // q = lt + n L walks (py, px) without divisions
    int py = lt / Ae, px = lt - py * Ae;
    for (int q = lt; q < AA; q += L) {
      const int gx = x0 + px, gy = y0 + py;
      const bool in = px < A && gx < gs.ext_x && gy < gs.ext_y;
      const int sq = SPLIT ? py * Rs + (px & 1) * He + (px >> 1) : q;
      px += dx;
      py += dy;
      if (px >= Ae) {
        px -= Ae;
        py++;
      }
      const float2* src = in ? grid + (int64_t)gy * gs.pitch + gx : grid;
      const unsigned dst = (unsigned)__cvta_generic_to_shared(sg + GB_IDX(sq, stage_len));
      asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(dst), "l"(src),
                   "r"(in ? 8 : 0)
                   : "memory");
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  }
  constexpr int SUBS = 32 / SW;
  const bool gcf16 = (reinterpret_cast<uintptr_t>(gcf) & 15) == 0;
  const int nw = L >> 5, w = lt >> 5, lane = lt & 31;
  const int sub = lane / SW, sl = lane - sub * SW;
  const int end = it.start + it.count;
  for (int base = it.start; base < end; base += L) {
    const int nb = min(L, end - base);
    group_sync(bar, L, whole);  // previous batch consumed
    if (lt < nb) {
      const Rec r = a.recs[GB_IDX(base + lt, a.n_recs)];
      DegridRec d;
      d.gcf = (int32_t)r.gcf;
      d.pitch = r.sm1 + 1;
      d.vis = r.vis;
      d.wx = r.wx;
      d.wy = r.wy;
      // taps in pairs when the piece's rows, its GCF rows and its first tap
      // all start on 16-byte boundaries
      const bool paired = gcf16 && (r.wx & 1) == 0 && (d.pitch & 1) == 0 && (d.gcf & 1) == 0;
      const int steps = paired ? r.wx >> 1 : r.wx;  // steps per row
      d.dj = (int16_t)(SW / steps);
      d.di = (int16_t)(SW - d.dj * steps);
      d.rcp_w = 1.0f / (float)steps;
      d.flags = (r.sm1 > r.pm1 ? kRecCut : 0) | (paired ? kRecPaired : 0) |
                (r.xl & 1 ? kRecOdd : 0) | ((int32_t)r.xl << 8);
      // stage offset of the piece's first tap (row-major), or in the split
      // layout: of its first tap for pairs, of its first row for single taps
      if constexpr (SPLIT)
        d.q0 = r.yl * Rs + (paired ? (r.xl & 1) * He + (r.xl >> 1) : 0);
      else
        d.q0 = r.yl * Ae + r.xl;
      srec[lt] = d;
    }
    // the stage (issued before the first batch's record loads, so the two
    // latencies overlap); the barrier publishes per-thread copies to the group
    if (base == it.start) {
      if constexpr (TMA) {
        const unsigned parity = (*(volatile unsigned*)&g_stage_phase >> slot) & 1u;
        // once any wait has run out, later items do not wait again
        if (*(volatile int32_t*)sm.err == 0 && !mbar_wait(&g_stage_bar[slot], parity))
          atomicOr(sm.err, 1);
      } else {
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
      }
    }
    group_sync(bar, L, whole);
    // every thread of the group has read the phase: the next use of this
    // slot's barrier waits for the other parity
    if constexpr (TMA)
      if (base == it.start && lt == 0) atomicXor(&g_stage_phase, 1u << slot);
    for (int kk = w * SUBS; kk < nb; kk += nw * SUBS) {
      const int k = kk + sub;
      const bool live = k < nb;
      const DegridRec r = srec[live ? k : kk];
      float ar = 0.f, ai = 0.f, cr = 0.f, ci = 0.f;
      if (live) {
        const float2* sp = sg + r.q0;
        // sl / steps: (sl + 1/2) / steps is at least 1/(2 steps) from an
        // integer, far more than the float rounding of the product
        int j = (int)(((float)sl + 0.5f) * r.rcp_w);
        const int dj = r.dj, di = r.di;
        if (r.flags & kRecPaired) {
          const int w2 = r.wx >> 1, p2 = r.pitch >> 1;
          const float4* gp = reinterpret_cast<const float4*>(gcf + r.gcf);
          // the pair's second tap: the next pixel (row-major), or the other
          // half of the split row (one column on when the first is odd)
          const float2* sp1 = SPLIT ? sp + ((r.flags & kRecOdd) ? 1 - He : He) : sp + 1;
          int i = sl - j * w2;
          // this lane's pairs: sl, sl + SW, ... below w2 * wy (SW is a power of two)
          const int tot = w2 * r.wy;
          const int n = tot > sl ? (tot - sl + SW - 1) / SW : 0;
          constexpr int UN = 4;
          // one group of UN steps: positions first, then every load, then the
          // sums; CHECK only for the last, partial group (a missing step adds
          // zeros)
          auto group = [&](int t, auto check) {
            constexpr bool CHECK = decltype(check)::value;
            int off_g[UN], off_s[UN];
#pragma unroll
            for (int u = 0; u < UN; u++) {
              off_g[u] = j * p2 + i;
              off_s[u] = j * Rs + (SPLIT ? i : 2 * i);
              i += di;
              j += dj;
              if (i >= w2) {
                i -= w2;
                j++;
              }
            }
            float4 c[UN];
            float2 x0[UN], x1[UN];
#pragma unroll
            for (int u = 0; u < UN; u++) {
              const bool ok = !CHECK || t + u < n;
              c[u] = ok ? __ldg(gp + GB_IDX(off_g[u], gcf_pairs - r.gcf / 2))
                        : make_float4(0.f, 0.f, 0.f, 0.f);
              x0[u] = ok ? sp[GB_IDX(off_s[u], stage_len - r.q0)] : make_float2(0.f, 0.f);
              x1[u] = ok ? sp1[GB_IDX(off_s[u], stage_len - (sp1 - sg))] : make_float2(0.f, 0.f);
            }
            // the group's products summed by FMA chains, then one compensated
            // add of the group sum
            float br = 0.f, bi = 0.f;
#pragma unroll
            for (int u = 0; u < UN; u++) {
              tap_fma<MODE>(br, bi, x0[u], c[u].x, c[u].y);
              tap_fma<MODE>(br, bi, x1[u], c[u].z, c[u].w);
            }
            kahan(ar, cr, br);
            kahan(ai, ci, bi);
          };
          int t = 0;
          for (; t + UN <= n; t += UN) group(t, std::false_type{});
          if (t < n) group(t, std::true_type{});
        } else {
          const float2* gp = gcf + r.gcf;
          const int wx = r.wx, pitch = r.pitch, xl = (r.flags >> 8) & 0xFF;
          int i = sl - j * wx;
          // this lane's taps: sl, sl + SW, ... below wx * wy
          const int tot = wx * r.wy;
          const int n = tot > sl ? (tot - sl + SW - 1) / SW : 0;
          constexpr int UN = 4;
          auto group = [&](int t, auto check) {
            constexpr bool CHECK = decltype(check)::value;
            int off_g[UN], off_s[UN];
#pragma unroll
            for (int u = 0; u < UN; u++) {
              off_g[u] = j * pitch + i;
              if constexpr (SPLIT) {
                const int c = xl + i;
                off_s[u] = j * Rs + (c & 1) * He + (c >> 1);
              } else {
                off_s[u] = j * Ae + i;
              }
              i += di;
              j += dj;
              if (i >= wx) {
                i -= wx;
                j++;
              }
            }
            float2 c[UN], x[UN];
#pragma unroll
            for (int u = 0; u < UN; u++) {
              const bool ok = !CHECK || t + u < n;
              c[u] = ok ? __ldg(gp + GB_IDX(off_g[u], gcf_len - r.gcf)) : make_float2(0.f, 0.f);
              x[u] = ok ? sp[GB_IDX(off_s[u], stage_len - r.q0)] : make_float2(0.f, 0.f);
            }
            float br = 0.f, bi = 0.f;
#pragma unroll
            for (int u = 0; u < UN; u++) tap_fma<MODE>(br, bi, x[u], c[u].x, c[u].y);
            kahan(ar, cr, br);
            kahan(ai, ci, bi);
          };
          int t = 0;
          for (; t + UN <= n; t += UN) group(t, std::false_type{});
          if (t < n) group(t, std::true_type{});
        }
      }
      ar -= cr;
      ai -= ci;
      if (MODE == 1) {  // the reference's negated product
        ar = -ar;
        ai = -ai;
      }
#pragma unroll
      for (int o = SW / 2; o > 0; o >>= 1) {
        ar += __shfl_xor_sync(0xffffffffu, ar, o);
        ai += __shfl_xor_sync(0xffffffffu, ai, o);
      }
      if (live && sl == 0) {
        if (r.flags & kRecCut)
          atomicAdd(pred + GB_IDX(r.vis, gs.n_vis), make_float2(ar, ai));
        else
          pred[GB_IDX(r.vis, gs.n_vis)] = make_float2(ar, ai);
      }
    }
  }
}

// At most 64 registers per thread (1024 resident threads per SM): registers
// then do not cut the CTAs per SM below what shared memory allows.
template <int NT, int MODE, int STAGE>
__global__ void __launch_bounds__(NT, 1024 / NT)
    k_degrid_tiled(const __grid_constant__ TiledArgs a, const __grid_constant__ GridPtrs gp,
                   const __grid_constant__ StageMaps sm, const float2* __restrict__ gcf) {
  static_assert(NT / 64 <= kMaxGroupSlots, "one stage barrier per group slot");
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ int s_b;
  const int tid = threadIdx.x;
  if constexpr (STAGE == kStageTma) {
    if (tid < NT / 64) mbar_init(&g_stage_bar[tid], 1);
    if (tid == 0) g_stage_phase = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    __syncthreads();
  }
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
      unsigned char* base = smem + (size_t)g * degrid_group_bytes(ci.A, ci.L);
      float2* sg = (float2*)base;
      DegridRec* srec = (DegridRec*)(base + degrid_stage_bytes(ci.A));
      const Item it = a.items[bd.first_item + g];
      const bool whole = ci.L == NT;
      // sub-warp width by piece size: <= 64 taps -> 8 lanes, <= 256 -> 16, else 32
      if (ci.pmax <= 8)
        degrid_item<MODE, 8, STAGE>(a, it, lt, ci.L, 1 + g, whole, ci.A, sg, srec,
                                   gp.s[bd.grid], gcf, sm, bd.cls, g);
      else if (ci.pmax <= 16)
        degrid_item<MODE, 16, STAGE>(a, it, lt, ci.L, 1 + g, whole, ci.A, sg, srec,
                                   gp.s[bd.grid], gcf, sm, bd.cls, g);
      else
        degrid_item<MODE, 32, STAGE>(a, it, lt, ci.L, 1 + g, whole, ci.A, sg, srec,
                                   gp.s[bd.grid], gcf, sm, bd.cls, g);
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- host side
size_t tiled_smem_grid(const ClassInfo* cls, int n, int) {
  size_t m = 0;
  for (int c = 0; c < n; c++) m = std::max(m, (size_t)cls[c].G * grid_group_bytes(cls[c].A, cls[c].L));
  return m;
}

size_t tiled_smem_degrid(const ClassInfo* cls, int n, int) {
  size_t m = 0;
  for (int c = 0; c < n; c++)
    m = std::max(m, (size_t)cls[c].G * degrid_group_bytes(cls[c].A, cls[c].L));
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

typedef void (*GridFn)(const TiledArgs, const GridPtrs, const float2*);
typedef void (*DegridFn)(const TiledArgs, const GridPtrs, const StageMaps, const float2*);

static GridFn grid_fn(int NT) {
  return NT == 128 ? k_grid_tiled<128> : NT == 256 ? k_grid_tiled<256> : k_grid_tiled<512>;
}

template <int STAGE>
static DegridFn degrid_fn_t(int NT, int mode) {
  if (NT == 128) return mode ? k_degrid_tiled<128, 1, STAGE> : k_degrid_tiled<128, 0, STAGE>;
  if (NT == 256) return mode ? k_degrid_tiled<256, 1, STAGE> : k_degrid_tiled<256, 0, STAGE>;
  return mode ? k_degrid_tiled<512, 1, STAGE> : k_degrid_tiled<512, 0, STAGE>;
}

static DegridFn degrid_fn(int NT, int mode, int stage) {
  return stage == kStageTma    ? degrid_fn_t<kStageTma>(NT, mode)
         : stage == kStageRows ? degrid_fn_t<kStageRows>(NT, mode)
                               : degrid_fn_t<kStageSplit>(NT, mode);
}

int degrid_stage_choice(int pref, int64_t taps, int64_t taps_paired, const float* gcf,
                        bool tma_possible) {
  if (pref == kStageTma || pref == kStageRows)
    return pref == kStageTma && tma_possible ? kStageTma : kStageRows;
  if (pref == kStageSplit) return kStageSplit;
  const bool pairs = (reinterpret_cast<uintptr_t>(gcf) & 15) == 0 && 2 * taps_paired >= taps;
  if (pairs) return kStageSplit;
  return tma_possible ? kStageTma : kStageRows;
}

static int set_smem_attr(const void* fn) {
  GB_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   tiled_max_smem()));
  return GB_OK;
}

int tiled_ctas_per_sm(const gb_plan* P, bool grid, int stage) {
  const void* fn = grid ? (const void*)grid_fn(P->NT)
                        : (const void*)degrid_fn(P->NT, 0, stage);
  if (set_smem_attr(fn)) return 1;
  if (!grid) set_smem_attr((const void*)degrid_fn(P->NT, 1, stage));
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, P->NT,
                                                grid ? P->smem_grid : P->smem_degrid);
  return n > 0 ? n : 1;
}

static void set_bounds(TiledArgs& a, const TiledBounds& b) {
#ifdef GB_CHECKED
  a.n_recs = b.n_recs;
  a.gcf_len = b.gcf_len;
#else
  (void)a;
  (void)b;
#endif
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
  set_bounds(a, TiledBounds{P->n_recs, P->gcf_len, P->dev.n_vis});
  return a;
}

static GridPtrs one_grid(const float* grid, const float* vis, int ext_x, int ext_y,
                         int64_t pitch, int64_t n_vis) {
  GridPtrs gp;
  memset(&gp, 0, sizeof(gp));
  gp.s[0].grid = (float2*)grid;
  gp.s[0].vis = (float2*)vis;
  gp.s[0].pitch = pitch;
  gp.s[0].ext_x = ext_x;
  gp.s[0].ext_y = ext_y;
#ifdef GB_CHECKED
  gp.s[0].n_vis = n_vis;
#else
  (void)n_vis;
#endif
  return gp;
}

int launch_grid_tiled(gb_plan* P, const float* vis, const float* gcf, float* grid,
                      cudaStream_t s) {
  if (P->n_bundles == 0) return GB_OK;
  GB_CUDA_TRY(cudaMemsetAsync(P->d_queue, 0, sizeof(int32_t), s));
  const int blocks = std::min(P->n_bundles, sm_count() * P->ctas_per_sm_grid);
  GridFn fn = grid_fn(P->NT);
  fn<<<blocks, P->NT, P->smem_grid, s>>>(
      make_args(P), one_grid(grid, vis, P->dev.ext_x, P->dev.ext_y, P->dev.pitch, P->dev.n_vis),
      (const float2*)gcf);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  });
  return fn;
}

// Tensor maps of the grid for TMA staging, one per class (box = Ae x A
// pixels of 8 bytes, rows of pitch * 8 bytes, zero fill outside ext_x x
// ext_y), cached on the plan.  False where TMA does not apply: an odd tile
// edge (the box's x would not start on 16 bytes), an odd pitch, an unaligned
// grid, an oversized box or no encoder; degridding then stages with
// per-thread copies.
static bool stage_maps(gb_plan* P, const float* grid, StageMaps* out) {
  const int64_t pitch = P->dev.pitch;
  const int ex = P->dev.ext_x, ey = P->dev.ext_y;
  if ((P->T & 1) || (pitch & 1) || (reinterpret_cast<uintptr_t>(grid) & 15) || ex <= 0 ||
      ey <= 0 || P->NT / 64 > kMaxGroupSlots)
    return false;
  for (int c = 0; c < P->n_classes; c++)
    if (P->cls[c].A > 256 || stage_stride(P->cls[c].A) > 256 || P->cls[c].L < 64) return false;
  if (!(P->tma_ok && P->tma_grid == grid && P->tma_ext_x == ex && P->tma_ext_y == ey &&
        P->tma_pitch == pitch)) {
    P->tma_ok = false;
    EncodeTiledFn enc = encode_tiled();
    if (!enc) return false;
    for (int c = 0; c < P->n_classes; c++) {
      const int A = P->cls[c].A;
      const cuuint64_t dims[2] = {(cuuint64_t)ex, (cuuint64_t)ey};
      const cuuint64_t strides[1] = {(cuuint64_t)pitch * 8};
      const cuuint32_t box[2] = {(cuuint32_t)stage_stride(A), (cuuint32_t)A};
      const cuuint32_t estr[2] = {1, 1};
      if (enc(&P->tma_maps[c], CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, (void*)grid, dims, strides,
              box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
              CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    }
    P->tma_grid = grid;
    P->tma_ext_x = ex;
    P->tma_ext_y = ey;
    P->tma_pitch = pitch;
    P->tma_ok = true;
  }
  for (int c = 0; c < P->n_classes; c++) out->m[c] = P->tma_maps[c];
  return true;
}

int launch_degrid_tiled(gb_plan* P, const float* gcf, const float* grid, float* pred, int mode,
                        cudaStream_t s) {
  GB_CUDA_TRY(cudaMemsetAsync(pred, 0, sizeof(float2) * (size_t)P->dev.n_vis, s));
  if (P->n_bundles == 0) return GB_OK;
  GB_CUDA_TRY(cudaMemsetAsync(P->d_queue + 1, 0, sizeof(int32_t), s));
  StageMaps sm;
  memset(&sm, 0, sizeof(sm));
  // tensor maps only where the choice can fall on TMA
  int stage = degrid_stage_choice(P->stage_pref, P->taps, P->taps_paired, gcf, false);
  if (stage == kStageRows)
    stage = degrid_stage_choice(P->stage_pref, P->taps, P->taps_paired, gcf,
                                stage_maps(P, grid, &sm));
  sm.err = P->d_queue + 2;
  P->last_stage = stage;
  const int blocks = std::min(P->n_bundles, sm_count() * P->ctas_per_sm_degrid[stage]);
  DegridFn fn = degrid_fn(P->NT, mode, stage);
  fn<<<blocks, P->NT, P->smem_degrid, s>>>(
      make_args(P), one_grid(grid, pred, P->dev.ext_x, P->dev.ext_y, P->dev.pitch, P->dev.n_vis),
      sm, (const float2*)gcf);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

// Launch of the tiled gridding kernel on caller-supplied work tables (used by
// the allocation-free entry point, whose tables live in a static device
// array rather than in a plan).
int launch_grid_tiled_tables(const Bundle* bundles, int n_bundles, const Item* items,
                             const Rec* recs, int32_t* queue, const ClassInfo* cls, int n_classes,
                             int NT, int T, int ext_x, int ext_y, int64_t pitch, size_t smem,
                             const float* vis, const float* gcf, float* grid,
                             const TiledBounds& bounds, cudaStream_t s) {
  if (n_bundles <= 0) return GB_OK;
  GridFn fn = grid_fn(NT);
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
  set_bounds(a, bounds);
  GB_CUDA_TRY(cudaMemsetAsync(queue, 0, sizeof(int32_t), s));
  fn<<<blocks, NT, smem, s>>>(a, one_grid(grid, vis, ext_x, ext_y, pitch, bounds.n_vis),
                              (const float2*)gcf);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

// Batched launches: one persistent kernel over the bundles of several grids.
int launch_tiled_batch(bool grid_mode, int mode, int NT, size_t smem, int ctas_per_sm,
                       const Bundle* bundles, int n_bundles, const Item* items, const Rec* recs,
                       int32_t* queue, const ClassInfo* cls, int n_classes, int T,
                       const GridPtrs& gp, const float* gcf, int stage,
                       const TiledBounds& bounds, cudaStream_t s) {
  if (n_bundles <= 0) return GB_OK;
  TiledArgs a;
  a.bundles = bundles;
  a.items = items;
  a.recs = recs;
  a.queue = queue;
  for (int c = 0; c < kMaxClasses; c++) a.cls[c] = c < n_classes ? cls[c] : ClassInfo{64, 1, 1, 1};
  a.n_bundles = n_bundles;
  a.T = T;
  set_bounds(a, bounds);
  const int blocks = std::min(n_bundles, sm_count() * std::max(1, ctas_per_sm));
  // queue: the two work-queue heads (the grid kernel uses [0], degrid [1])
  GB_CUDA_TRY(cudaMemsetAsync(queue + (grid_mode ? 0 : 1), 0, sizeof(int32_t), s));
  if (grid_mode) {
    GridFn fn = grid_fn(NT);
    fn<<<blocks, NT, smem, s>>>(a, gp, (const float2*)gcf);
  } else {
    StageMaps sm;  // several grids: per-thread asynchronous staging (split or rows)
    memset(&sm, 0, sizeof(sm));
    DegridFn fn = degrid_fn(NT, mode, stage == kStageSplit ? kStageSplit : kStageRows);
    fn<<<blocks, NT, smem, s>>>(a, gp, sm, (const float2*)gcf);
  }
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

// Occupancy of the batched kernels (sets their shared-memory limit first).
int tiled_ctas_per_sm_for(int NT, bool grid, size_t smem, int stage) {
  const void* fn = grid ? (const void*)grid_fn(NT) : (const void*)degrid_fn(NT, 0, stage);
  if (set_smem_attr(fn)) return 1;
  if (!grid) set_smem_attr((const void*)degrid_fn(NT, 1, stage));
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, NT, smem);
  return n > 0 ? n : 1;
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

extern "C" int gb_grid_forward(gb_plan* P, const float* d_gcf, const float* d_vis, float* d_grid,
                               void* stream) {
  return gb_grid_f32(P, d_vis, d_gcf, d_grid, stream);
}

extern "C" int gb_grid_backward(gb_plan* P, const float* d_gcf, const float* d_grid_grad,
                                float* d_vis_grad, void* stream) {
  return gb_degrid_f32(P, d_gcf, d_grid_grad, d_vis_grad, 0, stream);
}

// ---------------------------------------------------------------- bounds-checked build
#ifdef GB_CHECKED
__global__ void k_checked_selftest() {
  // two indices out of range and one in range: no memory is touched
  (void)gb_checked_index(5, 3);
  (void)gb_checked_index(-1, 3);
  (void)gb_checked_index(2, 3);
}
#endif

extern "C" int gb_checked_violations(int64_t* out) {
  if (!out) {
    gb_set_error(GB_ERR_ARG, "gb_checked_violations: NULL argument");
    return GB_ERR_ARG;
  }
#ifdef GB_CHECKED
  unsigned long long v = 0, zero = 0;
  GB_CUDA_TRY(cudaMemcpyFromSymbol(&v, g_check_violations, sizeof(v)));
  GB_CUDA_TRY(cudaMemcpyToSymbol(g_check_violations, &zero, sizeof(zero)));
  *out = (int64_t)v;
#else
  *out = -1;
#endif
  return GB_OK;
}

extern "C" int gb_checked_selftest(void) {
#ifdef GB_CHECKED
  k_checked_selftest<<<1, 1>>>();
  GB_CUDA_TRY(cudaGetLastError());
  GB_CUDA_TRY(cudaDeviceSynchronize());
  return GB_OK;
#else
  gb_set_error(GB_ERR_ARG, "gb_checked_selftest: not a bounds-checked build");
  return GB_ERR_ARG;
#endif
}
