// Plain FP64 gridder / degridder (complex128) and the reference-ABI entry
// points built on them.
//
// "Plain" = no tiling: one warp per visibility, lanes over the S*S taps,
// FP64 atomics into the grid (gridding) or a warp-shuffle reduction
// (degridding, computed in double-float; see the section below).  Each lane
// computes the FP64 index math of one of up to 32 visibilities and the warp
// takes them in turn.  It is the FP64 GPU comparison path of the engine and
// the implementation behind kern_degrid_gpu1 / kern_degrid; the gridders
// kern_scatter_gpu1 / nvGridder / kern_scatter sum each 32 x 32 grid block's
// taps in shared memory in double-float first (k_scatter_blocks_df) and keep
// the warp kernel for inputs with an Inf, a NaN or a subnormal.  Semantics
// are the reference's (MS6/kernel/cpu/gridding/scatter.cpp:56-111,
// degrid.cpp:41-98) on Halide buffer_t host buffers.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <type_traits>
#include <thread>
#include <vector>

#include "gb_common.cuh"
#include "gb_plan.cuh"
#include "gb_runtime.cuh"
#include "rc_gb300_ms5.h"

namespace gb {

// Tap walk of a warp over an S x S footprint, lane-strided: tap k = lane +
// 32 m, (i, j) = (k mod S, k div S), advanced incrementally.
struct TapWalk {
  int i, j, di, dj, S;
  // lane: the lane's index among the L lanes that share the footprint
  __device__ __forceinline__ TapWalk(int S_, int lane, int L = 32) : S(S_) {
    j = lane / S_;
    i = lane - j * S_;
    dj = L / S_;
    di = L - dj * S_;
  }
  __device__ __forceinline__ void next() {
    i += di;
    j += dj;
    if (i >= S) {
      i -= S;
      j++;
    }
  }
};

// grid[y0+j][x0+i] += vis * gcf[j][i] for the S*S taps of one visibility.
__device__ __forceinline__ void warp_scatter64(double2* __restrict__ base, int64_t pitch,
                                               const double2* __restrict__ g, int S,
                                               double vr, double vi, int lane) {
  TapWalk w(S, lane);
  for (; w.j < S; w.next()) {
    const double2 c = __ldg(g + w.j * S + w.i);
    double2* p = base + (int64_t)w.j * pitch + w.i;
    atomicAdd(&p->x, vr * c.x - vi * c.y);
    atomicAdd(&p->y, vr * c.y + vi * c.x);
  }
}

// sum over taps of grid * gcf (conj_g: grid * conj(gcf)), reduced over the warp.
__device__ __forceinline__ double2 warp_gather64(const double2* __restrict__ base, int64_t pitch,
                                                 const double2* __restrict__ g, int S,
                                                 bool conj_g, int lane) {
  double ar = 0.0, ai = 0.0;
  const double sg = conj_g ? -1.0 : 1.0;
  TapWalk w(S, lane);
  for (; w.j < S; w.next()) {
    const double2 c = __ldg(g + w.j * S + w.i);
    const double2 u = base[(int64_t)w.j * pitch + w.i];
    const double ci = sg * c.y;
    ar += u.x * c.x - u.y * ci;
    ai += u.x * ci + u.y * c.x;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ar += __shfl_xor_sync(0xffffffffu, ar, o);
    ai += __shfl_xor_sync(0xffffffffu, ai, o);
  }
  return make_double2(ar, ai);
}

// ---------------------------------------------------------------- double-float gather
// The FP64 pipe of this part runs at a small fraction of its FP32 rate
// (nominal 1.25 TFLOP/s FP64 for the whole GPU), so the FP64 degridders do
// their tap arithmetic in double-float on the FP32 pipe.  Each operand array
// is scaled by the power of two that brings its largest magnitude into [1, 2)
// and every double x is held as hi + lo: hi = x rounded to 24 significant
// bits, lo = the remainder rounded to 24 (x to 2^-48 relative).  A product is
// hi*hi with its exact FMA error plus the hi*lo cross terms (lo*lo, under
// 2^-48 of the product, is left out); the running sums are TwoSum pairs (hi
// sum, low-order sum), so each addition errs by about 2^-48 of the running sum,
// as in a 48-bit floating-point format (FP64: 2^-53).  Scaled values below
// 2^-74 lose their low part and those below 2^-126 are dropped (an absolute
// error under 2^-98 of the array's largest value).  An Inf, a NaN or a
// subnormal in either array sends the launch down the native FP64 loop
// instead, so that those propagate as FP64 arithmetic would.

constexpr int kExpNonFinite = 0x7FF;

// Largest biased exponent field over rows x row doubles (rows `pitch` doubles
// apart), max-ed into *out, which the caller zeroes.  A subnormal counts as
// kExpNonFinite too: the split would drop it, so the native loop takes it.
__global__ void k_max_exponent(const double* __restrict__ x, int64_t rows, int64_t row,
                               int64_t pitch, int* __restrict__ out) {
  int m = 0;
  for (int64_t r = blockIdx.y; r < rows; r += gridDim.y) {
    const unsigned long long* xr = (const unsigned long long*)(x + r * pitch);
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < row;
         c += (int64_t)gridDim.x * blockDim.x) {
      const unsigned long long b = xr[c];
      const int e = (int)((b >> 52) & 0x7FF);
      m = max(m, e == 0 && (b & 0xFFFFFFFFFFFFFull) ? kExpNonFinite : e);
    }
  }
  m = __reduce_max_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

// The scale exponent of an array from its largest exponent field: the array
// is multiplied by 2^-k (k = 0 for an array of zeros).
__device__ __forceinline__ int df_scale_exp(int e) { return e > 0 && e < kExpNonFinite ? e - 1023 : 0; }

// x * 2^-k as (hi, lo) floats from x's bit pattern, no FP64 arithmetic: hi =
// the scaled x rounded to 24 significant bits (a carry out of the mantissa
// moves into the exponent field), lo = the remaining 29-bit signed remainder
// rounded to 24 bits.
__device__ __forceinline__ float2 df_split(unsigned long long b, int k) {
  const unsigned hi32 = (unsigned)(b >> 32), lo32 = (unsigned)b;
  const int e = (int)((hi32 >> 20) & 0x7FF);
  const int fe = e - k - 896;  // biased float exponent of the scaled value (1023 - 127 = 896)
  if (e == 0 || fe <= 0) return make_float2(0.f, 0.f);
  const unsigned sign = hi32 & 0x80000000u;
  const unsigned top = ((hi32 & 0xFFFFFu) << 3) | (lo32 >> 29);  // mantissa bits 51..29
  const unsigned up = (lo32 >> 28) & 1u;                          // bit 28: round up
  const float hi = __uint_as_float(sign | ((((unsigned)fe << 23) | top) + up));
  // mantissa bits 28..0, less 2^29 when hi was rounded up, are worth
  // rem * 2^(fe - 127 - 52) in magnitude
  float lo = 0.f;
  if (fe > 52) {
    const int rem = (int)(lo32 & 0x1FFFFFFFu) - (int)(up << 29);
    lo = __int2float_rn(rem) * __uint_as_float((unsigned)(fe - 52) << 23);
  }
  return make_float2(hi, __uint_as_float(__float_as_uint(lo) ^ sign));
}

// out[r * row + c] = split of x[r * pitch + c] under the scale of exps[which];
// nothing when either array of the launch holds an Inf or NaN.
__global__ void k_df_split(const double* __restrict__ x, int64_t rows, int64_t row, int64_t pitch,
                           const int* __restrict__ exps, int which, float2* __restrict__ out) {
  if (exps[0] == kExpNonFinite || exps[1] == kExpNonFinite) return;
  const int k = df_scale_exp(exps[which]);
  for (int64_t r = blockIdx.y; r < rows; r += gridDim.y) {
    const unsigned long long* xr = (const unsigned long long*)(x + r * pitch);
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < row;
         c += (int64_t)gridDim.x * blockDim.x)
      out[r * row + c] = df_split(xr[c], k);
  }
}

// s + p into the pair (s, c): s the rounded sum, c += its exact rounding error.
__device__ __forceinline__ void two_sum_acc(float& s, float& c, float p) {
  const float t = __fadd_rn(s, p);
  const float bp = __fsub_rn(t, s);
  const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  s = t;
  c = __fadd_rn(c, e);
}

// acc += a * b (CONJ: a * conj(b)) for complex double-floats laid out
// (re hi, re lo, im hi, im lo); acc = (re sum, im sum, re low-order, im low-order).
template <bool CONJ>
__device__ __forceinline__ void df_cmac(const float4 a, float4 b, float4& acc) {
  if (CONJ) {
    b.z = -b.z;
    b.w = -b.w;
  }
  const float p1 = __fmul_rn(a.x, b.x), e1 = __fmaf_rn(a.x, b.x, -p1);  // re re
  const float p2 = __fmul_rn(a.z, b.z), e2 = __fmaf_rn(a.z, b.z, -p2);  // im im
  const float p3 = __fmul_rn(a.x, b.z), e3 = __fmaf_rn(a.x, b.z, -p3);  // re im
  const float p4 = __fmul_rn(a.z, b.x), e4 = __fmaf_rn(a.z, b.x, -p4);  // im re
  float lr = __fmaf_rn(a.x, b.y, __fmaf_rn(a.y, b.x, __fsub_rn(e1, e2)));
  lr = __fmaf_rn(-a.z, b.w, __fmaf_rn(-a.w, b.z, lr));
  float li = __fmaf_rn(a.x, b.w, __fmaf_rn(a.y, b.z, __fadd_rn(e3, e4)));
  li = __fmaf_rn(a.z, b.y, __fmaf_rn(a.w, b.x, li));
  acc.z = __fadd_rn(acc.z, lr);
  acc.w = __fadd_rn(acc.w, li);
  two_sum_acc(acc.x, acc.z, p1);
  two_sum_acc(acc.x, acc.z, -p2);
  two_sum_acc(acc.y, acc.w, p3);
  two_sum_acc(acc.y, acc.w, p4);
}

// The footprint's double-float sum over a group of L lanes (an aligned part
// of the warp, `mask` its lanes; lane = the lane's index in the group).  A
// lane takes its taps U at a time, all 2U loads issued first, into U running
// sums (independent addition chains), which are added at the end: U = 4 where
// few warps share an SM (small reference-ABI calls), 1 where the registers
// are better spent on resident warps (the engine's FP64 degridder).
template <bool CONJ, int L = 32, int U = 1>
__device__ __forceinline__ float4 warp_gather_df(const float4* __restrict__ base, int64_t pitch,
                                                 const float4* __restrict__ g, int S, int lane,
                                                 unsigned mask = 0xffffffffu) {
  float4 acc[U];
#pragma unroll
  for (int u = 0; u < U; u++) acc[u] = make_float4(0.f, 0.f, 0.f, 0.f);
  TapWalk w(S, lane, L);
  if constexpr (U == 1) {
    for (; w.j < S; w.next())
      df_cmac<CONJ>(base[(int64_t)w.j * pitch + w.i], __ldg(g + w.j * S + w.i), acc[0]);
  }
  while (U > 1 && w.j < S) {
    int64_t ob[U];
    int og[U];
    bool ok[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      ok[u] = w.j < S;
      ob[u] = ok[u] ? (int64_t)w.j * pitch + w.i : 0;
      og[u] = ok[u] ? w.j * S + w.i : 0;
      w.next();
    }
    float4 x[U], c[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      x[u] = ok[u] ? base[ob[u]] : make_float4(0.f, 0.f, 0.f, 0.f);
      c[u] = ok[u] ? __ldg(g + og[u]) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < U; u++) df_cmac<CONJ>(x[u], c[u], acc[u]);
  }
#pragma unroll
  for (int u = 1; u < U; u++) {
    acc[0].z = __fadd_rn(acc[0].z, acc[u].z);
    acc[0].w = __fadd_rn(acc[0].w, acc[u].w);
    two_sum_acc(acc[0].x, acc[0].z, acc[u].x);
    two_sum_acc(acc[0].y, acc[0].w, acc[u].y);
  }
  float4 r = acc[0];
#pragma unroll
  for (int o = L / 2; o > 0; o >>= 1) {
    const float sr = __shfl_xor_sync(mask, r.x, o);
    const float si = __shfl_xor_sync(mask, r.y, o);
    r.z = __fadd_rn(r.z, __shfl_xor_sync(mask, r.z, o));
    r.w = __fadd_rn(r.w, __shfl_xor_sync(mask, r.w, o));
    two_sum_acc(r.x, r.z, sr);
    two_sum_acc(r.y, r.w, si);
  }
  return r;
}

// A double-float sum back to FP64, times 2^kt.
__device__ __forceinline__ double2 df_to_double(float4 a, int kt) {
  return make_double2(ldexp((double)a.x + (double)a.z, kt), ldexp((double)a.y + (double)a.w, kt));
}

// 2^kt as a double when it is a normal number (else 0: use df_to_double).
__device__ __forceinline__ double df_pow2(int kt) {
  return kt > -1023 && kt < 1024 ? __longlong_as_double((long long)(kt + 1023) << 52) : 0.0;
}

// df_to_double with the factor 2^kt given as sc = df_pow2(kt) (one multiply
// instead of ldexp's range handling; the same result while sc is normal).
__device__ __forceinline__ double2 df_to_double_sc(float4 a, int kt, double sc) {
  if (sc == 0.0) return df_to_double(a, kt);
  return make_double2(((double)a.x + (double)a.z) * sc, ((double)a.y + (double)a.w) * sc);
}

// Lane l of a warp indexes visibility t0 + l once; the warp then takes the
// visibilities one by one, fetching each index from its lane.
struct LaneIndex {
  int32_t x0, y0, phase, keep, plane;
  __device__ __forceinline__ LaneIndex from(int j) const {
    LaneIndex r;
    r.x0 = __shfl_sync(0xffffffffu, x0, j);
    r.y0 = __shfl_sync(0xffffffffu, y0, j);
    r.phase = __shfl_sync(0xffffffffu, phase, j);
    r.keep = __shfl_sync(0xffffffffu, keep, j);
    r.plane = __shfl_sync(0xffffffffu, plane, j);
    return r;
  }
};

// ---------------------------------------------------------------- single GCF (ABI form)
struct SingleGeo {
  double scale;
  int32_t grid_size, margin, S;
  int32_t min_x, min_y, ext_x, ext_y;
  int64_t pitch;  // complex elements per grid row
};

__device__ __forceinline__ LaneIndex single_index(const double* __restrict__ vis5, int64_t t,
                                                  int64_t n, const SingleGeo& geo) {
  LaneIndex li{0, 0, 0, 0, 0};
  if (t < n) {
    const VisIndex ix = vis_index(vis5[5 * t], vis5[5 * t + 1], geo.scale, geo.grid_size, geo.S,
                                  geo.margin, geo.min_x, geo.min_y, geo.ext_x, geo.ext_y);
    li.x0 = ix.x0 - geo.min_x;
    li.y0 = ix.y0 - geo.min_y;
    li.phase = ix.phase;
    li.keep = ix.keep;
  }
  return li;
}

// The record at visit position i: `order` (records by the grid block of their
// footprint corner, so that neighbouring warps share grid lines in L2) or
// index order.
__device__ __forceinline__ int64_t visit_rec(const int32_t* __restrict__ order, int64_t i,
                                             int64_t n) {
  return order && i < n ? (int64_t)order[i] : i;
}

__global__ void k_scatter_single64(int64_t n, const double* __restrict__ vis5,
                                   const double2* __restrict__ gcf, double2* __restrict__ grid,
                                   SingleGeo geo, const int32_t* __restrict__ order) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t t0 = 32 * (blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5)); t0 < n;
       t0 += 32 * warps) {
    const int64_t t = visit_rec(order, t0 + lane, n);
    const LaneIndex mine = single_index(vis5, t, n, geo);
    const int m = (int)min((int64_t)32, n - t0);
    for (int j = 0; j < m; j++) {
      const LaneIndex ix = mine.from(j);
      if (!ix.keep) continue;
      const double* r = vis5 + 5 * __shfl_sync(0xffffffffu, t, j);
      warp_scatter64(grid + (int64_t)ix.y0 * geo.pitch + ix.x0, geo.pitch,
                     gcf + (int64_t)ix.phase * geo.S * geo.S, geo.S, r[3], r[4], lane);
    }
  }
}

// vis_out = vis; in-bound: vis_out.re/im -= sum grid * gcf (degrid.cpp:78-98).
// exps: largest exponent fields of the grid and the GCF; grid_df / gcf_df
// their double-float splits (grid rows ext_x apart).
__global__ void k_degrid_single64(int64_t n, const double* __restrict__ vis5,
                                  const double2* __restrict__ gcf,
                                  const double2* __restrict__ grid,
                                  const float4* __restrict__ gcf_df,
                                  const float4* __restrict__ grid_df,
                                  const int* __restrict__ exps, double* __restrict__ out5,
                                  SingleGeo geo, const int32_t* __restrict__ order, int pw) {
  const int lane = threadIdx.x & 31;
  const bool df = exps[0] != kExpNonFinite && exps[1] != kExpNonFinite;
  const int kt = df_scale_exp(exps[0]) + df_scale_exp(exps[1]);
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t t0 = pw * (blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5)); t0 < n;
       t0 += pw * warps) {
    const int m = (int)min((int64_t)pw, n - t0);
    const bool mine_ok = lane < m;
    const int64_t t = visit_rec(order, t0 + lane, n);
    const LaneIndex mine = single_index(vis5, mine_ok ? t : n, n, geo);
    float4 acc_df = make_float4(0.f, 0.f, 0.f, 0.f);
    double2 acc = make_double2(0.0, 0.0);
    if (df && geo.S <= 8) {
      // small footprints: 8 lanes per visibility, four visibilities at a time
      const int grp = lane >> 3, gl = lane & 7;
      const unsigned gmask = 0xFFu << (8 * grp);
      for (int j0 = 0; j0 < m; j0 += 4) {
        const int jv = j0 + grp;
        const LaneIndex ix = mine.from(jv < m ? jv : m - 1);
        float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
        if (jv < m && ix.keep)  // uniform within the group
          a = warp_gather_df<false, 8, 4>(grid_df + (int64_t)ix.y0 * geo.ext_x + ix.x0, geo.ext_x,
                                       gcf_df + (int64_t)ix.phase * geo.S * geo.S, geo.S, gl,
                                       gmask);
        // lane j0 + q takes the sum of group q
        const int src = ((lane - j0) & 3) * 8;
        a.x = __shfl_sync(0xffffffffu, a.x, src);
        a.y = __shfl_sync(0xffffffffu, a.y, src);
        a.z = __shfl_sync(0xffffffffu, a.z, src);
        a.w = __shfl_sync(0xffffffffu, a.w, src);
        if (lane >= j0 && lane < j0 + 4) acc_df = a;
      }
    }
    for (int j = 0; j < m && !(df && geo.S <= 8); j++) {
      const LaneIndex ix = mine.from(j);
      if (!ix.keep) continue;
      const int64_t g0 = (int64_t)ix.phase * geo.S * geo.S;
      if (df) {
        const float4 a = warp_gather_df<false, 32, 4>(grid_df + (int64_t)ix.y0 * geo.ext_x + ix.x0,
                                               geo.ext_x, gcf_df + g0, geo.S, lane);
        if (lane == j) acc_df = a;
      } else {
        const double2 a = warp_gather64(grid + (int64_t)ix.y0 * geo.pitch + ix.x0, geo.pitch,
                                        gcf + g0, geo.S, false, lane);
        if (lane == j) acc = a;
      }
    }
    if (mine_ok) {
      if (df) acc = df_to_double(acc_df, kt);
      const double* r = vis5 + 5 * t;
      double* o = out5 + 5 * t;
      o[0] = r[0];
      o[1] = r[1];
      o[2] = r[2];
      o[3] = r[3] - acc.x;  // acc is zero for an out-of-bound record
      o[4] = r[4] - acc.y;
    }
  }
}

// ---------------------------------------------------------------- multi-plane (engine form)
__device__ __forceinline__ LaneIndex plane_index(const PlanDev& P, int64_t t) {
  LaneIndex li{0, 0, 0, 0, -1};
  if (t < P.n_vis) {
    const int32_t p = P.plane[t];
    if (p >= 0) {
      const double* r = P.uvw + t * P.uvw_stride;
      const VisIndex ix = vis_index(r[0], r[1], P.scale, P.grid_size, P.supports[p], P.margin, 0,
                                    0, P.ext_x, P.ext_y);
      li = LaneIndex{ix.x0, ix.y0, ix.phase, ix.keep, p};
    }
  }
  return li;
}

// The visibility at visit position i: the plan's order (by the tile of the
// footprint corner, so that a warp's and its neighbours' footprints share grid
// lines in L2), or index order.
__device__ __forceinline__ int64_t visit(const PlanDev& P, int64_t i) {
  return P.order && i < P.n_vis ? (int64_t)P.order[i] : i;
}

__global__ void k_grid_plain64(PlanDev P, const double2* __restrict__ vis,
                               const double2* __restrict__ gcf, double2* __restrict__ grid) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t t0 = 32 * (blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5));
       t0 < P.n_vis; t0 += 32 * warps) {
    const int64_t t = visit(P, t0 + lane);
    const LaneIndex mine = plane_index(P, t);
    const int m = (int)min((int64_t)32, P.n_vis - t0);
    for (int j = 0; j < m; j++) {
      const LaneIndex ix = mine.from(j);
      if (!ix.keep) continue;
      const int32_t S = P.supports[ix.plane];
      const double2 v = vis[__shfl_sync(0xffffffffu, t, j)];
      warp_scatter64(grid + (int64_t)ix.y0 * P.pitch + ix.x0, P.pitch,
                     gcf + P.gcf_offsets[ix.plane] + (int64_t)ix.phase * S * S, S, v.x, v.y,
                     lane);
    }
  }
}

// mode 0: pred = sum grid * conj(gcf); mode 1: pred = -sum grid * gcf.
// grid_df rows are ext_x apart.
__global__ void k_degrid_plain64(PlanDev P, const double2* __restrict__ gcf,
                                 const double2* __restrict__ grid,
                                 const float4* __restrict__ gcf_df,
                                 const float4* __restrict__ grid_df,
                                 const int* __restrict__ exps, double2* __restrict__ pred,
                                 int mode) {
  const int lane = threadIdx.x & 31;
  const bool df = exps[0] != kExpNonFinite && exps[1] != kExpNonFinite;
  const int kt = df_scale_exp(exps[0]) + df_scale_exp(exps[1]);
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t t0 = 32 * (blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5));
       t0 < P.n_vis; t0 += 32 * warps) {
    const bool mine_ok = t0 + lane < P.n_vis;
    const int64_t t = visit(P, t0 + lane);
    const LaneIndex mine = plane_index(P, t);
    const int m = (int)min((int64_t)32, P.n_vis - t0);
    float4 acc_df = make_float4(0.f, 0.f, 0.f, 0.f);
    double2 acc = make_double2(0.0, 0.0);
    for (int j = 0; j < m; j++) {
      const LaneIndex ix = mine.from(j);
      if (!ix.keep) continue;
      const int32_t S = P.supports[ix.plane];
      const int64_t g0 = P.gcf_offsets[ix.plane] + (int64_t)ix.phase * S * S;
      if (df) {
        const float4* base = grid_df + (int64_t)ix.y0 * P.ext_x + ix.x0;
        const float4 a = mode == 0 ? warp_gather_df<true>(base, P.ext_x, gcf_df + g0, S, lane)
                                   : warp_gather_df<false>(base, P.ext_x, gcf_df + g0, S, lane);
        if (lane == j) acc_df = a;
      } else {
        const double2 a = warp_gather64(grid + (int64_t)ix.y0 * P.pitch + ix.x0, P.pitch,
                                        gcf + g0, S, mode == 0, lane);
        if (lane == j) acc = a;
      }
    }
    if (mine_ok) {
      if (df) acc = df_to_double(acc_df, kt);
      if (mode == 1) {
        acc.x = -acc.x;
        acc.y = -acc.y;
      }
      pred[t] = acc;
    }
  }
}

// Launch shape of k_degrid_single64: pw records per warp (32, fewer for a
// call too small to occupy every SM with 32 warps), 8 warps per block.
static int single_degrid_dims(int64_t n, int* blocks, int* pw) {
  const int64_t target = (int64_t)sm_count() * 32;
  *pw = (int)std::clamp<int64_t>((n + target - 1) / target, 1, 32);
  const int64_t warps = (n + *pw - 1) / *pw;
  *blocks = (int)std::clamp<int64_t>((warps + 7) / 8, 1, (int64_t)sm_count() * 8);
  return 256;
}

static int plain_grid_dims(int64_t n, int* blocks) {
  const int64_t warps_needed = (n + 31) / 32;
  int64_t b = (warps_needed + 7) / 8;
  const int64_t cap = (int64_t)sm_count() * 8;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  *blocks = (int)b;
  return 256;
}

// a += b over n complex128 elements.
__global__ void k_add_c128(double2* __restrict__ a, const double2* __restrict__ b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double2 x = a[i], y = b[i];
    a[i] = make_double2(x.x + y.x, x.y + y.y);
  }
}

// ---------------------------------------------------------------- host-direct staging
// On a GPU that reaches pageable host memory through the host's own page
// tables (Grace with NVLink-C2C: cudaDevAttrPageableMemoryAccess and
// cudaDevAttrPageableMemoryAccessUsesHostPageTables), the synchronous ABI
// calls move only the grid blocks their visibilities touch instead of the
// whole grid: a mark kernel flags every kBlk x kBlk block that a kept
// footprint overlaps (the same index math and bounds rule as the gridder, so
// no kept tap falls outside a marked block); gridding accumulates into a
// device buffer zeroed on the marked blocks, and a flush kernel adds those
// blocks into the caller's grid in place, with loads and stores over the link;
// degridding gathers the marked blocks of the caller's grid into a device
// buffer whose other blocks are zeroed.  The kernels touch the caller's
// buffer only inside the region its buffer_t describes (rows of W complex
// elements, `row` doubles apart).  Elsewhere, for a host buffer that is not
// 16-byte aligned, or with RC_GB300_HOST_DIRECT=0 in the environment, the
// whole grid is copied as before (host_direct, gb_runtime.cu).
constexpr int kBlk = 32;

// marks[by * nbx + bx] = 1 for every block a kept footprint overlaps
__global__ void k_mark_blocks(int64_t n, const double* __restrict__ vis5, SingleGeo geo, int nbx,
                              unsigned char* __restrict__ marks) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const VisIndex ix = vis_index(vis5[5 * t], vis5[5 * t + 1], geo.scale, geo.grid_size, geo.S,
                                  geo.margin, geo.min_x, geo.min_y, geo.ext_x, geo.ext_y);
    if (!ix.keep) continue;
    const int x0 = ix.x0 - geo.min_x, y0 = ix.y0 - geo.min_y;
    const int bx1 = (x0 + geo.S - 1) / kBlk, by1 = (y0 + geo.S - 1) / kBlk;
    for (int by = y0 / kBlk; by <= by1; by++)
      for (int bx = x0 / kBlk; bx <= bx1; bx++) marks[by * nbx + bx] = 1;
  }
}

// One CTA per block of a W x H complex128 region (device rows W apart):
// zero the marked blocks.
__global__ void k_zero_marked(double2* __restrict__ d, int W, int H, int nbx,
                              const unsigned char* __restrict__ marks) {
  const int b = blockIdx.x;
  if (!marks[b]) return;
  const int bx = b % nbx, by = b / nbx;
  for (int k = threadIdx.x; k < kBlk * kBlk; k += blockDim.x) {
    const int x = bx * kBlk + (k % kBlk), y = by * kBlk + k / kBlk;
    if (x < W && y < H) d[(int64_t)y * W + x] = make_double2(0.0, 0.0);
  }
}

// host grid (rows `row` doubles apart) += d over the marked blocks
__global__ void k_flush_host(double* __restrict__ host, int64_t row,
                             const double2* __restrict__ d, int W, int H, int nbx,
                             const unsigned char* __restrict__ marks) {
  const int b = blockIdx.x;
  if (!marks[b]) return;
  const int bx = b % nbx, by = b / nbx;
  for (int k = threadIdx.x; k < kBlk * kBlk; k += blockDim.x) {
    const int x = bx * kBlk + (k % kBlk), y = by * kBlk + k / kBlk;
    if (x < W && y < H) {
      double2* hp = reinterpret_cast<double2*>(host + (int64_t)y * row) + x;
      const double2 a = *hp, v = d[(int64_t)y * W + x];
      *hp = make_double2(a.x + v.x, a.y + v.y);
    }
  }
}

// d = the host grid on the marked blocks (the other blocks are not written:
// nothing reads them), and *exp max-ed with the largest exponent field of
// what was read (k_max_exponent's rule)
__global__ void k_gather_host(double2* __restrict__ d, const double* __restrict__ host,
                              int64_t row, int W, int H, int nbx,
                              const unsigned char* __restrict__ marks, int* __restrict__ exp) {
  const int b = blockIdx.x;
  if (!marks[b]) return;
  const int bx = b % nbx, by = b / nbx;
  int m = 0;
  for (int k = threadIdx.x; k < kBlk * kBlk; k += blockDim.x) {
    const int x = bx * kBlk + (k % kBlk), y = by * kBlk + k / kBlk;
    if (x < W && y < H) {
      const double2 v = *(reinterpret_cast<const double2*>(host + (int64_t)y * row) + x);
      d[(int64_t)y * W + x] = v;
      const unsigned long long bits[2] = {(unsigned long long)__double_as_longlong(v.x),
                                          (unsigned long long)__double_as_longlong(v.y)};
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int e = (int)((bits[h] >> 52) & 0x7FF);
        m = max(m, e == 0 && (bits[h] & 0xFFFFFFFFFFFFFull) ? kExpNonFinite : e);
      }
    }
  }
  m = __reduce_max_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0 && m) atomicMax(exp, m);
}

// The double-float split of d (W x H, rows W apart) on the marked blocks,
// under the scale of exps[0] (nothing when either exponent is non-finite).
__global__ void k_df_split_marked(const double2* __restrict__ d, int W, int H, int nbx,
                                  const unsigned char* __restrict__ marks,
                                  const int* __restrict__ exps, float4* __restrict__ out) {
  const int b = blockIdx.x;
  if (!marks[b] || exps[0] == kExpNonFinite || exps[1] == kExpNonFinite) return;
  const int k0 = df_scale_exp(exps[0]);
  const int bx = b % nbx, by = b / nbx;
  for (int k = threadIdx.x; k < kBlk * kBlk; k += blockDim.x) {
    const int x = bx * kBlk + (k % kBlk), y = by * kBlk + k / kBlk;
    if (x < W && y < H) {
      const double2 v = d[(int64_t)y * W + x];
      const float2 re = df_split((unsigned long long)__double_as_longlong(v.x), k0);
      const float2 im = df_split((unsigned long long)__double_as_longlong(v.y), k0);
      out[(int64_t)y * W + x] = make_float4(re.x, re.y, im.x, im.y);
    }
  }
}

// Marks of the kept footprints of n device records over a W x H region.
static int mark_blocks(int64_t n, const void* d_vis, const SingleGeo& geo, int nbx, int nby,
                       unsigned char* marks, cudaStream_t s) {
  GB_CUDA_TRY(cudaMemsetAsync(marks, 0, (size_t)nbx * nby, s));
  const int blocks = (int)std::clamp<int64_t>((n + 255) / 256, 1, (int64_t)sm_count() * 8);
  k_mark_blocks<<<blocks, 256, 0, s>>>(n, (const double*)d_vis, geo, nbx, marks);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

// Counting sort of a call's records by the kBlk x kBlk block of their
// footprint corner (kept records; the others last), on the device: a
// histogram, a one-block exclusive scan, a scatter of record indices.
__device__ __forceinline__ int block_key(const double* __restrict__ vis5, int64_t t,
                                         const SingleGeo& geo, int nbx, int nkeys) {
  const VisIndex ix = vis_index(vis5[5 * t], vis5[5 * t + 1], geo.scale, geo.grid_size, geo.S,
                                geo.margin, geo.min_x, geo.min_y, geo.ext_x, geo.ext_y);
  return ix.keep ? ((ix.y0 - geo.min_y) / kBlk) * nbx + (ix.x0 - geo.min_x) / kBlk : nkeys - 1;
}

__global__ void k_key_hist(int64_t n, const double* __restrict__ vis5, SingleGeo geo, int nbx,
                           int nkeys, int32_t* __restrict__ hist) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&hist[block_key(vis5, t, geo, nbx, nkeys)], 1);
}

// offs = exclusive scan of hist over nkeys entries (one block of 1024 threads)
__global__ void __launch_bounds__(1024) k_scan_keys(const int32_t* __restrict__ hist,
                                                    int32_t* __restrict__ offs, int nkeys) {
  __shared__ int32_t part[1024];
  const int tid = threadIdx.x, chunk = (nkeys + 1023) / 1024;
  const int k0 = min(nkeys, tid * chunk), k1 = min(nkeys, k0 + chunk);
  int32_t sum = 0;
  for (int k = k0; k < k1; k++) sum += hist[k];
  part[tid] = sum;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    const int32_t a = tid >= off ? part[tid - off] : 0;
    __syncthreads();
    part[tid] += a;
    __syncthreads();
  }
  int32_t pre = part[tid] - sum;
  for (int k = k0; k < k1; k++) {
    offs[k] = pre;
    pre += hist[k];
  }
}

__global__ void k_key_scatter(int64_t n, const double* __restrict__ vis5, SingleGeo geo, int nbx,
                              int nkeys, const int32_t* __restrict__ offs,
                              int32_t* __restrict__ cursor, int32_t* __restrict__ order) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int k = block_key(vis5, t, geo, nbx, nkeys);
    order[offs[k] + atomicAdd(&cursor[k], 1)] = (int32_t)t;
  }
}

// The visit order of n device records (staging slots 7 and 8).
static int order_by_block(int64_t n, const void* d_vis, const SingleGeo& geo, int32_t** order,
                          cudaStream_t s) {
  const int nbx = (geo.ext_x + kBlk - 1) / kBlk, nby = (geo.ext_y + kBlk - 1) / kBlk;
  const int nkeys = nbx * nby + 1;
  void *d_keys, *d_order;
  int rc;
  if ((rc = stage_buffer(7, (size_t)3 * nkeys * sizeof(int32_t), &d_keys)) ||
      (rc = stage_buffer(8, (size_t)n * sizeof(int32_t), &d_order)))
    return rc;
  int32_t* hist = (int32_t*)d_keys;
  int32_t* offs = hist + nkeys;
  int32_t* cursor = offs + nkeys;
  GB_CUDA_TRY(cudaMemsetAsync(hist, 0, sizeof(int32_t) * nkeys, s));
  GB_CUDA_TRY(cudaMemsetAsync(cursor, 0, sizeof(int32_t) * nkeys, s));
  const int blocks = (int)std::clamp<int64_t>((n + 255) / 256, 1, (int64_t)sm_count() * 8);
  const double* v = (const double*)d_vis;
  k_key_hist<<<blocks, 256, 0, s>>>(n, v, geo, nbx, nkeys, hist);
  k_scan_keys<<<1, 1024, 0, s>>>(hist, offs, nkeys);
  k_key_scatter<<<blocks, 256, 0, s>>>(n, v, geo, nbx, nkeys, offs, cursor, (int32_t*)d_order);
  GB_CUDA_TRY(cudaGetLastError());
  *order = (int32_t*)d_order;
  return GB_OK;
}

// Exponents and double-float splits of a grid region (ext_y rows of ext_x
// complex elements, `pitch` apart) and of n_gcf complex GCF elements.
static int df_prepare(const double* grid, int32_t ext_x, int32_t ext_y, int64_t pitch,
                      const double* gcf, int64_t n_gcf, float4* grid_df, float4* gcf_df,
                      int* exps, cudaStream_t s) {
  GB_CUDA_TRY(cudaMemsetAsync(exps, 0, 2 * sizeof(int), s));
  const int64_t row = 2 * (int64_t)ext_x;
  const dim3 gg((unsigned)std::clamp<int64_t>((row + 255) / 256, 1, 64),
                (unsigned)std::clamp<int64_t>(ext_y, 1, 4096));
  const dim3 gc((unsigned)std::clamp<int64_t>((2 * n_gcf + 255) / 256, 1, (int64_t)sm_count() * 4),
                1);
  k_max_exponent<<<gg, 256, 0, s>>>(grid, ext_y, row, 2 * pitch, exps);
  k_max_exponent<<<gc, 256, 0, s>>>(gcf, 1, 2 * n_gcf, 2 * n_gcf, exps + 1);
  k_df_split<<<gg, 256, 0, s>>>(grid, ext_y, row, 2 * pitch, exps, 0, (float2*)grid_df);
  k_df_split<<<gc, 256, 0, s>>>(gcf, 1, 2 * n_gcf, 2 * n_gcf, exps, 1, (float2*)gcf_df);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

// ---------------------------------------------------------------- ABI gridding in shared memory
// kern_scatter_gpu1 and its siblings (every GCF size they accept: 8, 16, 32
// and 64).  A call's kept records, counting-sorted by the kBlk x kBlk block of
// their footprint corner (order_by_block), are cut into chunks of up to
// ScatShape<S>::CH consecutive records (fewer for a call with few records),
// one CTA per chunk.  A CTA accumulates the records of
// one block at a time in shared memory, over the block's footprint region
// ((kBlk + S - 1)^2 pixels), in the degridders' double-float arithmetic
// (products and sums err by about 2^-48 of their size); each thread owns the
// region's pixels of its residues (x mod S, y mod S), so that every tap is an
// exclusive read-modify-write, with no atomics.  When the block changes, the
// non-zero pixels of the segment's footprints are added into the device grid
// by FP64 atomics (regions of neighbouring blocks overlap, and a block's
// records may span two chunks) and cleared.  With an Inf, a NaN or a
// subnormal in the visibilities or the GCF, the chunk is gridded by the FP64
// atomics of warp_scatter64 instead, so that those propagate as FP64 would.
template <int S>
struct ScatShape {
  static constexpr int NT = S == 64 ? 1024 : S == 8 ? 64 : 256;  // threads per CTA
  static constexpr int R = S * S / NT;            // residue slots per thread
  static constexpr int DR = NT / S;               // residue rows between a thread's slots
  static constexpr int CH = S <= 16 ? 512 : S == 32 ? 256 : 128;  // at most, records per CTA
  static constexpr int CPS = S == 8 ? 8 : S == 16 ? 5 : S == 32 ? 3 : 1;  // CTAs per SM
  static constexpr int RA = kBlk + S - 1;         // region edge (pixels)
  static constexpr int As = (RA + 7) & ~7;        // region row stride (float4)
};

struct ScatRec {
  float4 vis;      // (re hi, re lo, im hi, im lo) under the visibilities' scale
  int32_t x0, y0;  // footprint corner relative to its block's origin (0 .. kBlk-1)
  int32_t phase;   // GCF oversampling phase
  int32_t key;     // block
};

template <int S>
constexpr size_t scatter_blocks_smem() {
  using Z = ScatShape<S>;
  return sizeof(float4) * Z::RA * Z::As + sizeof(ScatRec) * Z::NT;
}

template <int S>
__global__ void __launch_bounds__(ScatShape<S>::NT)
    k_scatter_blocks_df(const double* __restrict__ vis5, const int32_t* __restrict__ order,
                        const int32_t* __restrict__ offs, int nkeys, int nbx,
                        const double2* __restrict__ gcf, const float4* __restrict__ gcf_df,
                        const int* __restrict__ exps, double2* __restrict__ grid, SingleGeo geo,
                        int ch) {
  using Z = ScatShape<S>;
  extern __shared__ __align__(16) unsigned char smem[];
  float4* acc = (float4*)smem;
  ScatRec* srec = (ScatRec*)(acc + Z::RA * Z::As);
  const int64_t n_kept = offs[nkeys - 1];  // the records without a kept footprint come last
  const int64_t c0 = (int64_t)blockIdx.x * ch;
  if (c0 >= n_kept) return;
  const int64_t c1 = min(n_kept, c0 + ch);
  const int t = threadIdx.x;
  if (exps[0] == kExpNonFinite || exps[1] == kExpNonFinite) {
    const int lane = t & 31;
    for (int64_t k = c0 + (t >> 5); k < c1; k += Z::NT / 32) {
      const double* r = vis5 + 5 * (int64_t)order[k];
      const VisIndex ix = vis_index(r[0], r[1], geo.scale, geo.grid_size, S, geo.margin,
                                    geo.min_x, geo.min_y, geo.ext_x, geo.ext_y);
      warp_scatter64(grid + (int64_t)(ix.y0 - geo.min_y) * geo.pitch + (ix.x0 - geo.min_x),
                     geo.pitch, gcf + (int64_t)ix.phase * S * S, S, r[3], r[4], lane);
    }
    return;
  }
  const int kv = df_scale_exp(exps[0]);
  const int kt = kv + df_scale_exp(exps[1]);
  const double sc = df_pow2(kt);
  for (int q = t; q < Z::RA * Z::As; q += Z::NT) acc[q] = make_float4(0.f, 0.f, 0.f, 0.f);
  const int ra = t % S, rb0 = t / S;
  int cur = -1;                        // the segment's block
  int xlo = 0, ylo = 0, xhi = 0, yhi = 0;  // its footprint corners' bounds
  // the segment's pixels into the grid, and the region cleared
  auto flush = [&]() {
    __syncthreads();  // every tap of the segment is in
    const int ox = (cur % nbx) * kBlk, oy = (cur / nbx) * kBlk;
    const int w = xhi - xlo + S, h = yhi - ylo + S;
    for (int q = t; q < w * h; q += Z::NT) {
      const int yy = ylo + q / w, xx = xlo + q % w;
      float4* a = acc + yy * Z::As + xx;
      const float4 v = *a;
      if (v.x != 0.f || v.y != 0.f || v.z != 0.f || v.w != 0.f) {
        const int gx = ox + xx, gy = oy + yy;
        if (gx < geo.ext_x && gy < geo.ext_y) {
          double2* p = grid + (int64_t)gy * geo.pitch + gx;
          const double2 d = df_to_double_sc(v, kt, sc);
          atomicAdd(&p->x, d.x);
          atomicAdd(&p->y, d.y);
        }
        *a = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
    __syncthreads();  // cleared before the next segment's taps
  };
  for (int64_t b = c0; b < c1; b += Z::NT) {
    const int nb = (int)min((int64_t)Z::NT, c1 - b);
    __syncthreads();  // the previous batch is consumed
    if (t < nb) {
      const double* r = vis5 + 5 * (int64_t)order[b + t];
      const VisIndex ix = vis_index(r[0], r[1], geo.scale, geo.grid_size, S, geo.margin,
                                    geo.min_x, geo.min_y, geo.ext_x, geo.ext_y);
      const int x = ix.x0 - geo.min_x, y = ix.y0 - geo.min_y;
      ScatRec d;
      d.key = (y / kBlk) * nbx + x / kBlk;
      d.x0 = x % kBlk;
      d.y0 = y % kBlk;
      d.phase = ix.phase;
      const float2 re = df_split((unsigned long long)__double_as_longlong(r[3]), kv);
      const float2 im = df_split((unsigned long long)__double_as_longlong(r[4]), kv);
      d.vis = make_float4(re.x, re.y, im.x, im.y);
      srec[t] = d;
    }
    __syncthreads();
    for (int k = 0; k < nb; k++) {
      const ScatRec d = srec[k];  // the same record for every thread
      if (d.key != cur) {
        if (cur >= 0) flush();
        cur = d.key;
        xlo = xhi = d.x0;
        ylo = yhi = d.y0;
      } else {
        xlo = min(xlo, d.x0);
        xhi = max(xhi, d.x0);
        ylo = min(ylo, d.y0);
        yhi = max(yhi, d.y0);
      }
      const int i = (ra - d.x0) & (S - 1), ym = d.y0;
      const float4* g = gcf_df + (int64_t)d.phase * S * S + i;
      float4* a = acc + d.y0 * Z::As + d.x0 + i;
#pragma unroll 4
      for (int m = 0; m < Z::R; m++) {
        const int j = (rb0 + m * Z::DR - ym) & (S - 1);
        const float4 c = __ldg(g + j * S);
        float4 v = a[j * Z::As];
        df_cmac<false>(d.vis, c, v);
        a[j * Z::As] = v;
      }
    }
  }
  if (cur >= 0) flush();
}

// Gridding of a call's n device records into the device grid `grid` (W x H,
// rows W apart; zero, or zero on the blocks the records touch): the
// shared-memory double-float kernel for GCF sizes 8, 16, 32 and 64, the warp
// kernel with FP64 atomics otherwise.  Staging slots 5 (GCF split, exponents),
// 7 and 8 (the records' order).
static int scatter_records(int64_t n, const void* d_vis, const void* d_gcf, double2* grid,
                           const SingleGeo& geo, const int32_t* order, cudaStream_t s) {
  const int S = geo.S;
  int rc;
  if (!order && (rc = order_by_block(n, d_vis, geo, (int32_t**)&order, s))) return rc;
  if (S != 8 && S != 16 && S != 32 && S != 64) {
    int blocks;
    const int threads = plain_grid_dims(n, &blocks);
    k_scatter_single64<<<blocks, threads, 0, s>>>(n, (const double*)d_vis,
                                                  (const double2*)d_gcf, grid, geo, order);
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
  }
  const int64_t n_gcf = (int64_t)GB_PHASES * S * S;
  void* d_df;
  if ((rc = stage_buffer(5, (size_t)n_gcf * 16 + 16, &d_df))) return rc;
  float4* gcf_df = (float4*)d_df;
  int* exps = (int*)((char*)d_df + (size_t)n_gcf * 16);
  // exps[0]: the visibilities' (fields 3 and 4 of each record), exps[1]: the GCF's
  GB_CUDA_TRY(cudaMemsetAsync(exps, 0, 2 * sizeof(int), s));
  const int vb = (int)std::clamp<int64_t>((n + 255) / 256, 1, 4096);
  const dim3 gc((unsigned)std::clamp<int64_t>((2 * n_gcf + 255) / 256, 1, (int64_t)sm_count() * 4),
                1);
  k_max_exponent<<<dim3(1, vb), 32, 0, s>>>((const double*)d_vis + 3, n, 2, 5, exps);
  k_max_exponent<<<gc, 256, 0, s>>>((const double*)d_gcf, 1, 2 * n_gcf, 2 * n_gcf, exps + 1);
  k_df_split<<<gc, 256, 0, s>>>((const double*)d_gcf, 1, 2 * n_gcf, 2 * n_gcf, exps, 1,
                                (float2*)gcf_df);
  GB_CUDA_TRY(cudaGetLastError());
  const int nbx = (geo.ext_x + kBlk - 1) / kBlk, nby = (geo.ext_y + kBlk - 1) / kBlk;
  const int nkeys = nbx * nby + 1;
  // order_by_block keeps (hist, offs, cursor) in slot 7
  void* d_keys;
  if ((rc = stage_buffer(7, (size_t)3 * nkeys * sizeof(int32_t), &d_keys))) return rc;
  const int32_t* offs = (const int32_t*)d_keys + nkeys;
  // the shared-memory limit of each size's kernel, set once per device
  static std::once_flag attr[4][64];
  int dev = 0;
  GB_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    gb_set_error(GB_ERR_ARG, "device ordinal %d out of range", dev);
    return GB_ERR_ARG;
  }
  auto launch = [&](auto tag) -> int {
    constexpr int SS = decltype(tag)::value;
    using Z = ScatShape<SS>;
    std::call_once(attr[SS == 8 ? 3 : SS == 16 ? 0 : SS == 32 ? 1 : 2][dev], [] {
      cudaFuncSetAttribute(k_scatter_blocks_df<SS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)scatter_blocks_smem<SS>());
    });
    // chunks of up to CH records, smaller for a call too small to give every
    // SM two CTAs' worth (sparse w-bins: their records mostly have a block
    // each, and a CTA then grids one or a few)
    const int64_t ch = std::clamp<int64_t>((n + 2 * Z::CPS * sm_count() - 1) /
                                               (2 * Z::CPS * (int64_t)sm_count()),
                                           1, Z::CH);
    const int64_t chunks = (n + ch - 1) / ch;
    k_scatter_blocks_df<SS><<<(unsigned)chunks, Z::NT, scatter_blocks_smem<SS>(), s>>>(
        (const double*)d_vis, order, offs, nkeys, nbx, (const double2*)d_gcf, gcf_df, exps, grid,
        geo, (int)ch);
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
  };
  return S == 8    ? launch(std::integral_constant<int, 8>{})
         : S == 16 ? launch(std::integral_constant<int, 16>{})
         : S == 32 ? launch(std::integral_constant<int, 32>{})
                   : launch(std::integral_constant<int, 64>{});
}

int df_reserve(DfScratch& d, int64_t grid_elems, int64_t gcf_elems) {
  int rc;
  if (!d.exps && (rc = dev_alloc((void**)&d.exps, 2 * sizeof(int), "FP64 degrid scratch")))
    return rc;
  if ((size_t)grid_elems > d.grid_cap) {
    cudaFree(d.grid);
    d.grid = nullptr;
    d.grid_cap = 0;
    if ((rc = dev_alloc((void**)&d.grid, sizeof(float4) * grid_elems, "FP64 degrid scratch")))
      return rc;
    d.grid_cap = grid_elems;
  }
  if ((size_t)gcf_elems > d.gcf_cap) {
    cudaFree(d.gcf);
    d.gcf = nullptr;
    d.gcf_cap = 0;
    if ((rc = dev_alloc((void**)&d.gcf, sizeof(float4) * gcf_elems, "FP64 degrid scratch")))
      return rc;
    d.gcf_cap = gcf_elems;
  }
  return GB_OK;
}

void DfScratch::release() {
  cudaFree(grid);
  cudaFree(gcf);
  cudaFree(exps);
  grid = gcf = nullptr;
  exps = nullptr;
  grid_cap = gcf_cap = 0;
}

int launch_grid_plain64(const gb_plan* plan, const double* vis, const double* gcf, double* grid,
                        cudaStream_t s) {
  int blocks;
  const int threads = plain_grid_dims(plan->dev.n_vis, &blocks);
  k_grid_plain64<<<blocks, threads, 0, s>>>(plan->dev, (const double2*)vis, (const double2*)gcf,
                                            (double2*)grid);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

int launch_degrid_plain64(const gb_plan* plan, const double* gcf, const double* grid,
                          double* pred, int mode, DfScratch& scratch, cudaStream_t s) {
  const PlanDev& D = plan->dev;
  int rc;
  if ((rc = df_reserve(scratch, (int64_t)D.ext_x * D.ext_y, plan->gcf_len)) ||
      (rc = df_prepare(grid, D.ext_x, D.ext_y, D.pitch, gcf, plan->gcf_len, scratch.grid,
                       scratch.gcf, scratch.exps, s)))
    return rc;
  int blocks;
  const int threads = plain_grid_dims(D.n_vis, &blocks);
  k_degrid_plain64<<<blocks, threads, 0, s>>>(D, (const double2*)gcf, (const double2*)grid,
                                              scratch.gcf, scratch.grid, scratch.exps,
                                              (double2*)pred, mode);
  GB_CUDA_TRY(cudaGetLastError());
  return GB_OK;
}

// A CUDA call of an ABI entry point that has work queued on two streams: on an
// error both streams are drained before returning, so that nothing still
// reads or writes the caller's buffers afterwards.
#define GB_TRY_DRAIN(expr, s_a, s_b)                                              \
  do {                                                                            \
    const cudaError_t _e = (expr);                                                \
    if (_e != cudaSuccess) {                                                      \
      gb_set_error(GB_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #expr,        \
                   cudaGetErrorString(_e));                                       \
      cudaStreamSynchronize(s_a);                                                 \
      cudaStreamSynchronize(s_b);                                                 \
      return GB_ERR_CUDA;                                                         \
    }                                                                             \
  } while (0)

// ---------------------------------------------------------------- buffer_t validation
// GCF size as the reference dispatchers read it (gcf_common.h:8-14).
static int32_t check_size(const buffer_t* gcf) {
  const int32_t size = gcf->extent[1];
  if (gcf->extent[0] == 2 && gcf->extent[2] == size) return size;
  return -1;
}

static bool legacy_size(int32_t S) { return S == 8 || S == 16 || S == 32 || S == 64; }

// GCF constraints of the generated kernels (scatter.cpp:36-41).
static int check_gcf(const buffer_t* g, int32_t S, const char* who) {
  if (!g->host || g->elem_size != 8 || g->stride[0] != 1 || g->stride[1] != 2 ||
      g->stride[2] != 2 * S || g->stride[3] != 2 * S * S || g->extent[3] != GB_PHASES ||
      g->min[0] != 0 || g->min[1] != 0 || g->min[2] != 0 || g->min[3] != 0) {
    gb_set_error(GB_ERR_ARG, "%s: gcf buffer must be dense (2,%d,%d,64) doubles", who, S, S);
    return GB_ERR_ARG;
  }
  return GB_OK;
}

// Visibility buffer: (5, N) doubles, strides (1, 5), min(0) = 0 (scatter.cpp:30-32).
static int check_vis(const buffer_t* v, const char* who, const char* name) {
  if (v->elem_size != 8 || v->extent[0] != 5 || v->stride[0] != 1 || v->min[0] != 0 ||
      v->extent[1] < 0 || (v->extent[1] > 1 && v->stride[1] != 5) ||
      (v->extent[1] > 0 && !v->host)) {
    gb_set_error(GB_ERR_ARG, "%s: %s buffer must be (5,N) doubles with strides (1,5)", who,
                 name);
    return GB_ERR_ARG;
  }
  return GB_OK;
}

// Complex grid buffer: (2, W, H) doubles, strides (1, 2, stride2), stride2 even
// and >= 2W (scatter.cpp:52-54).
static int check_grid(const buffer_t* u, const char* who) {
  if (!u->host || u->elem_size != 8 || u->extent[0] != 2 || u->stride[0] != 1 ||
      u->stride[1] != 2 || u->extent[1] <= 0 || u->extent[2] <= 0 ||
      (u->extent[2] > 1 && (u->stride[2] < 2 * u->extent[1] || (u->stride[2] & 1)))) {
    gb_set_error(GB_ERR_ARG, "%s: grid buffer must be (2,W,H) doubles, strides (1,2,>=2W)", who);
    return GB_ERR_ARG;
  }
  return GB_OK;
}

static int64_t grid_row_doubles(const buffer_t* u) {
  return u->extent[2] > 1 ? (int64_t)u->stride[2] : 2 * (int64_t)u->extent[1];
}

// Synchronous single-GCF gridding on host buffers.
static int compat_scatter(const char* who, int size_err, double scale, int32_t grid_size,
                          int32_t margin, buffer_t* vis, buffer_t* gcf, buffer_t* uvg) {
  if (!vis || !gcf || !uvg) {
    gb_set_error(GB_ERR_ARG, "%s: NULL buffer", who);
    return GB_ERR_ARG;
  }
  const int32_t S = check_size(gcf);
  if (!legacy_size(S)) return size_err;
  int rc;
  if ((rc = check_gcf(gcf, S, who)) || (rc = check_vis(vis, who, "vis")) ||
      (rc = check_grid(uvg, who)))
    return rc;
  const int64_t n = vis->extent[1];
  const int32_t W = uvg->extent[1], H = uvg->extent[2];
  const int64_t row = grid_row_doubles(uvg);
  if (n == 0) return GB_OK;  // the grid is unchanged
  if (host_direct(uvg->host, row)) {
    cudaStream_t s;
    if ((rc = stage_stream(&s))) return rc;
    void *d_vis, *d_gcf, *d_acc, *d_marks;
    const size_t gcf_bytes = (size_t)GB_PHASES * S * S * 16;
    const int nbx = (W + kBlk - 1) / kBlk, nby = (H + kBlk - 1) / kBlk;
    if ((rc = stage_buffer(0, (size_t)n * 40, &d_vis)) ||
        (rc = stage_buffer(1, gcf_bytes, &d_gcf)) ||
        (rc = stage_buffer(4, (size_t)W * H * 16, &d_acc)) ||
        (rc = stage_buffer(6, (size_t)nbx * nby, &d_marks)))
      return rc;
    GB_CUDA_TRY(cudaMemcpyAsync(d_vis, vis->host, (size_t)n * 40, cudaMemcpyHostToDevice, s));
    GB_CUDA_TRY(cudaMemcpyAsync(d_gcf, gcf->host, gcf_bytes, cudaMemcpyHostToDevice, s));
    SingleGeo geo{scale, grid_size, margin, S, uvg->min[1], uvg->min[2], W, H, (int64_t)W};
    unsigned char* marks = (unsigned char*)d_marks;
    int32_t* order = nullptr;
    if ((rc = mark_blocks(n, d_vis, geo, nbx, nby, marks, s)) ||
        (rc = order_by_block(n, d_vis, geo, &order, s)))
      return rc;
    k_zero_marked<<<nbx * nby, 256, 0, s>>>((double2*)d_acc, W, H, nbx, marks);
    if ((rc = scatter_records(n, d_vis, d_gcf, (double2*)d_acc, geo, order, s))) {
      cudaStreamSynchronize(s);
      return rc;
    }
    k_flush_host<<<nbx * nby, 256, 0, s>>>((double*)uvg->host, row, (const double2*)d_acc, W, H,
                                           nbx, marks);
    GB_CUDA_TRY(cudaGetLastError());
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    return GB_OK;
  }
  cudaStream_t s, s2;
  cudaEvent_t* evs;
  if ((rc = stage_stream(&s)) || (rc = stage_aux(&s2, &evs))) return rc;
  const cudaEvent_t ev = evs[0];
  void *d_vis, *d_gcf, *d_grid, *d_acc;
  const size_t gcf_bytes = (size_t)GB_PHASES * S * S * 16;
  const size_t grid_bytes = (size_t)W * H * 16;
  if ((rc = stage_buffer(0, (size_t)n * 40, &d_vis)) || (rc = stage_buffer(1, gcf_bytes, &d_gcf)) ||
      (rc = stage_buffer(2, grid_bytes, &d_grid)) || (rc = stage_buffer(4, grid_bytes, &d_acc)))
    return rc;
  // Visibilities and GCF first.  The kernel then grids into a zeroed buffer on
  // the second stream while the caller's grid comes up on the first; the two
  // are added before the grid goes back.
  GB_CUDA_TRY(cudaMemcpyAsync(d_vis, vis->host, (size_t)n * 40, cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemcpyAsync(d_gcf, gcf->host, gcf_bytes, cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemsetAsync(d_acc, 0, grid_bytes, s));
  GB_CUDA_TRY(cudaEventRecord(ev, s));
  GB_CUDA_TRY(cudaStreamWaitEvent(s2, ev, 0));
  SingleGeo geo{scale, grid_size, margin, S, uvg->min[1], uvg->min[2], W, H, (int64_t)W};
  if ((rc = scatter_records(n, d_vis, d_gcf, (double2*)d_acc, geo, nullptr, s2))) {
    cudaStreamSynchronize(s);
    cudaStreamSynchronize(s2);
    return rc;
  }
  GB_TRY_DRAIN(cudaEventRecord(ev, s2), s, s2);
  GB_TRY_DRAIN(cudaMemcpy2DAsync(d_grid, (size_t)W * 16, uvg->host, (size_t)row * 8,
                                 (size_t)W * 16, H, cudaMemcpyHostToDevice, s),
               s, s2);
  GB_TRY_DRAIN(cudaStreamWaitEvent(s, ev, 0), s, s2);
  const int64_t cells = (int64_t)W * H;
  k_add_c128<<<(unsigned)std::clamp<int64_t>((cells + 255) / 256, 1, (int64_t)sm_count() * 8), 256,
               0, s>>>((double2*)d_grid, (const double2*)d_acc, cells);
  GB_CUDA_TRY(cudaGetLastError());
  GB_CUDA_TRY(cudaMemcpy2DAsync(uvg->host, (size_t)row * 8, d_grid, (size_t)W * 16, (size_t)W * 16,
                                H, cudaMemcpyDeviceToHost, s));
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GB_OK;
}

// Synchronous single-GCF degridding on host buffers.
static int compat_degrid(const char* who, int size_err, double scale, int32_t grid_size,
                         int32_t margin, buffer_t* gcf, buffer_t* uvg, buffer_t* vis,
                         buffer_t* vis_out) {
  if (!vis || !gcf || !uvg || !vis_out) {
    gb_set_error(GB_ERR_ARG, "%s: NULL buffer", who);
    return GB_ERR_ARG;
  }
  const int32_t S = check_size(gcf);
  if (!legacy_size(S)) return size_err;
  int rc;
  if ((rc = check_gcf(gcf, S, who)) || (rc = check_vis(vis, who, "vis")) ||
      (rc = check_vis(vis_out, who, "vis_out")) || (rc = check_grid(uvg, who)))
    return rc;
  // vis_out(f, t) = vis(f, t) over vis_out's region: vis must cover it
  // (degrid.cpp:80-82).
  const int64_t n = vis_out->extent[1];
  const int64_t first = (int64_t)vis_out->min[1] - vis->min[1];
  if (n > 0 && (first < 0 || first + n > vis->extent[1])) {
    gb_set_error(GB_ERR_ARG, "%s: vis does not cover the vis_out region", who);
    return GB_ERR_ARG;
  }
  if (n == 0) return GB_OK;  // nothing to write
  const int32_t W = uvg->extent[1], H = uvg->extent[2];
  const int64_t row = grid_row_doubles(uvg);
  cudaStream_t s;
  if ((rc = stage_stream(&s))) return rc;
  void *d_vis, *d_gcf, *d_grid, *d_out;
  const size_t gcf_bytes = (size_t)GB_PHASES * S * S * 16;
  const size_t grid_bytes = (size_t)W * H * 16;
  // slots 4 / 5: the grid and the GCF as double-float pairs (same sizes), the
  // two exponent words after the GCF's
  void *d_grid_df, *d_gcf_df;
  if ((rc = stage_buffer(0, (size_t)n * 40, &d_vis)) || (rc = stage_buffer(1, gcf_bytes, &d_gcf)) ||
      (rc = stage_buffer(2, grid_bytes, &d_grid)) || (rc = stage_buffer(3, (size_t)n * 40, &d_out)) ||
      (rc = stage_buffer(4, grid_bytes, &d_grid_df)) ||
      (rc = stage_buffer(5, gcf_bytes + 16, &d_gcf_df)))
    return rc;
  int* d_exps = (int*)((char*)d_gcf_df + gcf_bytes);
  GB_CUDA_TRY(cudaMemcpyAsync(d_vis, (const double*)vis->host + 5 * first, (size_t)n * 40,
                              cudaMemcpyHostToDevice, s));
  GB_CUDA_TRY(cudaMemcpyAsync(d_gcf, gcf->host, gcf_bytes, cudaMemcpyHostToDevice, s));
  SingleGeo geo{scale, grid_size, margin, S, uvg->min[1], uvg->min[2], W, H, (int64_t)W};
  const bool direct = host_direct(uvg->host, row);
  if (direct) {
    // only the blocks the visibilities read, straight from the caller's grid
    void* d_marks;
    const int nbx = (W + kBlk - 1) / kBlk, nby = (H + kBlk - 1) / kBlk;
    if ((rc = stage_buffer(6, (size_t)nbx * nby, &d_marks))) return rc;
    unsigned char* marks = (unsigned char*)d_marks;
    if ((rc = mark_blocks(n, d_vis, geo, nbx, nby, marks, s))) return rc;
    // the grid's blocks gathered with their exponent, then split; the GCF's
    // exponent and split as df_prepare makes them
    const int64_t n_gcf = (int64_t)GB_PHASES * S * S;
    const dim3 gc((unsigned)std::clamp<int64_t>((2 * n_gcf + 255) / 256, 1,
                                                (int64_t)sm_count() * 4),
                  1);
    GB_CUDA_TRY(cudaMemsetAsync(d_exps, 0, 2 * sizeof(int), s));
    k_gather_host<<<nbx * nby, 256, 0, s>>>((double2*)d_grid, (const double*)uvg->host, row, W, H,
                                            nbx, marks, d_exps);
    k_max_exponent<<<gc, 256, 0, s>>>((const double*)d_gcf, 1, 2 * n_gcf, 2 * n_gcf, d_exps + 1);
    k_df_split_marked<<<nbx * nby, 256, 0, s>>>((const double2*)d_grid, W, H, nbx, marks, d_exps,
                                                (float4*)d_grid_df);
    k_df_split<<<gc, 256, 0, s>>>((const double*)d_gcf, 1, 2 * n_gcf, 2 * n_gcf, d_exps, 1,
                                  (float2*)d_gcf_df);
    GB_CUDA_TRY(cudaGetLastError());
  } else {
    GB_CUDA_TRY(cudaMemcpy2DAsync(d_grid, (size_t)W * 16, uvg->host, (size_t)row * 8,
                                  (size_t)W * 16, H, cudaMemcpyHostToDevice, s));
    if ((rc = df_prepare((const double*)d_grid, W, H, W, (const double*)d_gcf,
                         (int64_t)GB_PHASES * S * S, (float4*)d_grid_df, (float4*)d_gcf_df,
                         d_exps, s)))
      return rc;
  }
  if (direct) {
    // one launch over the records in grid-block order (neighbouring warps
    // gather from the same grid lines), then one download of the results
    int32_t* order = nullptr;
    if ((rc = order_by_block(n, d_vis, geo, &order, s))) return rc;
    int blocks, pw;
    const int threads = single_degrid_dims(n, &blocks, &pw);
    k_degrid_single64<<<blocks, threads, 0, s>>>(
        n, (const double*)d_vis, (const double2*)d_gcf, (const double2*)d_grid,
        (const float4*)d_gcf_df, (const float4*)d_grid_df, d_exps, (double*)d_out, geo, order,
        pw);
    GB_CUDA_TRY(cudaGetLastError());
    GB_CUDA_TRY(cudaMemcpyAsync(vis_out->host, d_out, (size_t)n * 40, cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    return GB_OK;
  }
  // In chunks of visibilities: every chunk's kernel is queued first, each
  // followed by its event; a chunk's results then go down on the second stream
  // while the later chunks are degridded.  (A copy into pageable memory returns
  // only when done, so a copy issued between two launches would hold back the
  // second.)
  cudaStream_t s2;
  cudaEvent_t* evs;
  if ((rc = stage_aux(&s2, &evs))) return rc;
  const int chunks = n >= (1 << 18) ? kAuxEvents : 1;
  for (int c = 0; c < chunks; c++) {
    const int64_t c0 = n * c / chunks, c1 = n * (c + 1) / chunks;
    int blocks, pw;
    const int threads = single_degrid_dims(c1 - c0, &blocks, &pw);
    k_degrid_single64<<<blocks, threads, 0, s>>>(
        c1 - c0, (const double*)d_vis + 5 * c0, (const double2*)d_gcf, (const double2*)d_grid,
        (const float4*)d_gcf_df, (const float4*)d_grid_df, d_exps, (double*)d_out + 5 * c0, geo,
        nullptr, pw);
    GB_TRY_DRAIN(cudaGetLastError(), s, s2);
    GB_TRY_DRAIN(cudaEventRecord(evs[c], s), s, s2);
  }
  for (int c = 0; c < chunks; c++) {
    const int64_t c0 = n * c / chunks, c1 = n * (c + 1) / chunks;
    GB_TRY_DRAIN(cudaStreamWaitEvent(s2, evs[c], 0), s, s2);
    GB_TRY_DRAIN(cudaMemcpyAsync((double*)vis_out->host + 5 * c0, (const double*)d_out + 5 * c0,
                                 (size_t)(c1 - c0) * 40, cudaMemcpyDeviceToHost, s2),
                 s, s2);
  }
  GB_TRY_DRAIN(cudaStreamSynchronize(s2), s, s2);
  GB_CUDA_TRY(cudaStreamSynchronize(s));
  return GB_OK;
}

}  // namespace gb

using namespace gb;

extern "C" int kern_scatter_gpu1(double scale, int32_t grid_size, int32_t margin_size,
                                 buffer_t* vis, buffer_t* gcf, buffer_t* uvg) {
  return compat_scatter("kern_scatter_gpu1", GB_ERR_SCATTER_GPU_SIZE, scale, grid_size,
                        margin_size, vis, gcf, uvg);
}

#ifdef GB_MS5_ABI
// MS5's gridder binding (MS5/programs/Kernel/Gridder.hs:28-35; the kernel is
// generated by MS5/kernel/cpu/gridding/scatter.cpp:10-121): no margin argument
// and the GCF size fixed at 16.  Its bounds, min .. min + extent - 16 - 1, are
// the MS6 rule with the margin equal to the support.
extern "C" int kern_scatter(double scale, int32_t grid_size, buffer_t* vis, buffer_t* gcf,
                            buffer_t* uvg) {
  if (gcf && check_size(gcf) != 16) {
    gb_set_error(GB_ERR_ARG, "kern_scatter: the GCF must be (2,16,16,64) (MS5/scatter.cpp:36-41)");
    return GB_ERR_ARG;
  }
  return compat_scatter("kern_scatter", GB_ERR_ARG, scale, grid_size, 16, vis, gcf, uvg);
}
#else
extern "C" int kern_scatter(double scale, int32_t grid_size, int32_t margin_size, buffer_t* vis,
                            buffer_t* gcf, buffer_t* uvg) {
  return compat_scatter("kern_scatter", GB_ERR_SCATTER_SIZE, scale, grid_size, margin_size, vis,
                        gcf, uvg);
}
#endif

extern "C" int nvGridder(double scale, int32_t grid_size, int32_t margin_size, buffer_t* vis,
                         buffer_t* gcf, buffer_t* uvg) {
  return compat_scatter("nvGridder", GB_ERR_SCATTER_GPU_SIZE, scale, grid_size, margin_size, vis,
                        gcf, uvg);
}

extern "C" int kern_degrid_gpu1(double scale, int32_t grid_size, int32_t margin_size,
                                buffer_t* gcf, buffer_t* uvg, buffer_t* vis, buffer_t* vis_out) {
  return compat_degrid("kern_degrid_gpu1", GB_ERR_DEGRID_GPU_SIZE, scale, grid_size, margin_size,
                       gcf, uvg, vis, vis_out);
}

extern "C" int kern_degrid(double scale, int32_t grid_size, int32_t margin_size, buffer_t* gcf,
                           buffer_t* uvg, buffer_t* vis, buffer_t* vis_out) {
  return compat_degrid("kern_degrid", GB_ERR_DEGRID_SIZE, scale, grid_size, margin_size, gcf, uvg,
                       vis, vis_out);
}

// kern_init (init.cpp:8-15): zero the complex grid region described by uvg.
// The buffer is host memory and the reference's result is wanted there, so
// this is a host memset of the region (no device round trip), on up to eight
// host threads for a large grid.
extern "C" int kern_init(buffer_t* uvg) {
  if (!uvg) {
    gb_set_error(GB_ERR_ARG, "kern_init: NULL buffer");
    return GB_ERR_ARG;
  }
  int rc = check_grid(uvg, "kern_init");
  if (rc) return rc;
  const int64_t row = grid_row_doubles(uvg);
  double* p = (double*)uvg->host;
  // A large grid is zeroed by several host threads, rows split between them:
  // zeroing is also the first touch of a freshly allocated buffer, so it stays
  // on the host (a GPU touching pages first through the host page tables pays
  // a fault per page).
  const int32_t H = uvg->extent[2];
  const size_t rowb = (size_t)uvg->extent[1] * 16;
  const int nt = (int)std::min<int64_t>(8, (int64_t)H * rowb >> 24);  // one per 16 MB
  auto zero_rows = [p, row, rowb](int32_t y0, int32_t y1) {
    for (int32_t y = y0; y < y1; y++) memset(p + (int64_t)y * row, 0, rowb);
  };
  if (nt < 2) {
    zero_rows(0, H);
    return GB_OK;
  }
  std::vector<std::thread> ts;
  for (int k = 1; k < nt; k++) {
    const int32_t y0 = (int32_t)((int64_t)H * k / nt), y1 = (int32_t)((int64_t)H * (k + 1) / nt);
    try {
      ts.emplace_back(zero_rows, y0, y1);
    } catch (...) {  // no thread to be had: this one does those rows too
      zero_rows(y0, y1);
    }
  }
  zero_rows(0, (int32_t)((int64_t)H / nt));
  for (auto& t : ts) t.join();
  return GB_OK;
}

// kern_psf_vis (psf_vis.cpp:16-27): out = vis with re = 1, im = 0, over
// out's region.  Host buffers, host loop (a 40-byte record copy).
extern "C" int kern_psf_vis(buffer_t* vis, buffer_t* out) {
  if (!vis || !out) {
    gb_set_error(GB_ERR_ARG, "kern_psf_vis: NULL buffer");
    return GB_ERR_ARG;
  }
  int rc;
  if ((rc = check_vis(vis, "kern_psf_vis", "vis")) || (rc = check_vis(out, "kern_psf_vis", "out")))
    return rc;
  const int64_t n = out->extent[1];
  const int64_t first = (int64_t)out->min[1] - vis->min[1];
  if (n > 0 && (first < 0 || first + n > vis->extent[1])) {
    gb_set_error(GB_ERR_ARG, "kern_psf_vis: vis does not cover the output region");
    return GB_ERR_ARG;
  }
  const double* src = (const double*)vis->host + 5 * first;
  double* dst = (double*)out->host;
  for (int64_t t = 0; t < n; t++) {
    dst[5 * t + 0] = src[5 * t + 0];
    dst[5 * t + 1] = src[5 * t + 1];
    dst[5 * t + 2] = src[5 * t + 2];
    dst[5 * t + 3] = 1.0;
    dst[5 * t + 4] = 0.0;
  }
  return GB_OK;
}
