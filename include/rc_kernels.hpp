// rc_kernels.hpp -- C++17 host layer over librc_gb300's reference ABI for the
// gridding path, mirroring the MS6 Haskell kernel bindings that drive it
// (MS6/programs/Kernel/{Config,Data,Binning,IO,Gridder,Degrid,FFT}.hs): the
// same kernel names and argument meanings, the same buffer layouts passed to
// the same C symbols, and an exception where the Haskell marshaller gives up
// with `error "Could not call Halide kernel!"` (MS6/dna/flow/Flow/Halide/
// Marshal.hs:119-124).  Header only; link librc_gb300.so.
//
// The Haskell layer runs these kernels under the Flow scheduler, one call per
// region (a u/v tile, a w-bin); here the caller makes those calls, e.g. the
// gridding strategy of MS6/programs/gridding.hs:
//
//   for each (u, v) tile:   bins = binSizer(gp, vis, u, v)
//                           vb   = binner(gp, vis, u, v, bins)
//                           tile = gridInit(gcfp, u, v)
//                           for each bin b: gridKernel(kt, gp, gcfp, vb[b], gcfKernel(gcfp, b.bin), tile)
//                           gridDetiling(tile, full)            (full = gridInitDetile(...))
//   image = ifftKern(gp, full)
//
// Built with -DGB_MS5_ABI (against librc_gb300_ms5.so) the CPU gridder binds
// MS5's kern_scatter, which takes no margin (MS5/programs/Kernel/Gridder.hs:
// 28-35), and ifftKern binds MS5's kern_fft (MS5/programs/Kernel/FFT.hs:15-16);
// MS5 has no fftKern.
#pragma once

#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "rc_gb300.h"
#include "rc_gb300_ms5.h"
#include "rc_oskar.h"

namespace rc {

// A non-zero status from a kernel call (the status and gb_last_error()).
struct KernelError : std::runtime_error {
  int code;
  KernelError(const std::string& what, int c) : std::runtime_error(what), code(c) {}
};

inline void check(int status, const char* kernel) {
  if (status != 0)
    throw KernelError(std::string("Could not call kernel ") + kernel + " (" +
                          std::to_string(status) + "): " + gb_last_error(),
                      status);
}

// ------------------------------------------------------------ Kernel.Config
// MS6/programs/Kernel/Config.hs:84-95
struct GridPar {
  int width = 0, height = 0, pitch = 0;
  double theta = 0;  // field of view in radians
  int tiles = 1, facets = 1, bins = 1;
};

// Config.hs:106-122
struct GCFFile {
  std::string file;
  int size = 0;
  double w = 0;
};
struct GCFPar {
  std::vector<GCFFile> files;
  int over = 8;
};

// Config.hs:52-66: the symbol each kernel type binds (Gridder.hs:58-63, Degrid.hs:148-152)
enum class GridKernelType { CPU, GPU, NV };
enum class DegridKernelType { CPU, GPU };

// Config.hs:124-125
inline int gcfMaxSize(const GCFPar& p) {
  int m = 0;
  for (const GCFFile& f : p.files) m = std::max(m, f.size);
  return m;
}

// Config.hs:128-132: the file with the largest w <= max(|w0|, |w1|) (the
// last of equal ones); none is an error there too (maximumBy of an empty list).
inline const GCFFile& gcfGet(const GCFPar& p, double w0, double w1) {
  std::vector<double> ws;
  for (const GCFFile& f : p.files) ws.push_back(f.w);
  int32_t index = -1, conj = 0;
  check(gb_gcf_select((int32_t)ws.size(), ws.data(), w0, w1, &index, &conj), "gcfGet");
  return p.files[index];
}

// Config.hs:199-212
inline int gridImageWidth(const GridPar& gp) { return gp.width * gp.facets; }
inline int gridImageHeight(const GridPar& gp) { return gp.height * gp.facets; }
inline double gridScale(const GridPar& gp) { return gp.theta / (double)gp.facets; }
inline double gridXY2UV(const GridPar& gp, int z) {
  return (double)(z - gp.height / 2) / gridScale(gp);
}

// ------------------------------------------------------------ Kernel.Data
// A region of a range domain: pixels [low, high).
struct Range {
  int low = 0, high = 0;
  int size() const { return high - low; }
};

// A region of a bin domain (Flow.Domain RegionBinDesc): w in [low, high),
// `count` records.
struct WBin {
  double low = 0, high = 0;
  int64_t count = 0;
};

namespace detail {
// An allocator whose value-initialisation leaves doubles uninitialised: grid
// and visibility buffers are allocated like Flow's (posix_memalign,
// Flow/Vector.hs:173-190); a grid is zeroed once, by kern_init, and a kernel's
// output records are written whole by the kernel, so neither is zeroed twice.
template <class T>
struct NoInit : std::allocator<T> {
  template <class U>
  struct rebind {
    using other = NoInit<U>;
  };
  NoInit() = default;
  template <class U>
  NoInit(const NoInit<U>&) {}
  template <class U, class... A>
  void construct(U* p, A&&... a) {
    if constexpr (sizeof...(A) == 0)
      ::new ((void*)p) U;
    else
      ::new ((void*)p) U(std::forward<A>(a)...);
  }
};
}  // namespace detail

// Visibilities: 5-double records u, v, w, re, im (Data.hs:115-123).
struct Vis {
  std::vector<double, detail::NoInit<double>> rec;
  int64_t size() const { return (int64_t)rec.size() / 5; }
};

// The visibilities of one (u, v, w-bin) region, zero-padded to its count.
struct VisBin {
  WBin bin;
  Vis vis;
};


// A complex grid region: dims (2, width, height), strides (1, 2, 2 width),
// mins (0, min_u, min_v) (Data.hs:64-76, 93-97).
struct UVGrid {
  std::vector<double, detail::NoInit<double>> data;
  int min_u = 0, min_v = 0, width = 0, height = 0;
};

// GCFs: dims (2, S, S, 64) (Data.hs:125-133).
struct GCFs {
  std::vector<double> data;
  int size = 0;
};

// A real image: dims (width, height), strides (1, width) (Data.hs:81-91).
struct Image {
  std::vector<double> data;
  int width = 0, height = 0;
};

namespace detail {
inline buffer_t make_buffer(double* host, std::initializer_list<int> ext,
                            std::initializer_list<int> str, std::initializer_list<int> mins) {
  buffer_t b{};
  b.host = (uint8_t*)host;
  int k = 0;
  for (int e : ext) b.extent[k++] = e;
  k = 0;
  for (int s : str) b.stride[k++] = s;
  k = 0;
  for (int m : mins) b.min[k++] = m;
  b.elem_size = 8;
  b.host_dirty = true;
  return b;
}
// Flow/Halide.hs:154-171: vis dims (5, N) plus the u/v placeholder dims
inline buffer_t vis_buffer(Vis& v) {
  return make_buffer(v.rec.data(), {5, (int)v.size(), 1, 1}, {1, 5, 0, 0}, {0, 0, 0, 0});
}
inline buffer_t gcf_buffer(GCFs& g) {
  const int S = g.size;
  return make_buffer(g.data.data(), {2, S, S, 64}, {1, 2, 2 * S, 2 * S * S}, {0, 0, 0, 0});
}
inline buffer_t uvg_buffer(UVGrid& g) {
  return make_buffer(g.data.data(), {2, g.width, g.height}, {1, 2, 2 * g.width},
                     {0, g.min_u, g.min_v});
}
inline buffer_t image_buffer(Image& im) {
  return make_buffer(im.data.data(), {im.width, im.height}, {1, im.width}, {0, 0});
}
// A grid region whose values the caller zeroes (kern_init) or overwrites.
inline UVGrid alloc_grid(int min_u, int min_v, int width, int height) {
  UVGrid g;
  g.min_u = min_u;
  g.min_v = min_v;
  g.width = width;
  g.height = height;
  g.data.resize((size_t)2 * width * height);
  return g;
}
inline UVGrid zero_grid(int min_u, int min_v, int width, int height) {
  UVGrid g = alloc_grid(min_u, min_v, width, height);
  std::fill(g.data.begin(), g.data.end(), 0.0);
  return g;
}
}  // namespace detail

// ------------------------------------------------------------ Kernel.Binning
// binSizer (Binning.hs:34-99) for one (u, v) tile: the w range of the
// visibilities inside the tile's u/v range (the fold starts from (0, 0)),
// widened by 1e-4 of itself at the top, cut into gp.bins equal bins, and each
// bin's count by bin = clamp(floor((w - low) / (high - low) * bins)).
inline std::vector<WBin> binSizer(const GridPar& gp, const Vis& vis, Range u, Range v) {
  const double umin = gridXY2UV(gp, u.low), umax = gridXY2UV(gp, u.high);
  const double vmin = gridXY2UV(gp, v.low), vmax = gridXY2UV(gp, v.high);
  auto inside = [&](const double* r) {
    return r[0] >= umin && r[0] < umax && r[1] >= vmin && r[1] < vmax;
  };
  double low = 0, high0 = 0;
  for (int64_t i = 0; i < vis.size(); i++) {
    const double* r = &vis.rec[5 * i];
    if (inside(r)) {
      low = std::min(r[2], low);
      high0 = std::max(r[2], high0);
    }
  }
  const double high = high0 + (high0 - low) * 0.0001;
  const int bins = gp.bins;
  auto start = [&](int b) { return low + (double)b * (high - low) / (double)bins; };
  std::vector<WBin> out(bins);
  for (int b = 0; b < bins; b++) out[b] = WBin{start(b), start(b + 1), 0};
  for (int64_t i = 0; i < vis.size(); i++) {
    const double* r = &vis.rec[5 * i];
    if (!(inside(r) && r[2] >= low && r[2] <= high)) continue;
    // a zero-width range (every w equal) puts everything in bin 0
    const double f = high > low ? std::floor((r[2] - low) / (high - low) * (double)bins) : 0.0;
    const int b = (int)std::max(0.0, std::min((double)(bins - 1), f));
    out[b].count++;
  }
  return out;
}

// binner (Binning.hs:102-181) for one (u, v) tile: each visibility inside the
// tile goes to the bin with the largest low <= w, if w < that bin's high;
// every bin is then padded with zero records to its count.
inline std::vector<VisBin> binner(const GridPar& gp, const Vis& vis, Range u, Range v,
                                  const std::vector<WBin>& bins) {
  const double ul = gridXY2UV(gp, u.low), uh = gridXY2UV(gp, u.high);
  const double vl = gridXY2UV(gp, v.low), vh = gridXY2UV(gp, v.high);
  std::vector<VisBin> out(bins.size());
  for (size_t b = 0; b < bins.size(); b++) out[b].bin = bins[b];
  // binSizer's lows never decrease: lookupLE is then a binary search (the last
  // low <= w is the last of equal lows too)
  std::vector<double> lows(bins.size());
  bool sorted = true;
  for (size_t b = 0; b < bins.size(); b++) {
    lows[b] = bins[b].low;
    sorted = sorted && (b == 0 || !(lows[b] < lows[b - 1])) && lows[b] == lows[b];
  }
  for (int64_t i = 0; i < vis.size(); i++) {
    const double* r = &vis.rec[5 * i];
    if (!(ul <= r[0] && r[0] < uh && vl <= r[1] && r[1] < vh)) continue;
    int k = -1;  // Map.lookupLE over the bins' lows (the last of equal lows)
    if (sorted) {
      k = (int)(std::upper_bound(lows.begin(), lows.end(), r[2]) - lows.begin()) - 1;
    } else {
      for (size_t b = 0; b < bins.size(); b++)
        if (bins[b].low <= r[2] && (k < 0 || bins[b].low >= bins[k].low)) k = (int)b;
    }
    if (k < 0 || !(r[2] < bins[k].high)) continue;
    out[k].vis.rec.insert(out[k].vis.rec.end(), r, r + 5);
  }
  for (VisBin& vb : out)
    if (vb.vis.size() < vb.bin.count) vb.vis.rec.resize((size_t)5 * vb.bin.count, 0.0);
  return out;
}

// ------------------------------------------------------------ Kernel.IO
// gcfKernel (IO.hs:97-115): the GCF file gcfGet picks for the bin's w range,
// read as size^2 * 64 complex doubles, conjugated when the range lies mostly
// at negative w (low < -high).
inline GCFs gcfKernel(const GCFPar& p, const WBin& bin) {
  const GCFFile& f = gcfGet(p, bin.low, bin.high);
  GCFs g;
  g.size = f.size;
  g.data.resize((size_t)2 * f.size * f.size * 64);
  FILE* fp = std::fopen(f.file.c_str(), "rb");
  if (!fp) throw KernelError("gcfKernel: cannot open " + f.file, -1);
  const size_t got = std::fread(g.data.data(), sizeof(double), g.data.size(), fp);
  std::fclose(fp);
  if (got != g.data.size()) throw KernelError("gcfKernel: short read of " + f.file, -1);
  if (bin.low < -bin.high)
    for (size_t i = 1; i < g.data.size(); i += 2) g.data[i] = -g.data[i];
  return g;
}

// The reader's task data (MS6/kernel/oskar/OskarReader.hs:45-80): the file's
// counts and its reshuffled arrays, amplitudes [baseline][time][channel][pol]
// as complex doubles, u,v,w [baseline][time][channel][3] in wavelengths.
struct TaskData {
  int baselines = 0, times = 0, channels = 0, points = 0;
  Metrix metrix{};
  std::vector<WMaxMin> bl_max_min;
  std::vector<double> vis;  // points x 4 complex
  std::vector<double> uvws;  // points x 3
  // tdVisibilityPtr / tdUVWPtr (OskarReader.hs:64-80); the u,v,w address
  // ignores the channel stride, as there.
  const double* visibility(int bl, int t, int ch, int pol) const {
    return &vis[2 * ((size_t)pol + 4 * ((size_t)ch + (size_t)channels * (t + (size_t)times * bl)))];
  }
  const double* uvw(int bl, int t, int o) const {
    return &uvws[(size_t)o + 3 * ((size_t)t + (size_t)times * bl)];
  }
};

// readOskarData (OskarReader.hs:96-131): mkFromFile, readAndReshuffle,
// freeBinHandler; a non-zero status throws with the reader's message.
inline TaskData readOskarData(const std::string& fname) {
  VisData vd;
  const int st = mkFromFile(&vd, fname.c_str());
  if (st != 0)
    throw KernelError("While trying to read binary file " + fname + " : " + std::to_string(st), st);
  TaskData td;
  td.baselines = vd.num_baselines;
  td.times = vd.num_times;
  td.channels = vd.num_channels;
  td.points = vd.num_points;
  td.bl_max_min.resize(td.baselines);
  td.vis.resize((size_t)td.points * 8);
  td.uvws.resize((size_t)td.points * 3);
  const int rd = readAndReshuffle(&vd, td.vis.data(), td.uvws.data(), &td.metrix,
                                  td.bl_max_min.data());
  freeBinHandler(&vd);
  if (rd != 0)
    throw KernelError("While trying to read binary file " + fname + " : " + std::to_string(rd), rd);
  return td;
}

// oskarReader (MS6/programs/Kernel/IO.hs:22-74): 5-double records of points
// [low, high) of one channel and polarisation, [baseline][time] order; the
// region must lie inside the file and start on a baseline, as there.  Two
// differences, both on input the Haskell kernel would read or write out of
// bounds with: freq == channels (its check is freq > channels) and a pol
// outside 0..3 are rejected, and a high that is not baseline-aligned ends the
// records there (the Haskell kernel writes whole baselines past it).
inline Vis oskarReader(const TaskData& td, int freq, int pol, int64_t low, int64_t high) {
  if (freq < 0 || freq >= td.channels)
    throw KernelError("Attempted to read non-existent frequency channel from Oskar data!", -1);
  if (pol < 0 || pol > 3) throw KernelError("oskarReader: polarisation out of range", -1);
  const int64_t total = (int64_t)td.times * td.baselines;
  if (low < 0 || high > total)
    throw KernelError("oskarReader: region out of bounds: " + std::to_string(low) + "-" +
                          std::to_string(high) + " (only have " + std::to_string(total) +
                          " points)",
                      -1);
  if (td.times == 0 || low % td.times != 0)
    throw KernelError("oskarReader: region not baseline-aligned: " + std::to_string(low) + "-" +
                          std::to_string(high),
                      -1);
  Vis out;
  out.rec.reserve((size_t)5 * std::max<int64_t>(0, high - low));
  for (int64_t i = low; i < high; i++) {
    const int bl = (int)(i / td.times), t = (int)(i % td.times);
    out.rec.push_back(*td.uvw(bl, t, 0));
    out.rec.push_back(*td.uvw(bl, t, 1));
    out.rec.push_back(*td.uvw(bl, t, 2));
    const double* v = td.visibility(bl, t, freq, pol);
    out.rec.push_back(v[0]);
    out.rec.push_back(v[1]);
  }
  return out;
}

// ------------------------------------------------------------ Kernel.Gridder
// gridInit (Gridder.hs:25-27): the tile with a margin of gcfMaxSize / 2 on
// every side (Data.hs:71-76), zeroed by kern_init.
inline UVGrid gridInit(const GCFPar& gcfp, Range u, Range v) {
  const int m = gcfMaxSize(gcfp) / 2;
  UVGrid g = detail::alloc_grid(u.low - m, v.low - m, u.size() + 2 * m, v.size() + 2 * m);
  buffer_t b = detail::uvg_buffer(g);
  check(kern_init(&b), "gridInit");
  return g;
}

// gridKernel (Gridder.hs:30-43): grid += vis * gcf through the symbol of the
// kernel type, bound to (gridScale, gridHeight, gcfMaxSize).
inline void gridKernel(GridKernelType kt, const GridPar& gp, const GCFPar& gcfp, VisBin& vb,
                       GCFs& gcf, UVGrid& grid) {
  buffer_t bv = detail::vis_buffer(vb.vis), bg = detail::gcf_buffer(gcf),
           bu = detail::uvg_buffer(grid);
  const double scale = gridScale(gp);
  const int32_t gs = gp.height, margin = gcfMaxSize(gcfp);
  switch (kt) {
    case GridKernelType::CPU:
#ifdef GB_MS5_ABI
      check(kern_scatter(scale, gs, &bv, &bg, &bu), "kern_scatter");
#else
      check(kern_scatter(scale, gs, margin, &bv, &bg, &bu), "kern_scatter");
#endif
      break;
    case GridKernelType::GPU:
      check(kern_scatter_gpu1(scale, gs, margin, &bv, &bg, &bu), "kern_scatter_gpu1");
      break;
    case GridKernelType::NV:
      check(nvGridder(scale, gs, margin, &bv, &bg, &bu), "nvGridder");
      break;
  }
}

// gridInitDetile (Gridder.hs:76-77): the full grid without margins, zeroed.
inline UVGrid gridInitDetile(Range u, Range v) {
  UVGrid g = detail::alloc_grid(u.low, v.low, u.size(), v.size());
  buffer_t b = detail::uvg_buffer(g);
  check(kern_init(&b), "gridInitDetile");
  return g;
}

// gridDetiling (Gridder.hs:81-85): full += tile over their overlap.
inline void gridDetiling(UVGrid& tile, UVGrid& full) {
  buffer_t bi = detail::uvg_buffer(tile), bo = detail::uvg_buffer(full);
  check(kern_detile(&bi, &bo), "gridDetiling");
}

// ------------------------------------------------------------ Kernel.Degrid
// degridKernel (Degrid.hs:34-47): vis_out = vis - sum grid * gcf over the full
// grid, through the symbol of the kernel type.
inline Vis degridKernel(DegridKernelType kt, const GridPar& gp, const GCFPar& gcfp, GCFs& gcf,
                        UVGrid& full, Vis& vis) {
  Vis out;
  out.rec.resize(vis.rec.size());  // every record is written by the call
  buffer_t bg = detail::gcf_buffer(gcf), bu = detail::uvg_buffer(full),
           bv = detail::vis_buffer(vis), bo = detail::vis_buffer(out);
  const double scale = gridScale(gp);
  const int32_t gs = gp.height, margin = gcfMaxSize(gcfp);
  if (kt == DegridKernelType::CPU)
    check(kern_degrid(scale, gs, margin, &bg, &bu, &bv, &bo), "kern_degrid");
  else
    check(kern_degrid_gpu1(scale, gs, margin, &bg, &bu, &bv, &bo), "kern_degrid_gpu1");
  return out;
}

// ------------------------------------------------------------ Kernel.Cleaning
// Config.hs:134-138
struct CleanPar {
  double gain = 0.1, threshold = 0;
  int cycles = 0;
};

// psfVisKernel (Cleaning.hs:15-19): the visibilities with re = 1, im = 0.
inline Vis psfVisKernel(Vis& vis) {
  Vis out;
  out.rec.assign(vis.rec.size(), 0.0);
  buffer_t bi = detail::vis_buffer(vis), bo = detail::vis_buffer(out);
  check(kern_psf_vis(&bi, &bo), "kern_psf_vis");
  return out;
}

// cleanModel (Cleaning.hs:22-32): Hogbom CLEAN of `res` with `psf`,
// accumulating into `model` (written in place, as halideKernel2Write does).
inline void cleanModel(const CleanPar& cp, Image& psf, Image& res, Image& model) {
  buffer_t bp = detail::image_buffer(psf), br = detail::image_buffer(res),
           bm = detail::image_buffer(model);
  check(kern_hogbom_model(cp.gain, cp.threshold, &bp, &br, &bm), "kern_hogbom_model");
}

// cleanResidual (Cleaning.hs:35-44): the residual image of the same CLEAN.
inline Image cleanResidual(const CleanPar& cp, Image& psf, Image& res) {
  Image out;
  out.width = res.width;
  out.height = res.height;
  out.data.assign(res.data.size(), 0.0);
  buffer_t bp = detail::image_buffer(psf), br = detail::image_buffer(res),
           bo = detail::image_buffer(out);
  check(kern_hogbom_residual(cp.gain, cp.threshold, &bp, &br, &bo), "kern_hogbom_residual");
  return out;
}

// ------------------------------------------------------------ Kernel.Facet
// rotateKernel (Facet.hs:19-54) for the facet of pixel ranges (l, m): phase
// rotation of raw visibilities from the phase centre (lon, lat) to the
// facet's centre, without uvw reprojection (the binding fixes doRep = False).
inline Vis rotateKernel(const GridPar& gp, double lon, double lat, Range l, Range m, Vis& vis) {
  const double facets = (double)gp.facets;
  const double lon_incr = gp.theta / (double)gp.width / facets;  // radians per pixel
  const double lat_incr = gp.theta / (double)gp.height / facets;
  const double lon0 = lon - lon_incr * (double)(gridImageWidth(gp) / 2 - gp.width / 2);
  const double lat0 = lat - lat_incr * (double)(gridImageHeight(gp) / 2 - gp.height / 2);
  Vis out;
  out.rec.assign(vis.rec.size(), 0.0);
  buffer_t bi = detail::vis_buffer(vis);
  // RotatedVisRepr (Data.hs:109-113): the facet's l / m region lows in dims 2 / 3
  buffer_t bo = detail::make_buffer(out.rec.data(), {5, (int)out.size(), 1, 1}, {1, 5, 0, 0},
                                    {0, 0, l.low, m.low});
  check(kern_rotate(lon, lat, lon0, lat0, lon_incr, lat_incr, 0, &bi, &bo), "kern_rotate");
  return out;
}

// ------------------------------------------------------------ Kernel.FFT
// ifftKern (FFT.hs:18-20): grid -> facet image (kern_ifft; the facet is
// width x height, Data.hs:81-85).  MS5: its kern_fft, grid -> image.
inline Image ifftKern(const GridPar& gp, UVGrid& full) {
  Image im;
  im.width = gp.width;
  im.height = gp.height;
  im.data.assign((size_t)im.width * im.height, 0.0);
  buffer_t bu = detail::uvg_buffer(full), bi = detail::image_buffer(im);
#ifdef GB_MS5_ABI
  check(kern_fft(&bu, &bi), "kern_fft");
#else
  check(kern_ifft(&bu, &bi), "kern_ifft");
#endif
  return im;
}

#ifndef GB_MS5_ABI
// fftKern (FFT.hs:14-16): image -> full grid (kern_fft; both of the image size,
// Data.hs:87-97).
inline UVGrid fftKern(const GridPar& gp, Image& im) {
  UVGrid g = detail::zero_grid(0, 0, gridImageWidth(gp), gridImageHeight(gp));
  buffer_t bi = detail::image_buffer(im), bu = detail::uvg_buffer(g);
  check(kern_fft(&bi, &bu), "kern_fft");
  return g;
}
#endif

}  // namespace rc
