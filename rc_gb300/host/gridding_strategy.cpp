// The gridding strategy of MS6/programs/gridding.hs:40-103, restated on the
// C++ host layer (include/rc_kernels.hpp) for the parity tests and the
// drop-in timing of the benchmark: for every
// (u, v) tile, binSizer + binner, gridInit, one gridKernel per w-bin with
// the bin's GCF (gcfKernel), gridDetiling into the full grid; then ifftKern.
// With a model grid it also degrids every binned visibility (degridKernel),
// as the continuum strategy does against its model; `clean` images the
// visibilities and their PSF (psfVisKernel) and CLEANs (cleanModel,
// cleanResidual); `rotate` phase-rotates them to a facet (rotateKernel);
// `oskar` reads an OSKAR file's records (readOskarData, oskarReader).
//
// `time` runs gridding (every tile's w-bins, detiled into the full grid) and
// degridding (every binned visibility against the model grid) K times after W
// warm-up passes, the binning and the GCF reads done once beforehand (they
// belong to the observation, not to a pass), and prints one JSON line of
// per-pass wall times.
//
// `continuum` runs the major loop of MS6/programs/continuum.hs over these
// kernels (fftKern, degridKernel, gridKernel, ifftKern, cleanModel,
// cleanResidual) and writes the model and the final residual.
//
// usage: gridding_strategy DIR MODE
//        MODE = bins | grid | degrid | clean | continuum | rotate | oskar | time
//   DIR/params.txt   width height theta tiles bins n_gcf grid_kernel degrid_kernel
//                    then n_gcf lines "file size w"
//   DIR/vis.bin      N x 5 doubles (u v w re im)
//   DIR/model.bin    width x height complex doubles (degrid)
//   DIR/clean.txt    gain threshold (clean)
//   DIR/rotate.txt   facets lon lat l_low m_low (rotate)
//   DIR/oskar.txt    file freq pol low high (oskar)
//   DIR/time.txt     warmup steps (time; needs DIR/model.bin)
//   DIR/continuum.txt  loops (continuum; with DIR/clean.txt)
// writes DIR/bins.bin (per tile, per bin: low high count, then the binned
// records), DIR/grid.bin, DIR/image.bin, DIR/pred.bin (the degridded records
// in tile, bin order), DIR/clean_model.bin + DIR/clean_residual.bin,
// DIR/rot.bin, DIR/oskar.bin, DIR/cont_model.bin + DIR/cont_residual.bin.
#include <chrono>
#include <cstdio>
#include <string>
#include <vector>

#include "rc_kernels.hpp"

static std::vector<double> read_doubles(const std::string& path) {
  std::vector<double> v;
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return v;
  double x[4096];
  size_t k;
  while ((k = std::fread(x, sizeof(double), 4096, f)) > 0) v.insert(v.end(), x, x + k);
  std::fclose(f);
  return v;
}

template <class V>
static void write_doubles(const std::string& path, const V& v) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) throw rc::KernelError("cannot write " + path, -1);
  std::fwrite(v.data(), sizeof(double), v.size(), f);
  std::fclose(f);
}

// Tiles, bins, per-bin gridding, detiling (gridding.hs:58-97): the full grid.
static rc::UVGrid grid_tiles(rc::GridKernelType kt, const rc::GridPar& gp, const rc::GCFPar& gcfp,
                             const rc::Vis& vis) {
  rc::UVGrid full = rc::gridInitDetile({0, gp.width}, {0, gp.height});
  for (int tv = 0; tv < gp.tiles; tv++)
    for (int tu = 0; tu < gp.tiles; tu++) {
      // split of a range domain: low + (high - low) * i div n (Flow/Domain.hs:36-39)
      const rc::Range u{tu * gp.width / gp.tiles, (tu + 1) * gp.width / gp.tiles};
      const rc::Range v{tv * gp.height / gp.tiles, (tv + 1) * gp.height / gp.tiles};
      std::vector<rc::VisBin> vb = rc::binner(gp, vis, u, v, rc::binSizer(gp, vis, u, v));
      rc::UVGrid tile = rc::gridInit(gcfp, u, v);
      for (rc::VisBin& b : vb) {
        if (b.vis.size() == 0) continue;
        rc::GCFs g = rc::gcfKernel(gcfp, b.bin);
        rc::gridKernel(kt, gp, gcfp, b, g, tile);
      }
      rc::gridDetiling(tile, full);
    }
  return full;
}

static double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

// `time` mode: the gridding and degridding passes of the strategy, timed.
static void time_passes(const std::string& dir, rc::GridKernelType gkt, rc::DegridKernelType dkt,
                        const rc::GridPar& gp, const rc::GCFPar& gcfp, const rc::Vis& vis,
                        rc::UVGrid& model) {
  int warmup = 1, steps = 3;
  FILE* tf = std::fopen((dir + "/time.txt").c_str(), "r");
  if (!tf || std::fscanf(tf, "%d %d", &warmup, &steps) != 2)
    throw rc::KernelError("bad time.txt", -1);
  std::fclose(tf);
  struct Region {
    rc::Range u, v;
    std::vector<rc::VisBin> vb;
    std::vector<rc::GCFs> g;
  };
  // the observation's regions: binSizer + binner per tile, then the GCF reads
  const double tb0 = now_ms();
  std::vector<Region> regions;
  for (int tv = 0; tv < gp.tiles; tv++)
    for (int tu = 0; tu < gp.tiles; tu++) {
      Region r;
      r.u = {tu * gp.width / gp.tiles, (tu + 1) * gp.width / gp.tiles};
      r.v = {tv * gp.height / gp.tiles, (tv + 1) * gp.height / gp.tiles};
      r.vb = rc::binner(gp, vis, r.u, r.v, rc::binSizer(gp, vis, r.u, r.v));
      regions.push_back(std::move(r));
    }
  const double tb1 = now_ms();
  long long calls = 0, records = 0;
  for (Region& r : regions)
    for (rc::VisBin& b : r.vb) {
      r.g.push_back(b.vis.size() ? rc::gcfKernel(gcfp, b.bin) : rc::GCFs{});
      if (b.vis.size()) {
        calls++;
        records += b.vis.size();
      }
    }
  const double tb2 = now_ms();
  std::vector<double> t_grid, t_degrid;
  rc::UVGrid full;
  std::vector<double> pred_out;
  pred_out.reserve((size_t)5 * records);
  for (int it = 0; it < warmup + steps; it++) {
    const double t0 = now_ms();
    full = rc::gridInitDetile({0, gp.width}, {0, gp.height});
    for (Region& r : regions) {
      rc::UVGrid tile = rc::gridInit(gcfp, r.u, r.v);
      for (size_t k = 0; k < r.vb.size(); k++)
        if (r.vb[k].vis.size()) rc::gridKernel(gkt, gp, gcfp, r.vb[k], r.g[k], tile);
      rc::gridDetiling(tile, full);
    }
    const double t1 = now_ms();
    pred_out.clear();
    for (Region& r : regions)
      for (size_t k = 0; k < r.vb.size(); k++)
        if (r.vb[k].vis.size()) {
          const rc::Vis out = rc::degridKernel(dkt, gp, gcfp, r.g[k], model, r.vb[k].vis);
          pred_out.insert(pred_out.end(), out.rec.begin(), out.rec.end());
        }
    const double t2 = now_ms();
    if (it >= warmup) {
      t_grid.push_back(t1 - t0);
      t_degrid.push_back(t2 - t1);
    }
  }
  write_doubles(dir + "/grid.bin", full.data);
  write_doubles(dir + "/pred.bin", pred_out);
  auto list = [](const std::vector<double>& v) {
    std::string s = "[";
    for (size_t i = 0; i < v.size(); i++) s += (i ? ", " : "") + std::to_string(v[i]);
    return s + "]";
  };
  std::printf(
      "{\"bin_ms\": %.3f, \"gcf_read_ms\": %.3f, \"calls_per_direction\": %lld, "
      "\"records\": %lld, \"grid_ms\": %s, \"degrid_ms\": %s}\n",
      tb1 - tb0, tb2 - tb1, calls, records, list(t_grid).c_str(), list(t_degrid).c_str());
}

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s DIR bins|grid|degrid\n", argv[0]);
    return 2;
  }
  const std::string dir = argv[1], mode = argv[2];
  try {
    if (mode == "oskar") {
      char name[4096];
      int freq = 0, pol = 0;
      long long low = 0, high = 0;
      FILE* of = std::fopen((dir + "/oskar.txt").c_str(), "r");
      if (!of || std::fscanf(of, "%4095s %d %d %lld %lld", name, &freq, &pol, &low, &high) != 5)
        throw rc::KernelError("bad oskar.txt", -1);
      std::fclose(of);
      const rc::TaskData td = rc::readOskarData(name);
      write_doubles(dir + "/oskar.bin", rc::oskarReader(td, freq, pol, low, high).rec);
      return 0;
    }
    rc::GridPar gp;
    rc::GCFPar gcfp;
    int n_gcf = 0, gk = 1, dk = 1;
    FILE* pf = std::fopen((dir + "/params.txt").c_str(), "r");
    if (!pf || std::fscanf(pf, "%d %d %lf %d %d %d %d %d", &gp.width, &gp.height, &gp.theta,
                           &gp.tiles, &gp.bins, &n_gcf, &gk, &dk) != 8)
      throw rc::KernelError("bad params.txt", -1);
    gp.pitch = gp.width;
    for (int i = 0; i < n_gcf; i++) {
      char name[4096];
      rc::GCFFile f;
      if (std::fscanf(pf, "%4095s %d %lf", name, &f.size, &f.w) != 3)
        throw rc::KernelError("bad GCF line", -1);
      f.file = name;
      gcfp.files.push_back(f);
    }
    std::fclose(pf);
    const auto gkt = gk == 0 ? rc::GridKernelType::CPU
                     : gk == 1 ? rc::GridKernelType::GPU
                               : rc::GridKernelType::NV;
    const auto dkt = dk == 0 ? rc::DegridKernelType::CPU : rc::DegridKernelType::GPU;

    rc::Vis vis;
    {
      const std::vector<double> v = read_doubles(dir + "/vis.bin");
      vis.rec.assign(v.begin(), v.end());
    }
    rc::UVGrid model;
    if (mode == "degrid" || mode == "time") {
      model.width = gp.width;
      model.height = gp.height;
      const std::vector<double> m = read_doubles(dir + "/model.bin");
      model.data.assign(m.begin(), m.end());
      if (model.data.size() != (size_t)2 * gp.width * gp.height)
        throw rc::KernelError("bad model.bin", -1);
    }

    if (mode == "time") {
      time_passes(dir, gkt, dkt, gp, gcfp, vis, model);
      return 0;
    }
    if (mode == "grid") {
      rc::UVGrid full = grid_tiles(gkt, gp, gcfp, vis);
      write_doubles(dir + "/grid.bin", full.data);
      write_doubles(dir + "/image.bin", rc::ifftKern(gp, full).data);
      return 0;
    }
    if (mode == "clean") {
      rc::CleanPar cp;
      FILE* cf = std::fopen((dir + "/clean.txt").c_str(), "r");
      if (!cf || std::fscanf(cf, "%lf %lf", &cp.gain, &cp.threshold) != 2)
        throw rc::KernelError("bad clean.txt", -1);
      std::fclose(cf);
      rc::UVGrid g_dirty = grid_tiles(gkt, gp, gcfp, vis);
      rc::Image dirty = rc::ifftKern(gp, g_dirty);
      rc::Vis psf_vis = rc::psfVisKernel(vis);
      rc::UVGrid g_psf = grid_tiles(gkt, gp, gcfp, psf_vis);
      rc::Image psf = rc::ifftKern(gp, g_psf);
      rc::Image model = dirty;
      std::fill(model.data.begin(), model.data.end(), 0.0);
      rc::cleanModel(cp, psf, dirty, model);
      write_doubles(dir + "/clean_model.bin", model.data);
      write_doubles(dir + "/clean_residual.bin", rc::cleanResidual(cp, psf, dirty).data);
      return 0;
    }
#ifndef GB_MS5_ABI  // MS5 binds no image -> grid transform (fftKern)
    if (mode == "continuum") {
      // the major loop of MS6/programs/continuum.hs:80-98: each iteration
      // degrids the model's grid (fftKern) from the visibilities
      // (degridModel: vis - D fft(model)), grids and images the result
      // (idft of grid), and CLEANs it against the PSF of the visibilities:
      // the model grows (cleanModel) until the last iteration, which returns
      // the residual (cleanResidual against an empty model)
      rc::CleanPar cp;
      int loops = 0;
      FILE* cf = std::fopen((dir + "/clean.txt").c_str(), "r");
      if (!cf || std::fscanf(cf, "%lf %lf", &cp.gain, &cp.threshold) != 2)
        throw rc::KernelError("bad clean.txt", -1);
      std::fclose(cf);
      FILE* lf = std::fopen((dir + "/continuum.txt").c_str(), "r");
      if (!lf || std::fscanf(lf, "%d", &loops) != 1 || loops < 1)
        throw rc::KernelError("bad continuum.txt", -1);
      std::fclose(lf);
      rc::Vis psf_vis = rc::psfVisKernel(vis);
      rc::UVGrid g_psf = grid_tiles(gkt, gp, gcfp, psf_vis);
      rc::Image psf = rc::ifftKern(gp, g_psf);
      rc::Image mdl;
      mdl.width = gp.width;
      mdl.height = gp.height;
      mdl.data.assign((size_t)gp.width * gp.height, 0.0);
      rc::Image res;
      for (int it = 0; it < loops; it++) {
        rc::UVGrid mgrid = rc::fftKern(gp, mdl);
        rc::Vis corrected;  // degridModel over every (u, v) tile and w-bin region
        for (int tv = 0; tv < gp.tiles; tv++)
          for (int tu = 0; tu < gp.tiles; tu++) {
            const rc::Range u{tu * gp.width / gp.tiles, (tu + 1) * gp.width / gp.tiles};
            const rc::Range v{tv * gp.height / gp.tiles, (tv + 1) * gp.height / gp.tiles};
            std::vector<rc::VisBin> vb = rc::binner(gp, vis, u, v, rc::binSizer(gp, vis, u, v));
            for (rc::VisBin& b : vb) {
              if (b.vis.size() == 0) continue;
              rc::GCFs g = rc::gcfKernel(gcfp, b.bin);
              const rc::Vis o = rc::degridKernel(dkt, gp, gcfp, g, mgrid, b.vis);
              corrected.rec.insert(corrected.rec.end(), o.rec.begin(), o.rec.end());
            }
          }
        rc::UVGrid g_dirty = grid_tiles(gkt, gp, gcfp, corrected);
        rc::Image dirty = rc::ifftKern(gp, g_dirty);
        if (it + 1 < loops)
          rc::cleanModel(cp, psf, dirty, mdl);
        else
          res = rc::cleanResidual(cp, psf, dirty);
      }
      write_doubles(dir + "/cont_model.bin", mdl.data);
      write_doubles(dir + "/cont_residual.bin", res.data);
      return 0;
    }
#endif
    if (mode == "rotate") {
      double lon = 0, lat = 0;
      int l_low = 0, m_low = 0;
      FILE* rf = std::fopen((dir + "/rotate.txt").c_str(), "r");
      if (!rf || std::fscanf(rf, "%d %lf %lf %d %d", &gp.facets, &lon, &lat, &l_low, &m_low) != 5)
        throw rc::KernelError("bad rotate.txt", -1);
      std::fclose(rf);
      const rc::Vis out = rc::rotateKernel(gp, lon, lat, {l_low, l_low + gp.width},
                                           {m_low, m_low + gp.height}, vis);
      write_doubles(dir + "/rot.bin", out.rec);
      return 0;
    }

    std::vector<double> bins_out, pred_out;
    for (int tv = 0; tv < gp.tiles; tv++)
      for (int tu = 0; tu < gp.tiles; tu++) {
        // split of a range domain: low + (high - low) * i div n (Flow/Domain.hs:36-39)
        const rc::Range u{tu * gp.width / gp.tiles, (tu + 1) * gp.width / gp.tiles};
        const rc::Range v{tv * gp.height / gp.tiles, (tv + 1) * gp.height / gp.tiles};
        const std::vector<rc::WBin> bins = rc::binSizer(gp, vis, u, v);
        std::vector<rc::VisBin> vb = rc::binner(gp, vis, u, v, bins);
        if (mode == "bins") {
          for (const rc::VisBin& b : vb) {
            bins_out.push_back(b.bin.low);
            bins_out.push_back(b.bin.high);
            bins_out.push_back((double)b.bin.count);
            bins_out.push_back((double)b.vis.size());
            bins_out.insert(bins_out.end(), b.vis.rec.begin(), b.vis.rec.end());
          }
          continue;
        }
        for (rc::VisBin& b : vb) {  // degrid
          if (b.vis.size() == 0) continue;
          rc::GCFs g = rc::gcfKernel(gcfp, b.bin);
          const rc::Vis out = rc::degridKernel(dkt, gp, gcfp, g, model, b.vis);
          pred_out.insert(pred_out.end(), out.rec.begin(), out.rec.end());
        }
      }
    if (mode == "bins") write_doubles(dir + "/bins.bin", bins_out);
    if (mode == "degrid") write_doubles(dir + "/pred.bin", pred_out);
  } catch (const rc::KernelError& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
