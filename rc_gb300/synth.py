"""Seeded synthetic observations for the gridding workloads.

No dataset ships with the reference (its OSKAR .vis and gcf*.dat inputs are
not public), so every workload is generated: antenna layouts, baselines,
earth-rotation uvw tracks over hour angle +-4 h at latitude -30 deg towards
declination -45 deg, and visibilities of 20 point sources (l, m uniform in
+-0.05 rad, flux log-uniform 0.1-10 Jy) plus complex Gaussian noise
sigma = 0.01.  uvw are converted from metres to wavelengths (f / c), as the
reference's OSKAR reader does (MS6/kernel/oskar/OskarBinReader.cpp:318-385),
and records are ordered baseline-major, time-minor.

Workloads (sizes as the benchmark configurations state them):
  c1  64 antennas uniform in a 3 km disk, 2016 bl x 256 t x 1 ch @150 MHz
      = 516,096 vis, 2048^2 grid, one plane, 7x7 PSWF GCF padded to S=8.
  c2  256 antennas log-radial (dense 1 km core, out to 10 km),
      32,640 bl x 128 t = 4,177,920 vis, 4096^2 grid, 32 w-planes, S 8..64.
  c4  c1's array, 2,064,384 vis (2016 bl x 1024 t), 2048^2 grid,
      16 w-planes, S 8..64 (the least-squares imaging layout).
  c5  512 stations log-radial to 40 km, 130,816 bl x 64 t x 4 ch,
      8192^2 grid, 64 w-planes, S 8..128; its sources lie within +-0.2 of the
      field of view (the field is only +-0.046 rad wide).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

C_LIGHT = 299792458.0
SEED0 = 20261203


@dataclasses.dataclass
class Observation:
    name: str
    uvw: np.ndarray  # (N, 3) float64, wavelengths
    vis: np.ndarray  # (N,) complex128
    grid_size: int
    scale: float  # reference `scale`: FoV in radians (pixel = 1/scale wavelengths)
    n_planes: int
    supports: np.ndarray  # int32 per plane
    w_planes: np.ndarray  # float64 GCF w per plane
    w_low: float
    w_high: float
    max_support: int
    n_bl: int
    n_t: int
    n_ch: int

    @property
    def n(self):
        return self.uvw.shape[0]

    def vis5(self):
        """The reference's 5-double record (u, v, w, re, im) per visibility."""
        out = np.empty((self.n, 5), np.float64)
        out[:, :3] = self.uvw
        out[:, 3] = self.vis.real
        out[:, 4] = self.vis.imag
        return out


def antennas_disk(rng, n, diameter_m):
    r = 0.5 * diameter_m * np.sqrt(rng.uniform(0, 1, n))
    a = rng.uniform(0, 2 * np.pi, n)
    return np.stack([r * np.cos(a), r * np.sin(a)], 1)


def antennas_logradial(rng, n, r_core_m, r_max_m):
    """Radii log-uniform between r_core/20 and r_max: half the stations fall
    inside ~sqrt(r_core r_max)/..., a dense core with a sparse tail."""
    r = np.exp(rng.uniform(np.log(r_core_m / 20.0), np.log(r_max_m), n))
    a = rng.uniform(0, 2 * np.pi, n)
    return np.stack([r * np.cos(a), r * np.sin(a)], 1)


def uvw_tracks(ant_en, n_t, lat_deg=-30.0, dec_deg=-45.0, ha_hours=4.0):
    """(n_bl, n_t, 3) metres; baselines i<j, hour angle linspace(-ha, ha, n_t)."""
    na = ant_en.shape[0]
    i, j = np.triu_indices(na, 1)
    d = ant_en[j] - ant_en[i]  # east, north
    lat = math.radians(lat_deg)
    dec = math.radians(dec_deg)
    X = -math.sin(lat) * d[:, 1]
    Y = d[:, 0]
    Z = math.cos(lat) * d[:, 1]
    H = np.linspace(-ha_hours, ha_hours, n_t) * (np.pi / 12.0)
    sH, cH = np.sin(H)[None, :], np.cos(H)[None, :]
    X, Y, Z = X[:, None], Y[:, None], Z[:, None]
    u = sH * X + cH * Y
    v = -math.sin(dec) * cH * X + math.sin(dec) * sH * Y + math.cos(dec) * Z
    w = math.cos(dec) * cH * X - math.cos(dec) * sH * Y + math.sin(dec) * Z
    return np.stack([u, v, w], -1)


def sky(rng, n_src=20, lm_max=0.05):
    l = rng.uniform(-lm_max, lm_max, n_src)
    m = rng.uniform(-lm_max, lm_max, n_src)
    flux = np.exp(rng.uniform(np.log(0.1), np.log(10.0), n_src))
    return l, m, flux


def predict(uvw, l, m, flux, rng, noise=0.01, chunk=1 << 20):
    n = uvw.shape[0]
    nn = np.sqrt(1.0 - l * l - m * m) - 1.0
    out = np.empty(n, np.complex128)
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        ph = -2.0 * np.pi * (np.outer(uvw[a:b, 0], l) + np.outer(uvw[a:b, 1], m)
                             + np.outer(uvw[a:b, 2], nn))
        out[a:b] = (np.exp(1j * ph) * flux[None, :]).sum(1)
    out += noise * (rng.standard_normal(n) + 1j * rng.standard_normal(n)) / np.sqrt(2.0)
    return out


def sky_image(n, rng, n_blobs=20, sigma=(1.0, 5.0), flux=(0.1, 10.0), margin=0.25):
    """Real float32 n x n sky of Gaussian blobs (sigma uniform in px, peak
    log-uniform) on a zero background, centres within the inner 1 - 2*margin."""
    img = np.zeros((n, n), np.float64)
    yy, xx = np.mgrid[0:n, 0:n]
    lo, hi = margin * n, (1 - margin) * n
    for _ in range(n_blobs):
        cy, cx = rng.uniform(lo, hi, 2)
        s = rng.uniform(*sigma)
        a = np.exp(rng.uniform(np.log(flux[0]), np.log(flux[1])))
        y0, y1 = int(max(0, cy - 6 * s)), int(min(n, cy + 6 * s + 1))
        x0, x1 = int(max(0, cx - 6 * s)), int(min(n, cx + 6 * s + 1))
        img[y0:y1, x0:x1] += a * np.exp(-((yy[y0:y1, x0:x1] - cy) ** 2 +
                                          (xx[y0:y1, x0:x1] - cx) ** 2) / (2 * s * s))
    return img.astype(np.float32)


def _finish(name, rng, uvw_m, freqs, grid_size, n_planes, s_min, s_max, lm_field=None):
    """metres -> wavelengths per channel, sky, scale, w-planes.  lm_field: if
    given, sources lie within +-lm_field * (field of view) instead of +-0.05 rad."""
    from .gcf import plane_supports

    n_bl, n_t, _ = uvw_m.shape
    per_ch = [uvw_m.reshape(-1, 3) * (f / C_LIGHT) for f in freqs]
    # channel-minor ordering within each (baseline, time): [bl][t][ch]
    uvw = np.stack(per_ch, 1).reshape(-1, 3) if len(freqs) > 1 else per_ch[0]
    maxuv = float(np.sqrt(uvw[:, 0] ** 2 + uvw[:, 1] ** 2).max())
    scale = 0.9 * (grid_size / 2) / maxuv
    l, m, flux = sky(rng, lm_max=0.05 if lm_field is None else lm_field * scale)
    vis = predict(uvw, l, m, flux, rng)
    if n_planes > 1:
        w = uvw[:, 2]
        low = min(0.0, float(w.min()))
        high0 = max(0.0, float(w.max()))
        high = high0 + (high0 - low) * 1e-4  # MS6/programs/Kernel/Binning.hs:60
        supports, centres = plane_supports(low, high, n_planes, s_min, s_max)
    else:
        low, high = -np.inf, np.inf
        supports, centres = np.array([s_min], np.int32), np.zeros(1)
    return Observation(name, np.ascontiguousarray(uvw), vis, grid_size, scale, n_planes,
                       supports, centres, low, high, int(supports.max()), n_bl, n_t, len(freqs))


def config3(seed: int | None = None, n_t: int = 216, n_ch: int = 64, n_facets: int = 9,
            n_planes: int = 48, s_max: int = 96):
    """The batched workload: the 64-antenna 3 km array on n_ch channels from 100
    to 200 MHz (uv scaled by frequency, one grid per channel: 1024^2, 2048^2 or
    4096^2 by channel band) plus n_facets facets (1024^2, 2048^2, 4096^2) of the
    150 MHz data; one field of view for all (pixel size scales with the grid),
    so all members share one set of n_planes w-planes (S 8..s_max) over the
    global w range.  Default: 73 grids x 435,456 vis = 31.8 M visibilities.
    Returns (members, scale, supports, w_planes, w_low, w_high)."""
    from .gcf import plane_supports

    rng = np.random.default_rng(SEED0 + 3 if seed is None else seed)
    ant = antennas_disk(rng, 64, 3000.0)
    uvw_m = uvw_tracks(ant, n_t).reshape(-1, 3)
    freqs = np.linspace(100e6, 200e6, n_ch)
    sizes = [1024 if k < n_ch // 3 else 2048 if k < 2 * n_ch // 3 else 4096 for k in range(n_ch)]
    l, m, flux = sky(rng)
    uvws, grids = [], []
    for f, G in zip(freqs, sizes):
        uvws.append(uvw_m * (f / C_LIGHT))
        grids.append(G)
    f150 = uvw_m * (150e6 / C_LIGHT)
    for k in range(n_facets):
        uvws.append(f150)
        grids.append([1024, 2048, 4096][k % 3])
    # one FoV: every member's max |uv| fits 90 % of its half-grid
    scale = min(0.9 * (G / 2) / float(np.sqrt(u[:, 0] ** 2 + u[:, 1] ** 2).max())
                for u, G in zip(uvws, grids))
    wmin = min(0.0, min(float(u[:, 2].min()) for u in uvws))
    wmax0 = max(0.0, max(float(u[:, 2].max()) for u in uvws))
    w_high = wmax0 + (wmax0 - wmin) * 1e-4
    supports, centres = plane_supports(wmin, w_high, n_planes, 8, s_max)
    members = []
    for k, (u, G) in enumerate(zip(uvws, grids)):
        vis = predict(u, l, m, flux, rng)
        members.append(Observation(f"c3.{k}", np.ascontiguousarray(u), vis, G, scale, n_planes,
                                   supports, centres, wmin, w_high, int(supports.max()),
                                   u.shape[0] // n_t, n_t, 1))
    return members, scale, supports, centres, wmin, w_high


def config(name: str, seed: int | None = None, n_t: int | None = None) -> Observation:
    """Build a workload by name ('c1', 'c2', 'c4', 'c5'; 'small' for tests).
    n_t overrides the number of time samples (for reduced test sizes)."""
    idx = {"c1": 1, "c2": 2, "c4": 4, "c5": 5, "small": 0}[name]
    rng = np.random.default_rng(SEED0 + idx if seed is None else seed)
    if name == "c1":
        ant = antennas_disk(rng, 64, 3000.0)
        uvw_m = uvw_tracks(ant, n_t or 256)
        return _finish(name, rng, uvw_m, [150e6], 2048, 1, 8, 8)
    if name == "c2":
        ant = antennas_logradial(rng, 256, 1000.0, 10000.0)
        uvw_m = uvw_tracks(ant, n_t or 128)
        return _finish(name, rng, uvw_m, [150e6], 4096, 32, 8, 64)
    if name == "c4":
        ant = antennas_disk(rng, 64, 3000.0)
        uvw_m = uvw_tracks(ant, n_t or 1024)
        return _finish(name, rng, uvw_m, [150e6], 2048, 16, 8, 64)
    if name == "c5":
        ant = antennas_logradial(rng, 512, 1000.0, 40000.0)
        uvw_m = uvw_tracks(ant, n_t or 64)
        freqs = [150e6 * (1 + 0.01 * k) for k in range(4)]
        # the 40 km array's field is +-0.046 rad: keep the sources in its inner half
        return _finish(name, rng, uvw_m, freqs, 8192, 64, 8, 128, lm_field=0.2)
    # small: quick w-projection case for tests
    ant = antennas_logradial(rng, 24, 300.0, 3000.0)
    uvw_m = uvw_tracks(ant, n_t or 32)
    return _finish(name, rng, uvw_m, [150e6], 512, 8, 8, 32)


def abi_gcf_files(ob: Observation):
    """GCF files for driving the reference-ABI strategy on a workload whose
    plane supports follow S = 8 + 56 sqrt(|w| / w_max): the reference's own
    support set 16 / 32 / 64 (MS6/cfg/continuum.yaml) with each file's w at
    the point where the rule passes the previous size, so that gcfGet's choice
    (the largest file w <= the bin's largest |w|) never has a smaller support
    than the rule asks for below the next file.  [(w, support)]."""
    wmax = max(abs(ob.w_low), abs(ob.w_high))
    return [(0.0, 16), (wmax * (8.0 / 56.0) ** 2, 32), (wmax * (24.0 / 56.0) ** 2, 64)]


def write_oskar_vis(path, ob: Observation, max_times_per_block: int = 8,
                    freq_hz: float = 150e6) -> int:
    """Store a single-channel observation as an OSKAR 2.6 visibility file, the
    layout MS6/kernel/oskar/OskarBinReader.cpp reads (header tags in group 11,
    blocks of max_times_per_block times in group 12, tag numbers of
    OskarBinReader.cpp:67-100): cross-correlations [time][channel][baseline]
    x (XX, XY, YX, YY) with XX = YY = vis and XY = YX = 0, baseline u,v,w in
    metres (wavelengths x c / f) [time][baseline].  Every chunk carries its
    CRC-32C, computed on the GPU.  Returns the file size in bytes."""
    import torch

    from .oskar import crc32c

    assert ob.n_ch == 1, "one channel per file"
    B, T, M = ob.n_bl, ob.n_t, int(max_times_per_block)
    S = int(round((1 + math.sqrt(1 + 8 * B)) / 2))
    assert S * (S - 1) // 2 == B, "baselines must be all pairs of some station count"
    metres = (ob.uvw * (C_LIGHT / freq_hz)).reshape(B, T, 3)
    vis = ob.vis.reshape(B, T)
    ntpb = 7

    def crc(b: bytes, code=0xFFFFFFFF):
        if not b:
            return code
        t = torch.frombuffer(bytearray(b), dtype=torch.uint8).to("cuda")
        return crc32c(t, code)

    def chunk(ty, group, tag, user, payload: bytes):
        es = {0x01: 1, 0x02: 4, 0x08: 8, 0x68: 64}[ty]
        hdr = (b"T\x42G" + bytes([es, 0x40, ty, group, tag]) +
               int(user).to_bytes(4, "little", signed=True) +
               (len(payload) + 4).to_bytes(8, "little"))
        code = crc(payload, crc(hdr))
        return hdr + payload + int(code).to_bytes(4, "little")

    i4 = lambda *x: np.array(x, np.int32).tobytes()  # noqa: E731
    f8 = lambda *x: np.array(x, np.float64).tobytes()  # noqa: E731
    size = 0
    with open(path, "wb") as f:
        parts = [b"OSKARBIN\0\x02" + bytes(54),
                 chunk(0x01, 11, 1, 0, b"synthetic.tm\0"), chunk(0x02, 11, 2, 0, i4(ntpb)),
                 chunk(0x02, 11, 3, 0, i4(0)), chunk(0x02, 11, 4, 0, i4(0x68)),
                 chunk(0x02, 11, 5, 0, i4(M)), chunk(0x02, 11, 6, 0, i4(T)),
                 chunk(0x02, 11, 7, 0, i4(1)), chunk(0x02, 11, 8, 0, i4(S)),
                 chunk(0x08, 11, 9, 0, f8(freq_hz)), chunk(0x08, 11, 10, 0, f8(0.0)),
                 chunk(0x08, 11, 11, 0, f8(1e6)), chunk(0x08, 11, 12, 0, f8(57000.0)),
                 chunk(0x08, 11, 13, 0, f8(10.0)), chunk(0x08, 11, 14, 0, f8(10.0)),
                 chunk(0x08, 11, 15, 0, f8(0.0, -45.0)),
                 chunk(0x08, 11, 16, 0, f8(21.44, -30.0, 0.0))]
        parts += [chunk(0x08, 11, 17 + k, 0, np.zeros(S).tobytes()) for k in range(3)]
        for p in parts:
            f.write(p)
            size += len(p)
        for blk in range((T + M - 1) // M):
            t0 = blk * M
            nt = min(M, T - t0)
            amps = np.zeros((nt, 1, B, 4), np.complex128)
            amps[:, 0, :, 0] = vis[:, t0:t0 + nt].T
            amps[:, 0, :, 3] = vis[:, t0:t0 + nt].T
            m = metres[:, t0:t0 + nt, :].transpose(2, 1, 0)  # [uvw][t][b]
            for p in (chunk(0x02, 12, 1, blk, i4(t0, 0, nt, 1, B, S)),
                      chunk(0x08, 12, 2, blk, f8(freq_hz, 0.0)),
                      chunk(0x08, 12, 3, blk, f8(57000.0 + t0 * 10.0 / 86400.0, 10.0 / 86400.0)),
                      chunk(0x68, 12, 5, blk, amps.tobytes()),
                      chunk(0x08, 12, 6, blk, np.ascontiguousarray(m[0]).tobytes()),
                      chunk(0x08, 12, 7, blk, np.ascontiguousarray(m[1]).tobytes()),
                      chunk(0x08, 12, 8, blk, np.ascontiguousarray(m[2]).tobytes())):
                f.write(p)
                size += len(p)
    return size
