"""Parity at the full sizes of the gridding workloads.

Config 2 (4.18 M visibilities, 4096^2 grid, 32 w-planes with supports 8-64,
oversample 8) goes against the oracle on the whole observation:
- w-planes and per-visibility indices are bit-exact;
- the plain FP64 pair is within relative L2 1e-12;
- the FP32 pair is within 1e-5, with degridding's default staging (split
  rows: every support is even) and with the TMA form (rows as in the grid;
  per-thread copies on the odd tile edge);
- the adjoint identity holds to FP32 rounding;
- the GCFs generated on the GPU match the oracle's generator.

Config 5 (33.5 M visibilities, 8192^2 grid, 64 w-planes with supports 8-128)
goes through checks that do not depend on size:
- indices are bit-exact;
- the grid's sum equals sum_i vis_i * (sum of the taps of visibility i's GCF
  layer);
- degridding a grid of ones returns conj of that tap sum;
- the FP32 pair is within 1e-5 of the plain FP64 pair;
- the adjoint identity holds;
- the oracle itself runs on a 1 M-visibility sample on the full grid, with
  every support up to 128.

Config 1 (516,096 visibilities, 2048^2) goes through the reference's buffer_t
symbols against the oracle.  Config 3 (73 grids, 31.8 M visibilities) runs in
one batched launch per direction against the FP64 pair and, for two members,
the oracle.
"""
import os
from types import SimpleNamespace

import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 1e-5
# degridding in the oracle is per visibility: it runs on all host cores
NTHREADS = max(1, min(16, os.cpu_count() or 1))


def _gcf_oracle(ob):
    from rc_gb300 import gcf as Gm

    tp = Gm.pswf_taper(ob.max_support)
    return np.concatenate([O.gcf_layers(w, int(S), ob.max_support, ob.scale / 2, taper=tp).ravel()
                           for w, S in zip(ob.w_planes, ob.supports)]), tp


def _expected_index(ob, plane, margin):
    """x0, y0, phase (ou + 8 ov), plane, kept per visibility from the oracle."""
    v5 = np.zeros((ob.n, 5))
    v5[:, :3] = ob.uvw
    out = np.zeros((ob.n, 5), np.int32)
    G = ob.grid_size
    for p, S in enumerate(ob.supports):
        m = plane == p
        if not m.any():
            continue
        ix = O.index(v5[m], ob.scale, G, int(S), margin, 0, 0, G, G)
        out[m, 0], out[m, 1] = ix[:, 0], ix[:, 1]
        out[m, 2] = ix[:, 2] + 8 * ix[:, 3]
        out[m, 3] = p
        out[m, 4] = ix[:, 4]
    return out


def _check_index(ob, P, plane, margin):
    got = P.export_index().cpu().numpy()
    exp = _expected_index(ob, plane, margin)
    kept = exp[:, 4] == 1
    assert np.array_equal(got[:, 3:5], exp[:, 3:5])
    assert np.array_equal(got[kept, :3], exp[kept, :3])
    st = P.stats()
    assert st["kept"] == int(kept.sum())
    assert st["taps"] == int((ob.supports[plane[kept]].astype(np.int64) ** 2).sum())
    return got


def _plan(ob, d_uvw, **kw):
    from rc_gb300.engine import Plan

    G = ob.grid_size
    return Plan(d_uvw, scale=ob.scale, grid_size=G, grid_shape=(G, G), supports=ob.supports,
                w_range=(ob.w_low, ob.w_high), **kw)


def _adjoint(P, ob, d_gcf32, seed):
    import torch

    G = ob.grid_size
    g = torch.Generator(device="cuda").manual_seed(seed)
    x = torch.randn((G, G), dtype=torch.complex64, device="cuda", generator=g)
    y = torch.randn(ob.n, dtype=torch.complex64, device="cuda", generator=g)
    Dx = P.degrid(d_gcf32, x)
    Gy = torch.zeros((G, G), dtype=torch.complex64, device="cuda")
    P.grid(y, d_gcf32, Gy)
    lhs = torch.vdot(Dx.to(torch.complex128), y.to(torch.complex128)).item()
    rhs = torch.vdot(x.to(torch.complex128).reshape(-1),
                     Gy.to(torch.complex128).reshape(-1)).item()
    return lhs, rhs


# ---------------------------------------------------------------- config 2, whole observation
@pytest.fixture(scope="module")
def c2():
    import torch

    from rc_gb300 import synth

    ob = synth.config("c2")
    gcf, tp = _gcf_oracle(ob)
    from rc_gb300.gcf import layout

    offs, _ = layout(ob.supports)
    plane = O.wbin(ob.uvw, ob.w_low, ob.w_high, ob.n_planes)
    margin = int(ob.supports.max())
    G = ob.grid_size
    grid = np.zeros((G, G), np.complex128)
    O.scatter_planes(ob.scale, G, margin, ob.uvw, ob.vis, plane, ob.supports, gcf, offs, grid)
    pred = O.degrid_planes(ob.scale, G, margin, ob.uvw, plane, ob.supports, gcf, offs, grid,
                           nthreads=NTHREADS)
    assert np.abs(grid).max() > 0 and np.abs(pred).max() > 0
    return SimpleNamespace(ob=ob, gcf=gcf, taper=tp, offs=offs, plane=plane, margin=margin,
                           grid=grid, pred=pred,
                           d_uvw=torch.tensor(ob.uvw, device="cuda"))


def test_c2_planes_and_indices_bit_exact(c2):
    P = _plan(c2.ob, c2.d_uvw)
    _check_index(c2.ob, P, c2.plane, c2.margin)


def test_c2_gcf_generated_on_the_gpu_matches_the_oracle(c2):
    from rc_gb300 import gcf as Gm

    ob = c2.ob
    g64, g32, offs = Gm.generate(ob.w_planes, ob.supports, ob.max_support, ob.scale / 2,
                                 taper=c2.taper)
    assert np.array_equal(np.asarray(offs), np.asarray(c2.offs))
    got = g64.cpu().numpy()
    for p, S in enumerate(ob.supports):
        a, b = c2.offs[p], c2.offs[p] + 64 * int(S) ** 2
        assert rel_l2(got[a:b], c2.gcf[a:b]) < TOL64, p
    assert rel_l2(g32.cpu().numpy(), c2.gcf) < 1e-6


def test_c2_plain_fp64_pair_matches_the_oracle(c2):
    import torch

    ob = c2.ob
    G = ob.grid_size
    P = _plan(ob, c2.d_uvw)
    d_gcf = torch.tensor(c2.gcf, device="cuda")
    grid = torch.zeros((G, G), dtype=torch.complex128, device="cuda")
    P.grid64(torch.tensor(ob.vis, dtype=torch.complex128, device="cuda"), d_gcf, grid)
    assert rel_l2(grid.cpu().numpy(), c2.grid) < TOL64
    d_grid = torch.tensor(c2.grid, device="cuda")
    pred = P.degrid64(d_gcf, d_grid).cpu().numpy()
    assert rel_l2(pred, c2.pred) < TOL64
    # mode 1: the reference kern_degrid product, -sum grid * gcf (no conjugate),
    # FP64 and FP32 against the oracle on the whole observation
    exp1 = O.degrid_planes(ob.scale, G, c2.margin, ob.uvw, c2.plane, ob.supports, c2.gcf, c2.offs,
                           c2.grid, mode=1, nthreads=NTHREADS)
    assert rel_l2(P.degrid64(d_gcf, d_grid, mode=1).cpu().numpy(), exp1) < TOL64
    pred32 = P.degrid(d_gcf.to(torch.complex64), d_grid.to(torch.complex64), mode=1)
    assert rel_l2(pred32.cpu().numpy(), exp1) < TOL32


@pytest.mark.parametrize("tile,threads,cap", [(24, 256, 32), (25, 256, 32), (32, 512, 64)])
def test_c2_fp32_pair_matches_the_oracle(c2, tile, threads, cap):
    import torch

    ob = c2.ob
    G = ob.grid_size
    P = _plan(ob, c2.d_uvw, tile=tile, threads=threads, period_cap=cap)
    d_gcf = torch.tensor(c2.gcf, dtype=torch.complex64, device="cuda")
    grid = torch.zeros((G, G), dtype=torch.complex64, device="cuda")
    P.grid(torch.tensor(ob.vis, dtype=torch.complex64, device="cuda"), d_gcf, grid)
    assert rel_l2(grid.cpu().numpy(), c2.grid) < TOL32
    pred = P.degrid(d_gcf, torch.tensor(c2.grid, dtype=torch.complex64, device="cuda"))
    assert rel_l2(pred.cpu().numpy(), c2.pred) < TOL32
    # every support is even: split rows by default; the TMA form on even tiles
    from rc_gb300 import lib

    assert P.device_status() == (0, lib.STAGE_SPLIT)
    P.set_stage(lib.STAGE_TMA)
    pred_t = P.degrid(d_gcf, torch.tensor(c2.grid, dtype=torch.complex64, device="cuda"))
    assert rel_l2(pred_t.cpu().numpy(), c2.pred) < TOL32
    assert P.device_status() == (0, lib.STAGE_TMA if tile % 2 == 0 else lib.STAGE_ROWS)
    P.set_stage(lib.STAGE_AUTO)
    lhs, rhs = _adjoint(P, ob, d_gcf, seed=tile)
    assert abs(lhs - rhs) <= TOL32 * abs(lhs)


# ---------------------------------------------------------------- config 5, properties
@pytest.fixture(scope="module")
def c5():
    import torch

    from rc_gb300 import synth
    from rc_gb300.gcf import layout

    ob = synth.config("c5")
    gcf, tp = _gcf_oracle(ob)
    offs, _ = layout(ob.supports)
    plane = O.wbin(ob.uvw, ob.w_low, ob.w_high, ob.n_planes)
    # per-(plane, phase) sums of the taps: [n_planes][64]
    tsum = np.stack([gcf[o:o + 64 * int(S) ** 2].reshape(64, -1).sum(1)
                     for o, S in zip(offs, ob.supports)])
    return SimpleNamespace(ob=ob, gcf=gcf, taper=tp, offs=offs, plane=plane,
                           margin=int(ob.supports.max()), tsum=tsum,
                           d_uvw=torch.tensor(ob.uvw, device="cuda"))


def test_c5_properties_at_full_size(c5):
    import torch

    ob = c5.ob
    G = ob.grid_size
    assert G == 8192 and int(ob.supports.max()) == 128 and ob.n > 33_000_000
    P = _plan(ob, c5.d_uvw)
    idx = _check_index(ob, P, c5.plane, c5.margin)
    kept = idx[:, 4] == 1
    T = np.zeros(ob.n, np.complex128)
    T[kept] = c5.tsum[idx[kept, 3], idx[kept, 2]]

    d_gcf64 = torch.tensor(c5.gcf, device="cuda")
    d_gcf32 = d_gcf64.to(torch.complex64)
    d_vis64 = torch.tensor(ob.vis, dtype=torch.complex128, device="cuda")

    # checksum: sum over the grid of G(vis) = sum_i vis_i T_i
    want = np.sum(ob.vis * T)
    scale = np.sum(np.abs(ob.vis) * np.abs(T))
    grid64 = torch.zeros((G, G), dtype=torch.complex128, device="cuda")
    P.grid64(d_vis64, d_gcf64, grid64)
    assert abs(grid64.sum().item() - want) <= TOL64 * scale
    grid32 = torch.zeros((G, G), dtype=torch.complex64, device="cuda")
    P.grid(d_vis64.to(torch.complex64), d_gcf32, grid32)
    assert abs(grid32.to(torch.complex128).sum().item() - want) <= TOL32 * scale
    assert rel_l2(grid32.cpu().numpy(), grid64.cpu().numpy()) < TOL32

    # degridding a grid of ones returns conj(T_i)
    ones64 = torch.ones((G, G), dtype=torch.complex128, device="cuda")
    assert rel_l2(P.degrid64(d_gcf64, ones64).cpu().numpy(), np.conj(T)) < TOL64
    assert rel_l2(P.degrid(d_gcf32, ones64.to(torch.complex64)).cpu().numpy(),
                  np.conj(T)) < TOL32
    del ones64

    # the FP32 pair against the plain FP64 pair on the dirty grid of the data
    pred64 = P.degrid64(d_gcf64, grid64).cpu().numpy()
    pred32 = P.degrid(d_gcf32, grid64.to(torch.complex64)).cpu().numpy()
    assert rel_l2(pred32, pred64) < TOL32
    assert P.device_status()[0] == 0

    lhs, rhs = _adjoint(P, ob, d_gcf32, seed=5)
    assert abs(lhs - rhs) <= TOL32 * abs(lhs)


def test_c5_sample_matches_the_oracle_on_the_full_grid(c5):
    """1 M visibilities of config 5 (every w-plane, supports 8-128) on the
    8192^2 grid: plain FP64 pair within 1e-12 and FP32 pair within 1e-5 of
    the oracle."""
    import torch

    ob = c5.ob
    G = ob.grid_size
    rng = np.random.default_rng(55)
    # a random 1 M plus up to 4096 of every w-plane, so the sparse outer
    # planes (the largest supports) are in the sample too
    per_plane = [rng.permutation(np.flatnonzero(c5.plane == p))[:4096]
                 for p in range(ob.n_planes)]
    sel = np.unique(np.concatenate([rng.choice(ob.n, 1 << 20, replace=False)] + per_plane))
    uvw, vis, plane = ob.uvw[sel], ob.vis[sel], c5.plane[sel]
    assert np.array_equal(np.unique(plane), np.unique(c5.plane))
    exp = np.zeros((G, G), np.complex128)
    O.scatter_planes(ob.scale, G, c5.margin, uvw, vis, plane, ob.supports, c5.gcf, c5.offs, exp)
    exp_pred = O.degrid_planes(ob.scale, G, c5.margin, uvw, plane, ob.supports, c5.gcf, c5.offs,
                               exp, nthreads=NTHREADS)

    d_uvw = torch.tensor(uvw, device="cuda")
    P = _plan(ob, d_uvw)
    d_gcf64 = torch.tensor(c5.gcf, device="cuda")
    d_gcf32 = d_gcf64.to(torch.complex64)
    grid64 = torch.zeros((G, G), dtype=torch.complex128, device="cuda")
    P.grid64(torch.tensor(vis, device="cuda"), d_gcf64, grid64)
    assert rel_l2(grid64.cpu().numpy(), exp) < TOL64
    d_exp = torch.tensor(exp, device="cuda")
    assert rel_l2(P.degrid64(d_gcf64, d_exp).cpu().numpy(), exp_pred) < TOL64
    grid32 = torch.zeros((G, G), dtype=torch.complex64, device="cuda")
    P.grid(torch.tensor(vis, dtype=torch.complex64, device="cuda"), d_gcf32, grid32)
    assert rel_l2(grid32.cpu().numpy(), exp) < TOL32
    assert rel_l2(P.degrid(d_gcf32, d_exp.to(torch.complex64)).cpu().numpy(), exp_pred) < TOL32
    assert P.device_status()[0] == 0


# ---------------------------------------------------------------- config 1, reference ABI
@pytest.mark.parametrize("scatter,degrid", [("kern_scatter_gpu1", "kern_degrid_gpu1"),
                                            ("kern_scatter", "kern_degrid"),
                                            ("nvGridder", "kern_degrid_gpu1")])
def test_c1_whole_observation_through_the_reference_abi(scatter, degrid):
    """Config 1 (516,096 visibilities, 2048^2 complex128 grid, the 7x7 PSWF in
    S = 8) through the reference's host buffer_t symbols, against the oracle's
    restatement of kern_scatter / kern_degrid: within relative L2 1e-12."""
    from rc_gb300 import compat
    from rc_gb300 import gcf as G
    from rc_gb300 import synth

    ob = synth.config("c1")
    assert ob.n == 516_096 and ob.grid_size == 2048
    vis5 = ob.vis5()
    gcf = G.pswf_uv_gcf(8, 7)
    grid = np.zeros((ob.grid_size, ob.grid_size), np.complex128)
    assert compat.call_scatter(scatter, ob.scale, ob.grid_size, 8, vis5, gcf, grid) == 0
    exp = np.zeros_like(grid)
    O.scatter(ob.scale, ob.grid_size, 8, vis5, gcf, exp)
    assert np.abs(exp).max() > 0
    assert rel_l2(grid, exp) < TOL64
    out = np.zeros_like(vis5)
    assert compat.call_degrid(degrid, ob.scale, ob.grid_size, 8, gcf, exp, vis5, out) == 0
    ref = O.degrid(ob.scale, ob.grid_size, 8, gcf, exp, vis5)
    assert np.array_equal(out[:, :3], vis5[:, :3])
    assert rel_l2(out[:, 3:], ref[:, 3:]) < TOL64


# ---------------------------------------------------------------- config 3, one batched launch
def test_c3_batched_launch_at_full_size():
    """Config 3 (73 grids of 1024^2-4096^2, 31.8 M visibilities, 48 shared
    w-planes with supports 8-96) in one persistent launch per direction: the
    FP32 pair within relative L2 1e-5 of the plain FP64 pair on every member,
    and two members (a 1024^2 channel grid and a 4096^2 facet) against the
    oracle itself."""
    import torch

    from rc_gb300 import gcf as Gm
    from rc_gb300 import synth
    from rc_gb300.engine import Batch
    from rc_gb300.gcf import layout

    members, scale, supports, w_planes, wlo, whi = synth.config3()
    assert len(members) == 73 and sum(m.n for m in members) > 31_000_000
    smax = int(supports.max())
    tp = Gm.pswf_taper(smax)
    g64, g32, offs = Gm.generate(w_planes, supports, smax, scale / 2, taper=tp)
    uvws = [torch.tensor(m.uvw, device="cuda") for m in members]
    B = Batch([dict(uvw=u, scale=scale, grid_size=m.grid_size,
                    grid_shape=(m.grid_size, m.grid_size), supports=supports, gcf_offsets=offs,
                    w_range=(wlo, whi)) for u, m in zip(uvws, members)],
              tile=24, threads=256, period_cap=32)
    vis64 = [torch.tensor(m.vis, dtype=torch.complex128, device="cuda") for m in members]
    grids64 = [torch.zeros((m.grid_size, m.grid_size), dtype=torch.complex128, device="cuda")
               for m in members]
    B.grid64(vis64, g64, grids64)
    preds64 = [torch.empty(m.n, dtype=torch.complex128, device="cuda") for m in members]
    B.degrid64(g64, grids64, preds64)
    grids = [torch.zeros((m.grid_size, m.grid_size), dtype=torch.complex64, device="cuda")
             for m in members]
    B.grid([v.to(torch.complex64) for v in vis64], g32, grids)
    preds = B.degrid(g32, [g.to(torch.complex64) for g in grids64])
    torch.cuda.synchronize()

    def rel(a, b):
        return float(torch.linalg.vector_norm(a.to(torch.complex128) - b) /
                     torch.linalg.vector_norm(b))

    for k in range(len(members)):
        assert rel(grids[k], grids64[k]) < TOL32, k
        assert rel(preds[k], preds64[k]) < TOL32, k
    # the oracle on two whole members
    offs_np, _ = layout(supports)
    gcf_np = g64.cpu().numpy()
    for k in (0, len(members) - 1):
        m = members[k]
        plane = O.wbin(m.uvw, wlo, whi, len(supports))
        exp = np.zeros((m.grid_size, m.grid_size), np.complex128)
        O.scatter_planes(scale, m.grid_size, smax, m.uvw, m.vis, plane, supports, gcf_np, offs_np,
                         exp)
        assert np.abs(exp).max() > 0
        assert rel_l2(grids64[k].cpu().numpy(), exp) < TOL64, k
        assert rel_l2(grids[k].cpu().numpy(), exp) < TOL32, k
    B.close()
