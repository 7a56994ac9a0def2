"""Engine API on the GPU against the oracle.

Bars: per-visibility indices (corner, phase, plane, kept) bit-exact; plain
FP64 gridding/degridding within relative L2 1e-12 of the FP64 oracle; FP32
tiled pair within relative L2 1e-5 of the FP64 oracle; <Dx, y> = <x, Gy> to
FP32 rounding (relative 1e-5)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 1e-5


def torch_mod():
    import torch

    return torch


def random_case(seed, n=3000, G=256, supports=(8, 12, 30), spread=0.45, out_frac=0.05,
                skip_frac=0.05):
    rng = np.random.default_rng(seed)
    scale = 1.0
    lim = spread * G
    uvw = np.column_stack([rng.uniform(-lim, lim, n), rng.uniform(-lim, lim, n),
                           rng.uniform(-1, 1, n)])
    # some far outside, some exactly on integer / half-integer coordinates
    k = int(out_frac * n)
    uvw[:k, 0] = rng.choice([-1, 1], k) * rng.uniform(G / 2, 2 * G, k)
    uvw[k:2 * k, :2] = np.round(uvw[k:2 * k, :2] * 2) / 2
    sup = np.asarray(supports, np.int32)
    plane = rng.integers(0, len(sup), n).astype(np.int32)
    plane[rng.uniform(0, 1, n) < skip_frac] = -1
    offs, total = O_layout(sup)
    gcf = (rng.standard_normal(total) + 1j * rng.standard_normal(total)) / 8
    vis = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    return dict(uvw=uvw, vis=vis, plane=plane, sup=sup, offs=offs, gcf=gcf, G=G, scale=scale,
                grid_size=G, margin=int(sup.max()))


def O_layout(sup):
    from rc_gb300.gcf import layout

    return layout(sup)


def make_plan(c, tile=0, threads=0, cap=0):
    torch = torch_mod()
    from rc_gb300.engine import Plan

    d_uvw = torch.tensor(c["uvw"], dtype=torch.float64, device="cuda")
    d_plane = torch.tensor(c["plane"], dtype=torch.int32, device="cuda")
    P = Plan(d_uvw, scale=c["scale"], grid_size=c["grid_size"], grid_shape=(c["G"], c["G"]),
             supports=c["sup"], gcf_offsets=c["offs"], margin=c["margin"], plane=d_plane,
             tile=tile, threads=threads, period_cap=cap)
    P._keep = (d_uvw, d_plane)
    return P


def oracle_grid(c, vis=None, gcf=None):
    g = np.zeros((c["G"], c["G"]), np.complex128)
    O.scatter_planes(c["scale"], c["grid_size"], c["margin"], c["uvw"],
                     c["vis"] if vis is None else vis, c["plane"], c["sup"],
                     c["gcf"] if gcf is None else gcf, c["offs"], g)
    return g


def oracle_degrid(c, grid, mode=0, gcf=None):
    return O.degrid_planes(c["scale"], c["grid_size"], c["margin"], c["uvw"], c["plane"], c["sup"],
                           c["gcf"] if gcf is None else gcf, c["offs"], grid, mode=mode)


def oracle_index(c):
    """x0, y0, phase, plane, kept per visibility (per-plane S)."""
    n = c["uvw"].shape[0]
    out = np.zeros((n, 5), np.int32)
    v5 = np.zeros((n, 5))
    v5[:, :3] = c["uvw"]
    for p, S in enumerate(c["sup"]):
        m = c["plane"] == p
        if not m.any():
            continue
        ix = O.index(v5[m], c["scale"], c["grid_size"], int(S), c["margin"], 0, 0, c["G"], c["G"])
        out[m, 0], out[m, 1] = ix[:, 0], ix[:, 1]
        out[m, 2] = ix[:, 2] + 8 * ix[:, 3]
        out[m, 3] = p
        out[m, 4] = ix[:, 4]
    skip = c["plane"] < 0
    out[skip] = 0
    out[skip, 3] = c["plane"][skip]
    return out


def expected_auto_stage(P, c, cap):
    """The automatic staging choice restated on the host: split rows when at
    least half of the kept taps are in pieces degridding can pair (even piece
    width, even support, even GCF offset of the piece), otherwise TMA (the
    caller maps TMA to rows for an odd tile edge)."""
    from rc_gb300 import lib

    idx = P.export_index().cpu().numpy()
    kept = idx[:, 4] == 1
    counts = np.bincount(idx[kept, 3], minlength=len(c["sup"]))
    taps = paired = 0
    for p, S in enumerate(c["sup"]):
        S = int(S)
        k = (S + cap - 1) // cap
        Pp = (S + k - 1) // k
        if k > 1 and S % 2 == 0 and Pp % 2 == 1 and Pp < cap:
            Pp += 1  # even supports are cut into even-width pieces
        for ky in range(k):
            for kx in range(k):
                if kx * Pp >= S or ky * Pp >= S:
                    continue
                wx, wy = min(Pp, S - kx * Pp), min(Pp, S - ky * Pp)
                taps += counts[p] * wx * wy
                if wx % 2 == 0 and S % 2 == 0 and (c["offs"][p] + kx * Pp) % 2 == 0:
                    paired += counts[p] * wx * wy
    assert taps == P.stats()["taps"]
    return lib.STAGE_SPLIT if 2 * paired >= taps else lib.STAGE_TMA


def test_index_bit_exact():
    c = random_case(1)
    P = make_plan(c)
    got = P.export_index().cpu().numpy()
    exp = oracle_index(c)
    kept = exp[:, 4] == 1
    assert np.array_equal(got[:, 3:5], exp[:, 3:5])
    assert np.array_equal(got[kept, :3], exp[kept, :3])
    st = P.stats()
    assert st["kept"] == int(kept.sum())
    assert st["taps"] == int((c["sup"][c["plane"][kept]].astype(np.int64) ** 2).sum())


def test_plain_fp64_grid_and_degrid():
    torch = torch_mod()
    c = random_case(2)
    P = make_plan(c)
    d_vis = torch.tensor(c["vis"], dtype=torch.complex128, device="cuda")
    d_gcf = torch.tensor(c["gcf"], dtype=torch.complex128, device="cuda")
    grid = torch.zeros((c["G"], c["G"]), dtype=torch.complex128, device="cuda")
    P.grid64(d_vis, d_gcf, grid)
    exp = oracle_grid(c)
    assert rel_l2(grid.cpu().numpy(), exp) < TOL64
    model = np.random.default_rng(5).standard_normal((c["G"], c["G"])) * (1 + 1j)
    d_model = torch.tensor(model, dtype=torch.complex128, device="cuda")
    for mode in (0, 1):
        pred = P.degrid64(d_gcf, d_model, mode=mode).cpu().numpy()
        assert rel_l2(pred, oracle_degrid(c, model, mode)) < TOL64


@pytest.mark.parametrize("tile,threads,cap", [(32, 256, 32), (16, 128, 16), (64, 512, 32),
                                              (8, 256, 8), (32, 512, 64), (25, 256, 32),
                                              (9, 128, 16)])
def test_fp32_tiled_grid_matches_fp64_oracle(tile, threads, cap):
    torch = torch_mod()
    c = random_case(3, supports=(8, 12, 30, 7, 1, 40, 70))
    P = make_plan(c, tile, threads, cap)
    d_vis = torch.tensor(c["vis"], dtype=torch.complex64, device="cuda")
    d_gcf = torch.tensor(c["gcf"], dtype=torch.complex64, device="cuda")
    grid = torch.zeros((c["G"], c["G"]), dtype=torch.complex64, device="cuda")
    P.grid(d_vis, d_gcf, grid)
    torch.cuda.synchronize()
    exp = oracle_grid(c)
    assert rel_l2(grid.cpu().numpy(), exp) < TOL32
    # degridding, both modes, every staging form: the same taps in the same
    # order, so the forms agree to the rounding of the cut pieces' atomics
    from rc_gb300 import lib

    model = (np.random.default_rng(6).standard_normal((c["G"], c["G"])) +
             1j * np.random.default_rng(7).standard_normal((c["G"], c["G"])))
    d_model = torch.tensor(model, dtype=torch.complex64, device="cuda")
    auto = expected_auto_stage(P, c, cap)
    if auto == lib.STAGE_TMA and tile % 2:
        auto = lib.STAGE_ROWS
    for stage, want in [(lib.STAGE_AUTO, auto), (lib.STAGE_SPLIT, lib.STAGE_SPLIT),
                        (lib.STAGE_TMA, lib.STAGE_TMA if tile % 2 == 0 else lib.STAGE_ROWS),
                        (lib.STAGE_ROWS, lib.STAGE_ROWS)]:
        P.set_stage(stage)
        preds = []
        for mode in (0, 1):
            pred = P.degrid(d_gcf, d_model, mode=mode).cpu().numpy()
            assert rel_l2(pred, oracle_degrid(c, model, mode)) < TOL32, (stage, mode)
            preds.append(pred)
        # the form it used (TMA only for an even tile edge); no stage wait ran out
        assert P.device_status() == (0, want), stage
        if stage == lib.STAGE_AUTO:
            first = preds
        else:
            for a, b in zip(preds, first):
                assert rel_l2(a, b) < 1e-6


def test_fp32_adjoint_identity():
    torch = torch_mod()
    c = random_case(4, supports=(8, 16, 33, 64))
    P = make_plan(c)
    rng = np.random.default_rng(8)
    x = rng.standard_normal((c["G"], c["G"])) + 1j * rng.standard_normal((c["G"], c["G"]))
    y = rng.standard_normal(len(c["vis"])) + 1j * rng.standard_normal(len(c["vis"]))
    d_gcf = torch.tensor(c["gcf"], dtype=torch.complex64, device="cuda")
    Dx = P.degrid(d_gcf, torch.tensor(x, dtype=torch.complex64, device="cuda")).cpu().numpy()
    Gy = torch.zeros((c["G"], c["G"]), dtype=torch.complex64, device="cuda")
    P.grid(torch.tensor(y, dtype=torch.complex64, device="cuda"), d_gcf, Gy)
    lhs = np.vdot(Dx.astype(np.complex128), y)
    rhs = np.vdot(x, Gy.cpu().numpy().astype(np.complex128))
    assert abs(lhs - rhs) <= TOL32 * abs(lhs)


def test_fp32_synthetic_w_projection_case():
    """The small synthetic observation (w-binned by the reference rule)."""
    torch = torch_mod()
    from rc_gb300 import synth
    from rc_gb300.engine import Plan
    from rc_gb300.gcf import layout

    ob = synth.config("small")
    offs, total = layout(ob.supports)
    rng = np.random.default_rng(9)
    gcf = (rng.standard_normal(total) + 1j * rng.standard_normal(total)) / 16
    d_uvw = torch.tensor(ob.uvw, device="cuda")
    P = Plan(d_uvw, scale=ob.scale, grid_size=ob.grid_size,
             grid_shape=(ob.grid_size, ob.grid_size), supports=ob.supports,
             w_range=(ob.w_low, ob.w_high))
    plane = O.wbin(ob.uvw, ob.w_low, ob.w_high, ob.n_planes)
    assert np.array_equal(P.export_index().cpu().numpy()[:, 3], plane)
    grid = torch.zeros((ob.grid_size, ob.grid_size), dtype=torch.complex64, device="cuda")
    P.grid(torch.tensor(ob.vis, dtype=torch.complex64, device="cuda"),
           torch.tensor(gcf, dtype=torch.complex64, device="cuda"), grid)
    exp = np.zeros((ob.grid_size, ob.grid_size), np.complex128)
    O.scatter_planes(ob.scale, ob.grid_size, int(ob.supports.max()), ob.uvw, ob.vis, plane,
                     ob.supports, gcf, offs, exp)
    assert rel_l2(grid.cpu().numpy(), exp) < TOL32


def test_empty_and_all_skipped():
    torch = torch_mod()
    from rc_gb300.engine import Plan

    for n, plane_val in [(0, 0), (50, -1)]:
        c = random_case(5, n=max(n, 1))
        uvw = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
        plane = torch.full((n,), plane_val, dtype=torch.int32, device="cuda")
        P = Plan(uvw, scale=1.0, grid_size=64, grid_shape=(64, 64), supports=c["sup"],
                 gcf_offsets=c["offs"], plane=plane)
        gcf = torch.zeros(int(c["offs"][-1] + 64 * 900), dtype=torch.complex64, device="cuda")
        grid = torch.zeros((64, 64), dtype=torch.complex64, device="cuda")
        P.grid(torch.zeros(n, dtype=torch.complex64, device="cuda"), gcf, grid)
        pred = P.degrid(gcf, grid)
        torch.cuda.synchronize()
        assert float(grid.abs().max()) == 0.0 if n else True
        assert pred.numel() == n and (n == 0 or float(pred.abs().max()) == 0.0)
        assert P.stats()["kept"] == 0


def test_fp32_repeat_is_stable():
    torch = torch_mod()
    c = random_case(6)
    P = make_plan(c)
    d_vis = torch.tensor(c["vis"], dtype=torch.complex64, device="cuda")
    d_gcf = torch.tensor(c["gcf"], dtype=torch.complex64, device="cuda")
    g1 = torch.zeros((c["G"], c["G"]), dtype=torch.complex64, device="cuda")
    g2 = torch.zeros_like(g1)
    P.grid(d_vis, d_gcf, g1)
    P.grid(d_vis, d_gcf, g2)
    assert rel_l2(g1.cpu().numpy(), g2.cpu().numpy()) < 1e-6


@pytest.mark.parametrize("tile,threads,cap", [(24, 0, 0), (8, 512, 64), (32, 256, 32)])
def test_largest_supports(tile, threads, cap):
    """Supports up to the library's limit (GB_MAX_SUPPORT = 256), odd and even,
    cut into pieces of up to cap x cap: indices, FP32 pair and FP64 pair
    against the oracle."""
    torch = torch_mod()
    c = random_case(11, n=600, G=1024, supports=(256, 255, 129, 2))
    P = make_plan(c, tile=tile, threads=threads, cap=cap)
    got = P.export_index().cpu().numpy()
    exp = oracle_index(c)
    kept = exp[:, 4] == 1
    assert kept.sum() > 300
    assert np.array_equal(got[:, 3:5], exp[:, 3:5])
    assert np.array_equal(got[kept, :3], exp[kept, :3])
    d_gcf32 = torch.tensor(c["gcf"], dtype=torch.complex64, device="cuda")
    grid = torch.zeros((c["G"], c["G"]), dtype=torch.complex64, device="cuda")
    P.grid(torch.tensor(c["vis"], dtype=torch.complex64, device="cuda"), d_gcf32, grid)
    ref = oracle_grid(c)
    assert rel_l2(grid.cpu().numpy(), ref) < TOL32
    model = np.random.default_rng(12).standard_normal((c["G"], c["G"])) * (1 - 2j)
    pred = P.degrid(d_gcf32, torch.tensor(model, dtype=torch.complex64, device="cuda"))
    assert rel_l2(pred.cpu().numpy(), oracle_degrid(c, model)) < TOL32
    g64 = torch.zeros((c["G"], c["G"]), dtype=torch.complex128, device="cuda")
    P.grid64(torch.tensor(c["vis"], device="cuda"), torch.tensor(c["gcf"], device="cuda"), g64)
    assert rel_l2(g64.cpu().numpy(), ref) < TOL64


def test_single_visibility_each_plane():
    """One visibility per plane, one of them at the last corner the bounds rule
    keeps and one a pixel past it (the rule's extra -1 drops it): the
    footprints land exactly where the oracle puts them."""
    torch = torch_mod()
    c = random_case(13, n=5, G=256, supports=(8, 31, 64, 1))
    G = c["G"]
    # S = 64 with margin 64: corner x0 = round(u) + G/2 - 32 is kept up to
    # G - 64 - 1 = 191, i.e. u = 95; u = 96 gives x0 = 192, dropped
    c["uvw"] = np.array([[0.0, 0.0, 0.0], [12.25, -7.5, 0.0], [95.0, 3.0, 0.0],
                         [-3.0, 40.375, 0.0], [96.0, 3.0, 0.0]])
    c["plane"] = np.array([0, 1, 2, 3, 2], np.int32)
    P = make_plan(c)
    exp_idx = oracle_index(c)
    assert exp_idx[2, 0] == 191 and exp_idx[2, 4] == 1 and exp_idx[4, 4] == 0
    got = P.export_index().cpu().numpy()
    assert np.array_equal(got[:, 3:5], exp_idx[:, 3:5])
    assert np.array_equal(got[:4, :3], exp_idx[:4, :3])
    d_gcf = torch.tensor(c["gcf"], dtype=torch.complex64, device="cuda")
    grid = torch.zeros((G, G), dtype=torch.complex64, device="cuda")
    P.grid(torch.tensor(c["vis"], dtype=torch.complex64, device="cuda"), d_gcf, grid)
    assert rel_l2(grid.cpu().numpy(), oracle_grid(c)) < TOL32


def test_gcf_on_an_8_byte_boundary():
    """A GCF array that starts 8 bytes past a 16-byte boundary: no tap pairs
    (their 16-byte loads need the alignment), so the automatic staging takes
    plain rows; forced split rows read every tap on its own.  Both against the
    oracle."""
    torch = torch_mod()
    from rc_gb300 import lib

    c = random_case(14, supports=(8, 16, 40))
    P = make_plan(c, tile=24, threads=256, cap=40)
    buf = torch.zeros(len(c["gcf"]) + 1, dtype=torch.complex64, device="cuda")
    buf[1:] = torch.tensor(c["gcf"], dtype=torch.complex64, device="cuda")
    d_gcf = buf[1:]
    assert d_gcf.data_ptr() % 16 == 8
    model = np.random.default_rng(15).standard_normal((c["G"], c["G"])) * (1 + 0.5j)
    d_model = torch.tensor(model, dtype=torch.complex64, device="cuda")
    for stage, want in [(lib.STAGE_AUTO, lib.STAGE_TMA), (lib.STAGE_SPLIT, lib.STAGE_SPLIT)]:
        P.set_stage(stage)
        for mode in (0, 1):
            pred = P.degrid(d_gcf, d_model, mode=mode).cpu().numpy()
            assert rel_l2(pred, oracle_degrid(c, model, mode)) < TOL32, (stage, mode)
        assert P.device_status() == (0, want)
    grid = torch.zeros((c["G"], c["G"]), dtype=torch.complex64, device="cuda")
    P.grid(torch.tensor(c["vis"], dtype=torch.complex64, device="cuda"), d_gcf, grid)
    assert rel_l2(grid.cpu().numpy(), oracle_grid(c)) < TOL32
