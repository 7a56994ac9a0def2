"""gb_grid_f32_noalloc: gridding without any device allocation, for callers
that cannot call cudaMalloc (a host framework that owns all device memory, a
fixed-budget or real-time pipeline).  Called through the C ABI and checked
against the planned entry point (gb_plan_create + gb_grid_f32) and against the
FP64 oracle, within the FP32 tolerance of the other tests, on two calls in a
row that share the static scratch array; once with every library allocation
made to fail (so the call provably allocates nothing), and once with the
w-planes computed from w (no plane array).  This file is collected last on
purpose."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL32 = 1e-5


def _case(seed, n, G=256, supports=(8, 12, 30, 70)):
    rng = np.random.default_rng(seed)
    lim = 0.45 * G
    uvw = np.column_stack([rng.uniform(-lim, lim, n), rng.uniform(-lim, lim, n),
                           rng.uniform(-1, 1, n)])
    uvw[: n // 50, 0] = 3 * G  # some out of bounds
    sup = np.asarray(supports, np.int32)
    plane = rng.integers(-1, len(sup), n).astype(np.int32)
    from rc_gb300.gcf import layout

    offs, total = layout(sup)
    gcf = (rng.standard_normal(total) + 1j * rng.standard_normal(total)) / 8
    vis = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    return uvw, plane, sup, offs, gcf, vis, G


def _geometry(sup, offs, G, w_range=None):
    from rc_gb300 import lib

    g = lib.Geometry()
    g.scale = 1.0
    g.grid_size = G
    g.margin = int(sup.max())
    g.ext_x = g.ext_y = g.pitch = G
    g.n_planes = len(sup)
    g.tile = g.threads = g.period_cap = g.bundles_per_cta = 0
    g._sup = np.ascontiguousarray(sup, np.int32)
    g._offs = np.ascontiguousarray(offs, np.int64)
    g.supports = g._sup.ctypes.data_as(C.POINTER(C.c_int32))
    g.gcf_offsets = g._offs.ctypes.data_as(C.POINTER(C.c_int64))
    g.w_low, g.w_high = w_range if w_range is not None else (-np.inf, np.inf)
    return g


def _noalloc(case, use_plane=True, w_range=None, fail_allocs=False):
    import torch

    from rc_gb300 import lib

    uvw, plane, sup, offs, gcf, vis, G = case
    L = lib.load()
    d_uvw = torch.tensor(uvw, device="cuda")
    d_plane = torch.tensor(plane, device="cuda")
    d_vis = torch.tensor(vis, dtype=torch.complex64, device="cuda")
    d_gcf = torch.tensor(gcf, dtype=torch.complex64, device="cuda")
    grid = torch.zeros((G, G), dtype=torch.complex64, device="cuda")
    g = _geometry(sup, offs, G, w_range)
    torch.cuda.synchronize()
    if fail_allocs:
        # from here on every device allocation of the library fails
        assert L.gb_debug_fail_allocs(0, 1 << 30) == 0
    try:
        rc = L.gb_grid_f32_noalloc(C.byref(g), len(vis), d_uvw.data_ptr(), 3,
                                   d_plane.data_ptr() if use_plane else None, d_vis.data_ptr(),
                                   d_gcf.data_ptr(), grid.data_ptr(),
                                   torch.cuda.current_stream().cuda_stream)
    finally:
        if fail_allocs:
            assert L.gb_debug_fail_allocs(0, 0) == 0
    lib.check(rc, "gb_grid_f32_noalloc")
    torch.cuda.synchronize()
    return grid.cpu().numpy()


def _planned(case, use_plane=True, w_range=None):
    import torch

    from rc_gb300.engine import Plan

    uvw, plane, sup, offs, gcf, vis, G = case
    d_uvw = torch.tensor(uvw, device="cuda")
    d_plane = torch.tensor(plane, device="cuda")
    P = Plan(d_uvw, scale=1.0, grid_size=G, grid_shape=(G, G), supports=sup, gcf_offsets=offs,
             margin=int(sup.max()), plane=d_plane if use_plane else None, w_range=w_range)
    grid = torch.zeros((G, G), dtype=torch.complex64, device="cuda")
    P.grid(torch.tensor(vis, dtype=torch.complex64, device="cuda"),
           torch.tensor(gcf, dtype=torch.complex64, device="cuda"), grid)
    torch.cuda.synchronize()
    out = grid.cpu().numpy()
    P.close()
    return out


def _oracle(case, plane=None):
    uvw, pl, sup, offs, gcf, vis, G = case
    g = np.zeros((G, G), np.complex128)
    O.scatter_planes(1.0, G, int(sup.max()), uvw, vis, pl if plane is None else plane, sup, gcf,
                     offs, g)
    return g


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_noalloc_matches_planned_entry_point_twice():
    a = _case(101, 20000)
    b = _case(202, 6000, supports=(16, 8, 64))
    ref_a, ref_b = _planned(a), _planned(b)
    assert np.abs(ref_a).sum() > 0 and np.abs(ref_b).sum() > 0
    # two calls in a row on the shared scratch array, different inputs
    got_a = _noalloc(a)
    got_b = _noalloc(b)
    assert _rel(got_a, ref_a) < TOL32
    assert _rel(got_b, ref_b) < TOL32
    # and the first input again after the second left its contents behind
    assert _rel(_noalloc(a), ref_a) < TOL32
    # both against the FP64 oracle itself
    assert _rel(got_a, _oracle(a)) < TOL32
    assert _rel(got_b, _oracle(b)) < TOL32


def test_noalloc_allocates_nothing():
    """Every device allocation of the library is made to fail for the call's
    duration; the call still succeeds, twice, and matches the oracle."""
    a = _case(303, 15000)
    exp = _oracle(a)
    for _ in range(2):
        assert _rel(_noalloc(a, fail_allocs=True), exp) < TOL32


def test_noalloc_bins_w_without_a_plane_array():
    """d_plane = NULL: the planes come from w by the binning rule over
    [w_low, w_high), as in gb_plan_create."""
    a = _case(404, 12000)
    w_range = (-1.0, 1.0)
    got = _noalloc(a, use_plane=False, w_range=w_range)
    ref = _planned(a, use_plane=False, w_range=w_range)
    assert np.abs(ref).sum() > 0
    assert _rel(got, ref) < TOL32
    sup = a[2]
    plane = O.wbin(a[0], w_range[0], w_range[1], len(sup)).astype(np.int32)
    plane[plane >= len(sup)] = -1
    assert _rel(got, _oracle(a, plane=plane)) < TOL32


def test_noalloc_rejects_sizes_beyond_its_limit():
    import torch

    from rc_gb300 import lib

    L = lib.load()
    n = lib.NOALLOC_MAX_VIS + 1
    sup = np.array([8], np.int32)
    offs = np.array([0], np.int64)
    g = _geometry(sup, offs, 64)
    d = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    v = torch.zeros(n, dtype=torch.complex64, device="cuda")
    gcf = torch.zeros(64 * 64, dtype=torch.complex64, device="cuda")
    grid = torch.ones((64, 64), dtype=torch.complex64, device="cuda")
    rc = L.gb_grid_f32_noalloc(C.byref(g), n, d.data_ptr(), 3, None, v.data_ptr(), gcf.data_ptr(),
                               grid.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == lib.ERR_CAPACITY
    assert b"allocation-free" in L.gb_last_error()
    torch.cuda.synchronize()
    assert float((grid - 1).abs().max()) == 0.0  # nothing ran
