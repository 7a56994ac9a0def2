"""The FP64 degridders' double-float arithmetic (gb_plain.cu) at the edges of
its range, against the oracle (relative L2 1e-12, the FP64 bar): grids and
GCFs scaled to extreme magnitudes, a grid spanning 40 decades, a GCF with
exact zeros and values 1e-300 below its largest; and Inf, NaN and subnormal
inputs, which take the native FP64 loop and must propagate as the oracle's
FP64 arithmetic does.  Through the engine (both modes), a batch and the
reference ABI (kern_degrid_gpu1)."""
import numpy as np
import pytest

from oracle import oracle as O
from rc_gb300 import compat
from tests.conftest import rel_l2
from tests.test_gpu_engine import make_plan, oracle_degrid, random_case, torch_mod

pytestmark = pytest.mark.gpu

TOL64 = 1e-12


def engine_pair(c, model, gcf):
    torch = torch_mod()
    P = make_plan(c)
    d_gcf = torch.tensor(gcf, dtype=torch.complex128, device="cuda")
    d_model = torch.tensor(model, dtype=torch.complex128, device="cuda")
    out = [P.degrid64(d_gcf, d_model, mode=m).cpu().numpy() for m in (0, 1)]
    P.close()
    return out


def model_grid(seed, G):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((G, G)) + 1j * rng.standard_normal((G, G))


@pytest.mark.parametrize("sg,sc", [(1e-250, 1e200), (1e250, 1e-240), (2.0 ** -1000, 1.0),
                                   (1e300, 1e-300), (3.0, 1e-100)])
def test_extreme_magnitudes(sg, sc):
    c = random_case(31)
    model = model_grid(1, c["G"]) * sg
    gcf = c["gcf"] * sc
    for mode, got in enumerate(engine_pair(c, model, gcf)):
        exp = oracle_degrid(c, model, mode, gcf=gcf)
        assert np.isfinite(exp).all()
        assert rel_l2(got, exp) < TOL64


def test_forty_decades_in_the_grid_and_zeros_in_the_gcf():
    c = random_case(32)
    rng = np.random.default_rng(2)
    G = c["G"]
    model = model_grid(3, G) * 10.0 ** rng.uniform(-40, 0, (G, G))
    gcf = c["gcf"].copy()
    gcf[rng.uniform(0, 1, gcf.size) < 0.2] = 0
    tiny = rng.uniform(0, 1, gcf.size) < 0.05
    gcf[tiny] *= 1e-300
    for mode, got in enumerate(engine_pair(c, model, gcf)):
        assert rel_l2(got, oracle_degrid(c, model, mode, gcf=gcf)) < TOL64


def _same_nonfinite(got, exp):
    bad = ~np.isfinite(exp)
    assert bad.any() and not bad.all()
    assert np.array_equal(~np.isfinite(got), bad)
    assert rel_l2(got[~bad], exp[~bad]) < TOL64


def test_nan_in_the_grid_and_inf_in_the_gcf_propagate():
    c = random_case(33)
    G = c["G"]
    model = model_grid(4, G)
    model[G // 2 + 3, G // 2 - 7] = np.nan
    for mode, got in enumerate(engine_pair(c, model, c["gcf"])):
        _same_nonfinite(got, oracle_degrid(c, model, mode))
    gcf = c["gcf"].copy()
    gcf[c["offs"][1] + 5 * c["sup"][1] ** 2 + 3] = np.inf  # one tap of one phase of plane 1
    model = model_grid(5, G)
    for mode, got in enumerate(engine_pair(c, model, gcf)):
        _same_nonfinite(got, oracle_degrid(c, model, mode, gcf=gcf))


def test_subnormal_grid_takes_the_native_loop():
    """A grid of double subnormals (which the split would drop): the native
    loop's results are the oracle's up to the subnormal range's own
    rounding (absolute, 2^-1074 per operation)."""
    c = random_case(34)
    model = model_grid(6, c["G"]) * 1e-310
    for mode, got in enumerate(engine_pair(c, model, c["gcf"])):
        exp = oracle_degrid(c, model, mode)
        assert np.abs(exp).max() > 0
        assert np.abs(got - exp).max() < 1e-318 * 64


def test_batch_members_share_the_scratch():
    torch = torch_mod()
    from rc_gb300.engine import Batch

    cases = [random_case(40 + i, G=G) for i, G in enumerate((128, 256, 64))]
    # one GCF layout for all members
    for cc in cases[1:]:
        cc["gcf"], cc["offs"], cc["sup"] = cases[0]["gcf"], cases[0]["offs"], cases[0]["sup"]
        cc["margin"] = cases[0]["margin"]
    members = [dict(uvw=torch.tensor(cc["uvw"], device="cuda"), scale=cc["scale"],
                    grid_size=cc["grid_size"], grid_shape=(cc["G"], cc["G"]),
                    supports=cc["sup"], gcf_offsets=cc["offs"], margin=cc["margin"],
                    plane=torch.tensor(cc["plane"], dtype=torch.int32, device="cuda"))
               for cc in cases]
    B = Batch(members)
    d_gcf = torch.tensor(cases[0]["gcf"], device="cuda")
    models = [model_grid(50 + i, cc["G"]) * 10.0 ** (40 * i - 40) for i, cc in enumerate(cases)]
    grids = [torch.tensor(m, device="cuda") for m in models]
    preds = [torch.empty(len(cc["vis"]), dtype=torch.complex128, device="cuda") for cc in cases]
    B.degrid64(d_gcf, grids, preds, mode=0)
    for cc, m, p in zip(cases, models, preds):
        assert rel_l2(p.cpu().numpy(), oracle_degrid(cc, m, 0)) < TOL64
    B.close()


def test_reference_abi_with_nan_and_extreme_scales():
    rng = np.random.default_rng(7)
    n, G, S = 3000, 256, 16
    vis5 = np.zeros((n, 5))
    vis5[:, :2] = rng.uniform(-0.45 * G, 0.45 * G, (n, 2))
    vis5[:, 3:] = rng.standard_normal((n, 2))
    gcf = (rng.standard_normal((64, S, S)) + 1j * rng.standard_normal((64, S, S))) * 1e-200
    grid = model_grid(8, G) * 1e150
    out = np.zeros_like(vis5)
    assert compat.call_degrid("kern_degrid_gpu1", 1.0, G, S, gcf, grid, vis5, out) == 0
    exp = O.degrid(1.0, G, S, gcf, grid, vis5)
    assert rel_l2(out[:, 3:] - vis5[:, 3:], exp[:, 3:] - vis5[:, 3:]) < TOL64
    grid[100, 120] = np.nan
    assert compat.call_degrid("kern_degrid_gpu1", 1.0, G, S, gcf, grid, vis5, out) == 0
    exp = O.degrid(1.0, G, S, gcf, grid, vis5)
    _same_nonfinite(out[:, 3], exp[:, 3])


def _scatter_case(seed, S, n=3000, G=256):
    rng = np.random.default_rng(seed)
    vis5 = np.zeros((n, 5))
    vis5[:, :2] = rng.uniform(-0.45 * G, 0.45 * G, (n, 2))
    vis5[:, 3:] = rng.standard_normal((n, 2))
    vis5[:40, 0] = 1e9  # out of bounds
    gcf = rng.standard_normal((64, S, S)) + 1j * rng.standard_normal((64, S, S))
    return vis5, gcf, G


def _abi_scatter(vis5, gcf, G, margin=64):
    # a zero grid: the increments span magnitudes a unit grid would absorb
    got = np.zeros((G, G), np.complex128)
    assert compat.call_scatter("kern_scatter_gpu1", 1.0, G, margin, vis5, gcf, got) == 0
    exp = np.zeros_like(got)
    O.scatter(1.0, G, margin, vis5, gcf, exp)
    return got, exp


@pytest.mark.parametrize("S", [8, 16, 32, 64])
@pytest.mark.parametrize("sv,sc", [(1e150, 1e-200), (2.0 ** -1000, 1.0), (1e-300, 1e300)])
def test_reference_abi_scatter_extreme_magnitudes(S, sv, sc):
    """The shared-memory double-float gridder behind kern_scatter_gpu1 with
    visibilities and GCFs scaled far apart."""
    vis5, gcf, G = _scatter_case(60 + S, S)
    vis5[:, 3:] *= sv
    got, exp = _abi_scatter(vis5, gcf * sc, G)
    assert np.isfinite(exp).all() and np.abs(exp).max() > 0
    assert rel_l2(got, exp) < TOL64


@pytest.mark.parametrize("S", [16, 64])
def test_reference_abi_scatter_forty_decades(S):
    vis5, gcf, G = _scatter_case(70 + S, S)
    rng = np.random.default_rng(3)
    vis5[:, 3:] *= 10.0 ** rng.uniform(-40, 0, (len(vis5), 1))
    gcf[rng.uniform(0, 1, gcf.shape) < 0.2] = 0
    got, exp = _abi_scatter(vis5, gcf, G)
    assert rel_l2(got, exp) < TOL64


@pytest.mark.parametrize("S", [8, 16, 32, 64])
def test_reference_abi_scatter_nonfinite_and_subnormal(S):
    """A NaN visibility or an Inf GCF tap sends the call down the FP64
    atomics, which propagate them as the oracle does; so does a subnormal."""
    vis5, gcf, G = _scatter_case(80 + S, S)
    v = vis5.copy()
    v[500, :2] = 0.0  # a kept footprint at the centre
    v[500, 3] = np.nan
    got, exp = _abi_scatter(v, gcf, G)
    _same_nonfinite(got, exp)
    g = gcf.copy()
    g[5, 3, 2] = np.inf
    got, exp = _abi_scatter(vis5, g, G)
    _same_nonfinite(got, exp)
    v = vis5.copy()
    v[:, 3:] *= 1e-310
    got, exp = _abi_scatter(v, gcf, G)
    assert np.abs(exp).max() > 0
    assert np.abs(got - exp).max() < 1e-318 * 4 * S * S
