"""Both ways the reference-ABI calls reach the caller's host buffers, against
the oracle (FP64, relative L2 1e-12; kern_detile exact):
- direct (the GB300's kernels reach pageable host memory through the host's
  page tables): only the 32 x 32 grid blocks the visibilities touch move, and
  kern_detile runs in place on the GPU;
- whole-buffer copies: in a child process with RC_GB300_HOST_DIRECT=0, and
  in this process for host buffers that are not 16-byte aligned."""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

from oracle import oracle as O
from rc_gb300 import compat, lib
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _case(seed, n=6000, G=384, S=32):
    rng = np.random.default_rng(seed)
    lim = 0.46 * G
    vis5 = np.zeros((n, 5))
    vis5[:, 0] = rng.uniform(-lim, lim, n)
    vis5[:, 1] = 0.3 * rng.uniform(-lim, lim, n)  # a band: many blocks untouched
    vis5[:, 2] = rng.uniform(-5, 5, n)
    vis5[:, 3:] = rng.standard_normal((n, 2))
    vis5[:40, 0] = 1e9
    gcf = rng.standard_normal((64, S, S)) + 1j * rng.standard_normal((64, S, S))
    grid0 = rng.standard_normal((G, G)) + 1j * rng.standard_normal((G, G))
    return vis5, gcf, grid0


def _misaligned(shape):
    """A complex128 array whose data starts 8 bytes past a 16-byte boundary."""
    n = int(np.prod(shape))
    raw = np.zeros(2 * n + 2)
    off = 1 if raw.ctypes.data % 16 == 0 else 0
    a = raw[off:off + 2 * n].view(np.complex128).reshape(shape)
    assert a.ctypes.data % 16 == 8
    return a


def check_all(aligned=True):
    """Scatter (in place, on a margin tile too), degrid and kern_detile, each
    against the oracle."""
    mk = (lambda s: np.zeros(s, np.complex128)) if aligned else _misaligned
    vis5, gcf, grid0 = _case(5)
    G = grid0.shape[0]
    got = mk(grid0.shape)
    got[...] = grid0
    assert compat.call_scatter("kern_scatter_gpu1", 1.0, G, 64, vis5, gcf, got) == 0
    exp = grid0.copy()
    O.scatter(1.0, G, 64, vis5, gcf, exp)
    assert rel_l2(got - grid0, exp - grid0) < TOL64
    # a margin tile with non-zero mins
    tile = mk((160, 224))
    tile[...] = 0
    assert compat.call_scatter("kern_scatter_gpu1", 1.0, G, 32, vis5, gcf, tile, 100, 80) == 0
    exp_t = np.zeros((160, 224), np.complex128)
    O.scatter(1.0, G, 32, vis5, gcf, exp_t, 100, 80)
    assert np.abs(exp_t).sum() > 0 and rel_l2(tile, exp_t) < TOL64
    # degridding against a model grid
    model = mk(grid0.shape)
    model[...] = grid0
    out = np.zeros_like(vis5)
    assert compat.call_degrid("kern_degrid_gpu1", 1.0, G, 64, gcf, model, vis5, out) == 0
    exp_d = O.degrid(1.0, G, 64, gcf, grid0, vis5)
    assert np.array_equal(out[:, :3], vis5[:, :3])
    assert rel_l2(out[:, 3:], exp_d[:, 3:]) < TOL64
    L = lib.load()
    # kern_detile: full += tile over the overlap
    full = mk((300, 300))
    full[...] = 1 + 1j
    src = mk((160, 224))
    src[...] = exp_t
    bi, bo = compat.grid_buf(src, 100, 80), compat.grid_buf(full, 0, 0)
    assert L.kern_detile(C.byref(bi), C.byref(bo)) == 0
    exp_f = O.detile(exp_t, (100, 80), np.full((300, 300), 1 + 1j), (0, 0))
    assert np.array_equal(full, exp_f)


def test_direct_path_on_this_gpu():
    """The GB300 reaches pageable host memory; the calls take the direct path."""
    assert lib.load().gb_host_direct() == 1
    check_all(aligned=True)


def test_unaligned_host_buffers_are_copied():
    check_all(aligned=False)


def test_whole_buffer_copies_when_switched_off():
    code = ("import sys; sys.path.insert(0, %r)\n"
            "from rc_gb300 import lib\n"
            "assert lib.load().gb_host_direct() == 0\n"
            "from tests.test_gpu_abi_paths import check_all\n"
            "check_all(aligned=True)\nprint('copy path ok')\n" % ROOT)
    env = dict(os.environ, RC_GB300_HOST_DIRECT="0")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env,
                       cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "copy path ok" in r.stdout
