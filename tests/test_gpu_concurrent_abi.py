"""Concurrent callers of the reference ABI.  The reference's programs are
built -threaded (MS6/ms6.cabal:71,97) and bind the kernels with
`foreign import ccall unsafe` (MS6/programs/Kernel/Gridder.hs:67-71), so
several Haskell capabilities can be inside kern_scatter_gpu1 /
kern_degrid_gpu1 at the same time.  Here 6 host threads (ctypes releases the
GIL for the call) each grid and degrid their own buffers several times over,
started together at a barrier, with different supports and grid sizes; every
result must equal the oracle's (FP64, relative L2 1e-12), exactly as a lone
call does."""
import threading

import numpy as np
import pytest

from oracle import oracle as O
from rc_gb300 import compat
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
THREADS = 6
ROUNDS = 4


def _case(k):
    rng = np.random.default_rng(900 + k)
    S = (8, 16, 32, 64)[k % 4]
    G = (256, 384, 512)[k % 3]
    n = 3000 + 1500 * k
    lim = 0.46 * G
    vis5 = np.zeros((n, 5))
    vis5[:, 0] = rng.uniform(-lim, lim, n)
    vis5[:, 1] = rng.uniform(-lim, lim, n)
    vis5[:, 2] = rng.uniform(-5, 5, n)
    vis5[:, 3:] = rng.standard_normal((n, 2))
    gcf = rng.standard_normal((64, S, S)) + 1j * rng.standard_normal((64, S, S))
    grid0 = rng.standard_normal((G, G)) + 1j * rng.standard_normal((G, G))
    model = rng.standard_normal((G, G)) + 1j * rng.standard_normal((G, G))
    exp_g = grid0.copy()
    O.scatter(1.0, G, 64, vis5, gcf, exp_g)
    exp_d = O.degrid(1.0, G, 64, gcf, model, vis5)
    return dict(vis5=vis5, gcf=gcf, grid0=grid0, model=model, G=G, exp_g=exp_g, exp_d=exp_d)


def test_threads_call_the_abi_at_once():
    cases = [_case(k) for k in range(THREADS)]
    start = threading.Barrier(THREADS)
    errors = [[] for _ in range(THREADS)]

    def worker(k):
        c = cases[k]
        try:
            start.wait()
            for r in range(ROUNDS):
                grid = c["grid0"].copy()
                rc = compat.call_scatter("kern_scatter_gpu1", 1.0, c["G"], 64, c["vis5"],
                                         c["gcf"], grid)
                out = np.zeros_like(c["vis5"])
                rc2 = compat.call_degrid("kern_degrid_gpu1", 1.0, c["G"], 64, c["gcf"],
                                         c["model"], c["vis5"], out)
                errors[k].append((rc, rc2, rel_l2(grid - c["grid0"], c["exp_g"] - c["grid0"]),
                                  rel_l2(out[:, 3:], c["exp_d"][:, 3:]),
                                  bool(np.array_equal(out[:, :3], c["vis5"][:, :3]))))
        except Exception as e:  # surfaced below, on the test's thread
            errors[k].append(e)

    ts = [threading.Thread(target=worker, args=(k,)) for k in range(THREADS)]
    for t in ts:
        t.start()
    for t in ts:
        t.join(timeout=600)
    assert not any(t.is_alive() for t in ts)
    for k in range(THREADS):
        assert len(errors[k]) == ROUNDS, errors[k]
        for res in errors[k]:
            assert not isinstance(res, Exception), res
            rc, rc2, eg, ed, uvw_same = res
            assert rc == 0 and rc2 == 0
            assert eg < TOL64 and ed < TOL64 and uvw_same
