"""On-GPU w-kernel generation (FP64 screens + cuFFT) against the oracle's
numpy restatement of the reference generator (MS4/kernel/cpu/gcf/GCF.cpp)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("smax,t2,taper", [(16, 0.05, False), (32, 0.1, True), (64, 0.09, True)])
def test_gcf_generation_matches_oracle(smax, t2, taper):
    from rc_gb300 import gcf as G

    ws = np.array([-900.0, -120.0, 0.0, 35.5, 600.0])
    sup = np.array([smax, smax // 2, 8, 6, smax - 2], np.int32)
    tp = G.pswf_taper(smax) if taper else None
    g64, g32, offs = G.generate(ws, sup, smax, t2, taper=tp)
    g64 = g64.cpu().numpy()
    g32 = g32.cpu().numpy()
    for p, (w, S) in enumerate(zip(ws, sup)):
        exp = O.gcf_layers(w, int(S), smax, t2, taper=tp).reshape(-1)
        got = g64[offs[p]:offs[p] + 64 * S * S]
        assert rel_l2(got, exp) < 1e-12, (p, w, S)
        got32 = g32[offs[p]:offs[p] + 64 * S * S]
        assert rel_l2(got32, exp) < 1e-6


def test_gcf_generation_rejects_bad_arguments():
    from rc_gb300 import gcf as G
    from rc_gb300 import lib

    with pytest.raises(lib.GbError):
        G.generate([0.0], [10], 8, 0.1)  # support > max_support
    with pytest.raises(lib.GbError):
        G.generate([0.0], [8], 9, 0.1)  # odd max_support


def test_gcf_conjugate_on_device():
    import ctypes as C

    import torch

    from rc_gb300 import lib

    L = lib.load()
    rng = np.random.default_rng(2)
    g = rng.standard_normal(1000) + 1j * rng.standard_normal(1000)
    for dt, fn in [(torch.complex64, L.gb_gcf_conjugate_f32), (torch.complex128,
                                                               L.gb_gcf_conjugate_f64)]:
        d = torch.tensor(g, dtype=dt, device="cuda")
        lib.check(fn(d.data_ptr(), d.numel(), torch.cuda.current_stream().cuda_stream), "conj")
        assert np.array_equal(d.cpu().numpy(), np.conj(g.astype(d.cpu().numpy().dtype)))
