"""Hogbom CLEAN on the GPU: the engine form against the numpy float32 oracle
(bit-exact residual, model and iteration count), its threshold stop and CUDA
graph capture; the reference-ABI form against the FP64 restatement of the
reference's Halide CLEAN."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _scene(seed, n=192, pn=128):
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:pn, 0:pn]
    c = pn // 2
    psf = (np.exp(-((yy - c) ** 2 + (xx - c) ** 2) / (2 * 3.0 ** 2)) +
           0.1 * np.cos(0.3 * (xx - c)) * np.exp(-((yy - c) ** 2 + (xx - c) ** 2) / 800.0))
    psf = (psf / psf[c, c]).astype(np.float32)
    img = np.zeros((n, n))
    for _ in range(12):
        y, x = rng.integers(0, n, 2)
        a = rng.uniform(0.5, 5.0) * rng.choice([-1, 1])
        y0, y1 = max(0, y - c), min(n, y - c + pn)
        x0, x1 = max(0, x - c), min(n, x - c + pn)
        img[y0:y1, x0:x1] += a * psf[y0 - (y - c):y1 - (y - c), x0 - (x - c):x1 - (x - c)]
    img += 0.01 * rng.standard_normal((n, n))
    return img.astype(np.float32), psf, c, c


def _run_engine(res, psf, ppx, ppy, gain, threshold, n_iter, graph=False):
    import torch

    from rc_gb300 import lib

    L = lib.load()
    ny, nx = res.shape
    d_res = torch.tensor(res, device="cuda")
    d_psf = torch.tensor(psf, device="cuda")
    d_model = torch.zeros_like(d_res)
    wb = C.c_int64()
    lib.check(L.gb_hogbom_work_bytes(nx, ny, C.byref(wb)), "work")
    work = torch.empty(wb.value, dtype=torch.uint8, device="cuda")

    def call():
        lib.check(L.gb_hogbom_f32(d_res.data_ptr(), nx, ny, d_psf.data_ptr(), psf.shape[1],
                                  psf.shape[0], ppx, ppy, gain, threshold, n_iter,
                                  d_model.data_ptr(), work.data_ptr(), wb.value,
                                  torch.cuda.current_stream().cuda_stream), "gb_hogbom_f32")

    if graph:
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                call()
        d_res.copy_(torch.tensor(res, device="cuda"))  # capture did not run the kernels
        g.replay()
    else:
        call()
    torch.cuda.synchronize()
    it = C.c_int32()
    lib.check(L.gb_hogbom_iterations(work.data_ptr(), C.byref(it),
                                     torch.cuda.current_stream().cuda_stream), "iterations")
    return d_res.cpu().numpy(), d_model.cpu().numpy(), it.value


@pytest.mark.parametrize("n_iter,threshold", [(300, 0.0), (3000, 0.2)])
def test_engine_clean_is_bit_exact(n_iter, threshold):
    res, psf, ppx, ppy = _scene(1)
    r, m, it = _run_engine(res, psf, ppx, ppy, 0.1, threshold, n_iter)
    er, em, eit = O.hogbom_f32(res, psf, ppx, ppy, 0.1, threshold, n_iter)
    assert it == eit
    assert np.array_equal(r, er)
    assert np.array_equal(m, em)
    if threshold > 0:
        assert it < n_iter and np.abs(r).max() < 0.2


def test_engine_clean_in_a_cuda_graph_and_off_centre_psf():
    res, psf, _, _ = _scene(2, n=160, pn=96)
    psf = np.ascontiguousarray(psf[:, 5:])  # peak no longer in the middle
    ppy, ppx = np.unravel_index(int(np.argmax(psf)), psf.shape)
    r, m, it = _run_engine(res, psf, int(ppx), int(ppy), 0.2, 0.0, 150, graph=True)
    er, em, eit = O.hogbom_f32(res, psf, int(ppx), int(ppy), 0.2, 0.0, 150)
    assert it == eit == 150
    assert np.array_equal(r, er) and np.array_equal(m, em)


def test_reference_abi_clean_matches_restatement():
    from rc_gb300 import compat
    from rc_gb300 import lib

    L = lib.load()
    res, psf, _, _ = _scene(3, n=96, pn=64)
    res64 = res.astype(np.float64)
    psf64 = psf.astype(np.float64)

    def img_buf(a):
        return compat.buf(a, [(a.shape[1], 1), (a.shape[0], a.shape[1])])

    for threshold in (0.0, 2.0):
        model = np.full_like(res64, 0.5)
        em, er = O.hogbom_reference(0.1, threshold, psf64, res64, model)
        rc = L.kern_hogbom_model(0.1, threshold, C.byref(img_buf(psf64)), C.byref(img_buf(res64)),
                                 C.byref(img_buf(model)))
        assert rc == 0
        assert rel_l2(model, em) < 1e-12
        out = np.zeros_like(res64)
        rc = L.kern_hogbom_residual(0.1, threshold, C.byref(img_buf(psf64)),
                                    C.byref(img_buf(res64)), C.byref(img_buf(out)))
        assert rc == 0
        assert rel_l2(out, er) < 1e-12
