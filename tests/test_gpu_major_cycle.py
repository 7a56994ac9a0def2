"""The imaging major cycle on the GPU (grid -> FFT -> CLEAN -> FFT -> degrid ->
subtract).  With the no-w-term array (the 64-antenna layout, 7x7 PSWF kernel),
visibilities of point sources predicted by the same forward model, and the grid
correction taken from the kernel itself, the residual falls every cycle and
CLEAN puts the flux on the true sources."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_major_cycle_converges_on_point_sources():
    import torch

    from rc_gb300 import gcf as G
    from rc_gb300 import synth
    from rc_gb300.engine import Plan
    from rc_gb300.major_cycle import MajorCycle

    ob = synth.config("c1", n_t=64)
    n = ob.grid_size
    gcf = G.pswf_uv_gcf(8, 7)
    g32 = torch.tensor(gcf.ravel(), dtype=torch.complex64, device="cuda")
    uvw = torch.tensor(ob.uvw, device="cuda")
    plan = Plan(uvw, scale=ob.scale, grid_size=n, grid_shape=(n, n), supports=[8])
    t = torch.tensor(G.grid_correction(gcf, n, offsets="centred"), dtype=torch.float32,
                     device="cuda")
    mc = MajorCycle(plan, g32, t)
    rng = np.random.default_rng(5)
    truth = torch.zeros((n, n), device="cuda")
    pos = []
    for _ in range(8):
        y, x = rng.integers(n // 3, 2 * n // 3, 2)
        truth[y, x] = float(rng.uniform(1.0, 10.0))
        pos.append((int(y), int(x)))
    vis = mc.forward(truth)
    model, resid, stats = mc.run(vis, n_major=3, n_minor=400, gain=0.1)
    r0 = float(torch.sqrt(torch.mean(vis.real ** 2 + vis.imag ** 2)))
    rms = [s["residual_rms"] for s in stats]
    assert all(b < a for a, b in zip(rms, rms[1:])), rms
    assert rms[-1] < 0.1 * r0, (rms, r0)
    m = model.cpu().numpy()
    for (y, x) in pos:
        assert m[y - 1:y + 2, x - 1:x + 2].sum() > 0.8 * float(truth[y, x])
