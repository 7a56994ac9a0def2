"""Image <-> grid transforms and the differentiable least-squares imaging
model (the 2048^2 / 2.06 M-visibility / 16-w-plane configuration): numpy
checks of the transforms, adjoint dot-product tests of the whole chain,
FP64 central finite differences on 64 random pixels against the autograd
gradient (which runs the hand-written adjoint kernels), and 50 iterations of
gradient descent."""
import numpy as np
import pytest

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def np_image_to_grid(x, t):
    xt = x / np.outer(t, t) if t is not None else x
    return np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(xt)))


def np_grid_to_image(y, t):
    n = y.shape[0]
    img = np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(y))).real * n * n
    return img / np.outer(t, t) if t is not None else img


@pytest.mark.parametrize("n,dt", [(64, "f64"), (256, "f32"), (128, "f64")])
def test_transforms_match_numpy_and_are_adjoint(n, dt):
    import torch

    from rc_gb300 import gcf as G
    from rc_gb300.autograd import ImageToGrid, grid_to_image

    rng = np.random.default_rng(n)
    x = rng.standard_normal((n, n))
    t = G.pswf_taper(n)
    y = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    rdt = torch.float32 if dt == "f32" else torch.float64
    cdt = torch.complex64 if dt == "f32" else torch.complex128
    tol = 1e-5 if dt == "f32" else 1e-12
    xt = torch.tensor(x, dtype=rdt, device="cuda")
    tt = torch.tensor(t, dtype=rdt, device="cuda")
    g = ImageToGrid.apply(xt, tt).cpu().numpy()
    assert rel_l2(g, np_image_to_grid(x, t)) < tol
    yt = torch.tensor(y, dtype=cdt, device="cuda")
    im = grid_to_image(yt, tt).cpu().numpy()
    assert rel_l2(im, np_grid_to_image(y, t)) < tol
    # <A x, y>_R == <x, A^H y>
    lhs = np.real(np.vdot(np_image_to_grid(x, t), y))
    assert abs(lhs - np.sum(x * np_grid_to_image(y, t))) < 1e-9 * abs(lhs)
    assert abs(np.real(np.vdot(g.astype(np.complex128), y)) - np.sum(x * im)) < tol * 10 * abs(lhs)


@pytest.fixture(scope="module")
def lsq_setup():
    import torch

    from rc_gb300 import gcf as G
    from rc_gb300 import synth
    from rc_gb300.autograd import forward_model
    from rc_gb300.engine import Plan

    ob = synth.config("c4")
    n = ob.grid_size
    g64, g32, offs = G.generate(ob.w_planes, ob.supports, ob.max_support, ob.scale / 2,
                                taper=G.pswf_taper(ob.max_support))
    uvw = torch.tensor(ob.uvw, device="cuda")
    plan = Plan(uvw, scale=ob.scale, grid_size=n, grid_shape=(n, n), supports=ob.supports,
                w_range=(ob.w_low, ob.w_high))
    t_img = torch.tensor(G.pswf_taper(n), device="cuda")
    rng = np.random.default_rng(44)
    x_true = torch.tensor(synth.sky_image(n, rng), device="cuda")
    with torch.no_grad():
        v_obs = forward_model(x_true, t_img.float(), plan, g32)
        v_obs = v_obs + 0.01 * torch.randn_like(v_obs)
    return dict(ob=ob, n=n, plan=plan, g32=g32, g64=g64, t=t_img, x_true=x_true, v=v_obs,
                keep=(uvw,))


def test_lsq_chain_adjoint_dot_product(lsq_setup):
    import torch

    from rc_gb300.autograd import Degrid, ImageToGrid, grid_to_image

    S = lsq_setup
    rng = np.random.default_rng(1)
    for rdt, cdt, gcf, tol in [(torch.float64, torch.complex128, S["g64"], 1e-10),
                               (torch.float32, torch.complex64, S["g32"], 1e-5)]:
        # random image inside the inner half of the field: at the edge the grid
        # correction multiplies by up to 1/t^2 ~ 3e7, which FP32 cannot carry
        xn = np.zeros((S["n"], S["n"]))
        q = S["n"] // 4
        xn[q:-q, q:-q] = rng.standard_normal((S["n"] - 2 * q, S["n"] - 2 * q))
        x = torch.tensor(xn, dtype=rdt, device="cuda")
        y = torch.tensor(rng.standard_normal(S["ob"].n) + 1j * rng.standard_normal(S["ob"].n),
                         dtype=cdt, device="cuda")
        Ax = Degrid.apply(ImageToGrid.apply(x, S["t"].to(rdt)), S["plan"], gcf)
        Gy = torch.zeros((S["n"], S["n"]), dtype=cdt, device="cuda")
        (S["plan"].grid if cdt == torch.complex64 else S["plan"].grid64)(y, gcf, Gy)
        AHy = grid_to_image(Gy, S["t"].to(rdt))
        lhs = float(torch.real(torch.vdot(Ax.to(torch.complex128), y.to(torch.complex128))))
        rhs = float(torch.sum(x.double() * AHy.double()))
        assert abs(lhs - rhs) <= tol * abs(lhs), (rdt, lhs, rhs)


def test_lsq_gradient_matches_fp64_finite_differences(lsq_setup):
    import torch

    from rc_gb300.autograd import forward_model

    S = lsq_setup
    t64 = S["t"].double()
    v64 = S["v"].to(torch.complex128)
    x0 = (0.5 * S["x_true"].double()).clone()

    def loss(x):
        r = forward_model(x, t64, S["plan"], S["g64"]) - v64
        return torch.sum(r.real ** 2 + r.imag ** 2)

    x = x0.clone().requires_grad_(True)
    loss(x).backward()
    g = x.grad.detach()
    rng = np.random.default_rng(64)
    n = S["n"]
    # 64 random pixels inside the sky region plus anywhere
    pix = np.column_stack([rng.integers(0, n, 64), rng.integers(0, n, 64)])
    eps = 1e-3
    fd = []
    with torch.no_grad():
        for (i, j) in pix:
            xp = x0.clone()
            xp[i, j] += eps
            xm = x0.clone()
            xm[i, j] -= eps
            fd.append((float(loss(xp)) - float(loss(xm))) / (2 * eps))
    fd = np.array(fd)
    ga = g[pix[:, 0], pix[:, 1]].cpu().numpy()
    assert rel_l2(ga, fd) < 1e-6


def test_lsq_fifty_gradient_descent_iterations(lsq_setup):
    """Gradient descent on the sky, restricted to its support (the inner half
    of the field, where the blobs are): outside it the grid correction's
    1/t^2 would set the Lipschitz constant and stall plain gradient descent."""
    import torch

    from rc_gb300.autograd import Degrid, ImageToGrid, forward_model, grid_to_image

    S = lsq_setup
    n = S["n"]
    t32 = S["t"].float()
    mask = torch.zeros((n, n), device="cuda")
    mask[n // 4:-n // 4, n // 4:-n // 4] = 1.0
    # step 1/L, L = 2 * largest eigenvalue of (A M)^H (A M) (power iteration, FP32 pair)
    z = torch.randn((n, n), device="cuda") * mask
    for _ in range(15):
        Az = Degrid.apply(ImageToGrid.apply(z * mask, t32), S["plan"], S["g32"])
        Gz = torch.zeros((n, n), dtype=torch.complex64, device="cuda")
        S["plan"].grid(Az, S["g32"], Gz)
        z2 = grid_to_image(Gz, t32) * mask
        lam = float(torch.linalg.vector_norm(z2) / torch.linalg.vector_norm(z))
        z = z2 / torch.linalg.vector_norm(z2)
    step = 1.0 / (2.0 * lam * 1.05)
    x = torch.zeros((n, n), device="cuda", requires_grad=True)
    losses = []
    for it in range(50):
        r = forward_model(x * mask, t32, S["plan"], S["g32"]) - S["v"]
        L = torch.sum(r.real ** 2 + r.imag ** 2)
        losses.append(float(L.detach()))
        x.grad = None
        L.backward()
        with torch.no_grad():
            x -= step * x.grad
    losses = np.array(losses)
    assert np.all(np.diff(losses) <= 1e-5 * losses[0])  # monotone (to FP32 rounding)
    assert losses[-1] < 0.5 * losses[0]
    # the estimate moves towards the true sky
    with torch.no_grad():
        e0 = float(torch.linalg.vector_norm(S["x_true"] * mask))
        e1 = float(torch.linalg.vector_norm((x - S["x_true"]) * mask))
    assert e1 < e0


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_lsq_grid_gradient_is_the_reference_gridder_on_the_residual(lsq_setup, prec):
    """The gradient of L = ||D g - v||^2 with respect to the grid, as autograd
    computes it (Degrid.backward: the hand-written gridding kernel on the
    residual, 2 G r), against the reference's CPU gridder used as the adjoint:
    the oracle's kern_scatter semantics (MS6/kernel/cpu/gridding/scatter.cpp:
    89-111, grid += vis * gcf over every w-plane) applied to the same residual
    r = D g - v, FP64.  FP64 within 1e-12, FP32 within 1e-5."""
    import os

    import torch

    from oracle import oracle as O
    from rc_gb300 import gcf as Gm
    from rc_gb300.autograd import Degrid, ImageToGrid

    S = lsq_setup
    ob, n = S["ob"], S["n"]
    rdt, cdt, gcf, tol = ((torch.float64, torch.complex128, S["g64"], 1e-12) if prec == "f64"
                          else (torch.float32, torch.complex64, S["g32"], 1e-5))
    with torch.no_grad():
        g0 = ImageToGrid.apply((0.5 * S["x_true"]).to(rdt), S["t"].to(rdt))
    g = g0.detach().clone().requires_grad_(True)
    r = Degrid.apply(g, S["plan"], gcf) - S["v"].to(cdt)
    L = torch.sum(r.real ** 2 + r.imag ** 2)
    L.backward()
    got = g.grad.detach().cpu().numpy().astype(np.complex128)

    r_np = r.detach().cpu().numpy().astype(np.complex128)
    offs, _ = Gm.layout(ob.supports)
    plane = O.wbin(ob.uvw, ob.w_low, ob.w_high, len(ob.supports))
    exp = np.zeros((n, n), np.complex128)
    O.scatter_planes(ob.scale, n, int(ob.supports.max()), ob.uvw, r_np, plane, ob.supports,
                     S["g64"].cpu().numpy(), offs, exp, nthreads=os.cpu_count() or 1)
    exp *= 2.0
    assert np.abs(exp).max() > 0
    assert rel_l2(got, exp) < tol
