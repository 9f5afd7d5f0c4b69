"""Autograd of the NUFFT: gradients with respect to the image and to the
trajectory omega, checked against central finite differences (step 1e-3 rad)
and against torch's FP64 autograd of a direct NUDFT.

Workload: the differentiable-NUFFT case -- 2-D 256^2 image, 512^2 grid,
J 6, variable-density spiral of 16 interleaves x 4096 samples, loss
||A(x; omega) - y||^2 with y = A(x_true; omega) + 1% Gaussian noise; the FP64
comparison runs on a 64^2 / 2048-sample subproblem of the same spiral.
"""
import numpy as np
import pytest
import torch

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _spiral(n_inter=16, n_samp=4096):
    from mrrt.nufft_gb300.trajectories import spiral_2d

    return spiral_2d(n_inter, n_samp)


def _nudft(x, omega, Nd):
    """FP64 direct NUDFT y[c, m] = sum_n x[c, n] exp(-i omega_m . n), n = 0..N-1
    (the reference operator with n_shift = 0), differentiable by torch."""
    grids = torch.meshgrid(*[torch.arange(n, dtype=torch.float64, device=x.device) for n in Nd],
                           indexing="ij")
    n = torch.stack([g.reshape(-1) for g in grids], -1)
    E = torch.exp(-1j * (omega @ n.T))
    return x.reshape(x.shape[0], -1) @ E.T


def _cplx(shape, seed, device="cuda", dtype=torch.complex64):
    g = torch.Generator(device="cpu").manual_seed(seed)
    return torch.randn(shape, dtype=torch.complex128, generator=g).to(device=device, dtype=dtype)


def _sub_problem():
    om = _spiral()
    rows = np.random.default_rng(5).choice(om.shape[0], 2048, replace=False)
    return om[np.sort(rows)]


def test_forward_adjoint_match_fp64_nudft_and_each_other(gpu_lib):
    from mrrt.nufft_gb300 import NufftOperator

    Nd, Kd = (64, 64), (128, 128)
    om = _sub_problem()
    op = NufftOperator(Nd, om, Jd=(6, 6), Kd=Kd, max_coils=2)
    x = _cplx((2,) + Nd, 1)
    y = op.forward(x)
    omt = torch.from_numpy(om).cuda()
    y_ex = _nudft(x.to(torch.complex128), omt, Nd)
    assert rel_l2(y.cpu().numpy(), y_ex.cpu().numpy()) < 1e-4
    w = _cplx((2, om.shape[0]), 2)
    xa = op.adjoint(w)
    lhs = torch.vdot(y.reshape(-1).to(torch.complex128), w.reshape(-1).to(torch.complex128))
    rhs = torch.vdot(x.reshape(-1).to(torch.complex128), xa.reshape(-1).to(torch.complex128))
    assert abs(lhs - rhs) / abs(lhs) < 1e-5


def test_gradients_match_fp64_autograd_nudft(gpu_lib):
    """Image and trajectory gradients of ||A(x; omega) - y||^2 vs torch autograd
    of the FP64 direct NUDFT on the 64^2 / 2048-sample subproblem."""
    from mrrt.nufft_gb300 import NufftOperator

    Nd, Kd = (64, 64), (128, 128)
    om = _sub_problem()
    x_true = _cplx((1,) + Nd, 3, dtype=torch.complex128)
    omt64 = torch.from_numpy(om).cuda()
    y_clean = _nudft(x_true, omt64, Nd)
    noise = _cplx(tuple(y_clean.shape), 4, dtype=torch.complex128)
    y_t = y_clean + 0.01 * noise * (y_clean.abs().pow(2).mean().sqrt() / noise.abs().pow(2).mean().sqrt())
    x0 = _cplx((1,) + Nd, 5, dtype=torch.complex128)

    # FP64 autograd of the direct NUDFT
    xe = x0.clone().requires_grad_(True)
    oe = omt64.clone().requires_grad_(True)
    ((_nudft(xe, oe, Nd) - y_t).abs() ** 2).sum().backward()

    # the GPU operator in single precision
    op = NufftOperator(Nd, om, Jd=(6, 6), Kd=Kd)
    xg = x0.to(torch.complex64).clone().requires_grad_(True)
    og = omt64.to(torch.float32).clone().requires_grad_(True)
    r = op.forward(xg, og).to(torch.complex128) - y_t
    (r.abs() ** 2).sum().backward()

    assert rel_l2(xg.grad.cpu().numpy(), xe.grad.cpu().numpy()) < 2e-4
    assert rel_l2(og.grad.cpu().numpy(), oe.grad.cpu().numpy()) < 2e-3


def test_omega_gradient_central_differences_full_spiral(gpu_lib):
    """256^2 / 512^2 / 16 x 4096 spiral: the trajectory gradient against central
    differences with step 1e-3 rad, along a random direction of all samples
    and on single coordinates."""
    from mrrt.nufft_gb300 import NufftOperator

    Nd, Kd = (256, 256), (512, 512)
    om = _spiral()
    M = om.shape[0]
    op = NufftOperator(Nd, om, Jd=(6, 6), Kd=Kd)
    omt = torch.from_numpy(om.astype(np.float32)).cuda()
    x_true = _cplx((1,) + Nd, 6)
    with torch.no_grad():
        y_clean = op.forward(x_true, omt)
    noise = _cplx(tuple(y_clean.shape), 7)
    y_t = (y_clean + 0.01 * noise * (y_clean.abs().pow(2).mean().sqrt() /
                                     noise.abs().pow(2).mean().sqrt())).to(torch.complex128)
    x = _cplx((1,) + Nd, 8)

    def loss(o):
        with torch.no_grad():
            return float(((op.forward(x, o).to(torch.complex128) - y_t).abs() ** 2).sum())

    og = omt.clone().requires_grad_(True)
    ((op.forward(x, og).to(torch.complex128) - y_t).abs() ** 2).sum().backward()
    g = og.grad.double()
    eps = 1e-3

    # Every coordinate moves by exactly +-1e-3 rad (random sign per coordinate).
    # The operator's phase runs over n = 0..N-1, so a sample's value turns at
    # up to 255 rad per rad of omega and the O(eps^2) truncation of a 1e-3 rad
    # central difference is about (255 eps)^2 / 6 ~ 1%.  Richardson
    # extrapolation with the half step removes that term and is held to 2e-3.
    v32 = torch.from_numpy(np.random.default_rng(9).choice([-1.0, 1.0], (M, 2))).cuda().to(torch.float32)

    def central(step, direction):
        return (loss(omt + step * direction) - loss(omt - step * direction)) / (2 * step)

    fd1 = central(eps, v32)
    fd2 = central(eps / 2, v32)
    rich = (4 * fd2 - fd1) / 3
    an = float((g * v32.double()).sum())
    assert abs(fd1 - an) / abs(an) < 3e-2, (fd1, an)
    assert abs(rich - an) / abs(an) < 2e-3, (rich, fd1, an)

    rng = np.random.default_rng(10)
    for m, d in zip(rng.choice(M, 6, replace=False), rng.integers(0, 2, 6)):
        e = torch.zeros_like(omt)
        e[m, d] = 1.0
        fd = central(eps, e)
        an = float(g[m, d])
        assert abs(fd - an) <= 3e-2 * abs(an) + 1e-5 * float(g.abs().max()), (m, d, fd, an)


def test_adjoint_function_gradients(gpu_lib):
    """x = A(omega)^H y: gradients with respect to y and omega against
    central differences (64^2, 2048 samples, 2 coils)."""
    from mrrt.nufft_gb300 import NufftOperator

    Nd, Kd = (64, 64), (128, 128)
    om = _sub_problem()
    op = NufftOperator(Nd, om, Jd=(6, 6), Kd=Kd, max_coils=2)
    omt = torch.from_numpy(om.astype(np.float32)).cuda()
    y = _cplx((2, om.shape[0]), 11)
    b = _cplx((2,) + Nd, 12, dtype=torch.complex128)

    def loss(yv, o):
        with torch.no_grad():
            return float(((op.adjoint(yv, o).to(torch.complex128) - b).abs() ** 2).sum())

    yg = y.clone().requires_grad_(True)
    og = omt.clone().requires_grad_(True)
    ((op.adjoint(yg, og).to(torch.complex128) - b).abs() ** 2).sum().backward()

    # y: the loss is quadratic in y, so the central difference is exact up to rounding
    dv = _cplx(tuple(y.shape), 13)
    h = 1e-2
    fd = (loss(y + h * dv, omt) - loss(y - h * dv, omt)) / (2 * h)
    an = float((yg.grad.conj() * dv).real.double().sum())
    assert abs(fd - an) / abs(an) < 1e-3, (fd, an)

    v = torch.from_numpy(np.random.default_rng(14).choice([-1.0, 1.0], tuple(omt.shape))).cuda().to(torch.float32)
    eps = 1e-3
    fd = (loss(y, omt + eps * v) - loss(y, omt - eps * v)) / (2 * eps)
    an = float((og.grad.double() * v.double()).sum())
    assert abs(fd - an) / abs(an) < 1e-2, (fd, an)
