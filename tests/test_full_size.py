"""Full-size checks: linearity and the adjoint identity <A x, y> = <x, A^H y>
at the 2-D 32-coil workload (256^2 / 512^2, 402 x 512 golden-angle radial) and
the 3-D kooshball (128^3 / 256^3, 12000 x 256 spokes); the 2-D workload's
geometry against the oracle on a few coils; series edge cases (a frame with
no samples, a frame with one)."""
import numpy as np
import pytest
import torch

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _cplx(shape, seed, dtype=torch.complex64):
    g = torch.Generator(device="cpu").manual_seed(seed)
    return torch.randn(shape, dtype=torch.complex128, generator=g).to(device="cuda", dtype=dtype)


def _check_linear_and_adjoint(P, Nd, coils):
    xshape = (coils,) + tuple(reversed(Nd))
    x1, x2 = _cplx(xshape, 1), _cplx(xshape, 2)
    a, b = 0.75 - 0.5j, -1.25 + 0.25j
    y = lambda x: P.forward(x.contiguous(), torch.empty((coils, P.M_total), dtype=torch.complex64,
                                                        device="cuda"), coils)
    y1, y2 = y(x1), y(x2)
    y12 = y(a * x1 + b * x2)
    assert rel_l2(y12.cpu().numpy(), (a * y1 + b * y2).cpu().numpy()) < 1e-5
    w = _cplx((coils, P.M_total), 3)
    xa = P.adjoint(w, torch.empty(xshape, dtype=torch.complex64, device="cuda"), coils)
    lhs = torch.vdot(y1.reshape(-1).to(torch.complex128), w.reshape(-1).to(torch.complex128))
    rhs = torch.vdot(x1.reshape(-1).to(torch.complex128), xa.reshape(-1).to(torch.complex128))
    assert abs(lhs - rhs) / abs(lhs) < 1e-5


def test_2d_multicoil_workload_linear_and_adjoint(gpu_lib):
    from mrrt.nufft_gb300 import NufftBase
    from mrrt.nufft_gb300.trajectories import radial_2d

    Nd, coils = (256, 256), 32
    A = NufftBase(Nd, radial_2d(402, 512, golden=True), Jd=(6, 6), Kd=(512, 512), on_gpu=True,
                  max_coils=coils)
    _check_linear_and_adjoint(A.plan, Nd, coils)


def test_2d_multicoil_workload_matches_oracle(gpu_lib):
    """The 2-D workload's full geometry (every row and tile the 32-coil batch
    touches) against the oracle, on 4 coils of the batched path."""
    from oracle import oracle as O
    from mrrt.nufft_gb300 import NufftBase
    from mrrt.nufft_gb300.trajectories import radial_2d

    Nd, coils = (256, 256), 4
    kw = dict(Nd=Nd, omega=radial_2d(402, 512, golden=True), Jd=(6, 6), Kd=(512, 512))
    A = NufftBase(on_gpu=False, max_coils=32, **kw)
    B = O.OracleNufft(**kw)
    rng = np.random.default_rng(11)
    x = (rng.standard_normal(Nd + (coils,)) + 1j * rng.standard_normal(Nd + (coils,))).astype(np.complex64)
    y = B.fft(x)
    assert rel_l2(A.fft(x), y) < 1e-5
    assert rel_l2(A.adj(y), B.adj(y)) < 1e-5


def test_3d_kooshball_workload_linear_and_adjoint(gpu_lib):
    from mrrt.nufft_gb300 import NufftBase
    from mrrt.nufft_gb300.trajectories import kooshball_3d

    Nd, coils = (128, 128, 128), 2
    A = NufftBase(Nd, kooshball_3d(12000, 256), Jd=(6, 6, 6), Kd=(256, 256, 256), on_gpu=True,
                  max_coils=coils)
    assert A.M == 3_072_000
    _check_linear_and_adjoint(A.plan, Nd, coils)


def test_series_with_empty_and_single_sample_frames(gpu_lib):
    """A frame without samples and a frame with one sample: the empty frame
    contributes nothing and its image is zero after the adjoint; the others
    match single-frame operators."""
    from mrrt.nufft_gb300 import NufftBase
    from mrrt.nufft_gb300.series import NufftSeries
    from mrrt.nufft_gb300.trajectories import radial_2d

    Nd, Kd, coils = (32, 32), (64, 64), 3
    oms = [radial_2d(5, 32, golden=True), np.zeros((0, 2)), np.array([[0.3, -1.1]]),
           radial_2d(7, 32, golden=True, first_spoke=5)]
    S = NufftSeries(Nd, oms, Jd=(6, 6), Kd=Kd, coils=coils)
    assert S.samples_per_frame.tolist() == [160, 0, 1, 224]
    x = _cplx(S.image_shape, 4)
    y = S.forward(x)
    xa = S.adjoint(y)
    assert float(xa[1].abs().max()) == 0.0
    ys = S.split_samples(y)
    for f in (0, 2, 3):
        A = NufftBase(Nd, oms[f], Jd=(6, 6), Kd=Kd, on_gpu=True, max_coils=coils)
        yf = torch.empty((coils, oms[f].shape[0]), dtype=torch.complex64, device="cuda")
        A.plan.forward(x[f].contiguous(), yf, coils)
        assert rel_l2(ys[f].cpu().numpy(), yf.cpu().numpy()) < 1e-5
        xf = torch.empty_like(x[f])
        A.plan.adjoint(ys[f].contiguous(), xf, coils)
        assert rel_l2(xa[f].cpu().numpy(), xf.cpu().numpy()) < 1e-5
