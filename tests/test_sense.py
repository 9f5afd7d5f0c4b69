"""Coil-sensitivity (SENSE) transforms with the coil-map multiply fused into
the deapodisation pass and the conjugate-map coil sum fused into the crop
pass, against the plain transforms with the maps applied separately."""
import numpy as np
import pytest
import torch

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _cplx(shape, seed, dtype):
    g = torch.Generator(device="cpu").manual_seed(seed)
    return torch.randn(shape, dtype=torch.complex128, generator=g).to(device="cuda", dtype=dtype)


@pytest.mark.parametrize("frames,precision", [(1, "single"), (3, "single"), (2, "double")])
def test_fused_sense_matches_separate_maps(gpu_lib, frames, precision):
    from mrrt.nufft_gb300.series import NufftSeries
    from mrrt.nufft_gb300.trajectories import uneven_series_2d

    Nd, Kd, coils = (48, 40), (96, 80), 6
    oms = uneven_series_2d(frames, 96, min_spokes=9, max_spokes=21, seed=7)
    S = NufftSeries(Nd, oms, Jd=(6, 6), Kd=Kd, coils=coils, precision=precision)
    ct = S.ctype
    img = _cplx((frames,) + tuple(reversed(Nd)), 1, ct)
    maps = _cplx((coils,) + tuple(reversed(Nd)), 2, ct)
    tol = 1e-6 if precision == "single" else 1e-12

    y = S.forward_sense(img, maps)
    coil_images = (img[:, None] * maps[None]).contiguous()          # [F, C, N1, N0]
    y_ref = S.forward(coil_images)
    assert rel_l2(y.cpu().numpy(), y_ref.cpu().numpy()) < tol

    w = _cplx((coils * S.M_total,), 3, ct)
    xa = S.adjoint_sense(w, maps)
    xa_ref = (S.adjoint(w) * maps[None].conj()).sum(dim=1)
    assert xa.shape == (frames,) + tuple(reversed(Nd))
    assert rel_l2(xa.cpu().numpy(), xa_ref.cpu().numpy()) < tol

    # the fused pair is adjoint: <A_s x, w> = <x, A_s^H w>
    lhs = torch.vdot(y.reshape(-1).to(torch.complex128), w.to(torch.complex128))
    rhs = torch.vdot(img.reshape(-1).to(torch.complex128), xa.reshape(-1).to(torch.complex128))
    assert abs(lhs - rhs) / abs(lhs) < (1e-5 if precision == "single" else 1e-12)


def test_sense_rejects_missing_maps(gpu_lib):
    import ctypes

    from mrrt.nufft_gb300 import _lib
    from mrrt.nufft_gb300.series import NufftSeries
    from mrrt.nufft_gb300.trajectories import uneven_series_2d

    S = NufftSeries((16, 16), uneven_series_2d(1, 32, 3, 5, seed=1), Jd=(6, 6), Kd=(32, 32), coils=2)
    img = torch.zeros((1, 16, 16), dtype=torch.complex64, device="cuda")
    y = S.empty_samples(2)
    rc = S.plan.lib.gbn_forward_sense(S.plan.handle, ctypes.c_void_p(img.data_ptr()), None,
                                      ctypes.c_void_p(y.data_ptr()), 2, None)
    assert rc == _lib.GBN_ERR_INVALID


@pytest.mark.parametrize("frames,coils", [(2, 5), (2, 9)])
def test_fused_sense_3d_matches_separate_maps(gpu_lib, frames, coils):
    """3-D series: 10 planes run the per-plane pruned FFT, 18 planes the full
    3-D FFT; the fused transforms equal the plain ones with the maps applied
    separately."""
    from mrrt.nufft_gb300.series import NufftSeries

    Nd, Kd = (12, 14, 10), (24, 28, 20)
    rng = np.random.default_rng(8)
    oms = [rng.uniform(-np.pi, np.pi, (600 + 100 * f, 3)) for f in range(frames)]
    S = NufftSeries(Nd, oms, Jd=(6, 6, 6), Kd=Kd, coils=coils)
    img = _cplx((frames,) + tuple(reversed(Nd)), 4, torch.complex64)
    maps = _cplx((coils,) + tuple(reversed(Nd)), 5, torch.complex64)
    y = S.forward_sense(img, maps)
    y_ref = S.forward((img[:, None] * maps[None]).contiguous())
    assert rel_l2(y.cpu().numpy(), y_ref.cpu().numpy()) < 1e-6
    w = _cplx((coils * S.M_total,), 6, torch.complex64)
    xa = S.adjoint_sense(w, maps)
    xa_ref = (S.adjoint(w) * maps[None].conj()).sum(dim=1)
    assert rel_l2(xa.cpu().numpy(), xa_ref.cpu().numpy()) < 1e-6
