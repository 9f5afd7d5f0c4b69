"""Host-buffer entry points (gbn_forward_host / gbn_adjoint_host): host
memory in, host memory out, batches of 32 coils or more as a copy / transform
pipeline of 16-coil chunks.  Each result is checked against the device entry
points on the same data, for pageable and pinned inputs, coil counts that
leave a short last chunk, an input the copy kernel cannot take (not 16-byte
aligned, so the copy engines move it), double precision and a multi-frame
plan (one piece).  Device pointers are rejected."""
import ctypes

import numpy as np
import pytest
import torch

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _operator(max_coils, precision="single", Nd=(64, 48), Kd=(128, 96)):
    from mrrt.nufft_gb300 import NufftBase
    from mrrt.nufft_gb300.trajectories import radial_2d

    return NufftBase(Nd, radial_2d(40, 128, golden=True), Jd=(6, 6), Kd=Kd, on_gpu=True,
                     max_coils=max_coils, precision=precision)


def _rand(shape, ctype, seed):
    g = torch.Generator(device="cpu").manual_seed(seed)
    return torch.randn(shape, dtype=torch.complex128, generator=g).to(ctype)


def _device_pair(P, x, y, coils):
    """Forward of x and adjoint of y through the device entry points."""
    yd = P.forward(x.cuda(), torch.empty((coils, P.M_total), dtype=P.ctype, device="cuda"), coils)
    xd = P.adjoint(y.cuda(), torch.empty(x.shape, dtype=P.ctype, device="cuda"), coils)
    return yd.cpu(), xd.cpu()


@pytest.mark.parametrize("coils", [1, 3, 32, 33, 50])
@pytest.mark.parametrize("pinned", [False, True])
def test_host_entry_points_match_device_path(gpu_lib, coils, pinned):
    A = _operator(coils)
    P = A.plan
    x = _rand((coils, 48, 64), P.ctype, 1)
    y = _rand((coils, P.M_total), P.ctype, 2)
    if pinned:
        x, y = x.pin_memory(), y.pin_memory()
    yd, xd = _device_pair(P, x, y, coils)
    yh = torch.empty((coils, P.M_total), dtype=P.ctype)
    xh = torch.empty(x.shape, dtype=P.ctype)
    P.forward_host(x, yh, coils)
    P.adjoint_host(y, xh, coils)
    # the same kernels; the pipelined batches run their FFTs 16 planes at a time
    assert rel_l2(yh.numpy(), yd.numpy()) < 1e-6
    assert rel_l2(xh.numpy(), xd.numpy()) < 1e-6
    # repeated calls reuse the staging and give the same bits
    yh2 = torch.empty_like(yh)
    P.forward_host(x, yh2, coils)
    assert torch.equal(yh, yh2)


def test_unaligned_pageable_input_takes_the_copy_engines(gpu_lib):
    coils = 32
    A = _operator(coils)
    P = A.plan
    n = coils * P.M_total
    raw = torch.empty(n + 1, dtype=torch.complex64)          # 8 bytes past a 16-byte boundary
    y = raw[1:]
    assert y.data_ptr() % 16 == 8
    y.copy_(_rand((n,), torch.complex64, 3))
    x = _rand((coils, 48, 64), torch.complex64, 4)
    _, xd = _device_pair(P, x, y.view(coils, P.M_total).clone(), coils)
    xh = torch.empty(x.shape, dtype=torch.complex64)
    P.adjoint_host(y, xh, coils)
    assert rel_l2(xh.numpy(), xd.numpy()) < 1e-6


def test_host_entry_points_double_precision(gpu_lib):
    coils = 32
    A = _operator(coils, precision="double")
    P = A.plan
    x = _rand((coils, 48, 64), torch.complex128, 5)
    y = _rand((coils, P.M_total), torch.complex128, 6)
    yd, xd = _device_pair(P, x, y, coils)
    yh, xh = torch.empty_like(yd), torch.empty_like(xd)
    P.forward_host(x, yh, coils)
    P.adjoint_host(y, xh, coils)
    assert rel_l2(yh.numpy(), yd.numpy()) < 1e-12
    assert rel_l2(xh.numpy(), xd.numpy()) < 1e-12


def test_host_entry_points_multi_frame_plan(gpu_lib):
    from mrrt.nufft_gb300.series import NufftSeries
    from mrrt.nufft_gb300.trajectories import uneven_series_2d

    coils = 4
    oms = uneven_series_2d(5, 64, min_spokes=3, max_spokes=9, seed=2)
    S = NufftSeries((32, 32), oms, Jd=(6, 6), Kd=(64, 64), coils=coils)
    P = S.plan
    x = _rand(S.image_shape, torch.complex64, 7)
    y = _rand((coils * S.M_total,), torch.complex64, 8)
    yd = S.forward(x.cuda()).cpu()
    xd = S.adjoint(y.cuda()).cpu()
    yh, xh = torch.empty_like(yd), torch.empty_like(xd)
    P.forward_host(x.contiguous(), yh, coils)
    P.adjoint_host(y, xh, coils)
    assert torch.equal(yh, yd)
    assert torch.equal(xh, xd)


def test_host_entry_points_reject_device_memory(gpu_lib):
    from mrrt.nufft_gb300 import _lib

    coils = 2
    A = _operator(coils)
    P = A.plan
    x = torch.zeros((coils, 48, 64), dtype=torch.complex64, device="cuda")
    y = torch.zeros((coils, P.M_total), dtype=torch.complex64)
    rc = gpu_lib.gbn_forward_host(P.handle, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                                  coils, None)
    assert rc == _lib.GBN_ERR_INVALID
    assert b"host" in gpu_lib.gbn_last_error()
    with pytest.raises(ValueError):
        P.forward_host(x, y, coils)


def test_drop_in_host_arrays_use_the_host_entry_points(gpu_lib, monkeypatch):
    """NufftBase.fft / .adj on numpy arrays go through the host-buffer entry
    points and give the device path's result."""
    from mrrt.nufft_gb300 import NufftBase
    from mrrt.nufft_gb300.trajectories import complex_image, radial_2d

    Nd, Kd, reps = (64, 48), (128, 96), 34
    kw = dict(Nd=Nd, omega=radial_2d(40, 128, golden=True), Jd=(6, 6), Kd=Kd, max_coils=reps)
    Ah = NufftBase(on_gpu=False, **kw)
    calls = []
    for name in ("forward_host", "adjoint_host"):
        orig = getattr(Ah.plan, name)
        monkeypatch.setattr(Ah.plan, name, lambda *a, _o=orig, _n=name: (calls.append(_n), _o(*a))[1])
    x = np.asfortranarray(np.stack([complex_image(Nd, seed=s) for s in range(reps)], axis=-1))
    y = Ah.fft(x)
    xa = Ah.adj(y)
    assert calls == ["forward_host", "adjoint_host"]
    Ad = NufftBase(on_gpu=True, **kw)
    assert rel_l2(y, Ad.fft(x).cpu().numpy()) < 1e-6
    assert rel_l2(xa, Ad.adj(y).cpu().numpy()) < 1e-6
