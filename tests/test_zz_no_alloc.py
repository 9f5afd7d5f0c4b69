"""gbn_interp_adjoint_noalloc: the adjoint spread with its split-tile partial
sums in a fixed static device array instead of a per-plan buffer.

Called through the C ABI and compared with gbn_interp_adjoint on the same
plan and inputs.  The file name sorts last so that the tests also run after
every other GPU test in one session; each test passes on its own as well.
"""
import ctypes

import numpy as np
import pytest
import torch

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

NOALLOC_CAP = 64 * 1024 * 1024   # GBN_NOALLOC_SCRATCH_BYTES
TOL = 1e-6                       # same kernels, same part order: results agree to rounding


def _plan(tm, N, K, J, L=512, max_coils=1, rdt=np.float32):
    from mrrt.nufft_gb300._kernels import kernel_table
    from mrrt.nufft_gb300._plan import GpuPlan

    h = [kernel_table(N[d], J[d], K[d], L, "real", rdt) for d in range(len(N))]
    return GpuPlan(N, K, J, L, rdt, h, None, np.ones(int(np.prod(N)), rdt),
                   np.ascontiguousarray(tm, dtype=rdt), None, max_coils=max_coils)


def _call(P, name, y, grid, coils):
    fn = getattr(P.lib, name)
    return fn(P.handle, ctypes.c_void_p(y.data_ptr()), ctypes.c_void_p(grid.data_ptr()), int(coils),
              ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


def _noalloc(P, y, coils):
    from mrrt.nufft_gb300 import _lib

    grid = torch.empty((coils, P.Kprod), dtype=y.dtype, device="cuda")
    _lib.check(_call(P, "gbn_interp_adjoint_noalloc", y, grid, coils))
    return grid


def _regular(P, y, coils):
    from mrrt.nufft_gb300 import _lib

    grid = torch.empty((coils, P.Kprod), dtype=y.dtype, device="cuda")
    _lib.check(_call(P, "gbn_interp_adjoint", y, grid, coils))
    return grid


def _samples(coils, M, seed, dtype=torch.complex64):
    g = torch.Generator(device="cuda").manual_seed(seed)
    return torch.randn((coils, M), dtype=dtype, device="cuda", generator=g)


@pytest.mark.parametrize("case", ["2d-double", "3d-single"])
def test_noalloc_double_and_3d_match_interp_adjoint(gpu_lib, case):
    """The double-precision instantiation (2-D radial, 4 coils) and a 3-D
    geometry whose centre tiles are split (radial spokes through one point,
    3 coils): two consecutive no-alloc calls each match gbn_interp_adjoint."""
    from mrrt.nufft_gb300.trajectories import kooshball_3d, radial_2d

    if case == "2d-double":
        N, K, J, coils, rdt, ct = (64, 64), (128, 128), (6, 6), 4, np.float64, torch.complex128
        tm = radial_2d(160, 128, golden=True) / (2 * np.pi / 128.0)
    else:
        N, K, J, coils, rdt, ct = (24, 24, 24), (48, 48, 48), (6, 6, 6), 3, np.float32, torch.complex64
        tm = kooshball_3d(2000, 48) / (2 * np.pi / 48.0)
    P = _plan(tm, N, K, J, max_coils=coils, rdt=rdt)
    assert P.stats()["split_tiles"] > 0, "the case must exercise the split-tile scratch"
    tol = 1e-12 if rdt == np.float64 else TOL
    for seed in (5, 6):
        y = _samples(coils, P.M_total, seed, ct)
        g = _noalloc(P, y, coils)
        r = _regular(P, y, coils)
        torch.cuda.synchronize()
        assert rel_l2(g.cpu().numpy(), r.cpu().numpy()) < tol


def test_noalloc_matches_interp_adjoint_two_calls(gpu_lib):
    """Golden-angle radial 256^2 / 512^2 grid, 8 coils: two consecutive
    no-alloc calls on different samples each match gbn_interp_adjoint, and
    the plan's device memory does not grow."""
    from mrrt.nufft_gb300.trajectories import radial_2d

    N, K, J, coils = (256, 256), (512, 512), (6, 6), 8
    omega = radial_2d(402, 512, golden=True)
    tm = omega / (2 * np.pi / np.asarray(K, dtype=np.float64))
    P = _plan(tm, N, K, J, max_coils=coils)
    st = P.stats()
    assert st["split_tiles"] > 0, "the case must exercise the split-tile scratch"
    bytes_before = st["device_bytes"]

    y1, y2 = _samples(coils, P.M_total, 1), _samples(coils, P.M_total, 2)
    g1 = _noalloc(P, y1, coils)
    g2 = _noalloc(P, y2, coils)
    torch.cuda.synchronize()
    assert P.stats()["device_bytes"] == bytes_before

    r1 = _regular(P, y1, coils)
    r2 = _regular(P, y2, coils)
    torch.cuda.synchronize()
    assert rel_l2(g1.cpu().numpy(), r1.cpu().numpy()) < TOL
    assert rel_l2(g2.cpu().numpy(), r2.cpu().numpy()) < TOL


def test_noalloc_leaves_device_memory_unchanged(gpu_lib):
    """After the first call on the device (which may load the module that
    holds the fixed array), further calls change no device-memory figure."""
    from mrrt.nufft_gb300.trajectories import radial_2d

    N, K, J, coils = (64, 64), (128, 128), (6, 6), 4
    tm = radial_2d(96, 128, golden=True) / (2 * np.pi / 128.0)
    P = _plan(tm, N, K, J, max_coils=coils)
    y = _samples(coils, P.M_total, 3)
    first = _noalloc(P, y, coils)
    out = torch.empty_like(first)
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    from mrrt.nufft_gb300 import _lib

    for _ in range(2):
        _lib.check(_call(P, "gbn_interp_adjoint_noalloc", y, out, coils))
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
    assert rel_l2(out.cpu().numpy(), first.cpu().numpy()) < TOL


def test_noalloc_rejects_requests_beyond_its_capacity(gpu_lib):
    """2^18 samples on one k-space point: the four 16 x 8 spread tiles its
    window touches are each split into 342 parts.  128 coils would need far
    more than the fixed 64 MiB and are refused before any launch (the output
    keeps its sentinel); 16 coils fit and match gbn_interp_adjoint."""
    from mrrt.nufft_gb300 import _lib

    N, K, J, M = (32, 32), (64, 64), (6, 6), 1 << 18
    tm = np.zeros((M, 2), np.float32)
    P = _plan(tm, N, K, J, max_coils=16)
    assert P.stats()["split_tiles"] >= 4

    big = 128
    y = _samples(big, M, 4)
    grid = torch.full((big, P.Kprod), 7.0 + 0j, dtype=torch.complex64, device="cuda")
    rc = _call(P, "gbn_interp_adjoint_noalloc", y, grid, big)
    assert rc == _lib.GBN_ERR_TOOLARGE
    msg = P.lib.gbn_last_error().decode()
    assert "no-alloc" in msg and str(NOALLOC_CAP) in msg
    torch.cuda.synchronize()
    assert bool((grid == (7.0 + 0j)).all())

    small = 16
    ys = y[:small].contiguous()
    a = _noalloc(P, ys, small)
    b = _noalloc(P, ys, small)
    r = _regular(P, ys, small)
    torch.cuda.synchronize()
    assert rel_l2(a.cpu().numpy(), r.cpu().numpy()) < TOL
    assert rel_l2(b.cpu().numpy(), r.cpu().numpy()) < TOL
