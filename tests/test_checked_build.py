"""The bounds-checked build (libgbnufft_checked.so, compiled with
GBN_CHECKED): every global index the kernels form from plan data is tested
against its buffer's extent, and a failure is recorded in the plan's status
word instead of being performed.  Small oracle cases run through it -- 1-D,
2-D and 3-D, both precisions, real and complex phasing, a multi-frame plan
with the fused coil-sensitivity passes, coordinates on tile and period
edges, split spread tiles -- must match the oracle at the parity tolerance
and leave the status word at zero."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def checked():
    from mrrt.nufft_gb300 import _build, _lib

    _build.build(checked=True)
    return _lib.load_checked()


def _status(P):
    s = ctypes.c_uint(0xFFFFFFFF)
    rc = P.lib.gbn_debug_check_status(P.handle, ctypes.byref(s))
    assert rc == 0
    return s.value


def _edge_tm(K, M, seed):
    rng = np.random.default_rng(seed)
    tm = np.stack([rng.uniform(-1.5 * k, 2.5 * k, M) for k in K], -1)
    tm[:8] = np.round(tm[:8]) + 3.0
    tm[8:16] = np.round(tm[8:16])
    tm[16:24] = np.asarray(K) - 1e-3
    tm[24:1400] = 0.25           # a dense point: split spread tiles
    return tm


@pytest.mark.parametrize("K,J,coils,precision,phasing", [
    ((40,), (7,), 3, "single", "real"),
    ((64, 48), (6, 6), 32, "single", "real"),
    ((40, 34), (6, 5), 5, "double", "real"),
    ((36, 32), (6, 6), 4, "single", "complex"),
    ((24, 20, 16), (6, 6, 6), 3, "single", "real"),
])
def test_checked_interpolation_matches_oracle_with_no_violation(checked, K, J, coils, precision, phasing):
    from mrrt.nufft_gb300._kernels import kernel_table
    from mrrt.nufft_gb300._plan import GpuPlan

    rdt = np.float32 if precision == "single" else np.float64
    cdt = np.complex64 if precision == "single" else np.complex128
    ndim = len(K)
    N = tuple(k // 2 for k in K)
    M = 2500
    tm = _edge_tm(K, M, seed=sum(K) + coils).astype(rdt)
    L = 512
    tdt = cdt if phasing == "complex" else rdt
    h = [kernel_table(N[d], J[d], K[d], L, phasing, tdt) for d in range(ndim)]
    P = GpuPlan(N, K, J, L, rdt, [np.real(t) for t in h],
                [np.imag(t) for t in h] if phasing == "complex" else None,
                np.ones(int(np.prod(N)), rdt), tm, None, max_coils=coils, phasing=phasing, lib=checked)
    assert P.stats()["split_tiles"] > 0
    Kp = int(np.prod(K))
    rng = np.random.default_rng(2)
    grid = (rng.standard_normal((coils, Kp)) + 1j * rng.standard_normal((coils, Kp))).astype(cdt)
    y = torch.empty((coils, M), dtype=P.ctype, device="cuda")
    P.interp_forward(torch.from_numpy(grid).cuda(), y, coils)
    tol = 1e-5 if precision == "single" else 1e-12
    assert rel_l2(y.cpu().numpy().T, O.interp_forward(grid.T, h, J, L, tm, K)) < tol
    fm = (rng.standard_normal((coils, M)) + 1j * rng.standard_normal((coils, M))).astype(cdt)
    g = torch.empty((coils, Kp), dtype=P.ctype, device="cuda")
    P.interp_adjoint(torch.from_numpy(fm).cuda(), g, coils)
    assert rel_l2(g.cpu().numpy().T, O.interp_adjoint(fm.T, h, J, L, tm, K)) < tol
    # the full transforms (pad, FFT, crop around the interpolation)
    x = torch.randn((coils,) + tuple(reversed(N)), dtype=torch.complex128).to("cuda", P.ctype)
    y2 = torch.empty((coils, M), dtype=P.ctype, device="cuda")
    P.forward(x, y2, coils)
    xa = torch.empty_like(x)
    P.adjoint(y2, xa, coils)
    torch.cuda.synchronize()
    assert _status(P) == 0


def test_checked_series_sense_no_violation(checked):
    """A 3-frame plan with uneven sample counts through the fused
    coil-sensitivity pad and crop, and the plain transforms."""
    from mrrt.nufft_gb300._kernels import kernel_table
    from mrrt.nufft_gb300._plan import GpuPlan
    from mrrt.nufft_gb300.trajectories import uneven_series_2d

    N, K, J, coils = (48, 40), (96, 80), (6, 6), 6
    oms = uneven_series_2d(3, 96, 9, 23, seed=4)
    fo = np.concatenate([[0], np.cumsum([o.shape[0] for o in oms])])
    tm = np.concatenate(oms) / (2 * np.pi / np.asarray(K, dtype=np.float64))
    h = [kernel_table(N[d], J[d], K[d], 1024, "real", np.float32) for d in range(2)]
    P = GpuPlan(N, K, J, 1024, np.float32, h, None, np.ones(int(np.prod(N)), np.float32),
                tm.astype(np.float32), None, frame_offsets=fo, max_coils=coils, lib=checked)
    img = torch.randn((3,) + tuple(reversed(N)), dtype=torch.complex64, device="cuda")
    maps = torch.randn((coils,) + tuple(reversed(N)), dtype=torch.complex64, device="cuda")
    y = torch.empty((coils * P.M_total,), dtype=torch.complex64, device="cuda")
    P.forward_sense(img, maps, y, coils)
    xs = torch.empty_like(img)
    P.adjoint_sense(y, maps, xs, coils)
    x = torch.randn((3, coils) + tuple(reversed(N)), dtype=torch.complex64, device="cuda")
    P.forward(x, y, coils)
    xa = torch.empty_like(x)
    P.adjoint(y, xa, coils)
    torch.cuda.synchronize()
    assert _status(P) == 0
    ref = torch.empty_like(y)
    P.forward((img[:, None] * maps[None]).contiguous(), ref, coils)
    P.forward_sense(img, maps, y, coils)
    torch.cuda.synchronize()
    assert rel_l2(y.cpu().numpy(), ref.cpu().numpy()) < 1e-6
