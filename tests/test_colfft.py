"""The plan's own FFT passes (gbn_colfft.cu, gbn_rowfft.cu) against cuFFT.

Single-precision 2-D and 3-D plans run the FFT's pass along the slowest axis
on the library's kernel when that axis has a supported length, and 2-D plans
with a supported K0 also the row passes with the pad and crop folded in; a
plan made with cufft_only (GBN_FLAG_CUFFT_ONLY) runs every pass through cuFFT
around the separate pad and crop kernels.  Both
compute the same transform in float32 by different factorisations, so the
forward and adjoint NUFFTs agree to float32 rounding (relative L2 2e-6; the
measured differences are near 2e-7).  The cases cover every supported length,
column counts that are not a multiple of a CTA's 16 columns, image sizes
other than half the grid (the pruned rows), several coils and frames, the
3-D per-plane pass, and lengths and precisions that fall back to cuFFT.
"""
import numpy as np
import pytest
import torch

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 2e-6


def _pair(N, K, J, coils=2, frames=1, M=1500, seed=0, rdt=np.float32, **kw):
    from mrrt.nufft_gb300._kernels import kernel_table
    from mrrt.nufft_gb300._plan import GpuPlan

    ndim = len(K)
    rng = np.random.default_rng(seed)
    tm = np.stack([rng.uniform(-0.5 * k, 1.5 * k, M * frames) for k in K], -1).astype(rdt)
    h = [kernel_table(N[d], J[d], K[d], 256, "real", rdt) for d in range(ndim)]
    sn = rng.uniform(0.5, 1.5, int(np.prod(N))).astype(rdt)
    foff = np.arange(frames + 1, dtype=np.int64) * M
    return [GpuPlan(N, K, J, 256, rdt, h, None, sn, tm, None, frame_offsets=foff, max_coils=coils,
                    cufft_only=flag, **kw) for flag in (False, True)]


def _run(plans, coils, frames, seed=1):
    P = plans[0]
    ctype = P.ctype
    rng = np.random.default_rng(seed)
    nx = frames * coils * P.Nprod
    x = torch.from_numpy((rng.standard_normal(nx) + 1j * rng.standard_normal(nx)).astype(np.complex64)).to(
        ctype).cuda()
    ny = coils * P.M_total
    y0 = torch.from_numpy((rng.standard_normal(ny) + 1j * rng.standard_normal(ny)).astype(np.complex64)).to(
        ctype).cuda()
    ys = [Q.forward(x, torch.empty(ny, dtype=ctype, device="cuda"), coils) for Q in plans]
    xs = [Q.adjoint(y0, torch.empty(nx, dtype=ctype, device="cuda"), coils) for Q in plans]
    torch.cuda.synchronize()
    return [t.cpu().numpy() for t in ys], [t.cpu().numpy() for t in xs]


@pytest.mark.parametrize("L", [64, 96, 128, 192, 256, 384, 512, 768])
def test_2d_every_supported_length(gpu_lib, L):
    # K0 = 20 with 3 coils: 60 columns, not a multiple of 16
    N, K, J, coils = (10, L // 2), (20, L), (6, 6), 3
    plans = _pair(N, K, J, coils=coils, seed=L)
    ys, xs = _run(plans, coils, 1)
    assert rel_l2(ys[0], ys[1]) < TOL
    assert rel_l2(xs[0], xs[1]) < TOL


@pytest.mark.parametrize("N1", [3, 37, 63, 64])
def test_2d_pruned_rows_other_than_half(gpu_lib, N1):
    N, K, J = (24, N1), (48, 128), (4, 4)
    plans = _pair(N, K, J, coils=2, frames=3, seed=N1)
    ys, xs = _run(plans, 2, 3)
    assert rel_l2(ys[0], ys[1]) < TOL
    assert rel_l2(xs[0], xs[1]) < TOL


@pytest.mark.parametrize("K", [(12, 10, 64), (16, 16, 96), (8, 6, 128)])
def test_3d_per_plane_pass(gpu_lib, K):
    N = tuple(k // 2 for k in K)
    plans = _pair(N, K, (4, 4, 4), coils=2, seed=sum(K))
    ys, xs = _run(plans, 2, 1)
    assert rel_l2(ys[0], ys[1]) < TOL
    assert rel_l2(xs[0], xs[1]) < TOL


@pytest.mark.parametrize("K,rdt", [((32, 80), np.float32), ((16, 1024), np.float32), ((32, 64), np.float64)])
def test_fallback_to_cufft_is_exact(gpu_lib, K, rdt):
    """An unsupported length (80, 1024) or double precision runs cuFFT in both plans."""
    N = tuple(k // 2 for k in K)
    plans = _pair(N, K, (6, 6), coils=2, rdt=rdt)
    ys, xs = _run(plans, 2, 1)
    assert np.array_equal(ys[0], ys[1])
    assert np.array_equal(xs[0], xs[1])


def test_headline_geometry_against_cufft(gpu_lib):
    """The 256^2 / 512^2 grid with 32 coils (one plane per coil)."""
    N, K, J, coils = (256, 256), (512, 512), (6, 6), 32
    plans = _pair(N, K, J, coils=coils, M=4000)
    ys, xs = _run(plans, coils, 1)
    assert rel_l2(ys[0], ys[1]) < TOL
    assert rel_l2(xs[0], xs[1]) < TOL


@pytest.mark.parametrize("K0", [64, 96, 128, 192, 256, 384, 512, 768])
def test_2d_fused_row_passes(gpu_lib, K0):
    """A supported K0 runs the row passes with the pad and the crop folded in
    (gbn_rowfft.cu): image rows of N0 = K0/2 - 1 values, 30 of 64 rows, two
    frames of three coils."""
    N, K, J = (K0 // 2 - 1, 30), (K0, 64), (6, 6)
    plans = _pair(N, K, J, coils=3, frames=2, seed=K0)
    ys, xs = _run(plans, 3, 2)
    assert rel_l2(ys[0], ys[1]) < TOL
    assert rel_l2(xs[0], xs[1]) < TOL


def test_2d_fused_row_passes_orthonormal_scaling(gpu_lib):
    """The crop's scale (orthonormal FFT, adjoint_scale) is applied by the
    fused pass."""
    N, K, J = (64, 64), (128, 128), (6, 6)
    plans = _pair(N, K, J, coils=2, ortho=True, adjoint_scale=1.7)
    ys, xs = _run(plans, 2, 1)
    assert rel_l2(ys[0], ys[1]) < TOL
    assert rel_l2(xs[0], xs[1]) < TOL


@pytest.mark.parametrize("N,K,coils,frames", [
    ((32, 32, 32), (64, 64, 64), 2, 1),
    ((40, 30, 50), (96, 64, 128), 2, 1),
    ((20, 24, 16), (64, 96, 64), 3, 6),     # 18 planes: past the per-plane cuFFT path's limit
])
def test_3d_all_passes_on_own_kernels(gpu_lib, N, K, coils, frames):
    """Every axis supported: rows with the pad / crop folded in, then axes 1
    and 2 in place on the grid."""
    plans = _pair(N, K, (4, 4, 4), coils=coils, frames=frames, M=800, seed=sum(N))
    ys, xs = _run(plans, coils, frames)
    assert rel_l2(ys[0], ys[1]) < TOL
    assert rel_l2(xs[0], xs[1]) < TOL
