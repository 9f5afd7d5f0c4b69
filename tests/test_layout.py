"""The pruned FFTs.  2-D plans keep their transform grids row-interleaved,
[K1][planes][K0], so the row pass runs over the N1 rows that hold data only
and the column pass reads the other rows of its input as zero.  3-D plans
prune plane by plane: a 2-D FFT of the first N2 z-planes, then the z-pass.
These tests change the coil count between calls (in 2-D a call with more
coil planes writes rows that a call with fewer reads as padding) and replay a
CUDA graph captured with few coils after an eager call with more; every
result must equal single-coil calls on a fresh operator.  Non-square images
and grids catch swapped axes.  Grids of several sizes, in both precisions,
are checked against the oracle."""
import numpy as np
import pytest
import torch

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

COILS = 6
GEOMS = {
    "2d": ((40, 48), (80, 96)),
    "3d": ((20, 16, 12), (40, 32, 24)),
}


def _operator(geom, max_coils):
    from mrrt.nufft_gb300 import NufftBase

    Nd, Kd = GEOMS[geom]
    rng = np.random.default_rng(len(Nd))
    omega = rng.uniform(-np.pi, np.pi, (2000, len(Nd)))
    return NufftBase(Nd, omega, Jd=(6,) * len(Nd), Kd=Kd, on_gpu=True, max_coils=max_coils)


def _image_shape(geom, coils):
    return (coils,) + tuple(reversed(GEOMS[geom][0]))


def _images(geom, coils, seed):
    g = torch.Generator(device="cpu").manual_seed(seed)
    return torch.randn(_image_shape(geom, coils), dtype=torch.complex64, generator=g).cuda()


def _samples(coils, M, seed):
    g = torch.Generator(device="cpu").manual_seed(seed)
    return torch.randn((coils, M), dtype=torch.complex64, generator=g).cuda()


def _per_coil(geom, x, y):
    """Forward and adjoint of each coil alone on a fresh single-coil operator."""
    A1 = _operator(geom, 1)
    fw = [A1.plan.forward(x[c:c + 1].contiguous(),
                          torch.empty((1, A1.M), dtype=torch.complex64, device="cuda"), 1)
          for c in range(x.shape[0])]
    ad = [A1.plan.adjoint(y[c:c + 1].contiguous(), torch.empty_like(x[c:c + 1]), 1)
          for c in range(y.shape[0])]
    return torch.cat(fw), torch.cat(ad)


def _fw(A, x):
    c = x.shape[0]
    return A.plan.forward(x.contiguous(), torch.empty((c, A.M), dtype=torch.complex64,
                                                      device="cuda"), c)


def _ad(A, geom, y):
    c = y.shape[0]
    return A.plan.adjoint(y.contiguous(), torch.empty(_image_shape(geom, c), dtype=torch.complex64,
                                                      device="cuda"), c)


@pytest.mark.parametrize("geom", sorted(GEOMS))
def test_coil_count_changes_between_calls(gpu_lib, geom):
    A = _operator(geom, COILS)
    x, y = _images(geom, COILS, 1), _samples(COILS, A.M, 2)
    y_ref, x_ref = _per_coil(geom, x, y)
    for c in (COILS, 2, 5, 1, COILS, 3):
        assert rel_l2(_fw(A, x[:c]).cpu().numpy(), y_ref[:c].cpu().numpy()) < 1e-5, c
        assert rel_l2(_ad(A, geom, y[:c]).cpu().numpy(), x_ref[:c].cpu().numpy()) < 1e-5, c


@pytest.mark.parametrize("geom", sorted(GEOMS))
def test_graph_with_few_coils_replays_after_a_wider_call(gpu_lib, geom):
    A = _operator(geom, COILS)
    x, y = _images(geom, COILS, 3), _samples(COILS, A.M, 4)
    y_ref, x_ref = _per_coil(geom, x, y)
    c = 2
    xs, ys = x[:c].contiguous(), y[:c].contiguous()
    yo = torch.empty((c, A.M), dtype=torch.complex64, device="cuda")
    xo = torch.empty_like(xs)
    _fw(A, x)                                  # buffers sized for every coil
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):                 # plans and buffers for c coils
        A.plan.forward(xs, yo, c)
        A.plan.adjoint(ys, xo, c)
    torch.cuda.current_stream().wait_stream(s)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        A.plan.forward(xs, yo, c)
        A.plan.adjoint(ys, xo, c)
    for _ in range(2):
        _fw(A, x)                              # 2-D: writes rows the graph reads as padding
        _ad(A, geom, y)
        yo.zero_()
        xo.zero_()
        g.replay()
        torch.cuda.synchronize()
        assert rel_l2(yo.cpu().numpy(), y_ref[:c].cpu().numpy()) < 1e-5
        assert rel_l2(xo.cpu().numpy(), x_ref[:c].cpu().numpy()) < 1e-5
    np.testing.assert_array_equal(_fw(A, xs).cpu().numpy(), yo.cpu().numpy())


@pytest.mark.parametrize("Nd,Kd,precision", [
    ((24, 20), (48, 40), "single"),
    ((20, 24), (40, 48), "single"),
    ((12, 16), (24, 32), "double"),
    ((96, 10), (192, 20), "double"),
    ((512, 6), (1024, 12), "single"),
    ((1024, 6), (2048, 12), "single"),
    ((16, 20, 12), (32, 40, 24), "single"),
    ((12, 10, 14), (24, 20, 28), "double"),
])
def test_row_lengths_match_oracle(gpu_lib, Nd, Kd, precision):
    """The pruned FFTs (2-D rows, 3-D z-planes) for short and long rows, 3-D
    grids and both precisions, against the oracle."""
    from oracle import oracle as O
    from mrrt.nufft_gb300 import NufftBase

    rng = np.random.default_rng(7)
    omega = rng.uniform(-np.pi, np.pi, (700, len(Nd)))
    kw = dict(Nd=Nd, omega=omega, Jd=(6,) * len(Nd), Kd=Kd, precision=precision)
    A = NufftBase(**kw)
    B = O.OracleNufft(**kw)
    cdt = np.complex64 if precision == "single" else np.complex128
    x = (rng.standard_normal(Nd + (3,)) + 1j * rng.standard_normal(Nd + (3,))).astype(cdt)
    # the parity bars: 1e-5 in single; 1e-6 in double, where the reference
    # builds its tables in single precision and this library in double
    tol = 1e-5 if precision == "single" else 1e-6
    y = B.fft(x)
    assert rel_l2(A.fft(x), y) < tol
    assert rel_l2(A.adj(y), B.adj(y)) < tol


@pytest.mark.parametrize("reps", [16, 17])
def test_3d_pruning_limit_matches_oracle(gpu_lib, reps):
    """3-D batches of up to 16 planes take the per-plane pruned FFT, larger
    ones the full 3-D FFT; both against the oracle."""
    from oracle import oracle as O
    from mrrt.nufft_gb300 import NufftBase

    Nd, Kd = (10, 12, 8), (20, 24, 16)
    rng = np.random.default_rng(9)
    omega = rng.uniform(-np.pi, np.pi, (500, 3))
    kw = dict(Nd=Nd, omega=omega, Jd=(6, 6, 6), Kd=Kd)
    A = NufftBase(max_coils=reps, **kw)
    B = O.OracleNufft(**kw)
    x = (rng.standard_normal(Nd + (reps,)) + 1j * rng.standard_normal(Nd + (reps,))).astype(np.complex64)
    y = B.fft(x)
    assert rel_l2(A.fft(x), y) < 1e-5
    assert rel_l2(A.adj(y), B.adj(y)) < 1e-5
