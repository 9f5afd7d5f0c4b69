"""Dynamic series: all frames (uneven sample counts) and coils in one plan,
one launch per stage, CUDA-graph replay and the tile autotuner.

The series of the benchmark set -- 64 frames of a 2-D 192^2 image, 384^2 grid,
J 6, frame f with U{13..89} golden-angle spokes (seed 4) x 384 points, 8 coils
-- is checked frame by frame against single-frame operators and against the
FP64 NUDFT; smaller series cover graph replay and the autotuner.
"""
import numpy as np
import pytest
import torch

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _frames(n_frames, n_read, lo, hi, seed=4):
    from mrrt.nufft_gb300.trajectories import uneven_series_2d

    return uneven_series_2d(n_frames, n_read, min_spokes=lo, max_spokes=hi, seed=seed)


def _images(shape, seed):
    g = torch.Generator(device="cpu").manual_seed(seed)
    return torch.randn(shape, dtype=torch.complex64, generator=g).cuda()


def _per_frame_check(S, oms, Nd, Kd, coils, x, frames):
    from mrrt.nufft_gb300 import NufftBase

    y = S.forward(x)
    ys = S.split_samples(y)
    xa = S.adjoint(y)
    for f in frames:
        A = NufftBase(Nd, oms[f], Jd=(6, 6), Kd=Kd, on_gpu=True, max_coils=coils)
        yf = torch.empty((coils, oms[f].shape[0]), dtype=torch.complex64, device="cuda")
        A.plan.forward(x[f].contiguous(), yf, coils)
        # identical gather; the batched FFT over frames x coils may round
        # differently from the per-frame FFT, so float32 tolerance
        assert rel_l2(ys[f].cpu().numpy(), yf.cpu().numpy()) < 1e-5, f
        xf = torch.empty_like(x[f])
        A.plan.adjoint(ys[f].contiguous(), xf, coils)
        assert rel_l2(xa[f].cpu().numpy(), xf.cpu().numpy()) < 1e-5, f
    return y, xa


def test_small_series_matches_single_frame_operators(gpu_lib):
    from mrrt.nufft_gb300.series import NufftSeries

    Nd, Kd, coils = (48, 48), (96, 96), 3
    oms = _frames(6, 96, 5, 29, seed=1)
    S = NufftSeries(Nd, oms, Jd=(6, 6), Kd=Kd, coils=coils)
    assert S.n_frames == 6 and len(set(S.samples_per_frame.tolist())) > 1
    x = _images(S.image_shape, 0)
    _per_frame_check(S, oms, Nd, Kd, coils, x, range(6))


def test_series_workload_frames_and_fp64(gpu_lib):
    """The 64-frame series: frames 0, 31 and 63 against single-frame
    operators, frame 17 against the FP64 NUDFT, and the adjoint identity
    <A x, y> = <x, A^H y> over the whole series."""
    from mrrt.nufft_gb300 import dtft
    from mrrt.nufft_gb300.series import NufftSeries

    Nd, Kd, coils = (192, 192), (384, 384), 8
    oms = _frames(64, 384, 13, 89, seed=4)
    S = NufftSeries(Nd, oms, Jd=(6, 6), Kd=Kd, coils=coils)
    counts = S.samples_per_frame
    assert counts.min() >= 13 * 384 and counts.max() <= 89 * 384
    x = _images(S.image_shape, 1)
    y, xa = _per_frame_check(S, oms, Nd, Kd, coils, x, (0, 31, 63))

    f = 17
    rows = np.random.default_rng(2).choice(int(counts[f]), 1024, replace=False)
    x17 = x[f, 0].cpu().numpy().T.astype(np.complex128)    # [N0, N1] reference axis order
    y_ex = dtft(x17, oms[f][rows], shape=Nd)
    y17 = S.split_samples(y)[f][0].cpu().numpy()[rows]
    assert rel_l2(y17, y_ex) < 1e-4

    w = _images((coils * S.M_total,), 3)
    lhs = torch.vdot(y.to(torch.complex128), w.to(torch.complex128))
    xw = S.adjoint(w)
    rhs = torch.vdot(x.reshape(-1).to(torch.complex128), xw.reshape(-1).to(torch.complex128))
    assert abs(lhs - rhs) / abs(lhs) < 1e-5


def test_graph_replay_matches_eager(gpu_lib):
    from mrrt.nufft_gb300.series import NufftSeries

    Nd, Kd, coils = (64, 64), (128, 128), 4
    oms = _frames(8, 128, 7, 31, seed=5)
    S = NufftSeries(Nd, oms, Jd=(6, 6), Kd=Kd, coils=coils).capture()
    for seed in (10, 11):
        x = _images(S.image_shape, seed)
        S.x_static.copy_(x)
        y_graph = S.replay_forward().clone()
        xa_graph = S.replay_adjoint().clone()
        torch.cuda.synchronize()
        y_eager = S.forward(x)
        xa_eager = S.adjoint(y_eager)
        assert torch.equal(y_graph, y_eager)
        assert torch.equal(xa_graph, xa_eager)


def test_autotuner_picks_measured_candidates(gpu_lib, tmp_path):
    from mrrt.nufft_gb300 import autotune
    from mrrt.nufft_gb300.series import NufftSeries

    Nd, Kd, coils = (64, 64), (128, 128), 4
    oms = _frames(8, 128, 7, 31, seed=6)
    cache = str(tmp_path / "tune.json")
    tile, stile, report = autotune.tune_series(Nd, oms, Jd=(6, 6), Kd=Kd, coils=coils, reps=2,
                                               cache_path=cache)
    gathers, spreads = autotune.candidate_tiles(2)
    assert tile in [tuple(t) for t in gathers] and stile in [tuple(t) for t in spreads]
    assert len(report["gather"]) == len(gathers) and all(ms > 0 for _, ms in report["gather"])
    # the cache answers the second call without timing
    again = autotune.tune_series(Nd, oms, Jd=(6, 6), Kd=Kd, coils=coils, reps=2, cache_path=cache)
    assert again[:2] == (tile, stile)
    # the tuned plan computes the same transform
    S0 = NufftSeries(Nd, oms, Jd=(6, 6), Kd=Kd, coils=coils)
    S1 = NufftSeries(Nd, oms, Jd=(6, 6), Kd=Kd, coils=coils, tile=tile, stile=stile)
    x = _images(S0.image_shape, 12)
    y0, y1 = S0.forward(x), S1.forward(x)
    assert rel_l2(y1.cpu().numpy(), y0.cpu().numpy()) < 1e-6
    assert rel_l2(S1.adjoint(y0).cpu().numpy(), S0.adjoint(y0).cpu().numpy()) < 1e-5
