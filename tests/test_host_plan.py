"""Host-side plan math of the drop-in ``NufftBase`` on CPU (no GPU): the
device plan is replaced by a recorder, so these tests check what would be
uploaded -- deapodisation, tables, coordinates, phases and the sparse-mode
interpolation weights -- against values the reference itself computed
(tests/golden)."""
import numpy as np
import pytest

from tests.conftest import rel_l2
from tests.golden import cases


class _RecordingPlan:
    """Stands in for GpuPlan: records the upload, computes nothing."""

    def __init__(self, Nd, Kd, Jd, L, rdt, tables_re, tables_im, sn, tm, sample_phase, **kw):
        self.args = dict(Nd=Nd, Kd=Kd, Jd=Jd, L=L, rdt=rdt, tables_re=tables_re, tables_im=tables_im,
                         sn=sn, tm=tm, sample_phase=sample_phase, **kw)
        self.weights = None
        self.ctype = None
        self.device = None

    def set_weights(self, w_re, w_im=None):
        self.weights = (w_re, w_im)


@pytest.fixture
def host_nufft(monkeypatch):
    from mrrt.nufft_gb300 import _nufft

    monkeypatch.setattr(_nufft, "require_cuda", lambda: None)
    monkeypatch.setattr(_nufft, "GpuPlan", _RecordingPlan)
    return _nufft.NufftBase


def test_table_plan_matches_reference_sn_and_table(host_nufft):
    c = cases.radial_2d_128()
    g = cases.load("radial128")
    A = host_nufft(**c["kw"])
    assert A.sn.dtype == np.float32
    assert rel_l2(A.sn, g["radial128_sn"]) < 1e-6
    assert rel_l2(np.asarray(A.h[0]), g["radial128_h0"]) < 1e-6
    up = A.plan.args
    assert up["tm"].shape == (A.M, 2) and up["tm"].flags["C_CONTIGUOUS"]
    np.testing.assert_array_equal(up["tm"], A.tm)
    assert up["sample_phase"].dtype == np.complex64


@pytest.mark.parametrize("name", [n for n, _ in cases.sparse_cases() if n.startswith("sparse_2d")])
def test_sparse_weights_rebuild_reference_matrix(host_nufft, name):
    """The per-axis weights uploaded in sparse mode, multiplied out, give the
    reference's interpolation matrix ``p``: same pattern, values within
    single-precision rounding of the per-axis factors."""
    c = dict(cases.sparse_cases())[name]
    g = cases.load("sparse_cases")
    A = host_nufft(**c["kw"])
    assert A.plan.weights is not None
    w_re, w_im = A.plan.weights
    assert len(w_re) == 2 and w_re[0].shape == (A.M, A.Jd[0])
    assert (w_im is None) == (c["kw"]["phasing"] == "real")
    p = A.p.tocsc()
    p.sort_indices()
    np.testing.assert_array_equal(p.indptr, g[name + "_p_indptr"])
    np.testing.assert_array_equal(p.indices, g[name + "_p_indices"])
    tol = 1e-6 if c["kw"]["precision"] == "single" else 1e-13
    assert rel_l2(p.data, g[name + "_p_data"]) < tol


def test_sparse_mode_rejects_unknown_mode(host_nufft):
    c = cases.radial_2d_128()
    kw = dict(c["kw"])
    kw["mode"] = "lut"
    with pytest.raises(ValueError):
        host_nufft(**kw)


def test_series_plan_concatenates_frames(monkeypatch, host_nufft):
    """NufftSeries uploads one plan holding every frame: frame offsets, the
    frames' coordinates and phases in order, each equal to what a
    single-frame operator would upload."""
    from mrrt.nufft_gb300 import series
    from mrrt.nufft_gb300.trajectories import uneven_series_2d

    monkeypatch.setattr(series, "require_cuda", lambda: None)
    monkeypatch.setattr(series, "GpuPlan", _RecordingPlan)
    oms = uneven_series_2d(5, 64, min_spokes=3, max_spokes=9, seed=2)
    S = series.NufftSeries((32, 32), oms, Jd=(6, 6), Kd=(64, 64), coils=4)
    counts = [o.shape[0] for o in oms]
    np.testing.assert_array_equal(S.frame_offsets, np.concatenate([[0], np.cumsum(counts)]))
    up = S.plan.args
    assert up["frame_offsets"] is S.frame_offsets and up["max_coils"] == 4
    for f, om in enumerate(oms):
        A = host_nufft((32, 32), om, Jd=(6, 6), Kd=(64, 64))
        a, b = S.frame_offsets[f], S.frame_offsets[f + 1]
        np.testing.assert_array_equal(up["tm"][a:b], A.plan.args["tm"])
        np.testing.assert_array_equal(up["sample_phase"][a:b], A.plan.args["sample_phase"])
    np.testing.assert_array_equal(up["sn"], A.plan.args["sn"])


def test_autotune_cache_round_trip(tmp_path):
    from mrrt.nufft_gb300 import autotune

    path = str(tmp_path / "tune.json")
    rng = np.random.default_rng(0)
    om_a = [rng.uniform(-3, 3, (10, 2)), rng.uniform(-3, 3, (20, 2))]
    om_b = [om_a[0], om_a[1] + 1e-3]   # same counts, another trajectory
    da, db = autotune.trajectory_digest(om_a), autotune.trajectory_digest(om_b)
    assert da != db and da == autotune.trajectory_digest([o.copy() for o in om_a])
    key = autotune._key("series", (64, 64), (128, 128), (6, 6), [10, 20], 4, "single", da)
    assert key != autotune._key("series", (64, 64), (128, 128), (6, 6), [10, 20], 4, "single", db)
    assert autotune._load(path) == {}
    autotune._store(path, key, {"tile": [32, 16], "stile": [8, 8], "report": {}})
    autotune._store(path, key + "x", {"tile": [16, 8], "stile": [16, 8], "report": {}})
    got = autotune._load(path)
    assert got[key]["tile"] == [32, 16] and got[key + "x"]["stile"] == [16, 8]
    g2, s2 = autotune.candidate_tiles(2)
    g3, s3 = autotune.candidate_tiles(3)
    # spread tiles are whole 4 x 4 (x 1) register blocks, at most 8 per tile
    for t in s2:
        assert t[0] % 4 == 0 and t[1] % 4 == 0 and (t[0] // 4) * (t[1] // 4) <= 8
    for t in s3:
        assert t[0] % 4 == 0 and t[1] % 4 == 0 and (t[0] // 4) * (t[1] // 4) * t[2] <= 8


def test_reference_attributes_on_gpu_and_sparse_format(host_nufft):
    c = cases.radial_2d_128()
    A = host_nufft(**c["kw"])
    assert A.on_gpu is False and A.sparse_format is None
    with pytest.raises(ValueError):
        A.on_gpu = "yes"
    A.on_gpu = True
    assert A.on_gpu is True
    kw = dict(c["kw"], mode="sparse")
    assert host_nufft(**kw).sparse_format == "CSC"


class _HostIoPlan(_RecordingPlan):
    """A recording plan whose host-buffer transforms compute a fixed linear
    map in the device layouts: sample m of repetition r gets
    (r + 1) * sum(image r), and every pixel of image r gets (r + 1) * sum(samples r)."""

    def __init__(self, *a, **kw):
        super().__init__(*a, **kw)
        import torch

        self.ctype = torch.complex64
        self.calls = []

    def forward_host(self, x, y, coils):
        self.calls.append(("forward_host", tuple(x.shape), tuple(y.shape), coils, x.is_contiguous()))
        xs = x.reshape(coils, -1).sum(dim=1)
        for r in range(coils):
            y[r].fill_((r + 1) * xs[r])
        return y

    def adjoint_host(self, y, x, coils):
        self.calls.append(("adjoint_host", tuple(y.shape), tuple(x.shape), coils, y.is_contiguous()))
        ys = y.reshape(coils, -1).sum(dim=1)
        for r in range(coils):
            x[r].fill_((r + 1) * ys[r])
        return x


@pytest.mark.parametrize("order", ["F", "C"])
@pytest.mark.parametrize("reps", [1, 3])
def test_numpy_calls_route_through_host_entry_points(monkeypatch, order, reps):
    """NufftBase.fft/.adj on numpy arrays (on_gpu=False): one host-buffer call
    each, with the image handed over as [reps][N1][N0] and the result returned
    in the reference's layout for the order (reps last for 'F', first for
    'C', squeezed when there is one)."""
    import torch

    from mrrt.nufft_gb300 import _nufft

    monkeypatch.setattr(_nufft, "require_cuda", lambda: None)
    monkeypatch.setattr(_nufft, "GpuPlan", _HostIoPlan)
    monkeypatch.setattr(torch.cuda, "is_current_stream_capturing", lambda: False)
    real_empty = torch.empty
    monkeypatch.setattr(torch, "empty", lambda *a, pin_memory=False, **k: real_empty(*a, **k))

    Nd = (6, 4)
    omega = np.random.default_rng(1).uniform(-np.pi, np.pi, (10, 2))
    A = _nufft.NufftBase(Nd, omega, Jd=(4, 4), Kd=(12, 8), order=order)
    rng = np.random.default_rng(2)
    shape = (Nd + (reps,)) if order == "F" else ((reps,) + Nd)
    if reps == 1:
        shape = Nd
    x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    y = A.fft(x)
    expect_y = (10,) if reps == 1 else ((10, reps) if order == "F" else (reps, 10))
    assert isinstance(y, np.ndarray) and y.shape == expect_y and y.dtype == np.complex64
    assert A.plan.calls[-1] == ("forward_host", (reps * 24,), (reps, 10), reps, True)
    xr = x.reshape(Nd + (reps,)) if order == "F" else np.moveaxis(x.reshape((reps,) + Nd), 0, -1)
    yr = y.reshape(10, reps) if order == "F" else np.moveaxis(y.reshape(reps, 10), 0, -1)
    for r in range(reps):
        np.testing.assert_allclose(yr[:, r], (r + 1) * xr[..., r].sum(), rtol=1e-5)
    xa = A.adj(y)
    assert xa.shape == x.shape and A.plan.calls[-1][0] == "adjoint_host"
    xar = xa.reshape(Nd + (reps,)) if order == "F" else np.moveaxis(xa.reshape((reps,) + Nd), 0, -1)
    for r in range(reps):
        np.testing.assert_allclose(xar[..., r], (r + 1) * yr[:, r].sum(), rtol=1e-5)
