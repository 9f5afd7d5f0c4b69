"""Device binning (gbn_plan_set_points_device): tile lists built on the GPU
from device coordinates.  Checked against the host planner on the same
coordinates -- same list lengths, items and split tiles, and (2-D, 1-D: same
entry order) bitwise-equal transforms -- and through the differentiable
operator, whose set_omega keeps a CUDA trajectory on the device."""
import numpy as np
import pytest
import torch

from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _plans(Nd, Kd, Jd, tms, coils, frame_offsets=None, precision="single"):
    """A plan built on the host for tms[1], and one built for tms[0] then
    moved to tms[1] by device binning."""
    from mrrt.nufft_gb300._kernels import kernel_table
    from mrrt.nufft_gb300._plan import GpuPlan

    rdt = np.float32 if precision == "single" else np.float64
    cdt = np.complex64 if precision == "single" else np.complex128
    ndim = len(Nd)
    h = [kernel_table(Nd[d], Jd[d], Kd[d], 1024, "real", rdt) for d in range(ndim)]
    sn = np.random.default_rng(0).uniform(0.5, 1.5, int(np.prod(Nd))).astype(rdt)
    ph = [np.exp(1j * tm @ np.arange(1, ndim + 1)).astype(cdt) for tm in tms]
    kw = dict(frame_offsets=frame_offsets, max_coils=coils, pb_coef=[0.1] * ndim,
              pb_order=list(range(ndim)))
    host = GpuPlan(Nd, Kd, Jd, 1024, rdt, h, None, sn, tms[1].astype(rdt), ph[1], **kw)
    dev = GpuPlan(Nd, Kd, Jd, 1024, rdt, h, None, sn, tms[0].astype(rdt), ph[0], **kw)
    dev.set_points_device(torch.from_numpy(tms[1].astype(rdt)).cuda(), torch.from_numpy(ph[1]).cuda())
    return host, dev


def _transforms(P, coils, seed):
    g = torch.Generator(device="cpu").manual_seed(seed)
    F = len(P.frame_offsets) - 1
    x = torch.randn((F, coils) + tuple(reversed(P.Nd)), dtype=torch.complex128, generator=g).to(
        device="cuda", dtype=P.ctype)
    y = torch.empty((coils * P.M_total,), dtype=P.ctype, device="cuda")
    P.forward(x, y, coils)
    w = torch.randn((coils * P.M_total,), dtype=torch.complex128, generator=g).to(device="cuda", dtype=P.ctype)
    xa = torch.empty_like(x)
    P.adjoint(w, xa, coils)
    torch.cuda.synchronize()
    return y, xa


STAT_KEYS = ("gather_items", "spread_items", "split_tiles", "gather_len", "spread_len")


@pytest.mark.parametrize("case", ["2d-radial-32", "2d-series-8", "1d-4", "2d-double-3"])
def test_device_lists_equal_host_lists(gpu_lib, case):
    from mrrt.nufft_gb300.trajectories import radial_2d, uneven_series_2d

    rng = np.random.default_rng(1)
    fo = None
    precision = "single"
    if case == "2d-radial-32":
        Nd, Kd, Jd, coils = (64, 64), (128, 128), (6, 6), 32
        om = [radial_2d(150, 128, golden=True), radial_2d(150, 128, golden=True, first_spoke=7)]
    elif case == "2d-series-8":
        Nd, Kd, Jd, coils = (48, 48), (96, 96), (6, 6), 8
        a = uneven_series_2d(5, 96, 9, 21, seed=2)
        b = [o + 0.01 for o in a]
        fo = np.concatenate([[0], np.cumsum([o.shape[0] for o in a])])
        om = [np.concatenate(a), np.concatenate(b)]
    elif case == "1d-4":
        Nd, Kd, Jd, coils = (100,), (200,), (7,), 4
        om = [rng.uniform(-np.pi, np.pi, (3000, 1)), rng.uniform(-3 * np.pi, 3 * np.pi, (3000, 1))]
    else:
        Nd, Kd, Jd, coils, precision = (40, 36), (80, 72), (6, 5), 3, "double"
        om = [rng.uniform(-np.pi, np.pi, (2500, 2)), rng.uniform(-2 * np.pi, 2 * np.pi, (2500, 2))]
    tms = [o / (2 * np.pi / np.asarray(Kd, dtype=np.float64)) for o in om]
    host, dev = _plans(Nd, Kd, Jd, tms, coils, frame_offsets=fo, precision=precision)
    sh, sd = host.stats(), dev.stats()
    assert {k: sh[k] for k in STAT_KEYS} == {k: sd[k] for k in STAT_KEYS}
    yh, xh = _transforms(host, coils, 3)
    yd, xd = _transforms(dev, coils, 3)
    assert torch.equal(yh, yd)
    assert torch.equal(xh, xd)


def test_device_lists_3d_match_host(gpu_lib):
    """3-D: the host planner orders the entries of heavy tiles by a hash, the
    device lists keep sample order, so results agree to float rounding."""
    from mrrt.nufft_gb300.trajectories import kooshball_3d

    Nd, Kd, Jd, coils = (24, 24, 24), (48, 48, 48), (6, 6, 6), 4
    om = [kooshball_3d(600, 48), kooshball_3d(640, 45)[:600 * 48]]
    tms = [o / (2 * np.pi / 48.0) for o in om]
    host, dev = _plans(Nd, Kd, Jd, tms, coils)
    sh, sd = host.stats(), dev.stats()
    assert {k: sh[k] for k in STAT_KEYS} == {k: sd[k] for k in STAT_KEYS}
    yh, xh = _transforms(host, coils, 4)
    yd, xd = _transforms(dev, coils, 4)
    assert torch.equal(yh, yd)
    assert rel_l2(xd.cpu().numpy(), xh.cpu().numpy()) < 1e-6


def test_device_binning_rejects_invalid_coordinates(gpu_lib):
    from mrrt.nufft_gb300._lib import GbnValueError
    from mrrt.nufft_gb300.trajectories import radial_2d

    Nd, Kd, Jd, coils = (32, 32), (64, 64), (6, 6), 2
    om = radial_2d(20, 64)
    tm = om / (2 * np.pi / 64.0)
    host, dev = _plans(Nd, Kd, Jd, [tm, tm], coils)
    y0, x0 = _transforms(dev, coils, 5)
    for bad in (np.nan, np.inf, 1e7):
        t2 = tm.copy()
        t2[17, 1] = bad
        with pytest.raises(GbnValueError):
            dev.set_points_device(torch.from_numpy(t2.astype(np.float32)).cuda())
        y1, x1 = _transforms(dev, coils, 5)   # the previous lists still serve
        assert torch.equal(y0, y1) and torch.equal(x0, x1)


def test_operator_set_omega_on_device_matches_host_trajectory(gpu_lib):
    """NufftOperator with a CUDA omega (device binning) and with the same
    omega as a numpy array (host planner): same forward and adjoint, to
    float32 rounding -- the sample phase exp(i omega . (n_shift - n_mid)) has
    an argument of up to ~100 rad, whose float32 dot product rounds
    differently on the GPU (fused multiply-add) than in numpy."""
    from mrrt.nufft_gb300.autograd import NufftOperator
    from mrrt.nufft_gb300.trajectories import spiral_2d

    Nd = (64, 64)
    om0 = spiral_2d(8, 512)
    om1 = om0 * 0.97 + 0.002
    A = NufftOperator(Nd, om0, Jd=6, Kd=(128, 128), max_coils=4)
    B = NufftOperator(Nd, om1, Jd=6, Kd=(128, 128), max_coils=4)
    g = torch.Generator(device="cpu").manual_seed(2)
    x = torch.randn((4,) + Nd, dtype=torch.complex64, generator=g).cuda()
    om1_t = torch.from_numpy(om1.astype(np.float32)).cuda()
    ya = A.forward(x, om1_t)        # A moves to om1 on the device
    yb = B.forward(x)
    assert rel_l2(ya.detach().cpu().numpy(), yb.cpu().numpy()) < 1e-5
    xa = A.adjoint(ya, om1_t)
    xb = B.adjoint(yb)
    assert rel_l2(xa.detach().cpu().numpy(), xb.cpu().numpy()) < 1e-5
