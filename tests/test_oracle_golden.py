"""Pin the oracle: it must reproduce the golden vectors the reference itself
produced (tests/golden/make_golden.py), and, where the reference sources are
present, the reference on fresh inputs."""
import numpy as np
import pytest

from oracle import oracle as O
from oracle.ref_shim import reference_available
from tests.conftest import rel_l2
from tests.golden import cases


def test_radial128_forward_adjoint_match_golden():
    g = cases.load("radial128")
    c = cases.radial_2d_128()
    A = O.OracleNufft(**c["kw"])
    y = A.fft(c["x"])
    # same algorithm, same dtypes: equal to float32 rounding
    assert rel_l2(y, g["radial128_y"]) < 1e-6
    xa = A.adj(g["radial128_y"])
    assert rel_l2(xa, g["radial128_xadj"]) < 1e-6
    assert np.max(np.abs(A.sn - g["radial128_sn"])) == 0
    assert np.max(np.abs(A.h[0] - g["radial128_h0"])) < 1e-7


@pytest.mark.parametrize("name", [n for n, _ in cases.small_cases()])
def test_small_cases_match_golden(name):
    g = cases.load("small_cases")
    c = dict(cases.small_cases())[name]
    A = O.OracleNufft(**c["kw"])
    tol = 1e-5 if "single" in name else 1e-12
    y = A.fft(c["x"])
    assert rel_l2(y, g[name + "_y"]) < tol
    assert rel_l2(A.adj(y), g[name + "_xadj"]) < tol
    reps = np.stack((c["x"],) * 3, axis=-1)
    assert rel_l2(A.fft(reps), g[name + "_yreps"]) < tol


@pytest.mark.parametrize("name", [n for n, _ in cases.adj_shift_cases()])
def test_fractional_shift_adjoint_matches_golden(name):
    g = cases.load("small_cases")
    c = dict(cases.adj_shift_cases())[name]
    A = O.OracleNufft(**c["kw"])
    assert rel_l2(A.adj(c["y"]), g[name + "_xadj"]) < 1e-5


@pytest.mark.parametrize("n,phasing", [(64, "real"), (64, "complex"), (65, "real"), (65, "complex")])
def test_tables_match_golden(n, phasing):
    g = cases.load("tables")
    h, _ = O.table_make1(n, 6, 2 * n, 2048, phasing)
    ref = g["h_%d_%s" % (n, phasing)]
    assert h.shape == ref.shape
    assert np.max(np.abs(h - ref)) < 1e-6


def test_oracle_dtft_matches_golden():
    g = cases.load("dtft")
    c = cases.dtft_case()
    y = O.dtft(c["x"], c["omega"], c["Nd"], c["n_shift"])
    assert rel_l2(y, g["dtft_y"]) < 1e-12
    x = O.dtft_adj(c["y"], c["omega"], c["Nd"], c["n_shift"])
    assert rel_l2(x, g["dtft_xadj"]) < 1e-12


def test_oracle_nufft_accuracy_vs_exact():
    """The table NUFFT is within the reference test-suite tolerance of the
    exact NUDFT (mrrt/nufft/tests/test_nufft.py:184-244)."""
    c = dict(cases.small_cases())["2d_3232_J6_double_real"]
    A = O.OracleNufft(**c["kw"])
    y = A.fft(c["x"])
    yt = O.dtft(c["x"], c["kw"]["omega"], c["kw"]["Nd"], c["kw"]["n_shift"])
    np.testing.assert_allclose(y, yt, rtol=1e-3, atol=1e-5)


@pytest.mark.skipif(not reference_available(), reason="reference sources not present")
def test_oracle_interp_bit_identical_to_reference_c():
    """Where the reference compiles here, its C table interpolation and the
    oracle's restatement agree on identical inputs."""
    from oracle.ref_shim import load_reference

    load_reference()
    from mrrt.nufft._interp_table import interp2_table, interp2_table_adj

    rng = np.random.default_rng(3)
    K = (64, 48)
    tm = np.stack([rng.uniform(-40, 80, 500), rng.uniform(-30, 60, 500)], -1).astype(np.float32)
    h = [np.asarray(O.table_make1(32, 6, 64, 512, "real")[0]).astype(np.float32),
         np.asarray(O.table_make1(24, 6, 48, 512, "real")[0]).astype(np.float32)]
    ck = (rng.standard_normal(K + (2,)) + 1j * rng.standard_normal(K + (2,))).astype(np.complex64)
    y_ref = interp2_table(np.asfortranarray(ck), h[0], h[1], (6, 6), 512, tm)
    y_or = O.interp_forward(ck, h, (6, 6), 512, tm, K)
    assert np.array_equal(y_ref, y_or)
    fm = (rng.standard_normal((500, 2)) + 1j * rng.standard_normal((500, 2))).astype(np.complex64)
    g_ref = interp2_table_adj(np.asfortranarray(fm), h[0], h[1], (6, 6), 512, tm, K)
    g_or = O.interp_adjoint(fm, h, (6, 6), 512, tm, K)
    assert rel_l2(g_or, g_ref) < 1e-6


@pytest.mark.skipif(not __import__("oracle.refc").refc.available(), reason="oracle/_ref not built")
@pytest.mark.parametrize("ndim", [1, 2, 3])
def test_reference_c_library_matches_oracle_restatement(ndim):
    """The reference's own compiled kernels (oracle/_ref, built from its
    sources or from the preprocessed unit on a machine without them) and the
    oracle's C restatement: forward bit for bit, adjoint to rounding, on
    coordinates that wrap around both ends of the grid."""
    from oracle import refc

    rng = np.random.default_rng(11 + ndim)
    K = (40, 36, 20)[:ndim]
    N = (20, 18, 10)[:ndim]
    M = 700
    tm = np.stack([rng.uniform(-2 * k, 3 * k, M) for k in K], -1).astype(np.float32)
    h = [np.asarray(O.table_make1(N[d], 6, K[d], 256, "real")[0]).astype(np.float32) for d in range(ndim)]
    ck = (rng.standard_normal(K + (3,)) + 1j * rng.standard_normal(K + (3,))).astype(np.complex64)
    y_ref = refc.interp_forward(ck, h, (6,) * ndim, 256, tm, K)
    y_or = O.interp_forward(ck, h, (6,) * ndim, 256, tm, K)
    assert np.array_equal(y_ref, y_or)
    fm = (rng.standard_normal((M, 3)) + 1j * rng.standard_normal((M, 3))).astype(np.complex64)
    g_ref = refc.interp_adjoint(fm, h, (6,) * ndim, 256, tm, K)
    g_or = O.interp_adjoint(fm, h, (6,) * ndim, 256, tm, K)
    assert rel_l2(g_or, g_ref) < 1e-6
    A = O.OracleNufft(N, tm[:, :ndim] * (2 * np.pi / np.asarray(K)), Jd=6, Kd=K, Ld=256, interp=refc)
    B = O.OracleNufft(N, tm[:, :ndim] * (2 * np.pi / np.asarray(K)), Jd=6, Kd=K, Ld=256)
    x = (rng.standard_normal(N) + 1j * rng.standard_normal(N)).astype(np.complex64)
    assert rel_l2(A.fft(x), B.fft(x)) < 1e-6
    assert rel_l2(A.adj(fm[:, 0]), B.adj(fm[:, 0])) < 1e-6


def test_exported_kaiser_bessel_helpers_match_reference():
    """kaiser_bessel, kaiser_bessel_ft and BeattyKernel (exported like the
    reference's, mrrt/nufft/__init__.py) against values the reference
    computed on the parameter sets of its own tests."""
    import warnings

    from mrrt.nufft_gb300 import BeattyKernel, kaiser_bessel, kaiser_bessel_ft

    g = cases.load("kaiser")
    J, alpha = 8, 2.34 * 8
    x = np.linspace(-(J + 1) / 2.0, (J + 1) / 2.0, 1001)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        for m in (-4, 0, 2, 7):
            np.testing.assert_allclose(kaiser_bessel(x, J, alpha, m), g["kb_J8_m%d" % m], rtol=1e-12, atol=1e-15)
        J, alpha, N = 5, 6.8, 2 ** 10
        xx = np.arange(-N / 2.0, N / 2.0) / float(N) * (J + 3) / 2.0
        u = np.arange(-N / 2.0, N / 2.0) * (1 / float(N) / float(xx[1] - xx[0]))
        for m in (-2, 0, 2, 7):
            np.testing.assert_allclose(kaiser_bessel_ft(u, J, alpha, m, 1), g["kbft_J5_m%d" % m],
                                       rtol=1e-10, atol=1e-14)
    for d in (2, 3):
        np.testing.assert_allclose(kaiser_bessel_ft(np.linspace(-1.5, 1.5, 301), 6, 2.34 * 6, 0, d),
                                   g["kbft_J6_d%d" % d], rtol=1e-10, atol=1e-14)
    pts = np.random.default_rng(3).uniform(-4, 4, 64)
    for shape, grid, os_grid in (((6, 6), (256, 256), (512, 512)), ((4, 7), (64, 48), (96, 80)),
                                 ((6, 6, 6), (128, 128, 128), (256, 256, 256))):
        kern = BeattyKernel(shape=shape, grid_shape=grid, os_grid_shape=os_grid)
        tag = "x".join(map(str, shape)) + "_" + "x".join(map(str, grid)) + "_" + "x".join(map(str, os_grid))
        np.testing.assert_allclose(np.asarray(kern.alpha, dtype=np.float64), g["beatty_alpha_" + tag], rtol=1e-14)
        np.testing.assert_allclose(kern.kernels[0](pts), g["beatty_k0_" + tag], rtol=1e-12, atol=1e-15)
