"""Generate golden vectors from the reference package itself.

Run in a container that has the reference sources and the ``oracle/_ref``
build (``make -C oracle ref``):

    python tests/golden/make_golden.py

The reference is imported through ``oracle/ref_shim.py``.  Trajectories and
images are regenerated from their definitions in ``tests/golden/cases.py``
(seeded, platform-independent), so the fixtures store only what the
reference computed plus the inputs that are not bit-reproducible from a
formula.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle.ref_shim import load_reference  # noqa: E402
from tests.golden import cases  # noqa: E402


def main():
    ref = load_reference()
    from mrrt.nufft._nufft import _nufft_table_make1

    out = {}
    # 1. the CPU-runnable headline workload (2-D radial, 128^2 / 256^2)
    c = cases.radial_2d_128()
    A = ref.NufftBase(**c["kw"])
    y = A.fft(c["x"])
    out["radial128_y"] = y
    out["radial128_xadj"] = A.adj(y)
    out["radial128_h0"] = np.asarray(A.h[0])
    out["radial128_sn"] = np.asarray(A.sn)
    np.savez_compressed(os.path.join(HERE, "radial128.npz"), **out)

    # 2. the reference test-suite cases (perturbed Cartesian grids)
    small = {}
    for name, c in cases.small_cases():
        A = ref.NufftBase(**c["kw"])
        y = A.fft(c["x"])
        small[name + "_y"] = y
        small[name + "_xadj"] = A.adj(y)
        reps = np.stack((c["x"],) * 3, axis=-1)
        small[name + "_yreps"] = A.fft(reps)
    # adjoint with fractional shifts (reference test_nufft_adj)
    for name, c in cases.adj_shift_cases():
        A = ref.NufftBase(**c["kw"])
        small[name + "_xadj"] = A.adj(c["y"])
    np.savez_compressed(os.path.join(HERE, "small_cases.npz"), **small)

    # 3. lookup tables (reference test_nufft_table_make1 sizes)
    tabs = {}
    for n in (64, 65):
        for phasing in ("real", "complex"):
            h, t0 = _nufft_table_make1(how="fast", N=n, J=6, K=2 * n, L=2048,
                                       phasing=phasing, order="F")
            tabs["h_%d_%s" % (n, phasing)] = np.asarray(h)
    np.savez_compressed(os.path.join(HERE, "tables.npz"), **tabs)

    make_sparse(ref)
    make_kaiser(ref)

    # 4. exact NUDFT reference values
    d = {}
    c = cases.dtft_case()
    d["dtft_y"] = ref.dtft(c["x"], c["omega"], shape=c["Nd"], n_shift=c["n_shift"])
    d["dtft_xadj"] = ref.dtft_adj(c["y"], c["omega"], shape=c["Nd"], n_shift=c["n_shift"])
    np.savez_compressed(os.path.join(HERE, "dtft.npz"), **d)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


def make_kaiser(ref=None):
    """The exported Kaiser-Bessel helpers on the parameter sets of the
    reference's own tests (mrrt/nufft/tests/test_kaiser.py), the Beatty
    kernel shape parameters, and kernel values at random points."""
    ref = ref or load_reference()
    import warnings

    from mrrt.nufft import _kaiser_bessel as kb
    from mrrt.nufft._kernels import BeattyKernel

    out = {}
    J, alpha = 8, 2.34 * 8
    x = np.linspace(-(J + 1) / 2.0, (J + 1) / 2.0, 1001)
    for m in (-4, 0, 2, 7):
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            out["kb_J8_m%d" % m] = kb.kaiser_bessel(x, J, alpha, m)
    J, alpha, N = 5, 6.8, 2 ** 10
    xx = np.arange(-N / 2.0, N / 2.0) / float(N) * (J + 3) / 2.0
    du = 1 / float(N) / float(xx[1] - xx[0])
    u = np.arange(-N / 2.0, N / 2.0) * du
    for m in (-2, 0, 2, 7):
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            out["kbft_J5_m%d" % m] = kb.kaiser_bessel_ft(u, J, alpha, m, 1)
    for d in (2, 3):
        out["kbft_J6_d%d" % d] = kb.kaiser_bessel_ft(np.linspace(-1.5, 1.5, 301), 6, 2.34 * 6, 0, d)
    for shape, grid, os_grid in (((6, 6), (256, 256), (512, 512)), ((4, 7), (64, 48), (96, 80)),
                                 ((6, 6, 6), (128, 128, 128), (256, 256, 256))):
        kern = BeattyKernel(shape=shape, grid_shape=grid, os_grid_shape=os_grid)
        tag = "x".join(map(str, shape)) + "_" + "x".join(map(str, grid)) + "_" + "x".join(map(str, os_grid))
        out["beatty_alpha_" + tag] = np.asarray(kern.alpha, dtype=np.float64)
        pts = np.random.default_rng(3).uniform(-4, 4, 64)
        out["beatty_k0_" + tag] = np.asarray(kern.kernels[0](pts))
    np.savez_compressed(os.path.join(HERE, "kaiser.npz"), **out)


def make_sparse(ref=None):
    """Sparse-matrix mode on the reference test geometries: forward and
    adjoint outputs, and the interpolation matrix itself (CSC arrays) for the
    2-D cases."""
    ref = ref or load_reference()
    sp = {}
    for name, c in cases.sparse_cases():
        A = ref.NufftBase(**c["kw"])
        y = A.fft(c["x"])
        sp[name + "_y"] = y
        sp[name + "_xadj"] = A.adj(y)
        if name.startswith("sparse_2d"):
            p = A.p.tocsc()
            p.sort_indices()
            sp[name + "_p_data"] = p.data
            sp[name + "_p_indices"] = p.indices
            sp[name + "_p_indptr"] = p.indptr
    np.savez_compressed(os.path.join(HERE, "sparse_cases.npz"), **sp)


if __name__ == "__main__":
    if sys.argv[1:] == ["--sparse-only"]:
        make_sparse()
    elif sys.argv[1:] == ["--kaiser-only"]:
        make_kaiser()
    else:
        main()
