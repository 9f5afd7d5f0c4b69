"""Definitions of the golden-vector cases (inputs regenerated from seeds).

Shared by ``make_golden.py`` (which runs the reference on them) and by the
tests (which run the oracle and the CUDA path on them).
"""
import itertools
import os
import sys

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if REPO not in sys.path:
    sys.path.insert(0, REPO)

from mrrt.nufft_gb300.trajectories import (  # noqa: E402
    complex_image,
    perturbed_grid,
    radial_2d,
)

HERE = os.path.dirname(os.path.abspath(__file__))


def load(name):
    return dict(np.load(os.path.join(HERE, name + ".npz")))


def radial_2d_128():
    """128^2 image, 256^2 grid, J=6, L=1024; 128 uniform spokes x 256 points."""
    omega = radial_2d(128, 256)
    kw = dict(Nd=(128, 128), omega=omega, Jd=(6, 6), Kd=(256, 256), mode="table",
              Ld=1024, precision="single")
    return dict(kw=kw, x=complex_image((128, 128), seed=0))


def _small(Nd, Kd, Jd, precision, phasing):
    omega = perturbed_grid(Nd)
    rs = np.random.RandomState(1234)
    x = rs.standard_normal(Nd) + 1j * rs.standard_normal(Nd)
    kw = dict(Nd=Nd, omega=omega, Jd=Jd, Kd=Kd, n_shift=tuple(np.asarray(Nd) / 2),
              mode="table", Ld=1024, precision=precision, phasing=phasing)
    return dict(kw=kw, x=x)


def small_cases():
    """The reference test-suite geometries (mrrt/nufft/tests/test_nufft.py:99-324)."""
    out = []
    for precision, phasing in itertools.product(("single", "double"), ("real", "complex")):
        for Kd, Jd in (((32, 32), 6), ((33, 31), 7)):
            name = "2d_%d%d_J%d_%s_%s" % (Kd[0], Kd[1], Jd, precision, phasing)
            out.append((name, _small((16, 16), Kd, Jd, precision, phasing)))
        out.append(("3d_J6_%s_%s" % (precision, phasing),
                    _small((8, 8, 8), (16, 16, 16), 6, precision, phasing)))
        out.append(("1d_J6_%s_%s" % (precision, phasing),
                    _small((64,), (128,), 6, precision, phasing)))
    return out


def adj_shift_cases():
    """Fractional n_shift adjoint (mrrt/nufft/tests/test_nufft.py:60-96)."""
    o1 = 2 * np.pi * np.array([0.0, 0.1, 0.3, 0.4, 0.7, 0.9])
    omega = np.stack((o1, o1[::-1].copy()), axis=-1)
    data = np.arange(1, o1.size + 1).astype(np.float64) ** 2
    y = np.stack((data,) * 3, axis=-1)
    out = []
    for phasing in ("real", "complex"):
        kw = dict(Nd=(4, 8), omega=omega, Jd=(8, 8), Kd=(8, 16), Ld=1024,
                  n_shift=(2.7, 3.1), phasing=phasing, mode="table")
        out.append(("adjshift_%s" % phasing, dict(kw=kw, y=y)))
    return out


def dtft_case():
    rs = np.random.RandomState(7)
    Nd = (8, 12, 10)
    omega = rs.uniform(-np.pi, np.pi, size=(300, 3))
    x = rs.standard_normal(Nd) + 1j * rs.standard_normal(Nd)
    y = rs.standard_normal(300) + 1j * rs.standard_normal(300)
    return dict(Nd=Nd, omega=omega, x=x, y=y, n_shift=(1.0, 3.0, 2.0))


def sparse_cases():
    """The reference test-suite geometries in sparse-matrix mode
    (mrrt/nufft/tests/test_nufft.py:99-324 run both modes)."""
    out = []
    for name, c in small_cases():
        kw = dict(c["kw"])
        kw["mode"] = "sparse"
        out.append(("sparse_" + name, dict(kw=kw, x=c["x"])))
    return out

