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

    # 4. exact NUDFT reference values
    d = {}
    c = cases.dtft_case()
    d["dtft_y"] = ref.dtft(c["x"], c["omega"], shape=c["Nd"], n_shift=c["n_shift"])
    d["dtft_xadj"] = ref.dtft_adj(c["y"], c["omega"], shape=c["Nd"], n_shift=c["n_shift"])
    np.savez_compressed(os.path.join(HERE, "dtft.npz"), **d)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


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
    else:
        main()
