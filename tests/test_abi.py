"""C-ABI checks that need no GPU: the library loads, exports every entry
point include/gbnufft.h declares, its struct layout matches the ctypes
mirror, and argument validation returns status codes (no compute calls)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from tests.conftest import REPO

HEADER = os.path.join(REPO, "include", "gbnufft.h")


@pytest.fixture(scope="module")
def lib():
    from mrrt.nufft_gb300 import _build, _lib

    _build.build()
    return _lib.load()


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gbn_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_expected_api():
    names = declared_functions()
    for required in ("gbn_plan_create", "gbn_plan_destroy", "gbn_forward", "gbn_adjoint",
                     "gbn_interp_forward", "gbn_interp_adjoint", "gbn_grad_tm",
                     "gbn_dtft_forward", "gbn_dtft_adjoint", "gbn_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", lib._name], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\bT (gbn_[a-z0-9_]+)", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing


def test_ctypes_signatures_cover_header(lib):
    from mrrt.nufft_gb300 import _lib

    assert sorted(_lib.SIGNATURES) == declared_functions()


def test_geometry_struct_layout_matches_c(tmp_path):
    from mrrt.nufft_gb300._lib import GbnGeometry

    probe = tmp_path / "probe.c"
    fields = [f for f, _ in GbnGeometry._fields_]
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gbnufft.h"', "int main(void){",
             'printf("%zu\\n", sizeof(gbn_geometry));']
    lines += ['printf("%%zu\\n", offsetof(gbn_geometry, %s));' % f for f in fields]
    lines += ["return 0;}"]
    probe.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-I", os.path.join(REPO, "include"), str(probe), "-o", str(exe)], check=True)
    vals = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert vals[0] == ctypes.sizeof(GbnGeometry)
    for f, off in zip(fields, vals[1:]):
        assert getattr(GbnGeometry, f).offset == off, f


def test_header_constants_match_python_mirror():
    """Status codes, precision / phasing values and geometry flags: every
    #define of include/gbnufft.h against the constants of _lib.py."""
    from mrrt.nufft_gb300 import _lib

    defines = dict(re.findall(r"#define\s+(GBN_[A-Z_]+)\s+(\d+)", open(HEADER).read()))
    mirror = {k: getattr(_lib, k) for k in dir(_lib) if k.startswith("GBN_ERR_") or k == "GBN_OK"}
    mirror.update({"GBN_FLAG_" + k[5:]: getattr(_lib, k) for k in dir(_lib) if k.startswith("FLAG_")})
    mirror.update({"GBN_PRECISION_" + k.upper(): v for k, v in _lib.PRECISION.items()})
    mirror.update({"GBN_PHASING_" + k.upper(): v for k, v in _lib.PHASING.items()})
    numeric = {k: int(v) for k, v in defines.items() if not k.startswith("GBN_NOALLOC")}
    assert numeric == mirror


def _geom(**kw):
    from mrrt.nufft_gb300._lib import GbnGeometry

    g = GbnGeometry()
    g.ndim = kw.get("ndim", 2)
    for d in range(3):
        g.Nd[d] = kw.get("N", 16)
        g.Kd[d] = kw.get("K", 32)
        g.Jd[d] = kw.get("J", 6)
        g.pb_order[d] = d if d < g.ndim else 0
    g.L = kw.get("L", 1024)
    g.precision = kw.get("precision", 0)
    g.phasing = kw.get("phasing", 0)
    g.n_frames = kw.get("n_frames", 1)
    g.max_coils = kw.get("max_coils", 1)
    g.adjoint_scale = 1.0
    return g


@pytest.mark.parametrize("bad,code", [
    (dict(ndim=4), 5), (dict(J=9), 5), (dict(J=0), 1), (dict(K=8, N=16), 1), (dict(L=0), 1),
    (dict(precision=3), 1), (dict(phasing=2), 1), (dict(n_frames=0), 1), (dict(max_coils=0), 1),
])
def test_plan_create_rejects_bad_geometry(lib, bad, code):
    g = _geom(**bad)
    handle = ctypes.c_void_p()
    fo = (ctypes.c_int64 * 2)(0, 0)
    tabs = (ctypes.c_void_p * 3)()
    rc = lib.gbn_plan_create(ctypes.byref(handle), ctypes.byref(g), tabs, None, None, fo, None, None, 0)
    assert rc == code
    assert handle.value is None
    assert len(lib.gbn_last_error()) > 0


def test_null_arguments_are_rejected(lib):
    assert lib.gbn_plan_create(None, None, None, None, None, None, None, None, 0) == 1
    assert lib.gbn_forward(None, None, None, 1, None) == 1
    assert lib.gbn_adjoint(None, None, None, 1, None) == 1
    assert lib.gbn_plan_destroy(None) == 0
    nd = (ctypes.c_int * 3)(4, 4, 1)
    sh = (ctypes.c_double * 3)(0, 0, 0)
    assert lib.gbn_dtft_forward(0, nd, sh, None, 1, None, None, 1, None) == 1
    assert lib.gbn_dtft_forward(2, nd, sh, None, 5, None, None, 1, None) == 1
    assert lib.gbn_version().startswith(b"gbnufft")


def test_checked_build_exports_every_declared_symbol():
    """The bounds-checked build (GBN_CHECKED) exposes the same C ABI."""
    from mrrt.nufft_gb300 import _build

    path = _build.build(checked=True)
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\bT (gbn_[a-z0-9_]+)", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing


def test_check_status_rejects_a_null_plan(lib):
    status = ctypes.c_uint(7)
    assert lib.gbn_debug_check_status(None, ctypes.byref(status)) == 1   # GBN_ERR_INVALID
