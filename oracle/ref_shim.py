"""Loader for the reference Python package (test infrastructure only).

Used in the build container, where the reference sources exist, to validate
the oracle against the reference itself and to generate the golden vectors
under ``tests/golden``.  Nothing on the product path imports this module and
nothing here runs on a machine without the reference sources.

The reference imports a helper package ``mrrt.utils`` that is not part of its
tree (``mrrt/nufft/_nufft.py:35-50``).  The stand-in below restates the
behaviour its call sites rely on:

* ``fftn`` / ``ifftn`` -- zero-padded n-d FFT over ``axes`` (numpy pocketfft,
  which keeps complex64 in single precision);
* ``complexify(x, complex_dtype)`` -- cast exactly to ``complex_dtype`` (the C
  kernels receive ``float*`` planes, so the dtype must match the operator);
* ``reale(x)`` -- real part, raising ``ValueError`` if the imaginary part is
  not negligible;
* ``outer_sum``, ``get_array_module``, ``get_data_address``, ``prod``,
  ``nullcontext``, ``profile``, ``config.have_cupy = False`` and
  ``max_percent_diff``.

scipy >= 1.14 dropped ``spmatrix.H`` (used by the sparse-mode adjoint,
``_nufft.py:1505``); it is restored as the conjugate transpose.
"""
import contextlib
import importlib.machinery
import importlib.util
import math
import os
import sys
import sysconfig
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def _reference_root():
    """The reference checkout: MRRT_REFERENCE_ROOT, else the one the build
    recorded in oracle/_ref/REF_ROOT when it compiled the reference there."""
    root = os.environ.get("MRRT_REFERENCE_ROOT")
    if root:
        return root
    marker = os.path.join(HERE, "_ref", "REF_ROOT")
    if os.path.exists(marker):
        with open(marker) as f:
            return f.read().strip() or None
    return None


DEFAULT_REF = _reference_root()


def _standin_utils():
    m = types.ModuleType("mrrt.utils")

    def complexify(x, complex_dtype=None):
        x = np.asarray(x)
        if complex_dtype is None:
            complex_dtype = np.result_type(x.dtype, np.complex64)
        return x.astype(complex_dtype, copy=False)

    def reale(x, tol=1e-10):
        x = np.asarray(x)
        if np.iscomplexobj(x):
            mag = np.max(np.abs(x)) if x.size else 0.0
            if x.size and np.max(np.abs(x.imag)) > tol * max(mag, 1e-300):
                raise ValueError("non-negligible imaginary part")
            return x.real
        return x

    def fftn(x, s=None, axes=None):
        return np.fft.fftn(x, s=s, axes=None if axes is None else tuple(axes))

    def ifftn(x, s=None, axes=None):
        return np.fft.ifftn(x, s=s, axes=None if axes is None else tuple(axes))

    def outer_sum(a, b):
        return np.asarray(a)[:, None] + np.asarray(b)[None, :]

    def get_array_module(x, xp=None):
        return np, False

    def get_data_address(x):
        return x.__array_interface__["data"][0]

    def prod(seq):
        return math.prod(int(s) if float(s).is_integer() else s for s in seq)

    def profile(f):
        return f

    def max_percent_diff(a, b):
        a = np.asarray(a)
        b = np.asarray(b)
        return 100.0 * np.max(np.abs(a - b)) / max(np.max(np.abs(a)), 1e-300)

    class _Config:
        have_cupy = False

    m.complexify = complexify
    m.reale = reale
    m.fftn = fftn
    m.ifftn = ifftn
    m.outer_sum = outer_sum
    m.get_array_module = get_array_module
    m.get_data_address = get_data_address
    m.prod = prod
    m.profile = profile
    m.max_percent_diff = max_percent_diff
    m.nullcontext = contextlib.nullcontext
    m.config = _Config()
    return m


def reference_available(ref_root=DEFAULT_REF):
    if not ref_root:
        return False
    ext = os.path.join(HERE, "_ref", "_nufft_table" + sysconfig.get_config_var("EXT_SUFFIX"))
    return os.path.isdir(os.path.join(ref_root, "mrrt", "nufft")) and os.path.exists(ext)


def load_reference(ref_root=DEFAULT_REF):
    """Import and return the reference ``mrrt.nufft`` package."""
    if "mrrt.nufft" in sys.modules:
        return sys.modules["mrrt.nufft"]
    if not reference_available(ref_root):
        raise RuntimeError("reference sources or oracle/_ref build missing")
    import scipy.sparse

    for cls in (scipy.sparse.csc_matrix, scipy.sparse.csr_matrix, scipy.sparse.coo_matrix):
        if not hasattr(cls, "H"):
            cls.H = property(lambda s: s.conj().T)

    if REPO not in sys.path:
        sys.path.insert(0, REPO)
    import mrrt  # the project's namespace package

    ref_pkg = os.path.join(ref_root, "mrrt")
    if ref_pkg not in list(mrrt.__path__):
        mrrt.__path__.append(ref_pkg)
    utils = _standin_utils()
    sys.modules["mrrt.utils"] = utils
    mrrt.utils = utils

    ext_name = "mrrt.nufft._extensions._nufft_table"
    ext_path = os.path.join(HERE, "_ref", "_nufft_table" + sysconfig.get_config_var("EXT_SUFFIX"))
    loader = importlib.machinery.ExtensionFileLoader(ext_name, ext_path)
    spec = importlib.util.spec_from_file_location(ext_name, ext_path, loader=loader)
    ext = importlib.util.module_from_spec(spec)
    loader.exec_module(ext)
    sys.modules[ext_name] = ext

    import mrrt.nufft as ref

    return ref
