"""ctypes binding of libgbnufft.so (the C ABI in include/gbnufft.h).

The library is built in-tree by ``mrrt.nufft_gb300._build.build()``.  There is
no fallback: if the shared object is missing or fails to load, every entry
point raises.
"""
import ctypes
import os
import threading

from ._build import LIB_PATH

GBN_OK = 0
GBN_ERR_INVALID = 1
GBN_ERR_CUDA = 2
GBN_ERR_CUFFT = 3
GBN_ERR_NOMEM = 4
GBN_ERR_UNSUPPORTED = 5
GBN_ERR_TOOLARGE = 6

FLAG_TABLE_ONLY = 1
FLAG_CUFFT_ONLY = 2

PRECISION = {"single": 0, "double": 1}
PHASING = {"real": 0, "complex": 1}


class GbnGeometry(ctypes.Structure):
    _fields_ = [
        ("ndim", ctypes.c_int),
        ("Nd", ctypes.c_int * 3),
        ("Kd", ctypes.c_int * 3),
        ("Jd", ctypes.c_int * 3),
        ("L", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("phasing", ctypes.c_int),
        ("ortho", ctypes.c_int),
        ("adjoint_scale", ctypes.c_double),
        ("pb_coef", ctypes.c_double * 3),
        ("pb_order", ctypes.c_int * 3),
        ("n_frames", ctypes.c_int),
        ("tile", ctypes.c_int * 3),
        ("stile", ctypes.c_int * 3),
        ("max_coils", ctypes.c_int),
        ("flags", ctypes.c_int),
    ]


class GbnError(RuntimeError):
    """A libgbnufft entry point returned a non-zero status."""

    def __init__(self, code, msg):
        super().__init__("libgbnufft error %d: %s" % (code, msg))
        self.code = code


class GbnValueError(GbnError, ValueError):
    pass


# Entry points and their signatures (void* = ctypes.c_void_p).
_VP = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
SIGNATURES = {
    "gbn_plan_create": [ctypes.POINTER(_VP), ctypes.POINTER(GbnGeometry), ctypes.POINTER(_VP),
                        ctypes.POINTER(_VP), _VP, ctypes.POINTER(_I64), _VP, _VP, _I],
    "gbn_plan_set_points": [_VP, _VP, _VP],
    "gbn_plan_set_points_device": [_VP, _VP, _VP, _VP],
    "gbn_plan_destroy": [_VP],
    "gbn_forward": [_VP, _VP, _VP, _I, _VP],
    "gbn_adjoint": [_VP, _VP, _VP, _I, _VP],
    "gbn_forward_host": [_VP, _VP, _VP, _I, _VP],
    "gbn_adjoint_host": [_VP, _VP, _VP, _I, _VP],
    "gbn_interp_forward": [_VP, _VP, _VP, _I, _VP],
    "gbn_interp_adjoint": [_VP, _VP, _VP, _I, _VP],
    "gbn_interp_adjoint_noalloc": [_VP, _VP, _VP, _I, _VP],
    "gbn_plan_set_weights": [_VP, _VP, _VP],
    "gbn_forward_sense": [_VP, _VP, _VP, _VP, _I, _VP],
    "gbn_adjoint_sense": [_VP, _VP, _VP, _VP, _I, _VP],
    "gbn_plan_set_dtables": [_VP, ctypes.POINTER(_VP)],
    "gbn_grad_tm": [_VP, _VP, _VP, ctypes.POINTER(ctypes.c_double), _VP, _I, _VP],
    "gbn_forward_grid": [_VP, ctypes.POINTER(_VP)],
    "gbn_dtft_forward": [_I, ctypes.POINTER(_I), ctypes.POINTER(ctypes.c_double), _VP, _I64, _VP,
                         _VP, _I, _VP],
    "gbn_dtft_adjoint": [_I, ctypes.POINTER(_I), ctypes.POINTER(ctypes.c_double), _VP, _I64, _VP,
                         _VP, _I, _VP],
    "gbn_plan_stats": [_VP, ctypes.POINTER(_I64)],
    "gbn_last_error": [],
    "gbn_version": [],
    "gbn_debug_fail_alloc": [ctypes.c_longlong],
    "gbn_debug_check_status": [_VP, ctypes.POINTER(ctypes.c_uint)],
}

_lib = None
_lib_checked = None
_lock = threading.Lock()


def _open(path):
    if not os.path.exists(path):
        raise ImportError(
            "%s is not built; run mrrt.nufft_gb300._build.build() "
            "or __graft_entry__.build() first" % path)
    lib = ctypes.CDLL(path)
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_char_p if name in ("gbn_last_error", "gbn_version") else ctypes.c_int
    return lib


def load(path=None):
    """Load (once) and return the ctypes handle of libgbnufft.so."""
    global _lib
    with _lock:
        if _lib is None:
            _lib = _open(path or LIB_PATH)
        return _lib


def load_checked():
    """Load (once) the bounds-checked build, libgbnufft_checked.so (a
    separate library: plans made through it run the checked kernels)."""
    global _lib_checked
    with _lock:
        if _lib_checked is None:
            _lib_checked = _open(os.path.join(os.path.dirname(LIB_PATH), "libgbnufft_checked.so"))
        return _lib_checked


def check(rc, lib=None):
    if rc != GBN_OK:
        msg = (lib or load()).gbn_last_error().decode(errors="replace")
        if rc in (GBN_ERR_INVALID, GBN_ERR_UNSUPPORTED, GBN_ERR_TOOLARGE):
            raise GbnValueError(rc, msg)
        raise GbnError(rc, msg)
    return rc


def check_with(lib, rc):
    """check() with the error message taken from ``lib``."""
    return check(rc, lib)
