"""ctypes binding to the reference's own compiled table interpolation
(test infrastructure and CPU baseline only).

``oracle/_ref/libnufft_table_ref.so`` is the reference's
``mrrt/nufft/_extensions/c/nufft_table.c`` compiled by ``oracle/Makefile``:
from its sources where they lie (``make ref``), or, on a machine without the
sources, from the preprocessed unit that compile left in ``oracle/_ref/``
(``make ref-native``).  Nothing here restates the algorithm: the calls go to
the reference's C symbols ``{float,double}_interp{1,2,3}_table1_real_{forward,adj}``
(``nufft_table.template.h:48-280``) with the argument layout its Cython
wrappers use (``_extensions/_nufft_table.pyx:29-704``): split real/imaginary
planes in Fortran order, the forward called once per repetition, the adjoint
once with all repetitions (OpenMP over repetitions inside the C).

``OracleNufft(..., interp=refc)`` runs the oracle's restated orchestration
(pad, FFT, phases, crop) around these kernels, which is how the timed CPU
baseline measures the reference's own compiled code.
"""
import ctypes
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libnufft_table_ref.so")
_lib = None
_lock = threading.Lock()


def available():
    return os.path.exists(LIB_PATH)


def _load():
    global _lib
    with _lock:
        if _lib is None:
            if not available():
                raise RuntimeError("oracle/_ref/libnufft_table_ref.so missing: run make -C oracle ref "
                                   "(or ref-native)")
            lib = ctypes.CDLL(LIB_PATH)
            for T, pre in ((ctypes.c_float, "float"), (ctypes.c_double, "double")):
                P = ctypes.POINTER(T)
                I = ctypes.c_int
                for nd in (1, 2, 3):
                    fw = getattr(lib, "%s_interp%d_table1_real_forward" % (pre, nd))
                    fw.restype = None
                    fw.argtypes = [P, P] + [I] * nd + [P] * nd + [I] * nd + [I, P, I, P, P]
                    ad = getattr(lib, "%s_interp%d_table1_real_adj" % (pre, nd))
                    ad.restype = None
                    ad.argtypes = [P, P] + [I] * nd + [P] * nd + [I] * nd + [I, P, I, P, P, I]
            _lib = lib
    return _lib


def _ptr(a, T):
    return a.ctypes.data_as(ctypes.POINTER(T))


def _setup(h_list, tm, ndim):
    if any(np.iscomplexobj(h) for h in h_list):
        raise NotImplementedError("reference C binding: real (phasing 'real') tables only")
    rdt = np.result_type(*[np.asarray(h).dtype for h in h_list])
    T = ctypes.c_float if rdt == np.float32 else ctypes.c_double
    pre = "float" if rdt == np.float32 else "double"
    hs = [np.asfortranarray(np.asarray(h, dtype=rdt)) for h in h_list]
    tm = np.asfortranarray(np.asarray(tm, dtype=rdt).reshape((-1, ndim)))
    return rdt, T, pre, hs, tm


def interp_forward(ck, h_list, Jd, L, tm, Kd):
    """Grid ``[prod(Kd), N]`` (Fortran) -> samples ``[M, N]`` through the
    reference's ``*_interp{d}_table1_real_forward``, once per repetition."""
    lib = _load()
    ndim = len(Kd)
    rdt, T, pre, hs, tm = _setup(h_list, tm, ndim)
    cdt = np.result_type(rdt, np.complex64)
    Kprod = int(np.prod(Kd))
    ck = np.asarray(ck, dtype=cdt).reshape((Kprod, -1), order="F")
    M, N = tm.shape[0], ck.shape[1]
    fn = getattr(lib, "%s_interp%d_table1_real_forward" % (pre, ndim))
    out = np.empty((M, N), dtype=cdt, order="F")
    fr = np.empty(M, dtype=rdt)
    fi = np.empty(M, dtype=rdt)
    for n in range(N):
        r = np.ascontiguousarray(ck[:, n].real)
        i = np.ascontiguousarray(ck[:, n].imag)
        fn(_ptr(r, T), _ptr(i, T), *[int(k) for k in Kd], *[_ptr(h, T) for h in hs],
           *[int(j) for j in Jd], int(L), _ptr(tm, T), M, _ptr(fr, T), _ptr(fi, T))
        out[:, n].real = fr
        out[:, n].imag = fi
    return out


def interp_adjoint(fm, h_list, Jd, L, tm, Kd):
    """Samples ``[M, N]`` -> grid ``[prod(Kd), N]`` (Fortran) through the
    reference's ``*_interp{d}_table1_real_adj`` with all N repetitions."""
    lib = _load()
    ndim = len(Kd)
    rdt, T, pre, hs, tm = _setup(h_list, tm, ndim)
    cdt = np.result_type(rdt, np.complex64)
    Kprod = int(np.prod(Kd))
    M = tm.shape[0]
    fm = np.asarray(fm, dtype=cdt).reshape((M, -1), order="F")
    N = fm.shape[1]
    fr = np.asfortranarray(fm.real)
    fi = np.asfortranarray(fm.imag)
    ckr = np.zeros((Kprod, N), dtype=rdt, order="F")
    cki = np.zeros((Kprod, N), dtype=rdt, order="F")
    fn = getattr(lib, "%s_interp%d_table1_real_adj" % (pre, ndim))
    fn(_ptr(ckr, T), _ptr(cki, T), *[int(k) for k in Kd], *[_ptr(h, T) for h in hs],
       *[int(j) for j in Jd], int(L), _ptr(tm, T), M, _ptr(fr, T), _ptr(fi, T), N)
    out = np.empty((Kprod, N), dtype=cdt, order="F")
    out.real = ckr
    out.imag = cki
    return out
