"""Oracle: numpy restatement of the reference table-mode NUFFT (test infrastructure).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU legs use
this module, as the checker and as the timed CPU baseline.  The product
package never imports it.

Every function restates the reference algorithm it names (file:line within
the reference project) with the same numpy dtypes, so that float32 rounding
follows the reference.  The interpolation itself runs in the project's C
restatement ``nufft_table_oracle.cpp`` (built by ``oracle/Makefile`` into
``liboracle_nufft.so``), called through ctypes.

Parity pin: ``tests/test_oracle_golden.py`` checks this module against golden
vectors produced by the reference package itself (``tests/golden/make_golden.py``).
"""
import ctypes
import functools
import math
import os
import subprocess
import threading

import numpy as np
import scipy.sparse
from scipy.special import i0, iv, j0, jv

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(HERE, "liboracle_nufft.so")
_lib = None
_lib_lock = threading.Lock()


def build_oracle(force=False):
    """Compile ``liboracle_nufft.so`` (g++, OpenMP, the reference's -ffast-math;
    the same command as ``oracle/Makefile``'s default target)."""
    src = os.path.join(HERE, "nufft_table_oracle.cpp")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        tmp = _LIB_PATH + ".%d.tmp" % os.getpid()
        subprocess.run(["g++", "-O2", "-ffast-math", "-fopenmp", "-fPIC", "-shared", "-o", tmp, src],
                       check=True)
        os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def _load():
    global _lib
    with _lib_lock:
        if _lib is None:
            build_oracle()
            lib = ctypes.CDLL(_LIB_PATH)
            for name, T in (("f32", ctypes.c_float), ("f64", ctypes.c_double)):
                P = ctypes.POINTER(T)
                PP = ctypes.POINTER(P)
                for kind in ("forward", "adjoint"):
                    fn = getattr(lib, "oracle_interp_%s_%s" % (kind, name))
                    fn.restype = ctypes.c_int
                    fn.argtypes = [
                        ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                        ctypes.c_int, PP, PP, P, ctypes.c_int64, P, P, ctypes.c_int, P, P,
                    ]
            _lib = lib
    return _lib


# --------------------------------------------------------------------------
# plan-time kernel math
# --------------------------------------------------------------------------


def beatty_alpha(J, K, N):
    """Beatty et al. KB shape parameter (mrrt/nufft/_kernels.py:342-345)."""
    k_n = K / N
    return np.pi * math.sqrt(J ** 2 / k_n ** 2 * (k_n - 0.5) ** 2 - 0.8)


def kaiser_bessel(x, J=6, alpha=None, m=0):
    """Generalised KB function on [-J/2, J/2] (mrrt/nufft/_kaiser_bessel.py:78-149)."""
    x = np.asarray(x)
    if alpha is None:
        alpha = 2.34 * J
    m_bi = abs(m)
    ii = (2 * np.abs(x) < J).nonzero()
    tmp = 2 * x[ii] / J
    tmp *= tmp
    f = np.sqrt(1 - tmp)
    denom = iv(m_bi, alpha) if m_bi != 0 else i0(alpha)
    kb = np.zeros_like(x)
    if m_bi != 0:
        kb[ii] = (f ** m * iv(m_bi, alpha * f)) / float(denom)
    else:
        kb[ii] = i0(alpha * f) / float(denom)
    return kb.real


def kaiser_bessel_ft(u, J=6, alpha=None, m=0, d=1):
    """Fourier transform of the KB function (mrrt/nufft/_kaiser_bessel.py:153-226)."""
    u = np.asarray(u)
    if not alpha:
        alpha = 2.34 * J
    tmp = (np.pi * J) * u
    tmp *= tmp
    tmp -= alpha * alpha
    z = np.lib.scimath.sqrt(tmp)
    nu = d / 2.0 + m
    const1 = (2 * np.pi) ** (d / 2.0) * (J / 2.0) ** d * alpha ** m
    const1 /= i0(alpha) if m == 0 else iv(m, alpha)
    if nu == 0:
        y = const1 * j0(z)
        y /= z
    else:
        y = const1 * jv(nu, z)
        y /= z ** nu
    y = y.real
    return y


def nufft_offset(om, J, K):
    """Leftmost neighbour offset (mrrt/nufft/_utils.py:20-43)."""
    gam = 2 * np.pi / K
    return np.floor(om / gam - J / 2.0)


def nufft_coef(om, J, K, kernel):
    """Interpolation coefficients [J, M] and their arguments (mrrt/nufft/_utils.py:46-86)."""
    om = np.atleast_1d(np.squeeze(om))
    gam = 2 * np.pi / K
    dk = om / gam - nufft_offset(om, J, K)
    arg = -np.arange(1, J + 1)[:, None] + dk[None, :]
    return kernel(arg), arg


def _dtypes(precision):
    if precision == "single":
        return np.dtype(np.float32), np.dtype(np.complex64)
    if precision == "double":
        return np.dtype(np.float64), np.dtype(np.complex128)
    raise ValueError("precision must be 'single' or 'double'")


def sparse_interp_matrix(omega, Nd, Jd, Kd, alphas, n_shift, phasing, precision):
    """COO->CSC interpolation matrix [M, prod(Kd)] (mrrt/nufft/_nufft.py:751-877).

    ``omega`` must already carry the operator's real dtype, as in the reference
    (the constructor casts it before building the matrix).
    """
    rdt, cdt = _dtypes(precision)
    ndim = len(Nd)
    M = omega.shape[0]
    kd, ud = [], []
    for d in range(ndim):
        N, J, K = Nd[d], Jd[d], Kd[d]
        kern = functools.partial(kaiser_bessel, J=J, alpha=alphas[d], m=0)
        c, arg = nufft_coef(omega[:, d], J, K, kern)
        koff = nufft_offset(omega[:, d], J, K)
        kd.append(np.mod(np.arange(1, J + 1)[:, None] + koff[None, :], K))
        if phasing == "complex":
            gam = 2 * np.pi / K
            phase = np.exp(1j * gam * (N - 1) / 2.0 * arg)
        else:
            phase = 1.0
        ud.append(phase * c)
    kk, uu = kd[0], ud[0]
    for d in range(1, ndim):
        Jprod = int(np.prod(Jd[: d + 1]))
        tmp = kd[d] * int(np.prod(Kd[:d]))
        kk = (kk.reshape(kk.shape[0], 1, M) + tmp.reshape(1, tmp.shape[0], M)).reshape((Jprod, M), order="F")
        uu = (uu.reshape(uu.shape[0], 1, M) * ud[d].reshape(1, ud[d].shape[0], M)).reshape((Jprod, M), order="F")
    if np.iscomplexobj(uu):
        uu = uu.conj()
    if phasing == "complex":
        if any(s != 0 for s in n_shift):
            uu = uu * np.exp(1j * np.dot(omega, np.asarray(n_shift))).reshape((1, -1), order="F")
        sdt = cdt
    else:
        sdt = rdt
    mm = np.tile(np.arange(M), (int(np.prod(Jd)), 1))
    p = scipy.sparse.coo_matrix(
        (uu.ravel(order="F"), (mm.ravel(order="F"), kk.ravel(order="F"))),
        shape=(M, int(np.prod(Kd))),
        dtype=sdt,
    )
    return p.tocsc()


def table_make1(N, J, K, L, phasing):
    """Kernel lookup table of length J*L+1 via the reference's "fast" method
    (mrrt/nufft/_nufft.py:1195-1271): J columns of the sparse matrix of a dummy
    1-D single-precision operator sampled at L offsets."""
    t0 = np.arange(-J * L / 2.0, J * L / 2.0 + 1) / L
    if N % 2 == 0:
        t1 = J / 2.0 - 1 + np.arange(L) / L
    else:
        t1 = J / 2.0 - 1 + np.arange(1, L + 1) / L
    omega1 = (t1 * 2 * np.pi / K)[:, None].astype(np.float32)
    n_mid = (N // 2,) if phasing == "real" else ((N - 1) / 2.0,)
    p = sparse_interp_matrix(
        omega1, (N,), (J,), (K,), [beatty_alpha(J, K, N)], (0.0,), phasing, "single"
    )
    del n_mid
    h = np.asarray(p[:, np.arange(J - 1, -1, -1)].todense()).ravel(order="F")
    if N % 2 == 0:
        h = np.concatenate((h, np.atleast_1d(h[0])), axis=0)
    else:
        h = np.concatenate((np.atleast_1d(h[-1]), h), axis=0)
    return h, t0


# --------------------------------------------------------------------------
# table interpolation through the C restatement
# --------------------------------------------------------------------------


def _ptr(a, T):
    return a.ctypes.data_as(ctypes.POINTER(T))


def _tables(h_list, rdt):
    T = ctypes.c_float if rdt == np.float32 else ctypes.c_double
    hr = [np.ascontiguousarray(np.real(h), dtype=rdt) for h in h_list]
    cplx = any(np.iscomplexobj(h) for h in h_list)
    hi = [np.ascontiguousarray(np.imag(h), dtype=rdt) for h in h_list] if cplx else None
    keep = hr + (hi or [])
    PP = ctypes.POINTER(T) * 3
    hr_arr = PP(*[_ptr(h, T) for h in hr] + [None] * (3 - len(hr)))
    hi_arr = PP(*[_ptr(h, T) for h in hi] + [None] * (3 - len(hi))) if cplx else None
    return T, hr_arr, hi_arr, keep


def interp_forward(ck, h_list, Jd, L, tm, Kd):
    """interp{1,2,3}_table (mrrt/nufft/_interp_table.py:26-159): grid [prod(Kd), N]
    (or [*Kd, N], Fortran order) -> samples [M, N]."""
    lib = _load()
    rdt = np.result_type(*[np.real(h).dtype for h in h_list])
    cdt = np.result_type(rdt, np.complex64)
    ndim = len(Kd)
    Kprod = int(np.prod(Kd))
    ck = np.asarray(ck, dtype=cdt).reshape((Kprod, -1), order="F")
    N = ck.shape[1]
    tm = np.asfortranarray(np.asarray(tm, dtype=rdt).reshape((-1, ndim)))
    M = tm.shape[0]
    T, hr, hi, keep = _tables(h_list, rdt)
    ckr = np.asfortranarray(ck.real)
    cki = np.asfortranarray(ck.imag)
    fr = np.zeros((M, N), dtype=rdt, order="F")
    fi = np.zeros((M, N), dtype=rdt, order="F")
    Ka = (ctypes.c_int * 3)(*Kd)
    Ja = (ctypes.c_int * 3)(*Jd)
    fn = lib.oracle_interp_forward_f32 if rdt == np.float32 else lib.oracle_interp_forward_f64
    rc = fn(ndim, Ka, Ja, int(L), hr, hi, _ptr(tm, T), M, _ptr(ckr, T), _ptr(cki, T), N,
            _ptr(fr, T), _ptr(fi, T))
    if rc != 0:
        raise ValueError("oracle forward interpolation rejected its arguments")
    del keep
    out = np.empty((M, N), dtype=cdt, order="F")
    out.real = fr
    out.imag = fi
    return out


def interp_adjoint(fm, h_list, Jd, L, tm, Kd):
    """interp{1,2,3}_table_adj (mrrt/nufft/_interp_table.py:46-191): samples
    [M, N] -> grid [prod(Kd), N] (Fortran order)."""
    lib = _load()
    rdt = np.result_type(*[np.real(h).dtype for h in h_list])
    cdt = np.result_type(rdt, np.complex64)
    ndim = len(Kd)
    Kprod = int(np.prod(Kd))
    tm = np.asfortranarray(np.asarray(tm, dtype=rdt).reshape((-1, ndim)))
    M = tm.shape[0]
    fm = np.asarray(fm, dtype=cdt).reshape((M, -1), order="F")
    N = fm.shape[1]
    T, hr, hi, keep = _tables(h_list, rdt)
    fr = np.asfortranarray(fm.real)
    fi = np.asfortranarray(fm.imag)
    ckr = np.zeros((Kprod, N), dtype=rdt, order="F")
    cki = np.zeros((Kprod, N), dtype=rdt, order="F")
    Ka = (ctypes.c_int * 3)(*Kd)
    Ja = (ctypes.c_int * 3)(*Jd)
    fn = lib.oracle_interp_adjoint_f32 if rdt == np.float32 else lib.oracle_interp_adjoint_f64
    rc = fn(ndim, Ka, Ja, int(L), hr, hi, _ptr(tm, T), M, _ptr(fr, T), _ptr(fi, T), N,
            _ptr(ckr, T), _ptr(cki, T))
    if rc != 0:
        raise ValueError("oracle adjoint interpolation rejected its arguments")
    del keep
    out = np.empty((Kprod, N), dtype=cdt, order="F")
    out.real = ckr
    out.imag = cki
    return out


# --------------------------------------------------------------------------
# operator: construction and transforms
# --------------------------------------------------------------------------


def _as_tuple(seq, type=int, n=None):
    if np.isscalar(seq):
        return (type(seq),) * n
    if n is not None and len(seq) != n:
        raise ValueError("array did not have the expected size of {}".format(n))
    return tuple(type(s) for s in seq)


class OracleNufft:
    """Restatement of ``NufftBase`` in table (and sparse) mode
    (mrrt/nufft/_nufft.py:216-360, 425-482), CPU only."""

    def __init__(self, Nd, omega, Jd=4, Kd=None, precision="single", mode="table", Ld=1024,
                 ortho=False, n_shift=None, phasing="real", adjoint_scalefactor=1.0, order="F",
                 interp=None):
        # interp: a module with interp_forward / interp_adjoint of this
        # module's signatures (``oracle.refc`` runs the reference's own
        # compiled kernels); None uses the C restatement
        self._interp_fwd = interp.interp_forward if interp is not None else interp_forward
        self._interp_adj = interp.interp_adjoint if interp is not None else interp_adjoint
        if np.isscalar(Nd):
            Nd = (Nd,)
        self.Nd = _as_tuple(Nd)
        self.ndim = len(self.Nd)
        self.Jd = _as_tuple(Jd, n=self.ndim)
        if Kd is None:
            Kd = tuple(int(1.5 * n) for n in self.Nd)
        self.Kd = _as_tuple(Kd, n=self.ndim)
        self.Ld = int(Ld)
        self.mode = mode
        self.order = order
        self.phasing = phasing
        self.ortho = ortho
        self.scale_ortho = math.sqrt(math.prod(self.Kd)) if ortho else 1
        self.adjoint_scalefactor = adjoint_scalefactor
        omega = np.asarray(omega)
        if omega.ndim == 1:
            omega = omega[:, None]
        if omega.shape[1] != self.ndim:
            raise ValueError("number of cols must match NUFFT dimension")
        if omega.dtype not in (np.float32, np.float64):
            raise ValueError("omega must be float32 or float64")
        if precision == "auto":
            precision = "single" if omega.dtype == np.float32 else "double"
        self.precision = precision
        rdt, cdt = _dtypes(precision)
        self._real_dtype, self._cplx_dtype = rdt, cdt
        self.n_shift = (0.0,) * self.ndim if n_shift is None else _as_tuple(n_shift, float, self.ndim)
        if phasing == "real":
            self.n_mid = tuple(n // 2 for n in self.Nd)
        elif phasing == "complex":
            self.n_mid = tuple((n - 1) / 2.0 for n in self.Nd)
        else:
            raise ValueError("phasing must be 'real' or 'complex'")
        self.alpha = [beatty_alpha(j, k, n) for j, k, n in zip(self.Jd, self.Kd, self.Nd)]
        # deapodisation, computed in float64 then cast (_nufft.py:727-748, 654-678)
        sn = np.array([1.0])
        for d in range(self.ndim):
            nc = np.arange(-self.n_mid[d], -self.n_mid[d] + self.Nd[d])
            tmp = 1 / kaiser_bessel_ft(nc / self.Kd[d], self.Jd[d], self.alpha[d], 0, 1)
            sn = np.outer(sn.ravel(), tmp.conj())
        self.sn = sn.reshape(self.Nd).astype(rdt)
        # phases (_nufft.py:703-724); phase_after uses omega in its given dtype
        if phasing == "real":
            phase = (2 * np.pi / self.Kd[0] * self.n_mid[0]) * np.arange(self.Kd[0], dtype=rdt)
            for d in range(1, self.ndim):
                tmp = (2 * np.pi / self.Kd[d] * self.n_mid[d]) * np.arange(self.Kd[d], dtype=rdt)
                phase = phase.reshape(phase.shape + (1,)) + tmp.reshape((1,) * d + (tmp.size,))
            self.phase_before = np.exp(1j * phase).astype(cdt, copy=False)
            shift_vec = [(s - m) for s, m in zip(self.n_shift, self.n_mid)]
            self.phase_after = np.exp(1j * np.dot(omega, np.asarray(shift_vec, dtype=rdt))).astype(cdt, copy=False)
        else:
            self.phase_before = None
            self.phase_after = None
        self.omega = np.asfortranarray(omega.astype(rdt))
        self.M = self.omega.shape[0]
        if mode == "sparse":
            self.p = sparse_interp_matrix(self.omega, self.Nd, self.Jd, self.Kd, self.alpha,
                                          self.n_shift, phasing, precision)
            self.h = None
            self.tm = None
        elif mode == "table":
            self.p = None
            self.h = []
            for d in range(self.ndim):
                h, _ = table_make1(self.Nd[d], self.Jd[d], self.Kd[d], self.Ld, phasing)
                if phasing == "complex":
                    h = h.astype(cdt)
                else:
                    h = np.real(h).astype(rdt)
                self.h.append(h)
            tm = np.zeros_like(self.omega)
            for d in range(self.ndim):
                gam = 2 * np.pi / self.Kd[d]
                tm[:, d] = self.omega[:, d] / gam
            self.tm = tm
        else:
            raise ValueError("Invalid NUFFT mode: {}".format(mode))
        if phasing == "complex" and any(s != 0 for s in self.n_shift):
            self.phase_shift = np.exp(1j * np.dot(self.omega, np.asarray(self.n_shift))).astype(cdt)
        else:
            self.phase_shift = None
        self.nargin1 = math.prod(self.Nd)
        self.nargout1 = self.M

    # reps axis handling for order='C' (_nufft.py:415-423)
    def _swap(self, x, narg):
        if x.size != narg:
            x = x.transpose(tuple(range(1, x.ndim)) + (0,))
        return x

    def _unswap(self, x, narg):
        if x.size != narg:
            x = x.transpose((x.ndim - 1,) + tuple(range(x.ndim - 1)))
        return x

    def fft(self, x):
        if self.order == "C":
            x = self._swap(x, self.nargin1)
        y = self._forward(x)
        if self.order == "C":
            y = self._unswap(y, self.nargout1)
        return y

    def adj(self, y):
        if self.order == "C":
            y = self._swap(y, self.nargout1)
        x = self._adjoint(y)
        if self.order == "C":
            x = self._unswap(x, self.nargin1)
        return x

    def _forward(self, x):
        """nufft_forward (mrrt/nufft/_nufft.py:1275-1397)."""
        Nd, Kd = self.Nd, self.Kd
        x = np.asfortranarray(x).reshape(list(Nd) + [-1], order="F")
        x = x.astype(self._cplx_dtype, copy=False)
        n_reps = x.shape[-1]
        xk = x * self.sn[..., None]
        xk = np.fft.fftn(xk, s=Kd, axes=tuple(range(x.ndim - 1)))
        if self.phase_before is not None:
            xk *= self.phase_before[..., None]
        xk = xk.reshape((math.prod(Kd), n_reps), order="F")
        if self.ortho:
            xk /= self.scale_ortho
        if self.mode == "table":
            y = self._interp_fwd(xk, self.h, self.Jd, self.Ld, self.tm, self.Kd)
            if self.phase_shift is not None:
                y *= self.phase_shift[:, None]
            y = y.astype(xk.dtype, copy=False)
        else:
            y = self.p * xk
        y = np.reshape(y, (self.M, n_reps), order="F")
        if self.phase_after is not None:
            y *= self.phase_after[:, None]
        if n_reps == 1:
            y = y[..., 0]
        return y

    def _adjoint(self, y):
        """nufft_adj (mrrt/nufft/_nufft.py:1459-1578)."""
        Nd, Kd = self.Nd, self.Kd
        y = np.asfortranarray(y)
        if y.size % self.M != 0:
            raise ValueError("invalid size")
        xk = y.astype(self._cplx_dtype, copy=False).reshape((self.M, -1), order="F").copy(order="F")
        n_reps = xk.shape[-1]
        if self.phase_after is not None:
            xk *= self.phase_after.conj()[:, None]
        if self.mode == "table":
            if self.phase_shift is not None:
                xk *= self.phase_shift.conj()[:, None]
            xk_all = self._interp_adj(xk, self.h, self.Jd, self.Ld, self.tm, self.Kd)
        else:
            xk_all = self.p.conj().T * xk
        xk_all = xk_all.reshape(Kd + (n_reps,), order="F")
        if self.phase_before is not None:
            xk_all *= self.phase_before.conj()[..., None]
        x = np.fft.ifftn(xk_all, s=Kd, axes=tuple(range(xk_all.ndim - 1)))
        x = x[tuple([slice(d) for d in Nd] + [slice(None)])]
        if self.ortho:
            x *= self.scale_ortho * self.adjoint_scalefactor
        else:
            x *= math.prod(Kd) * self.adjoint_scalefactor
        x *= np.conj(self.sn)[..., None]
        if n_reps == 1:
            x = x[..., 0]
        return x


# --------------------------------------------------------------------------
# FP64 direct NUDFT (mrrt/nufft/_dtft.py:16-216), chunked and separable
# --------------------------------------------------------------------------


def _factors(omega, Nd, n_shift, sign, rows):
    out = []
    for d in range(len(Nd)):
        n = np.arange(Nd[d], dtype=np.float64) - float(n_shift[d])
        out.append(np.exp(sign * 1j * np.outer(omega[rows, d].astype(np.float64), n)))
    return out


def dtft(x, omega, Nd, n_shift=None, rows=None, chunk=4096):
    """Exact forward NUDFT y[m] = sum_n x[n] exp(-i omega_m . (n - n_shift)).

    ``x`` is one image (Fortran axis order, shape Nd) or [*Nd, reps].
    ``rows`` optionally restricts the samples evaluated.
    """
    Nd = tuple(Nd)
    ndim = len(Nd)
    omega = np.asarray(omega, dtype=np.float64).reshape(-1, ndim)
    n_shift = (0.0,) * ndim if n_shift is None else tuple(np.broadcast_to(n_shift, (ndim,)))
    x = np.asarray(x, dtype=np.complex128).reshape(Nd + (-1,), order="F")
    reps = x.shape[-1]
    rows = np.arange(omega.shape[0]) if rows is None else np.asarray(rows)
    out = np.empty((rows.size, reps), dtype=np.complex128)
    for s in range(0, rows.size, chunk):
        r = rows[s:s + chunk]
        E = _factors(omega, Nd, n_shift, -1.0, r)
        if ndim == 1:
            out[s:s + r.size] = E[0] @ x
        elif ndim == 2:
            for c in range(reps):
                t = E[0] @ x[:, :, c]
                out[s:s + r.size, c] = np.sum(t * E[1], axis=1)
        else:
            for c in range(reps):
                t = np.einsum("ma,abc->mbc", E[0], x[:, :, :, c], optimize=True)
                t = np.einsum("mbc,mb->mc", t, E[1], optimize=True)
                out[s:s + r.size, c] = np.sum(t * E[2], axis=1)
    return out[:, 0] if reps == 1 else out


def dtft_adj(y, omega, Nd, n_shift=None, chunk=4096):
    """Exact adjoint NUDFT x[n] = sum_m y[m] exp(+i omega_m . (n - n_shift))."""
    Nd = tuple(Nd)
    ndim = len(Nd)
    omega = np.asarray(omega, dtype=np.float64).reshape(-1, ndim)
    n_shift = (0.0,) * ndim if n_shift is None else tuple(np.broadcast_to(n_shift, (ndim,)))
    M = omega.shape[0]
    y = np.asarray(y, dtype=np.complex128).reshape((M, -1), order="F")
    reps = y.shape[1]
    x = np.zeros(Nd + (reps,), dtype=np.complex128, order="F")
    for s in range(0, M, chunk):
        r = np.arange(s, min(M, s + chunk))
        E = _factors(omega, Nd, n_shift, 1.0, r)
        for c in range(reps):
            v = y[r, c]
            if ndim == 1:
                x[:, c] += E[0].T @ v
            elif ndim == 2:
                x[:, :, c] += (E[0] * v[:, None]).T @ E[1]
            else:
                t = np.einsum("ma,mb->mab", E[0] * v[:, None], E[1], optimize=True)
                x[:, :, :, c] += np.einsum("mab,mc->abc", t, E[2], optimize=True)
    return x[..., 0] if reps == 1 else x


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))
