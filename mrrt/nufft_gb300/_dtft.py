"""Exact direct NUDFT (double precision, on the GPU).

Same names and argument meaning as the reference's validation transforms
(mrrt/nufft/_dtft.py:16-216):

    dtft(x, omega, shape, n_shift)      y[m] = sum_n x[n] exp(-i omega_m . (n - n_shift))
    dtft_adj(xk, omega, shape, n_shift) x[n] = sum_m xk[m] exp(+i omega_m . (n - n_shift))

Images use the reference's Fortran axis convention (``omega[:, d]`` pairs with
image axis ``d``); extra trailing axes are repetitions.  The sums run in
libgbnufft's FP64 kernels; numpy input gives numpy output, torch input gives
a torch tensor on the input's device.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from ._plan import _stream, require_cuda

__all__ = ["dtft", "dtft_adj"]


def _prep(omega, shape, n_shift):
    om = omega.detach().cpu().numpy() if isinstance(omega, torch.Tensor) else np.asarray(omega)
    if om.ndim == 1:
        om = om[:, None]
    if om.ndim != 2:
        raise ValueError("omega must be 2d")
    dd = om.shape[1]
    if dd > 3:
        raise NotImplementedError("dimensions > 3 not implemented")
    shape = tuple(int(s) for s in np.atleast_1d(shape))
    if len(shape) != dd:
        raise ValueError("length of shape must match number of columns in omega")
    if n_shift is None:
        n_shift = (0.0,) * dd
    n_shift = np.broadcast_to(np.atleast_1d(np.squeeze(np.asarray(n_shift, dtype=np.float64))), (dd,))
    return om.astype(np.float64), shape, n_shift


def _run(adjoint, data, omega, shape, n_shift):
    require_cuda()
    lib = _lib.load()
    om, shape, n_shift = _prep(omega, shape, n_shift)
    M, dd = om.shape
    is_torch = isinstance(data, torch.Tensor)
    dev = data.device if is_torch and data.is_cuda else torch.device("cuda")
    if is_torch:
        arr = data.detach().to(dev, torch.complex128)
        # Fortran convention: leading axes are the image (or sample) axes
        lead = (M,) if adjoint else shape
        nlead = len(lead)
        n = int(np.prod(lead))
        reps = arr.numel() // n
        arr = arr.reshape(lead + (reps,)).permute(*reversed(range(nlead + 1))).contiguous()
    else:
        a = np.asarray(data).astype(np.complex128)
        lead = (M,) if adjoint else shape
        n = int(np.prod(lead))
        reps = a.size // n
        a = np.asfortranarray(a.reshape(lead + (reps,), order="F"))
        arr = torch.from_numpy(a.ravel(order="F")).to(dev)
    om_t = torch.from_numpy(np.ascontiguousarray(om)).to(dev)
    nout = int(np.prod(shape)) if adjoint else M
    out = torch.empty((reps, nout), dtype=torch.complex128, device=dev)
    Nd = (ctypes.c_int * 3)(*list(shape) + [1] * (3 - dd))
    sh = (ctypes.c_double * 3)(*[float(s) for s in n_shift] + [0.0] * (3 - dd))
    fn = lib.gbn_dtft_adjoint if adjoint else lib.gbn_dtft_forward
    with torch.cuda.device(dev):
        _lib.check(fn(dd, Nd, sh, ctypes.c_void_p(om_t.data_ptr()), M,
                      ctypes.c_void_p(arr.data_ptr()), ctypes.c_void_p(out.data_ptr()), reps,
                      _stream()))
    lead_out = shape if adjoint else (M,)
    out = out.reshape((reps,) + tuple(reversed(lead_out)))
    out = out.permute(*reversed(range(len(lead_out) + 1)))
    if not is_torch:
        out = out.cpu().numpy()
    if reps == 1:
        out = out[..., 0]
    return out


def dtft(x, omega, shape=None, n_shift=None, useloop=False, xp=None):
    """Exact forward NUDFT of ``x`` (image ``shape`` [+ reps]) at ``omega``."""
    if shape is None:
        dd = np.asarray(omega.shape)[1] if not isinstance(omega, torch.Tensor) else omega.shape[1]
        shape = tuple(x.shape[:dd])
    return _run(False, x, omega, shape, n_shift)


def dtft_adj(xk, omega, shape=None, n_shift=None, useloop=False, xp=None):
    """Exact adjoint NUDFT of samples ``xk`` ([M] or [M, reps]) onto ``shape``."""
    if shape is None:
        raise ValueError("shape must be specified")
    return _run(True, xk, omega, shape, n_shift)
