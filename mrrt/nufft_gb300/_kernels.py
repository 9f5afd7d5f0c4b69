"""Interpolation kernel objects and lookup tables (plan-time host math).

The classes keep the reference's public names and constructor arguments
(mrrt/nufft/_kernels.py:14-162): ``NufftKernelBase``, ``KaiserBesselKernel``
and ``BeattyKernel`` (Kaiser-Bessel with the shape parameter of Beatty et al.,
IEEE TMI 24(6):799-808, 2005, eq. 5).

``kernel_table`` builds the per-axis lookup table the interpolation kernels
read: ``J*L + 1`` samples of the kernel at ``t0 = (i - J L / 2) / L``.  The
reference derives the same table from columns of a sparse interpolation
matrix (mrrt/nufft/_nufft.py:1195-1271); sampling the closed form directly is
equivalent (for phasing ``'complex'`` the kernel carries the phase
``exp(-i (2 pi / K) (N-1)/2 t)``) and is evaluated here in float64.
"""
import functools
from abc import ABC, abstractmethod
from math import pi, sqrt

import numpy as np

from ._kaiser_bessel import kaiser_bessel, kaiser_bessel_deriv

__all__ = ["BeattyKernel", "KaiserBesselKernel", "NufftKernelBase", "kernel_table",
           "kernel_deriv_table", "beatty_alpha"]


def _as_1d_ints(arr, n=None):
    arr = np.atleast_1d(np.squeeze(np.asarray(arr)))
    if arr.ndim > 1:
        raise ValueError("arr must be scalar or 1d")
    if not issubclass(arr.dtype.type, np.integer):
        if not np.all(np.mod(arr, 1) == 0):
            raise ValueError("arr contains non-integer values")
    if n is not None and arr.size != n:
        if arr.size == 1:
            arr = np.asarray([arr[0]] * n)
        else:
            raise ValueError("array did not have the expected size of {}".format(n))
    return arr.astype(np.intp)


def beatty_alpha(J, K, N):
    """Beatty KB shape: pi * sqrt(J^2 / r^2 * (r - 1/2)^2 - 0.8), r = K / N."""
    r = K / N
    return pi * sqrt(J ** 2 / r ** 2 * (r - 0.5) ** 2 - 0.8)


class NufftKernelBase(ABC):
    shape = ()
    kernels = []
    kernel_type = ""
    params = {}

    @abstractmethod
    def __init__(self):
        pass

    @property
    def ndim(self):
        return len(self.shape)

    @abstractmethod
    def _initialize_kernel(self, *args):
        """Set ``self.kernels``: one 1-D callable per axis of ``self.shape``."""

    def __str__(self):
        return "kernel type: {}\nkernel shape: {}\n".format(self.kernel_type, self.shape)


class KaiserBesselKernel(NufftKernelBase):
    """Separable KB kernel with user shape parameters ``alpha`` and order ``m``."""

    is_kaiser_scale = None

    def __init__(self, shape, alpha=None, m=None):
        self.kernel_type = "kb:user"
        self.params = {}
        if np.isscalar(shape):
            shape = (shape,)
        self.shape = tuple(shape)
        alpha = _as_1d_ints(alpha, self.ndim)
        m = _as_1d_ints(m, self.ndim)
        self.kernels = self._initialize_kernel(alpha, m)

    def _initialize_kernel(self, alpha, m):
        self.is_kaiser_scale = True
        if m is None or alpha is None:
            raise ValueError("kwargs must contain shape, m, alpha for %s case" % self.kernel_type)
        self.alpha = alpha
        self.m = m
        return [functools.partial(kaiser_bessel, J=j, alpha=a, m=mm)
                for j, a, mm in zip(self.shape, alpha, m)]


class BeattyKernel(KaiserBesselKernel):
    """KB kernel whose shape parameter follows Beatty et al. for the given
    grid (``grid_shape`` = Nd) and oversampled grid (``os_grid_shape`` = Kd)."""

    def __init__(self, shape, grid_shape, os_grid_shape):
        self.kernel_type = "kb:beatty"
        if np.isscalar(shape):
            shape = (shape,)
        self.shape = tuple(shape)
        self.grid_shape = _as_1d_ints(grid_shape, self.ndim)
        self.os_grid_shape = _as_1d_ints(os_grid_shape, self.ndim)
        self.is_kaiser_scale = True
        alpha = [beatty_alpha(j, k, n) for j, k, n in
                 zip(self.shape, self.os_grid_shape, self.grid_shape)]
        self.kernels = super()._initialize_kernel(alpha, [0] * self.ndim)


def table_points(J, L):
    """t0 = arange(-J L / 2, J L / 2 + 1) / L (length J*L + 1)."""
    return np.arange(-J * L / 2.0, J * L / 2.0 + 1) / L


def kernel_table(N, J, K, L, phasing="real", dtype=np.float32):
    """Lookup table of one axis, ``J*L + 1`` entries, cast to ``dtype``
    (real dtype for phasing 'real', complex dtype for 'complex')."""
    t0 = table_points(J, L)
    h = kaiser_bessel(t0, J=J, alpha=beatty_alpha(J, K, N), m=0)
    if phasing == "complex":
        h = h * np.exp(-1j * (2 * pi / K) * (N - 1) / 2.0 * t0)
    elif phasing != "real":
        raise ValueError("phasing must be 'real' or 'complex'")
    return h.astype(dtype)


def kernel_deriv_table(N, J, K, L, dtype=np.float32):
    """Table of the analytic derivative dh/dt on the same points (phasing 'real')."""
    t0 = table_points(J, L)
    return kaiser_bessel_deriv(t0, J=J, alpha=beatty_alpha(J, K, N)).astype(dtype)
