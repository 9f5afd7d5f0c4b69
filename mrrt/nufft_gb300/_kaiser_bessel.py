"""Kaiser-Bessel interpolation kernel, its Fourier transform and its derivative.

Plan-time host math in float64 (numpy / scipy).  The functions keep the
reference's names and argument meaning (mrrt/nufft/_kaiser_bessel.py:78-226):

* ``kaiser_bessel(x, J, alpha, m)``: generalised KB function on (-J/2, J/2),
  zero outside (Lewitt 1990, eq. A1);
* ``kaiser_bessel_ft(u, J, alpha, m, d)``: its d-dimensional Fourier
  transform (Lewitt 1990, eq. A3), used for the deapodisation ``sn``;
* ``kaiser_bessel_deriv(x, J, alpha)``: the analytic derivative d/dx of the
  order-0 KB function, used by the trajectory gradient (no counterpart in the
  reference).
"""
import warnings

import numpy as np
from scipy.special import i0, i1, iv, j0, jv

__all__ = ["kaiser_bessel", "kaiser_bessel_ft", "kaiser_bessel_deriv"]


def kaiser_bessel(x=None, J=6, alpha=None, m=0, K_N=None):
    """Generalised Kaiser-Bessel function for x in the support (-J/2, J/2).

    ``f(x) = s^m I_m(alpha s) / I_m(alpha)``, ``s = sqrt(1 - (2x/J)^2)``,
    and 0 for ``|x| >= J/2``.  Negative non-integer ``m`` uses ``|m|`` in the
    Bessel order, as the reference does.
    """
    x = np.asarray(x)
    if alpha is None:
        alpha = 2.34 * J
    if m < 0 and abs(round(m) - m) > np.finfo(float).eps:
        warnings.warn("Negative NonInt m=%g: using modified definition of KB function" % m)
    mb = abs(m)
    inside = 2 * np.abs(x) < J
    s2 = 1 - (2 * x[inside] / J) ** 2
    s = np.sqrt(s2)
    out = np.zeros_like(x)
    if mb != 0:
        out[inside] = (s ** m * iv(mb, alpha * s)) / float(iv(mb, alpha))
    else:
        out[inside] = i0(alpha * s) / float(i0(alpha))
    return out.real


def kaiser_bessel_ft(u, J=6, alpha=None, m=0, d=1):
    """Fourier transform of the generalised KB function in dimension d.

    ``F(u) = (2 pi)^(d/2) (J/2)^d alpha^m / I_m(alpha) * J_nu(z) / z^nu`` with
    ``z = sqrt((pi J u)^2 - alpha^2)`` (complex for small u) and
    ``nu = d/2 + m``.
    """
    u = np.asarray(u, dtype=np.float64)
    if not alpha:
        alpha = 2.34 * J
    if m < -1:
        warnings.warn("m=%g < -1 in kaiser_bessel_ft: validity of FT formula uncertain" % m)
    z = np.lib.scimath.sqrt((np.pi * J * u) ** 2 - alpha * alpha)
    nu = d / 2.0 + m
    const = (2 * np.pi) ** (d / 2.0) * (J / 2.0) ** d * alpha ** m
    const /= i0(alpha) if m == 0 else iv(m, alpha)
    if nu == 0:
        y = const * j0(z) / z
    else:
        y = const * jv(nu, z) / z ** nu
    return np.real(y)


def kaiser_bessel_deriv(x, J=6, alpha=None):
    """d/dx of the order-0 KB function:
    ``-(4 alpha x / J^2) I_1(alpha s) / (s I_0(alpha))``, ``s = sqrt(1-(2x/J)^2)``;
    0 outside the support.  At ``s = 0`` the limit ``I_1(alpha s)/s -> alpha/2``
    is used."""
    x = np.asarray(x, dtype=np.float64)
    if alpha is None:
        alpha = 2.34 * J
    out = np.zeros_like(x)
    inside = 2 * np.abs(x) < J
    s = np.sqrt(1 - (2 * x[inside] / J) ** 2)
    ratio = np.where(s > 1e-12, i1(alpha * np.maximum(s, 1e-300)) / np.maximum(s, 1e-300), alpha / 2.0)
    out[inside] = -(4 * alpha * x[inside] / J ** 2) * ratio / i0(alpha)
    return out
