"""mrrt.nufft_gb300 -- table-mode NUFFT for the NVIDIA GB300 (sm_103a).

A drop-in for mritools/mrrt.nufft's ``NufftBase(Nd, omega, Jd, Kd,
mode='table' | 'sparse', precision=...)`` with ``.fft()`` / ``.adj()``,
running on hand-written CUDA kernels behind the C ABI in
``include/gbnufft.h``.

Exports mirror the reference package (mrrt/nufft/__init__.py:1-15) plus the
batched torch operators and the autograd function.
"""
from ._dtft import dtft, dtft_adj  # noqa: F401
from ._kaiser_bessel import kaiser_bessel, kaiser_bessel_ft  # noqa: F401
from ._kernels import BeattyKernel, KaiserBesselKernel  # noqa: F401
from ._nufft import NufftBase  # noqa: F401
from .autograd import NufftOperator, nufft_adjoint, nufft_forward  # noqa: F401

__version__ = "0.1.0"

__all__ = [
    "dtft",
    "dtft_adj",
    "BeattyKernel",
    "KaiserBesselKernel",
    "NufftBase",
    "NufftOperator",
    "nufft_forward",
    "nufft_adjoint",
    "kaiser_bessel",
    "kaiser_bessel_ft",
]
