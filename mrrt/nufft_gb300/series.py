"""Dynamic series: many frames of one image geometry, each with its own
(uneven) sample set, transformed in one launch per stage.

The reference applies one ``NufftBase`` per frame (one plan, one FFT and
one interpolation call per frame and coil, mrrt/nufft/_nufft.py:1275-1578).
``NufftSeries`` builds a single plan whose sample lists hold every frame
(``frame_offsets``), so each stage -- pad, batched FFT over frames x coils,
gather, spread, crop -- is one kernel launch for the whole series.  The
per-frame plan math (tables, ``sn``, ``tm``, phases) is the reference's, as
in ``NufftBase``.

Layouts (the C ABI's memory order, which is the reference's Fortran order):

* images ``x``: ``[F, coils, N_{d-1}, ..., N_0]`` contiguous, i.e. the memory
  of a Fortran-order ``Nd + (coils, F)`` array;
* samples ``y``: frame-major, frame f holds ``[coils, M_f]`` starting at
  element ``coils * frame_offsets[f]`` (``split_samples`` gives the views).

``capture()`` records the forward and adjoint of a fixed coil count as CUDA
graphs on static buffers, so a step is two graph launches.
"""
import numpy as np
import torch

from ._kernels import BeattyKernel, kernel_table
from ._nufft import deapodisation, normalised_coordinates, sample_phase_of
from ._plan import GpuPlan, require_cuda

__all__ = ["NufftSeries"]


class NufftSeries(object):
    """Forward / adjoint table NUFFT of a series of frames on one GPU.

    Parameters
    ----------
    Nd, Jd, Kd, Ld, n_shift, precision : as for ``NufftBase`` (phasing 'real').
    omegas : list of ``[M_f, ndim]`` arrays, one trajectory per frame (radians).
    coils : coil count the plan's tiles are sized for.
    tile, stile : gather / spread tile edges per axis in the reference's axis
        order (``None``: the planner's defaults; ``autotune.tune_series``
        picks them by measurement).
    """

    def __init__(self, Nd, omegas, Jd=6, Kd=None, Ld=1024, n_shift=None, precision="single",
                 coils=1, tile=None, stile=None):
        require_cuda()
        Nd = tuple(int(n) for n in (Nd if not np.isscalar(Nd) else (Nd,)))
        ndim = len(Nd)
        Jd = tuple(int(j) for j in (Jd if not np.isscalar(Jd) else (Jd,) * ndim))
        Kd = tuple(int(k) for k in (Kd if Kd is not None else [int(1.5 * n) for n in Nd]))
        if precision not in ("single", "double"):
            raise ValueError("precision must be 'single' or 'double'")
        rdt = np.dtype(np.float32 if precision == "single" else np.float64)
        cdt = np.dtype(np.complex64 if precision == "single" else np.complex128)
        n_shift = tuple(float(s) for s in (n_shift if n_shift is not None else (0.0,) * ndim))
        self.Nd, self.Kd, self.Jd, self.Ld, self.ndim = Nd, Kd, Jd, int(Ld), ndim
        self.n_mid = tuple(n // 2 for n in Nd)
        self.precision = precision
        self.coils = int(coils)
        kernel = BeattyKernel(shape=Jd, grid_shape=Nd, os_grid_shape=Kd)
        self.sn = deapodisation(Nd, Kd, Jd, self.n_mid, kernel.alpha, rdt)
        self.h = [kernel_table(Nd[d], Jd[d], Kd[d], self.Ld, "real", rdt) for d in range(ndim)]
        tms, phases, counts = [], [], []
        for om in omegas:
            om = np.asarray(om.detach().cpu().numpy() if isinstance(om, torch.Tensor) else om)
            if om.ndim == 1:
                om = om[:, None]
            if om.shape[1] != ndim:
                raise ValueError("number of cols must match NUFFT dimension")
            if om.dtype not in (np.float32, np.float64):
                om = om.astype(np.float64)
            # as NufftBase: the phase from omega in its given dtype, the
            # coordinates from omega cast to the operator's real dtype
            phases.append(sample_phase_of(om, n_shift, self.n_mid, "real", rdt, cdt))
            tms.append(normalised_coordinates(om.astype(rdt), Kd, rdt))
            counts.append(om.shape[0])
        if not counts:
            raise ValueError("a series needs at least one frame")
        self.frame_offsets = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        self.n_frames = len(counts)
        self.M_total = int(self.frame_offsets[-1])
        pb_coef = [2 * np.pi / Kd[d] * self.n_mid[d] for d in range(ndim)]
        self.plan = GpuPlan(Nd, Kd, Jd, self.Ld, rdt, self.h, None, self.sn.ravel(order="F"),
                            np.ascontiguousarray(np.concatenate(tms)), np.concatenate(phases),
                            frame_offsets=self.frame_offsets, pb_coef=pb_coef,
                            pb_order=list(range(ndim)), max_coils=self.coils, tile=tile, stile=stile)
        self.ctype = self.plan.ctype
        self.device = self.plan.device
        self.image_shape = (self.n_frames, self.coils) + tuple(reversed(Nd))
        self._graphs = None

    # ---------------------------------------------------------------- layout
    def empty_images(self, coils=None):
        c = self.coils if coils is None else coils
        return torch.empty((self.n_frames, c) + tuple(reversed(self.Nd)), dtype=self.ctype,
                           device=self.device)

    def empty_samples(self, coils=None):
        c = self.coils if coils is None else coils
        return torch.empty(c * self.M_total, dtype=self.ctype, device=self.device)

    def split_samples(self, y, coils=None):
        """Per-frame ``[coils, M_f]`` views of a frame-major sample buffer."""
        c = self.coils if coils is None else coils
        fo = self.frame_offsets
        return [y[c * fo[f]:c * fo[f + 1]].view(c, int(fo[f + 1] - fo[f])) for f in range(self.n_frames)]

    # ------------------------------------------------------------ transforms
    def forward(self, x, y=None, coils=None):
        """Images ``[F, coils, *reversed(Nd)]`` -> frame-major samples."""
        c = x.shape[1] if coils is None else coils
        y = self.empty_samples(c) if y is None else y
        self.plan.forward(x, y, c)
        return y

    def adjoint(self, y, x=None, coils=None):
        """Frame-major samples -> images ``[F, coils, *reversed(Nd)]``.  The
        coil count comes from ``coils``, else from ``x``, else from the size
        of ``y`` (which must hold ``coils * M_total`` samples)."""
        if coils is None:
            if x is not None:
                coils = x.shape[1]
            elif y.numel() % self.M_total == 0 and self.M_total > 0:
                coils = y.numel() // self.M_total
            else:
                raise ValueError("y holds %d samples, not a multiple of the series' %d"
                                 % (y.numel(), self.M_total))
        c = int(coils)
        if y.numel() != c * self.M_total:
            raise ValueError("y holds %d samples but %d coils x %d samples were expected"
                             % (y.numel(), c, self.M_total))
        x = self.empty_images(c) if x is None else x
        self.plan.adjoint(y, x, c)
        return x

    # ------------------------------------------ coil sensitivities (fused)
    def forward_sense(self, image, maps, y=None):
        """One image per frame ``[F, *reversed(Nd)]`` and coil maps
        ``[coils, *reversed(Nd)]`` -> frame-major samples of every coil; the
        map multiply is fused into the deapodisation pass."""
        c = maps.shape[0]
        y = self.empty_samples(c) if y is None else y
        self.plan.forward_sense(image, maps, y, c)
        return y

    def adjoint_sense(self, y, maps, image=None):
        """Frame-major samples -> ``[F, *reversed(Nd)]``, the coil sum of
        conj(maps) times each coil's adjoint fused into the crop pass."""
        c = maps.shape[0]
        if image is None:
            image = torch.empty((self.n_frames,) + tuple(reversed(self.Nd)), dtype=self.ctype,
                                device=self.device)
        self.plan.adjoint_sense(y, maps, image, c)
        return image

    # ------------------------------------------------------------ CUDA graphs
    def capture(self, coils=None, warmup=2):
        """Record forward and adjoint as CUDA graphs on static buffers
        ``self.x_static`` / ``self.y_static`` / ``self.xa_static``.  The warm-up
        calls size every plan buffer and cuFFT plan first, so nothing is
        allocated while capturing."""
        c = self.coils if coils is None else coils
        self.x_static = self.empty_images(c).zero_()
        self.y_static = self.empty_samples(c).zero_()
        self.xa_static = self.empty_images(c)
        s = torch.cuda.Stream(device=self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            for _ in range(max(1, warmup)):
                self.plan.forward(self.x_static, self.y_static, c)
                self.plan.adjoint(self.y_static, self.xa_static, c)
        torch.cuda.current_stream(self.device).wait_stream(s)
        torch.cuda.synchronize(self.device)
        gf, ga = torch.cuda.CUDAGraph(), torch.cuda.CUDAGraph()
        with torch.cuda.graph(gf):
            self.plan.forward(self.x_static, self.y_static, c)
        with torch.cuda.graph(ga):
            self.plan.adjoint(self.y_static, self.xa_static, c)
        self._graphs = (gf, ga, c)
        return self

    def replay_forward(self):
        """x_static -> y_static (the captured forward)."""
        if self._graphs is None:
            raise RuntimeError("call capture() first")
        self._graphs[0].replay()
        return self.y_static

    def replay_adjoint(self):
        """y_static -> xa_static (the captured adjoint)."""
        if self._graphs is None:
            raise RuntimeError("call capture() first")
        self._graphs[1].replay()
        return self.xa_static

    @property
    def samples_per_frame(self):
        return np.diff(self.frame_offsets)

    def __repr__(self):
        return "NufftSeries(Nd=%s, Kd=%s, Jd=%s, frames=%d, samples=%d, coils=%d)" % (
            self.Nd, self.Kd, self.Jd, self.n_frames, self.M_total, self.coils)
