"""Thin owner of a libgbnufft plan handle (host side of the C ABI).

``GpuPlan`` turns host-side plan math (tables, deapodisation, coordinates,
sample phase) into a ``gbn_plan`` and calls the transforms on torch's current
CUDA stream: on CUDA tensors through the device entry points, and on CPU
tensors (pageable or pinned) through the host-buffer ones.  Everything here
is plumbing around the C ABI; the arithmetic runs in the CUDA kernels.
"""
import ctypes

import numpy as np
import torch

from . import _lib

_CPLX = {np.dtype(np.float32): torch.complex64, np.dtype(np.float64): torch.complex128}
_REAL = {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64}


def _vp(arr):
    return ctypes.c_void_p(arr.ctypes.data) if arr is not None else None


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("mrrt.nufft_gb300 needs a CUDA GPU: torch.cuda.is_available() is False")


class GpuPlan:
    """A ``gbn_plan`` for one geometry and one or more sample sets (frames).

    All array arguments are in MEMORY-AXIS order (axis 0 fastest), as the C
    ABI expects; callers translate from their own axis convention.
    """

    def __init__(self, Nd, Kd, Jd, L, rdt, tables_re, tables_im, sn, tm, sample_phase,
                 frame_offsets=None, ortho=False, adjoint_scale=1.0, pb_coef=None, pb_order=None,
                 phasing="real", max_coils=1, tile=None, stile=None, device=None, table_only=False,
                 cufft_only=False, lib=None):
        require_cuda()
        # lib: a loaded libgbnufft (default); _lib.load_checked() gives the
        # bounds-checked build
        self.lib = lib if lib is not None else _lib.load()
        self.rdt = np.dtype(rdt)
        self.ndim = len(Nd)
        self.Nd, self.Kd, self.Jd = tuple(Nd), tuple(Kd), tuple(Jd)
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        g = _lib.GbnGeometry()
        g.ndim = self.ndim
        for d in range(self.ndim):
            g.Nd[d], g.Kd[d], g.Jd[d] = int(Nd[d]), int(Kd[d]), int(Jd[d])
            g.tile[d] = int(tile[d]) if tile is not None else 0
            g.stile[d] = int(stile[d]) if stile is not None else 0
            g.pb_coef[d] = float(pb_coef[d]) if pb_coef is not None else 0.0
            g.pb_order[d] = int(pb_order[d]) if pb_order is not None else d
        g.L = int(L)
        g.precision = _lib.PRECISION["double" if self.rdt == np.float64 else "single"]
        g.phasing = _lib.PHASING[phasing]
        g.ortho = int(bool(ortho))
        g.adjoint_scale = float(adjoint_scale)
        g.n_frames = 1 if frame_offsets is None else len(frame_offsets) - 1
        g.max_coils = max(1, int(max_coils))
        g.flags = (_lib.FLAG_TABLE_ONLY if table_only else 0) | (_lib.FLAG_CUFFT_ONLY if cufft_only else 0)
        self.geom = g
        self._keep = []
        hre = [np.ascontiguousarray(t, dtype=self.rdt) for t in tables_re]
        him = [np.ascontiguousarray(t, dtype=self.rdt) for t in tables_im] if tables_im else None
        self._keep += hre + (him or [])
        Hre = (ctypes.c_void_p * 3)(*[_vp(h) for h in hre] + [None] * (3 - len(hre)))
        Him = (ctypes.c_void_p * 3)(*[_vp(h) for h in him] + [None] * (3 - len(him))) if him else None
        sn = np.ascontiguousarray(sn, dtype=self.rdt)
        tm = np.ascontiguousarray(tm, dtype=self.rdt).reshape(-1, self.ndim)
        self.M_total = tm.shape[0]
        if frame_offsets is None:
            frame_offsets = [0, self.M_total]
        fo = np.ascontiguousarray(frame_offsets, dtype=np.int64)
        self.frame_offsets = fo
        ph = None
        if sample_phase is not None:
            ph = np.ascontiguousarray(sample_phase, dtype=np.result_type(self.rdt, np.complex64))
        handle = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check_with(self.lib, self.lib.gbn_plan_create(
                ctypes.byref(handle), ctypes.byref(g), Hre, Him, _vp(sn),
                fo.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), _vp(tm), _vp(ph),
                self.device.index))
        self.handle = handle
        self.ctype = _CPLX[self.rdt]
        self.Nprod = int(np.prod(Nd))
        self.Kprod = int(np.prod(Kd))

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                self.lib.gbn_plan_destroy(h)
            except Exception:
                pass
            self.handle = None

    # -- transforms on device tensors in the plan's memory layout -------------
    def _check(self, t, numel, name):
        if not isinstance(t, torch.Tensor) or t.device.type != "cuda":
            raise ValueError("%s must be a CUDA tensor" % name)
        if t.dtype != self.ctype:
            raise ValueError("%s must be %s, got %s" % (name, self.ctype, t.dtype))
        if not t.is_contiguous():
            raise ValueError("%s must be contiguous" % name)
        if t.numel() != numel:
            raise ValueError("%s has %d elements, expected %d" % (name, t.numel(), numel))

    def forward(self, x, y, coils):
        F = len(self.frame_offsets) - 1
        self._check(x, F * coils * self.Nprod, "x")
        self._check(y, coils * self.M_total, "y")
        with torch.cuda.device(self.device):
            _lib.check_with(self.lib, self.lib.gbn_forward(self.handle, ctypes.c_void_p(x.data_ptr()),
                                            ctypes.c_void_p(y.data_ptr()), int(coils), _stream()))
        return y

    def adjoint(self, y, x, coils):
        F = len(self.frame_offsets) - 1
        self._check(y, coils * self.M_total, "y")
        self._check(x, F * coils * self.Nprod, "x")
        with torch.cuda.device(self.device):
            _lib.check_with(self.lib, self.lib.gbn_adjoint(self.handle, ctypes.c_void_p(y.data_ptr()),
                                            ctypes.c_void_p(x.data_ptr()), int(coils), _stream()))
        return x

    def _check_host(self, t, numel, name):
        if not isinstance(t, torch.Tensor) or t.device.type != "cpu":
            raise ValueError("%s must be a CPU tensor" % name)
        if t.dtype != self.ctype:
            raise ValueError("%s must be %s, got %s" % (name, self.ctype, t.dtype))
        if not t.is_contiguous():
            raise ValueError("%s must be contiguous" % name)
        if t.numel() != numel:
            raise ValueError("%s has %d elements, expected %d" % (name, t.numel(), numel))

    def forward_host(self, x, y, coils):
        """Forward transform of host memory into host memory (CPU tensors in
        the device layouts, pageable or pinned); returns when y holds the
        result."""
        F = len(self.frame_offsets) - 1
        self._check_host(x, F * coils * self.Nprod, "x")
        self._check_host(y, coils * self.M_total, "y")
        with torch.cuda.device(self.device):
            _lib.check_with(self.lib, self.lib.gbn_forward_host(self.handle, ctypes.c_void_p(x.data_ptr()),
                                                 ctypes.c_void_p(y.data_ptr()), int(coils), _stream()))
        return y

    def adjoint_host(self, y, x, coils):
        """Adjoint transform of host memory into host memory."""
        F = len(self.frame_offsets) - 1
        self._check_host(y, coils * self.M_total, "y")
        self._check_host(x, F * coils * self.Nprod, "x")
        with torch.cuda.device(self.device):
            _lib.check_with(self.lib, self.lib.gbn_adjoint_host(self.handle, ctypes.c_void_p(y.data_ptr()),
                                                 ctypes.c_void_p(x.data_ptr()), int(coils), _stream()))
        return x

    def forward_sense(self, image, maps, y, coils):
        """Coil-sensitivity forward: image [F, N...] and maps [coils, N...]
        (plan layout) -> samples, the map multiply fused into the pad."""
        F = len(self.frame_offsets) - 1
        self._check(image, F * self.Nprod, "image")
        self._check(maps, coils * self.Nprod, "maps")
        self._check(y, coils * self.M_total, "y")
        with torch.cuda.device(self.device):
            _lib.check_with(self.lib, self.lib.gbn_forward_sense(self.handle, ctypes.c_void_p(image.data_ptr()),
                                                  ctypes.c_void_p(maps.data_ptr()),
                                                  ctypes.c_void_p(y.data_ptr()), int(coils), _stream()))
        return y

    def adjoint_sense(self, y, maps, image, coils):
        """Coil-combining adjoint: samples -> image [F, N...] = sum over coils
        of conj(maps) times each coil's adjoint, fused into the crop."""
        F = len(self.frame_offsets) - 1
        self._check(y, coils * self.M_total, "y")
        self._check(maps, coils * self.Nprod, "maps")
        self._check(image, F * self.Nprod, "image")
        with torch.cuda.device(self.device):
            _lib.check_with(self.lib, self.lib.gbn_adjoint_sense(self.handle, ctypes.c_void_p(y.data_ptr()),
                                                  ctypes.c_void_p(maps.data_ptr()),
                                                  ctypes.c_void_p(image.data_ptr()), int(coils), _stream()))
        return image

    def interp_forward(self, grid, y, coils):
        F = len(self.frame_offsets) - 1
        self._check(grid, F * coils * self.Kprod, "grid")
        self._check(y, coils * self.M_total, "y")
        with torch.cuda.device(self.device):
            _lib.check_with(self.lib, self.lib.gbn_interp_forward(self.handle, ctypes.c_void_p(grid.data_ptr()),
                                                   ctypes.c_void_p(y.data_ptr()), int(coils),
                                                   _stream()))
        return y

    def interp_adjoint(self, y, grid, coils):
        F = len(self.frame_offsets) - 1
        self._check(y, coils * self.M_total, "y")
        self._check(grid, F * coils * self.Kprod, "grid")
        with torch.cuda.device(self.device):
            _lib.check_with(self.lib, self.lib.gbn_interp_adjoint(self.handle, ctypes.c_void_p(y.data_ptr()),
                                                   ctypes.c_void_p(grid.data_ptr()), int(coils),
                                                   _stream()))
        return grid

    def forward_grid(self, coils):
        """View of the plan's grid buffer after a forward call: [coils, Kprod]."""
        ptr = ctypes.c_void_p()
        _lib.check_with(self.lib, self.lib.gbn_forward_grid(self.handle, ctypes.byref(ptr)))
        return ptr.value

    def set_dtables(self, dtabs):
        arrs = [np.ascontiguousarray(t, dtype=self.rdt) for t in dtabs]
        self._keep += arrs
        D = (ctypes.c_void_p * 3)(*[_vp(a) for a in arrs] + [None] * (3 - len(arrs)))
        with torch.cuda.device(self.device):
            _lib.check_with(self.lib, self.lib.gbn_plan_set_dtables(self.handle, D))

    def grad_tm(self, grid_ptr, gy, phase_shift, gtm, coils):
        self._check(gy, coils * self.M_total, "gy")
        sh = (ctypes.c_double * 3)(*[float(s) for s in phase_shift] + [0.0] * (3 - len(phase_shift)))
        with torch.cuda.device(self.device):
            _lib.check_with(self.lib, self.lib.gbn_grad_tm(self.handle, ctypes.c_void_p(grid_ptr),
                                            ctypes.c_void_p(gy.data_ptr()), sh,
                                            ctypes.c_void_p(gtm.data_ptr()), int(coils), _stream()))
        return gtm

    def set_weights(self, w_re, w_im=None):
        """Sparse-matrix mode: per-axis weights [M_total, J_d] (plan precision)
        replace the table interpolation; ``None`` returns to table mode."""
        if w_re is None:
            with torch.cuda.device(self.device):
                _lib.check_with(self.lib, self.lib.gbn_plan_set_weights(self.handle, None, None))
            return
        wr = [np.ascontiguousarray(w, dtype=self.rdt) for w in w_re]
        wi = [np.ascontiguousarray(w, dtype=self.rdt) for w in w_im] if w_im is not None else None
        Wr = (ctypes.c_void_p * 3)(*[_vp(w) for w in wr] + [None] * (3 - len(wr)))
        Wi = (ctypes.c_void_p * 3)(*[_vp(w) for w in wi] + [None] * (3 - len(wi))) if wi else None
        with torch.cuda.device(self.device):
            _lib.check_with(self.lib, self.lib.gbn_plan_set_weights(self.handle, Wr, Wi))

    def set_points(self, tm, sample_phase):
        tm = np.ascontiguousarray(tm, dtype=self.rdt).reshape(-1, self.ndim)
        if tm.shape[0] != self.M_total:
            raise ValueError("set_points keeps the sample count; got %d, expected %d"
                             % (tm.shape[0], self.M_total))
        ph = None
        if sample_phase is not None:
            ph = np.ascontiguousarray(sample_phase, dtype=np.result_type(self.rdt, np.complex64))
        with torch.cuda.device(self.device):
            _lib.check_with(self.lib, self.lib.gbn_plan_set_points(self.handle, _vp(tm), _vp(ph)))

    def set_points_device(self, tm, sample_phase=None):
        """Replace the coordinates from device tensors (``tm`` [M_total, ndim]
        in the plan's real dtype, ``sample_phase`` [M_total] complex or None):
        the tile lists are rebuilt by kernels on the plan's device, on the
        current stream."""
        rt = torch.float32 if self.rdt == np.float32 else torch.float64
        tm = tm.to(device=self.device, dtype=rt).contiguous()
        if tm.numel() != self.M_total * self.ndim:
            raise ValueError("set_points keeps the sample count; got %d coordinates, expected %d"
                             % (tm.numel(), self.M_total * self.ndim))
        ph = None
        if sample_phase is not None:
            ph = sample_phase.to(device=self.device, dtype=self.ctype).contiguous()
            if ph.numel() != self.M_total:
                raise ValueError("sample_phase needs %d values" % self.M_total)
        with torch.cuda.device(self.device):
            _lib.check_with(self.lib, self.lib.gbn_plan_set_points_device(
                self.handle, ctypes.c_void_p(tm.data_ptr()),
                ctypes.c_void_p(ph.data_ptr()) if ph is not None else None, _stream()))

    def stats(self):
        out = (ctypes.c_int64 * 8)()
        _lib.check_with(self.lib, self.lib.gbn_plan_stats(self.handle, out))
        keys = ("gather_items", "spread_items", "split_tiles", "gather_len", "spread_len",
                "tiles", "device_bytes", "samples")
        return dict(zip(keys, list(out)))
