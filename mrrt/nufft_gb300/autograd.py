"""Differentiable NUFFT for torch: gradients with respect to the image and
the trajectory.

``NufftOperator`` wraps one table-mode operator (the same plan math as
``NufftBase``, phasing 'real') for batched torch tensors on the GPU:

* image ``x``: ``[coils, *Nd]`` complex, C order (the reference's axis order);
* trajectory ``omega``: ``[M, ndim]`` real, radians (the reference's omega);
* samples ``y``: ``[coils, M]`` complex.

``op.forward(x, omega)`` computes y = A(omega) x and ``op.adjoint(y, omega)``
computes x = A(omega)^H y, both through ``torch.autograd.Function``s:

* d/dx of the forward is the adjoint transform and d/dy of the adjoint is
  the forward transform (torch's convention for complex gradients,
  grad = dL/dRe + i dL/dIm);
* d/domega of either uses the derivative of the table kernel: a
  derivative table dh/dt (the analytic derivative of the Beatty
  Kaiser-Bessel kernel, sampled like h) is interpolated like h by the
  ``gbn_grad_tm`` kernel, which adds the derivative of the per-sample phase
  exp(i omega . (n_shift - n_mid)).

The reference has no autograd; its forward / adjoint definitions are
mrrt/nufft/_nufft.py:1275-1397 and 1459-1578.  When omega changes between
calls the plan's sample lists are rebuilt: for a CUDA tensor omega by the
device binning (``gbn_plan_set_points_device``: tm = omega / gamma and the
sample phase computed on the GPU, the samples sorted by tile there, the
coordinates never copied to the host); for a host array by the host planner.
"""
import numpy as np
import torch

from ._nufft import NufftBase

__all__ = ["NufftOperator", "nufft_forward", "nufft_adjoint"]


class NufftOperator(object):
    """Batched, differentiable table NUFFT on one GPU (see module docstring).

    Parameters follow ``NufftBase`` (``Nd, omega, Jd, Kd, Ld, n_shift,
    precision``); ``max_coils`` sizes the tiles for the widest batch.
    """

    def __init__(self, Nd, omega, Jd=6, Kd=None, Ld=1024, n_shift=None, precision="single",
                 max_coils=1):
        om = omega.detach().cpu().numpy() if isinstance(omega, torch.Tensor) else np.asarray(omega)
        rdt = np.float32 if precision == "single" else np.float64
        om = np.ascontiguousarray(om, dtype=rdt)
        self.base = NufftBase(Nd, om, Jd=Jd, Kd=Kd, Ld=Ld, n_shift=n_shift, precision=precision,
                              mode="table", phasing="real", on_gpu=True, max_coils=max_coils)
        b = self.base
        self.plan = b.plan
        self.ndim = b.ndim
        self.Nd, self.Kd = tuple(b.Nd), tuple(b.Kd)
        self.M = b.M
        self.rdt = np.dtype(rdt)
        self.cdt = np.dtype(np.complex64 if precision == "single" else np.complex128)
        self.tdtype = torch.complex64 if precision == "single" else torch.complex128
        self.rtdtype = torch.float32 if precision == "single" else torch.float64
        self.device = self.plan.device
        self.gamma = np.array([2 * np.pi / k for k in self.Kd])
        self.shift_vec = np.asarray([s - m for s, m in zip(b.n_shift, b.n_mid)], dtype=rdt)
        # d(sample phase)/d(tm_d) / i  =  (n_shift_d - n_mid_d) * gamma_d
        self.phase_shift = [float(self.shift_vec[d]) * float(self.gamma[d]) for d in range(self.ndim)]
        self.plan.set_dtables(b.kernel_deriv_tables())
        self._omega = om.copy()
        self._omega_t = torch.as_tensor(om, device=self.device)   # the plan's current trajectory
        self._gamma_t = torch.tensor(self.gamma, dtype=torch.float64, device=self.device)
        self._shift_t = torch.as_tensor(self.shift_vec, device=self.device)

    # ----------------------------------------------------------- trajectory
    def set_omega(self, omega):
        """Move the samples to ``omega`` ([M, ndim], radians); rebuilds the
        plan's tile lists if the coordinates changed.  A CUDA tensor stays on
        the device (device binning); a host array goes through the host
        planner."""
        if isinstance(omega, torch.Tensor) and omega.is_cuda:
            om = omega.detach().to(device=self.device, dtype=self.rtdtype).reshape(self.M, self.ndim)
            if om.data_ptr() == self._omega_t.data_ptr() or torch.equal(om, self._omega_t):
                return
            # tm = omega / gamma (in double, rounded to the operator's dtype) and
            # exp(i omega . (n_shift - n_mid)), as the host path computes them
            tm = (om.to(torch.float64) / self._gamma_t).to(self.rtdtype).contiguous()
            phase = torch.exp(1j * (om @ self._shift_t)).to(self.tdtype)
            self.plan.set_points_device(tm, phase)
            self._omega_t = om.clone()
            self._omega = None
            return
        om = omega.detach().cpu().numpy() if isinstance(omega, torch.Tensor) else np.asarray(omega)
        om = np.ascontiguousarray(om, dtype=self.rdt).reshape(self.M, self.ndim)
        if self._omega is not None and np.array_equal(om, self._omega):
            return
        tm = np.zeros_like(om)
        for d in range(self.ndim):
            tm[:, d] = om[:, d] / self.gamma[d]
        phase = np.exp(1j * np.dot(om, self.shift_vec)).astype(self.cdt, copy=False)
        self.plan.set_points(tm, phase)
        self._omega = om.copy()
        self._omega_t = torch.as_tensor(om, device=self.device)

    # ---------------------------------------------------------- layout glue
    def _image_to_plan(self, x):
        """[coils, *Nd] (C order) -> contiguous [coils, N_{d-1}, ..., N_0]."""
        perm = (0,) + tuple(range(self.ndim, 0, -1))
        return x.to(device=self.device, dtype=self.tdtype).permute(*perm).contiguous()

    def _image_from_plan(self, xp):
        perm = (0,) + tuple(range(self.ndim, 0, -1))
        return xp.permute(*perm)

    def _apply_forward(self, x):
        xp = self._image_to_plan(x)
        C = xp.shape[0]
        y = torch.empty((C, self.M), dtype=self.tdtype, device=self.device)
        self.plan.forward(xp, y, C)
        return y

    def _apply_adjoint(self, y):
        yc = y.to(device=self.device, dtype=self.tdtype).contiguous()
        C = yc.shape[0]
        xp = torch.empty((C,) + tuple(reversed(self.Nd)), dtype=self.tdtype, device=self.device)
        self.plan.adjoint(yc, xp, C)
        return self._image_from_plan(xp)

    def _grad_omega(self, x, gy):
        """sum_c Re(conj(gy[c, m]) d(A x)[c, m] / d omega_m): runs the forward
        on x to fill the plan's grid, then the derivative-table gather."""
        xp = self._image_to_plan(x)
        C = xp.shape[0]
        scratch = torch.empty((C, self.M), dtype=self.tdtype, device=self.device)
        self.plan.forward(xp, scratch, C)
        gtm = torch.empty((self.M, self.ndim), dtype=self.rtdtype, device=self.device)
        gyc = gy.to(device=self.device, dtype=self.tdtype).contiguous()
        self.plan.grad_tm(self.plan.forward_grid(C), gyc, self.phase_shift, gtm, C)
        inv_gamma = torch.tensor(1.0 / self.gamma, dtype=self.rtdtype, device=self.device)
        return gtm * inv_gamma

    # ------------------------------------------------------------ public API
    def forward(self, x, omega=None):
        """y = A(omega) x, differentiable in x and omega."""
        return nufft_forward(x, omega, self)

    def adjoint(self, y, omega=None):
        """x = A(omega)^H y, differentiable in y and omega."""
        return nufft_adjoint(y, omega, self)


def _omega_arg(omega, op):
    if omega is None:
        return op._omega_t
    return omega


class _Forward(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, omega, op):
        op.set_omega(omega)
        ctx.op = op
        ctx.save_for_backward(x, omega)
        return op._apply_forward(x)

    @staticmethod
    def backward(ctx, gy):
        x, omega = ctx.saved_tensors
        op = ctx.op
        op.set_omega(omega)
        gx = gom = None
        if ctx.needs_input_grad[0]:
            gx = op._apply_adjoint(gy).to(x.dtype)
        if ctx.needs_input_grad[1]:
            gom = op._grad_omega(x, gy).to(device=omega.device, dtype=omega.dtype)
        return gx, gom, None


class _Adjoint(torch.autograd.Function):
    @staticmethod
    def forward(ctx, y, omega, op):
        op.set_omega(omega)
        ctx.op = op
        ctx.save_for_backward(y, omega)
        return op._apply_adjoint(y)

    @staticmethod
    def backward(ctx, gx):
        y, omega = ctx.saved_tensors
        op = ctx.op
        op.set_omega(omega)
        gy = gom = None
        if ctx.needs_input_grad[0]:
            gy = op._apply_forward(gx).to(y.dtype)
        if ctx.needs_input_grad[1]:
            # x = sum_m conj(a_m) y_m  =>  dL/domega_m = Re(conj(y_m) (A' gx)_m)
            gom = op._grad_omega(gx, y).to(device=omega.device, dtype=omega.dtype)
        return gy, gom, None


def nufft_forward(x, omega, op):
    """Differentiable forward NUFFT ``y = A(omega) x`` (``x``: [coils, *Nd])."""
    return _Forward.apply(x, _omega_arg(omega, op), op)


def nufft_adjoint(y, omega, op):
    """Differentiable adjoint NUFFT ``x = A(omega)^H y`` (``y``: [coils, M])."""
    return _Adjoint.apply(y, _omega_arg(omega, op), op)
