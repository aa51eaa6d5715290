"""Differentiable rho and grad rho: a torch.autograd.Function over the GPU kernels.

Forward: okg_rho (FP64 path), or the tensor-core mixed path for precision="fp32".
Backward: the hand-written adjoint kernel okg_rho_backward (FP64 or FP32
arithmetic), which recomputes AO tiles instead of storing them and returns
dL/dC (MO coefficients, in the output AO basis), dL/dalpha and dL/dc (primitive
exponents and contraction coefficients, in ao_spec.get_prim_coeffs() order) and
dL/dR (nuclear coordinates).

    model = DensityModel(qc, x, y, z, is_vector=False, precision="fp64")
    C = torch.tensor(qc.mo_spec.get_coeffs(), device="cuda", requires_grad=True)
    rho, grad = model(C, alpha, coef, geo)
    loss = density_fit_loss(rho, grad, rho_t, grad_t, w)
    loss.backward()
"""
import ctypes

import numpy

from . import _lib
from .basis import DeviceBasis
from .qcinfo import unpack

_SIGS = {
    "okg_rho_backward_workspace": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(_lib.OkgGrid), ctypes.c_int,
                                                  ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]),
    "okg_rho_backward": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(_lib.OkgGrid), ctypes.c_int,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_int64, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
}


def _L():
    L = _lib.load()
    for n, (r, a) in _SIGS.items():
        f = getattr(L, n)
        f.restype = r
        f.argtypes = a
    return L


def density_fit_loss(rho, grad, rho_t, grad_t, w, grad_weight=0.1):
    """sum_r w (rho - rho_t)^2 + grad_weight * sum_r |grad rho - grad rho_t|^2."""
    return (w * (rho - rho_t) ** 2).sum() + grad_weight * ((grad - grad_t) ** 2).sum()


class DensityModel:
    """rho / grad rho of one basis structure on a fixed grid, differentiable in
    (C, alpha, c, R).  precision: "fp64" (FP64 forward and backward) or "fp32"
    (mixed tensor-core forward, FP32 backward)."""

    def __init__(self, qc, x, y, z, is_vector, precision="fp64", device=None):
        import torch
        from .core import _DeviceGrid
        geo, ao_spec, mo_spec = unpack(qc)
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        self.basis = DeviceBasis(geo, ao_spec, self.device)
        self.occ = torch.as_tensor(numpy.array([m["occ_num"] for m in mo_spec], dtype=numpy.float64),
                                   device=self.device)
        self.grid = _DeviceGrid(numpy.asarray(x, dtype=numpy.float64), numpy.asarray(y, dtype=numpy.float64),
                                numpy.asarray(z, dtype=numpy.float64), is_vector, self.device)
        self.gd, self._keep = self.grid.slice(0, self.grid.npts)
        self.npts = self.grid.npts
        if precision not in ("fp64", "fp32"):
            raise ValueError("precision must be 'fp64' or 'fp32'")
        self.precision = precision
        self._L = _L()
        self._work = None
        self._mixed = None
        self.nmo = len(self.occ)

    def __call__(self, C, alpha, coef, geo):
        return _RhoGrad.apply(C, alpha, coef, geo, self)

    # ---- raw device operations
    def _set(self, alpha, coef, geo):
        import torch
        prim = torch.stack([alpha.detach(), coef.detach()], dim=1).to(torch.float64).contiguous()
        self.basis.set_params(geo=geo.detach().to(torch.float64), prim=prim)

    def _forward(self, C):
        import torch
        Ceff = self.basis.c_eff(C.detach())
        rho = torch.empty(self.npts, dtype=torch.float64, device=self.device)
        grad = torch.empty((3, self.npts), dtype=torch.float64, device=self.device)
        if self.precision == "fp64":
            _lib.check(self._L.okg_rho(self.basis.handle, self.gd, self.nmo, _lib.ptr(Ceff), _lib.ptr(self.occ), 3,
                                       _lib.int_array([1, 2, 3]), 1, _lib.ptr(rho), _lib.ptr(grad), self.npts, None,
                                       _lib.stream_handle()))
        else:
            from .mixed import MixedPlan
            if self._mixed is None:
                self._mixed = MixedPlan(self.basis, C.detach(), self.occ.cpu().numpy())
            p = self._mixed
            p.C = Ceff
            _lib.check(p._L.okg_mixed_set_coeffs(p.handle, _lib.ptr(Ceff), _lib.ptr(self.occ), _lib.stream_handle()))
            p.rho(self.gd, rho, grad, self.npts)
        return rho, grad

    def _backward(self, C, g_rho, g_grad):
        import torch
        Ceff = self.basis.c_eff(C.detach())
        prec = 64 if self.precision == "fp64" else 32
        nbytes = ctypes.c_size_t(0)
        _lib.check(self._L.okg_rho_backward_workspace(self.basis.handle, self.gd, self.nmo, prec, ctypes.byref(nbytes)))
        if self._work is None or self._work.numel() < nbytes.value:
            self._work = torch.empty(nbytes.value, dtype=torch.uint8, device=self.device)
        g_rho = g_rho.to(torch.float64).contiguous()
        g_grad = g_grad.to(torch.float64).contiguous()
        dC = torch.empty_like(Ceff)
        dprim = torch.empty((self.basis.nprim, 2), dtype=torch.float64, device=self.device)
        dgeo = torch.empty((self.basis.natom, 3), dtype=torch.float64, device=self.device)
        _lib.check(self._L.okg_rho_backward(self.basis.handle, self.gd, self.nmo, _lib.ptr(Ceff), _lib.ptr(self.occ),
                                            _lib.ptr(g_rho), _lib.ptr(g_grad), self.npts, prec, _lib.ptr(dC),
                                            _lib.ptr(dprim), _lib.ptr(dgeo), _lib.ptr(self._work), nbytes.value,
                                            _lib.stream_handle()))
        if self.basis.spherical:
            dC = dC @ self.basis.T_dev.T
        return dC, dprim, dgeo


def _grad_fn():
    import torch

    class RhoGrad(torch.autograd.Function):
        @staticmethod
        def forward(ctx, C, alpha, coef, geo, model):
            model._set(alpha, coef, geo)
            rho, grad = model._forward(C)
            ctx.save_for_backward(C, alpha, coef, geo)
            ctx.model = model
            return rho, grad

        @staticmethod
        def backward(ctx, g_rho, g_grad):
            C, alpha, coef, geo = ctx.saved_tensors
            model = ctx.model
            model._set(alpha, coef, geo)
            if g_rho is None:
                g_rho = torch.zeros(model.npts, dtype=torch.float64, device=model.device)
            if g_grad is None:
                g_grad = torch.zeros((3, model.npts), dtype=torch.float64, device=model.device)
            dC, dprim, dgeo = model._backward(C, g_rho, g_grad)
            return (dC.to(C.dtype), dprim[:, 0].to(alpha.dtype), dprim[:, 1].to(coef.dtype),
                    dgeo.to(geo.dtype), None)

    return RhoGrad


class _Lazy:
    fn = None

    @classmethod
    def apply(cls, *args):
        if cls.fn is None:
            cls.fn = _grad_fn()
        return cls.fn.apply(*args)


_RhoGrad = _Lazy
