"""Plain PyTorch float64 reference of rho and grad rho, differentiable in every
parameter (test infrastructure).

AO values are written out directly from the definition (orbkit/c_grid-based.c and
orbkit/c_support.c: primitive normalisation, contraction, Cartesian polynomial),
independently of the CUDA kernels' factorisation; grad rho comes from autograd
with respect to the point coordinates (create_graph=True), so the reference
gradient of a loss on (rho, grad rho) needs no hand-written adjoint.
"""
import math

import numpy
import torch


def _dfact(n):
    r = 1
    while n > 0:
        r *= n
        n -= 2
    return r


class Structure:
    def __init__(self, ao_spec, T=None):
        self.lxlylz = numpy.asarray(ao_spec.get_lxlylz())
        self.ncart = numpy.asarray(ao_spec.get_nlxlylz_per_cont())
        self.nprim = numpy.asarray(ao_spec.get_nprim_per_cont())
        self.atoms = numpy.asarray(ao_spec.get_assign_cont_to_atoms())
        self.normalized = bool(ao_spec.get_normalized())
        self.renorm = numpy.asarray(ao_spec[0]["N"]).reshape(-1) if "N" in ao_spec[0] else None
        self.T = T


def rho_grad(C, alpha, coef, geo, st, occ, pts):
    """pts: (3, n) float64 leaf (requires_grad is set here).  Returns rho (n,), grad (3, n)."""
    pts = pts.detach().clone().requires_grad_(True)
    chis = []
    k = 0
    p0 = 0
    for s in range(len(st.ncart)):
        X = pts - geo[int(st.atoms[s])][:, None]
        rr = (X * X).sum(0)
        L = int(st.lxlylz[k].sum())
        R = torch.zeros_like(rr)
        for q in range(int(st.nprim[s])):
            a = alpha[p0 + q]
            nrm = 1.0 if st.normalized else (2.0 / math.pi) ** 0.75 * 2.0 ** L * a ** ((2.0 * L + 3.0) / 4.0)
            R = R + coef[p0 + q] * nrm * torch.exp(-a * rr)
        for r in range(int(st.ncart[s])):
            lx, ly, lz = (int(v) for v in st.lxlylz[k + r])
            g = 1.0 if st.normalized else 1.0 / math.sqrt(_dfact(2 * lx - 1) * _dfact(2 * ly - 1) * _dfact(2 * lz - 1))
            if st.renorm is not None:
                g *= float(st.renorm[k + r])
            chis.append(g * X[0] ** lx * X[1] ** ly * X[2] ** lz * R)
        k += int(st.ncart[s])
        p0 += int(st.nprim[s])
    chi = torch.stack(chis)
    Ceff = C @ torch.as_tensor(st.T, dtype=C.dtype, device=C.device) if st.T is not None else C
    phi = Ceff @ chi
    rho = (occ[:, None] * phi * phi).sum(0)
    grad = torch.autograd.grad(rho.sum(), pts, create_graph=True)[0]
    return rho, grad
