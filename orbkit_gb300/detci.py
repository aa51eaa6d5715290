"""CI (transition) densities and flux densities on a grid from MO grids, on the GPU:
the grid part of orbkit's detCI module (orbkit/detci/ci_core.py:84-267) with the
same arguments and return shapes.

``zero`` and ``sing`` are the two lists produced by orbkit's determinant comparison
(orbkit/detci/occ_check.py compare): zero = [coefficient lists, orbital lists],
sing = [coefficients, orbital pairs].  ``molist`` is (NMO,) + N (orbkit's calc_mo
output) and ``molistdrv`` (3, NMO) + N; numpy arrays or CUDA tensors.  The sums run
over the terms in orbkit's order with orbkit's rounding (okg_ci_* in
include/orbkit_gb300.h); one launch covers every point, numproc is accepted for
compatibility.

orbkit's drivers slice the points with arange(0, npts + 1, s), s = min(npts,
slice_length) (orbkit/detci/ci_core.py:120-125), so the trailing npts % s points are
never evaluated and stay 0 -- its own test data (test/detci/refdata_h3+.npz) hold
that zero at the last grid point.  By default (reference_slicing=True) those points
are set to 0 as orbkit leaves them; reference_slicing=False returns every point.

Two evaluations: exact=True walks the terms in orbkit's order with orbkit's
rounding (okg_ci_rho / okg_ci_jab / okg_ci_a_nabla_b: bit-identical to orbkit for
the same MO grids, work proportional to the number of terms); the default folds
the terms into NMO x NMO coefficient matrices on the host (summed in term order)
and evaluates the quadratic forms (okg_ci_rho_matrix / okg_ci_flux_matrix: NMO^2
FMAs per point whatever the number of terms, FP64, a different summation order).
"""
import ctypes

import numpy

from . import _lib

_vp = ctypes.c_void_p
_SIGS = {
    "okg_ci_rho": (ctypes.c_int, [ctypes.c_int64, _vp, ctypes.c_int64, ctypes.c_int, _vp, _vp, ctypes.c_int, _vp, _vp,
                                  _vp, _vp]),
    "okg_ci_jab": (ctypes.c_int, [ctypes.c_int64, _vp, _vp, ctypes.c_int64, ctypes.c_int, ctypes.c_int, _vp, _vp,
                                  _vp, _vp]),
    "okg_ci_a_nabla_b": (ctypes.c_int, [ctypes.c_int64, _vp, _vp, ctypes.c_int64, ctypes.c_int, ctypes.c_int, _vp,
                                        _vp, _vp, _vp]),
    "okg_ci_rho_matrix": (ctypes.c_int, [ctypes.c_int64, _vp, ctypes.c_int64, ctypes.c_int, _vp, _vp, _vp]),
    "okg_ci_flux_matrix": (ctypes.c_int, [ctypes.c_int64, _vp, _vp, ctypes.c_int64, ctypes.c_int, _vp,
                                          ctypes.c_double, _vp, _vp]),
}


def _L():
    L = _lib.load()
    for n, (r, a) in _SIGS.items():
        f = getattr(L, n)
        f.restype = r
        f.argtypes = a
    return L


def _dev():
    import torch
    return torch.device("cuda", torch.cuda.current_device())


def _grid_tensor(a, nlead):
    """(tensor (nlead..., npts) float64 contiguous on the device, point shape, was_tensor)."""
    import torch
    if isinstance(a, torch.Tensor):
        t = a.to(device=_dev(), dtype=torch.float64)
        shape = tuple(a.shape[nlead:])
        return t.reshape(a.shape[:nlead] + (-1,)).contiguous(), shape, True
    arr = numpy.asarray(a, dtype=numpy.float64)
    shape = arr.shape[nlead:]
    t = torch.from_numpy(numpy.ascontiguousarray(arr.reshape(arr.shape[:nlead] + (-1,)))).to(_dev())
    return t, shape, False


def _zero_terms(zero):
    coef, idx = [], []
    for cs, js in zip(zero[0], zero[1]):
        coef.extend(float(c) for c in cs)
        idx.extend(int(j) for j in js)
    return numpy.asarray(coef, dtype=numpy.float64), numpy.asarray(idx, dtype=numpy.int32)


def _sing_terms(sing):
    coef = numpy.asarray([float(c) for c in sing[0]], dtype=numpy.float64)
    pairs = numpy.asarray([[int(p[0]), int(p[1])] for p in sing[1]], dtype=numpy.int32).reshape(-1, 2)
    return coef, pairs


def _to_dev(a):
    import torch
    return torch.from_numpy(numpy.ascontiguousarray(a)).to(_dev()) if a.size else None


def _covered(npts, slice_length):
    s = int(min(npts, abs(int(slice_length))))
    return (npts // s) * s if s > 0 else 0


def _out(t, shape, was_tensor):
    return t.reshape(tuple(t.shape[:-1]) + tuple(shape)) if was_tensor else t.cpu().numpy().reshape(
        tuple(t.shape[:-1]) + tuple(shape))


def _qt_device(qt_rows, nmo):
    """(nmo, ldq) zero-padded copy of Q^T on the device, ldq = nmo rounded up to 16."""
    import torch
    ldq = (nmo + 15) // 16 * 16
    q = numpy.zeros((nmo, ldq))
    q[:, :nmo] = qt_rows
    return torch.from_numpy(q).to(_dev())


def density_matrix(zero, sing, nmo):
    """M with rho = sum_ab M_ab MO_a MO_b: the zero terms on the diagonal, the single
    terms at (a, b), each entry summed in term order."""
    zc, zi = _zero_terms(zero)
    sc, sp = _sing_terms(sing)
    _check_indices(zi, sp, nmo)
    M = numpy.zeros((nmo, nmo))
    numpy.add.at(M, (zi, zi), zc)
    numpy.add.at(M, (sp[:, 0], sp[:, 1]), sc)
    return M


def flux_matrix(sing, nmo):
    """C with C_ab = sum of the coefficients of the single terms (a, b)."""
    sc, sp = _sing_terms(sing)
    _check_indices(numpy.zeros(0, dtype=numpy.int32), sp, nmo)
    C = numpy.zeros((nmo, nmo))
    numpy.add.at(C, (sp[:, 0], sp[:, 1]), sc)
    return C


def rho(zero, sing, molist, slice_length=1e4, numproc=1, reference_slicing=True, exact=False):
    """Electron (transition) density on the grid (orbkit/detci/ci_core.py:88-134)."""
    import torch
    L = _L()
    mo, shape, was_t = _grid_tensor(molist, 1)
    nmo, npts = mo.shape
    out = torch.empty((npts,), dtype=torch.float64, device=mo.device)
    if exact:
        zc, zi = _zero_terms(zero)
        sc, sp = _sing_terms(sing)
        _check_indices(zi, sp, nmo)
        keep = [_to_dev(a) for a in (zc, zi, sc, sp)]
        _lib.check(L.okg_ci_rho(npts, _lib.ptr(mo), npts, len(zc), _lib.ptr(keep[0]), _lib.ptr(keep[1]), len(sc),
                                _lib.ptr(keep[2]), _lib.ptr(keep[3]), _lib.ptr(out), _lib.stream_handle()))
    else:
        M = density_matrix(zero, sing, nmo)
        S = M + M.T
        S[numpy.diag_indices(nmo)] = numpy.diag(M)
        qt = _qt_device(numpy.tril(S), nmo)
        _lib.check(L.okg_ci_rho_matrix(npts, _lib.ptr(mo), npts, nmo, _lib.ptr(qt), _lib.ptr(out),
                                       _lib.stream_handle()))
    if reference_slicing:
        out[_covered(npts, slice_length):] = 0.0
    return _out(out, shape, was_t)


def _flux(name, zero, sing, molist, molistdrv, slice_length, reference_slicing, exact):
    import torch
    L = _L()
    mo, shape, was_t = _grid_tensor(molist, 1)
    drv, dshape, _ = _grid_tensor(molistdrv, 2)
    nmo, npts = mo.shape
    if tuple(drv.shape) != (3, nmo, npts):
        raise ValueError("molistdrv must have shape (3,) + molist.shape")
    out = torch.empty((3, npts), dtype=torch.float64, device=mo.device)
    if exact:
        sc, sp = _sing_terms(sing)
        _check_indices(numpy.zeros(0, dtype=numpy.int32), sp, nmo)
        keep = [_to_dev(a) for a in (sc, sp)]
        _lib.check(getattr(L, name)(npts, _lib.ptr(mo), _lib.ptr(drv), npts, nmo, len(sc), _lib.ptr(keep[0]),
                                    _lib.ptr(keep[1]), _lib.ptr(out), _lib.stream_handle()))
    else:
        C = flux_matrix(sing, nmo)
        # j = scale sum_b dMO_b sum_a Q_ab MO_a: jab Q = C - C^T, scale -1/2; a_nabla_b Q = C
        Q, scale = (C - C.T, -0.5) if name == "okg_ci_jab" else (C, 1.0)
        qt = _qt_device(Q.T, nmo)
        _lib.check(L.okg_ci_flux_matrix(npts, _lib.ptr(mo), _lib.ptr(drv), npts, nmo, _lib.ptr(qt), scale,
                                        _lib.ptr(out), _lib.stream_handle()))
    if reference_slicing:
        out[:, _covered(npts, slice_length):] = 0.0
    return _out(out, shape, was_t)


def jab(zero, sing, molist, molistdrv, slice_length=1e4, numproc=1, reference_slicing=True, exact=False):
    """Imaginary part of the electronic (transition) flux density, (3,) + N
    (orbkit/detci/ci_core.py:143-192)."""
    return _flux("okg_ci_jab", zero, sing, molist, molistdrv, slice_length, reference_slicing, exact)


def a_nabla_b(zero, sing, molist, molistdrv, slice_length=1e4, numproc=1, reference_slicing=True, exact=False):
    """sum_k c_k MO_a grad MO_b over the single-excitation terms, (3,) + N
    (orbkit/detci/ci_core.py:200-267)."""
    return _flux("okg_ci_a_nabla_b", zero, sing, molist, molistdrv, slice_length, reference_slicing, exact)


def _check_indices(zi, sp, nmo):
    for a in (zi, sp):
        if a.size and (a.min() < 0 or a.max() >= nmo):
            raise IndexError("orbital index outside 0..%d" % (nmo - 1))
