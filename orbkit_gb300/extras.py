"""Grid quantities built on the MO grids of the hot path (orbkit/extras.py).

Only the numerical parts: orbkit's output writers (Gaussian cube, HDF5, VMD ...)
are not part of this package, so an output type raises NotImplementedError.
"""
import numpy

from . import core


def calc_jmo(qc, ij, drv=("x", "y", "z"), numproc=1, otype=None, ofid="", exact_mixed=False, **kwargs):
    """Components of the transition electronic flux density between MO pairs,
    j_ij(r) = -1/2 (MO_i dMO_j - MO_j dMO_i), on the grid module's grid
    (orbkit/extras.py:441-492).

    ij: a pair (i, j) or an (n, 2) array of pairs of MO indices; drv: components.
    Returns an array of shape (len(drv), n_pairs) + grid shape.  The MO grids of the
    selected MOs and the flux densities are computed on the device
    (okg_eval_mo, okg_mo_pair_flux) with orbkit's rounding of the products."""
    import torch
    from . import _lib
    from .tools import validate_drv
    if otype is not None:
        raise NotImplementedError("output writers are not part of the GPU path; call with otype=None")
    ij = numpy.asarray(ij)
    if ij.ndim == 1 and len(ij) == 2:
        ij = ij.reshape(1, 2)
    if ij.ndim != 2 or ij.shape[1] != 2:
        raise ValueError("ij must be a pair or an (n, 2) array of MO index pairs")
    drv = list(drv)
    u, indices = numpy.unique(ij, return_inverse=True)
    indices = numpy.ascontiguousarray(indices.reshape(-1, 2), dtype=numpy.intc)
    codes = [0] + [validate_drv(d) for d in drv]
    grid = core.grid  # orbkit.grid once install(orbkit) routed the package
    if not grid.is_initialized:
        grid.grid_init()
    x, y, z, vec, N = core._grid_arrays(grid.x, grid.y, grid.z, grid.is_vector, use_module=False)
    mo = core._MoGrids(qc, x, y, z, vec, exact_mixed, mo_index=u)
    nd, npair, nmo = len(drv), len(indices), mo.nmo
    npts = mo.g.npts
    pairs = torch.from_numpy(indices.reshape(-1)).to(mo.dev)
    L = _lib.load()
    jmo = numpy.empty((nd, npair, npts))
    for (i, j) in core._point_steps(npts, 8 * (nd * npair + (nd + 1) * nmo)):
        m = mo(codes, i, j)
        o = torch.empty((nd, npair, j - i), dtype=torch.float64, device=mo.dev)
        _lib.check(L.okg_mo_pair_flux(nd, nmo, npair, _lib.ptr(pairs), _lib.ptr(m[0]), j - i, _lib.ptr(m[1:]), j - i,
                                      j - i, _lib.ptr(o), j - i, _lib.stream_handle()))
        jmo[:, :, i:j] = o.cpu().numpy()
    return jmo.reshape((nd, npair) + tuple(grid.get_shape()))
