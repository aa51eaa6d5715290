"""Grid quantities built on the MO grids of the hot path (orbkit/extras.py).

Only the numerical parts: orbkit's output writers (Gaussian cube, HDF5, VMD ...)
are not part of this package, so an output type raises NotImplementedError.
"""
import copy

import numpy

from . import core, grid


def _select_mos(qc, idx):
    """A shallow copy of qc (QCinfo or dict) holding only the MOs idx, in order."""
    if isinstance(qc, dict):
        out = dict(qc)
        out["mo_spec"] = qc["mo_spec"][idx]
        return out
    out = copy.copy(qc)
    out.mo_spec = qc.mo_spec[idx]
    return out


def calc_jmo(qc, ij, drv=("x", "y", "z"), numproc=1, otype=None, ofid="", **kwargs):
    """Components of the transition electronic flux density between MO pairs,
    j_ij(r) = -1/2 (MO_i dMO_j - MO_j dMO_i), on the grid module's grid
    (orbkit/extras.py:441-492).

    ij: a pair (i, j) or an (n, 2) array of pairs of MO indices; drv: components.
    Returns an array of shape (len(drv), n_pairs) + grid shape."""
    if otype is not None:
        raise NotImplementedError("output writers are not part of the GPU path; call with otype=None")
    ij = numpy.asarray(ij)
    if ij.ndim == 1 and len(ij) == 2:
        ij = ij.reshape(1, 2)
    if ij.ndim != 2 or ij.shape[1] != 2:
        raise ValueError("ij must be a pair or an (n, 2) array of MO index pairs")
    drv = list(drv)
    u, indices = numpy.unique(ij, return_inverse=True)
    indices = indices.reshape(-1, 2)
    mo_matrix = core.calc_mo_matrix(_select_mos(qc, u), drv=drv, numproc=numproc, **kwargs)
    jmo = numpy.zeros((len(drv), len(indices)) + tuple(grid.get_shape()))
    for n, (i, j) in enumerate(indices):
        jmo[:, n] = -0.5 * (mo_matrix[:, i, j] - mo_matrix[:, j, i])
    return jmo
