"""orbkit_gb300: orbkit's grid-evaluation path (AOs, MOs, density and its
derivatives) as hand-written sm_103a CUDA behind orbkit's own Python API.

    from orbkit_gb300 import core          # ao_creator, mo_creator, rho_compute, ...
    import orbkit_gb300; orbkit_gb300.install(orbkit)   # swap orbkit.core's grid path

See include/orbkit_gb300.h for the C ABI underneath.
"""
__version__ = "0.1.0"

from . import grid, tools  # noqa: F401
from .orbitals import AOClass, MOClass  # noqa: F401
from .qcinfo import QCinfo  # noqa: F401


def install(orbkit_module):
    """Route orbkit.core's grid functions to this package.

    ``orbkit_module`` is the imported orbkit package.  ao_creator, mo_creator,
    cartesian2spherical, rho_compute, rho_compute_no_slice and calc_mo_matrix of
    orbkit.core (and the names re-exported at the package level) are replaced;
    they read orbkit.grid.  Returns a function that restores the originals."""
    from . import core as ours
    okc = orbkit_module.core
    names = ["ao_creator", "mo_creator", "cartesian2spherical", "rho_compute", "rho_compute_no_slice",
             "calc_mo_matrix"]
    saved = {n: getattr(okc, n) for n in names}
    saved_pkg = {n: getattr(orbkit_module, n) for n in names if hasattr(orbkit_module, n)}
    saved_grid = ours.grid
    ours.grid = orbkit_module.grid
    for n in names:
        setattr(okc, n, getattr(ours, n))
        if n in saved_pkg:
            setattr(orbkit_module, n, getattr(ours, n))

    def restore():
        for n, f in saved.items():
            setattr(okc, n, f)
        for n, f in saved_pkg.items():
            setattr(orbkit_module, n, f)
        ours.grid = saved_grid

    return restore
