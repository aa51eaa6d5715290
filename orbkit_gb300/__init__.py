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


# orbkit submodule -> (module of this package, functions replaced)
ROUTES = [
    ("core", "core", ["ao_creator", "mo_creator", "cartesian2spherical", "rho_compute", "rho_compute_no_slice",
                      "calc_mo_matrix"]),
    ("extras", "extras", ["calc_jmo"]),
    ("detci.ci_core", "detci", ["rho", "jab", "a_nabla_b"]),
    ("analytical_integrals", "analytical_integrals",
     ["get_ao_overlap", "cartesian2spherical_aoom", "get_mo_overlap", "get_mo_overlap_matrix", "get_moom_atoms",
      "check_mo_norm", "get_dipole_moment", "get_ao_dipole_matrix", "get_nuclear_dipole_moment", "get_atom2mo",
      "get_lc"]),
]


def install(orbkit_module):
    """Route orbkit's grid and analytic-integral functions to this package.

    ``orbkit_module`` is the imported orbkit package.  Replaced: ao_creator,
    mo_creator, cartesian2spherical, rho_compute, rho_compute_no_slice and
    calc_mo_matrix of orbkit.core (they read orbkit.grid); calc_jmo of orbkit.extras;
    rho, jab and a_nabla_b of orbkit.detci.ci_core; the overlap, MO-overlap and dipole
    functions of orbkit.analytical_integrals -- and the same names where the package
    re-exports them.  Submodules orbkit cannot import are left alone.  Terminal
    output (MO norms, electron count) then goes through orbkit's display.  Returns a
    function that restores the originals."""
    import importlib
    from . import core as ours_core
    saved = []
    for sub, mine, names in ROUTES:
        try:
            target = importlib.import_module(orbkit_module.__name__ + "." + sub)
        except ImportError:
            continue
        ours = importlib.import_module(__name__ + "." + mine)
        for n in names:
            orig = getattr(target, n, None)
            if orig is None:
                continue
            saved.append((target, n, orig))
            setattr(target, n, getattr(ours, n))
            if getattr(orbkit_module, n, None) is orig:  # re-exported at the package level
                saved.append((orbkit_module, n, orig))
                setattr(orbkit_module, n, getattr(ours, n))
    saved_grid = ours_core.grid
    ours_core.grid = orbkit_module.grid
    saved_display = ours_core.display
    saved_options = ours_core._orbkit_options
    try:
        ours_core.display = importlib.import_module(orbkit_module.__name__ + ".display").display
        ours_core._orbkit_options = importlib.import_module(orbkit_module.__name__ + ".options")
    except (ImportError, AttributeError):
        pass

    def restore():
        for obj, n, f in reversed(saved):
            setattr(obj, n, f)
        ours_core.grid = saved_grid
        ours_core.display = saved_display
        ours_core._orbkit_options = saved_options

    return restore
