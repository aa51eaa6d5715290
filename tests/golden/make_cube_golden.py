"""Generate tests/golden/h2o_gaussian_cube.npz from the reference's Gaussian cube test.

Run in a container that has the reference tree (read-only) and Cython:

    python tests/golden/make_cube_golden.py

This follows the reference's test test/grid_based/cube_files.py: H2O RHF/cc-pVDZ with a
spherical basis read from Gaussian's formatted checkpoint file
(test/outputs_for_testing/gaussian/h2o_rhf_sph.fchk) by the reference's reader, on the
3 x 3 x 3 regular grid of that test.  Stored next to the molecule
(orbkit_gb300.qcinfo.to_arrays) and the grid:

  * Gaussian's own values from the cube files that test compares against (written by
    cubegen, i.e. computed by a code independent of orbkit, 6 significant digits):
    cube_rho / cube_drho (h2o_rhf_sph_grad.cube), cube_lapl (h2o_rhf_sph_laplace.cube),
    cube_rho_valence (h2o_rhf_sph.cube: density without the core MO, as Gaussian writes
    it) and cube_homo (h2o_rhf_sph_mo.cube);
  * the unmodified reference's rho_compute outputs for the same quantities (ref_*),
    checked here against the cube values with that test's tolerances.
"""
import os
import sys

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)

import refpkg  # noqa: E402

from orbkit_gb300.qcinfo import to_arrays  # noqa: E402


def main():
    ok = refpkg.load()
    if ok is None:
        raise SystemExit("reference not available")
    from orbkit import grid, read
    from orbkit.core import rho_compute
    folder = os.path.join(refpkg.REF_ROOT, "orbkit/test/outputs_for_testing/gaussian")
    dx = 4.970736
    x = numpy.arange(3) * dx - 4.970736
    y = numpy.arange(3) * dx - 4.970736
    z = numpy.arange(3) * dx - 4.732975
    grid.x, grid.y, grid.z = x.copy(), y.copy(), z.copy()
    grid.is_initialized = True
    grid.is_regular = True
    grid.is_vector = False
    qc = read.main_read(os.path.join(folder, "h2o_rhf_sph.fchk"), all_mo=False)
    arrs = to_arrays(qc)
    arrs.update({"x": x, "y": y, "z": z})

    rho, drho = rho_compute(qc, drv="xyz", slice_length=0)
    _, _, lapl = rho_compute(qc, laplacian=True, slice_length=0)
    grad = numpy.genfromtxt(os.path.join(folder, "h2o_rhf_sph_grad.cube"), skip_header=9).reshape(-1, 4)
    cube_rho = grad[:, 0].reshape(rho.shape)
    cube_drho = numpy.moveaxis(grad[:, 1:], 1, 0).reshape((3,) + rho.shape)
    cube_lapl = numpy.genfromtxt(os.path.join(folder, "h2o_rhf_sph_laplace.cube"), skip_header=9).reshape(lapl.shape)

    nmo = len(qc.mo_spec)
    qc.mo_spec = qc.mo_spec[1:]  # Gaussian's "Total SCF Density" cube leaves out the core MO
    rho_val = rho_compute(qc, slice_length=0)
    cube_val = numpy.genfromtxt(os.path.join(folder, "h2o_rhf_sph.cube"), skip_header=9).reshape(rho_val.shape)
    homo = qc.mo_spec["homo"]
    qc.mo_spec = homo
    mo = rho_compute(qc, calc_mo=True, slice_length=0)
    cube_mo = numpy.genfromtxt(os.path.join(folder, "h2o_rhf_sph_mo.cube"), skip_header=10).reshape(mo.shape)
    homo_coeffs = numpy.asarray(homo.get_coeffs(), dtype=numpy.float64)

    def close(a, b, tol):
        # test/tools.py equal(): numpy.allclose(a, b, rtol=100 tol, atol=tol)
        assert numpy.allclose(a, b, rtol=tol * 1e2, atol=tol), numpy.abs(a - b).max()
    close(rho, cube_rho, 1e-5)
    close(drho, cube_drho, 1e-3)
    close(lapl, cube_lapl, 1e-5)
    close(rho_val, cube_val, 1e-5)
    close(mo, cube_mo, 1e-5)
    arrs.update({"cube_rho": cube_rho, "cube_drho": cube_drho, "cube_lapl": cube_lapl,
                 "cube_rho_valence": cube_val, "cube_homo": cube_mo, "ref_rho": rho, "ref_drho": drho,
                 "ref_lapl": lapl, "ref_rho_valence": rho_val, "ref_homo": mo, "homo_coeffs": homo_coeffs,
                 "nmo_all": numpy.array(nmo)})
    print("max |ref - cube|: rho %.2e drho %.2e lapl %.2e valence %.2e mo %.2e" % (
        numpy.abs(rho - cube_rho).max(), numpy.abs(drho - cube_drho).max(), numpy.abs(lapl - cube_lapl).max(),
        numpy.abs(rho_val - cube_val).max(), numpy.abs(mo - cube_mo).max()))
    numpy.savez_compressed(os.path.join(HERE, "h2o_gaussian_cube.npz"), **arrs)
    print("wrote", os.path.join(HERE, "h2o_gaussian_cube.npz"))


if __name__ == "__main__":
    main()
