"""Generate tests/golden/h3p_detci.npz by running the reference's detCI test case.

Run in a container that has the reference tree (read-only) and Cython:

    python tests/golden/make_detci_golden.py

This follows the reference's own test (test/detci/h3+.py): H3+ FCI/cc-pVTZ from
psi4 (test/detci/read/outputs_for_testing/h3+_fci_cc-pVTZ.out and its molden
file), all 42 MOs, the 51 x 51 x 1 grid from min (-2.5, -2.5, 0) to max (2.5, 2.5, 0)
in steps of 0.1, and for the three state pairs the determinant-comparison terms
(detci.occ_check.compare), the CI transition density (ci_core.rho), the flux
density (ci_core.jab) and its divergence from the MOs' second derivatives.  The
reference's extensions are built from source (oracle/build_ref.py) and the
unmodified reference is imported (oracle/refpkg.py); the values computed here
are checked against the reference's golden file test/detci/refdata_h3+.npz and
stored together with the molecule (orbkit_gb300.qcinfo.to_arrays), the grid and
the terms.

Harness-only shim: the reference's psi4 CI reader converts a one-element index
array with int() (orbkit/detci/ci_read/psi4.py:143), which numpy 2 rejects;
during that call numpy.argwhere returns an array subclass whose int() takes the
single element.
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


class _IntArray(numpy.ndarray):
    def __int__(self):
        return int(self.reshape(-1)[0])


def main():
    ok = refpkg.load()
    if ok is None:
        raise SystemExit("reference not available")
    from orbkit import core, detci, grid, main_read
    folder = os.path.join(refpkg.REF_ROOT, "orbkit/test/detci/read/outputs_for_testing")
    file_ci = os.path.join(folder, "h3+_fci_cc-pVTZ.out")
    qc = main_read(file_ci + ".default.molden", all_mo=True)
    argwhere = numpy.argwhere
    numpy.argwhere = lambda a: argwhere(a).view(_IntArray)
    try:
        qc, ci = detci.ci_read.main_ci_read(qc, file_ci, itype="psi4_detci", threshold=0.0)
    finally:
        numpy.argwhere = argwhere

    grid.min_ = [-2.5, -2.5, 0.0]
    grid.max_ = [2.5, 2.5, 0.0]
    grid.delta_ = [0.1, 0.1, 0.1]
    grid.grid_init()
    x, y, z = grid.x.copy(), grid.y.copy(), grid.z.copy()
    molist = core.rho_compute(qc, calc_mo=True, slice_length=1e2, drv=[None, "x", "y", "z", "xx", "yy", "zz"])
    mo, mod, mod2 = molist[0], molist[1:4], molist[-3:]

    arrs = to_arrays(qc)
    arrs.update({"x": x, "y": y, "z": z})
    rho_01, j_01, nabla_j_01 = [], [], []
    k = 0
    for a in range(len(ci)):
        for b in range(a + 1, len(ci)):
            zero, sing = detci.occ_check.compare(ci[a], ci[b], numproc=1)
            rho_01.append(detci.ci_core.rho(zero, sing, mo, slice_length=1e2))
            j_01.append(detci.ci_core.jab(zero, sing, mo, mod, slice_length=1e2))
            nabla_j_01.append(-numpy.sum(detci.ci_core.jab(zero, sing, mo, mod2, slice_length=1e2), axis=0))
            arrs["zero_coef_%d" % k] = numpy.array([c for cs in zero[0] for c in cs], dtype=numpy.float64)
            arrs["zero_orb_%d" % k] = numpy.array([j for js in zero[1] for j in js], dtype=numpy.int32)
            arrs["zero_len_%d" % k] = numpy.array([len(cs) for cs in zero[0]], dtype=numpy.int32)
            arrs["sing_coef_%d" % k] = numpy.array(sing[0], dtype=numpy.float64)
            arrs["sing_pair_%d" % k] = numpy.array(sing[1], dtype=numpy.int32).reshape(-1, 2)
            k += 1
    ref = numpy.load(os.path.join(refpkg.REF_ROOT, "orbkit/test/detci/refdata_h3+.npz"))
    for name, mine in (("rho_01", rho_01), ("j_01", j_01), ("nabla_j_01", nabla_j_01)):
        d = numpy.abs(numpy.array(mine) - ref[name]).max() / numpy.abs(ref[name]).max()
        print("%s: reference now vs its golden file, max normwise diff %.2e" % (name, d))
        assert d < 1e-12
        arrs[name] = ref[name]
    arrs["npairs"] = numpy.array(k)
    numpy.savez_compressed(os.path.join(HERE, "h3p_detci.npz"), **arrs)
    print("wrote", os.path.join(HERE, "h3p_detci.npz"))


if __name__ == "__main__":
    main()
