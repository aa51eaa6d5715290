"""Generate tests/golden/h2o_analytic.npz from the reference's analytic-integral tests.

Run in a container that has the reference tree (read-only) and Cython:

    python tests/golden/make_analytic_golden.py

The reference's test/analytical_properties/analytical_integral_norm.py and dipole.py read
H2O (RHF and UHF, Cartesian and spherical basis) from Molpro molden, Gaussian log and
fchk, and Turbomole aomix files, and check that the MOs are orthonormal under
get_ao_overlap / get_mo_overlap_matrix and that get_dipole_moment reproduces the dipole
moments the quantum-chemistry programs printed (dipole.py keeps them in `ref_dip`, plus
three more for the molden file with shifted and moved atoms).  The cclib-parsed variant
is left out (cclib is not installed).  For every case this stores, under the prefix
c<k>__: the molecule (orbkit_gb300.qcinfo.to_arrays), the nuclear charges of geo_info,
the MO indices of each spin, and the unmodified reference's outputs: the AO overlap, the
MO overlap matrix of each spin, and the dipole moment; and `kat_dip`, the programs' own
dipole moment parsed from dipole.py.
"""
import ast
import os
import re
import sys

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)

import refpkg  # noqa: E402

from orbkit_gb300.qcinfo import to_arrays  # noqa: E402

TESTS = ["h2o_rhf_cart", "h2o_rhf_sph", "h2o_uhf_cart", "h2o_uhf_sph"]
READERS = [("molden", "molpro", ".molden"), ("gaussian.log", "gaussian", ".inp.log"),
           ("gaussian.fchk", "gaussian", ".fchk"), ("aomix", "turbomole", "/aomix.in")]


def kat_dipoles(path):
    """ref_dip of dipole.py (program dipoles per folder) and the three checks of its
    molden section (original, shifted molecule, one atom moved)."""
    src = open(path).read()
    progs = ast.literal_eval(re.search(r"ref_dip = (\{.*?\})", src, re.S).group(1))
    old = ast.literal_eval(re.search(r"ref_dip = (\[[^\]]*\])\s*\nequal", src).group(1))
    moved = ast.literal_eval(re.findall(r"equal\(dip, (\[[^\]]*\])\)", src)[-1])
    return progs, old, moved


def main():
    ok = refpkg.load()
    if ok is None:
        raise SystemExit("reference not available")
    from orbkit import analytical_integrals as ai
    from orbkit import read
    out_dir = os.path.join(refpkg.REF_ROOT, "orbkit/test/outputs_for_testing")
    progs, old, moved = kat_dipoles(os.path.join(refpkg.REF_ROOT, "orbkit/test/analytical_properties/dipole.py"))
    arrs = {}
    cases = []

    def store(qc, name, kat):
        k = len(cases)
        d = to_arrays(qc)
        d["charges"] = numpy.array([float(r[2]) for r in qc.geo_info])
        aoom = ai.get_ao_overlap(qc.geo_spec, qc.geo_spec, qc.ao_spec)
        d["aoom"] = aoom
        for spin in ("alpha", "beta"):
            mos = qc.mo_spec["all_mo " + spin]
            idx = numpy.array([next(i for i, x in enumerate(qc.mo_spec.data) if x is m) for m in mos],
                              dtype=numpy.intc) if mos != [] else numpy.zeros(0, dtype=numpy.intc)
            d["idx_" + spin] = idx
            d["moom_" + spin] = (ai.get_mo_overlap_matrix(mos, mos, aoom) if len(idx) else numpy.zeros((0, 0)))
        d["dipole"] = ai.get_dipole_moment(qc, component=["x", "y", "z"])
        d["kat_dip"] = numpy.asarray(kat, dtype=numpy.float64)
        for key, v in d.items():
            arrs["c%d__%s" % (k, key)] = numpy.array(v)  # a copy: the molden case moves atoms afterwards
        cases.append(name)
        print(name, "dipole", d["dipole"], "program", kat)

    for t in TESTS:
        for itype, folder, ext in READERS:
            fid = os.path.join(out_dir, "%s/%s%s" % (folder, t, ext))
            if "uhf" in t and folder == "molpro":
                qc = read.main_read(fid, itype=itype, all_mo=True, spin=None, i_md=0, interactive=False)
                qc_b = read.main_read(fid, itype=itype, all_mo=True, spin=None, i_md=1, interactive=False)
                qc.mo_spec.extend(qc_b.mo_spec)
                qc.mo_spec.update()
            else:
                qc = read.main_read(fid, itype=itype, interactive=False, all_mo=True)
            store(qc, "%s %s" % (t, itype), progs[folder])
    # the molden checks of dipole.py: as read, shifted by (1, 1, 0), then atom 1 moved by (1, 1, 0)
    qc = read.main_read(os.path.join(out_dir, "molpro/h2o_rhf_sph.molden"), all_mo=True)
    store(qc, "h2o_rhf_sph molden as read", old)
    qc.geo_spec += numpy.array([1, 1, 0])
    store(qc, "h2o_rhf_sph molden shifted", old)
    qc.geo_spec[1] += numpy.array([1, 1, 0])
    store(qc, "h2o_rhf_sph molden atom moved", moved)
    arrs["names"] = numpy.array(cases)
    numpy.savez_compressed(os.path.join(HERE, "h2o_analytic.npz"), **arrs)
    print("wrote", os.path.join(HERE, "h2o_analytic.npz"), len(cases), "cases")


if __name__ == "__main__":
    main()
