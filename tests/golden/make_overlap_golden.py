"""Generate tests/golden/overlap.npz by running the reference's analytic integrals.

Run in a container that has the reference tree (read-only) and Cython:

    python tests/golden/make_overlap_golden.py

For the molecules of the grid fixtures (h2o_molden.npz: the reference's H2O molden
test file; small_cart.npz: Cartesian s/p/d; sph_fg_N.npz: spherical f/g shells with
a per-AO 'N' factor; normalized.npz: pre-normalised contractions) it stores, under
the fixture's name as prefix, what the unmodified reference
(orbkit/analytical_integrals.py, over its compiled cy_overlap extension built from
source by oracle/build_ref.py) returns for:

  S        get_ao_overlap(geo, geo, ao_spec)
  Sd       get_ao_overlap(geo, geo, ao_spec, drv=['x', 'y', 'z'])     (3 matrices)
  S2       get_ao_overlap(geo, geo2, ao_spec) with geo2 = geo + a seeded shift
  S2d      the same with drv=['x', 'y', 'z']
  Sket     get_ao_overlap(geo, geo, ao_spec, lxlylz_b=lxlylz + (0, 1, 0))
  dip      get_ao_dipole_matrix(qc, ['x', 'y', 'z'])                  (3 matrices)
  moom     get_mo_overlap_matrix(mo, mo, S)
  moom2    get_mo_overlap_matrix(mo, mo, S2)
  dipole   get_dipole_moment(qc) with nuclear charges `charges`
  geo2, charges, lxlylz_ket
"""
import os
import sys

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)

import refpkg  # noqa: E402

from orbkit_gb300.qcinfo import from_arrays  # noqa: E402

FIXTURES = ("h2o_molden", "small_cart", "sph_fg_N", "normalized")


def main():
    ok = refpkg.load()
    if ok is None:
        raise SystemExit("reference not available")
    from orbkit import analytical_integrals as ai
    from orbkit.tools import exp, lquant
    rng = numpy.random.default_rng(2024)
    out = {}
    for name in FIXTURES:
        d = numpy.load(os.path.join(HERE, name + ".npz"))
        qc = refpkg.to_reference_qc(ok, from_arrays(d))
        # shells listed in the default Cartesian order drop their explicit 'lxlylz'
        # list, as the reference's readers leave them (its get_ao_dipole_matrix
        # counts a shell's AOs from that list when present)
        for s in qc.ao_spec:
            if "lxlylz" in s and [tuple(r) for r in s["lxlylz"]] == list(exp[lquant[s["type"]]]):
                del s["lxlylz"]
        qc.ao_spec.update()
        geo = numpy.array(qc.geo_spec)
        charges = rng.integers(1, 10, len(geo)).astype(numpy.float64)
        qc.geo_info = numpy.array([["X", str(i + 1), "%d" % z] for i, z in enumerate(charges)])
        geo2 = geo + rng.uniform(-0.4, 0.4, geo.shape)
        lx_ket = numpy.array(qc.ao_spec.get_lxlylz(), dtype=numpy.intc)
        lx_ket[:, 1] += 1
        S = ai.get_ao_overlap(geo, geo, qc.ao_spec)
        S2 = ai.get_ao_overlap(geo, geo2, qc.ao_spec)
        mo = qc.mo_spec.get_coeffs()
        res = {
            "S": S,
            "Sd": numpy.array(ai.get_ao_overlap(geo, geo, qc.ao_spec, drv=["x", "y", "z"])),
            "S2": S2,
            "S2d": numpy.array(ai.get_ao_overlap(geo, geo2, qc.ao_spec, drv=["x", "y", "z"])),
            "Sket": ai.get_ao_overlap(geo, geo, qc.ao_spec, lxlylz_b=lx_ket),
            "dip": numpy.array(ai.get_ao_dipole_matrix(qc, component=["x", "y", "z"])),
            "moom": ai.get_mo_overlap_matrix(mo, mo, S),
            "moom2": ai.get_mo_overlap_matrix(mo, mo, S2),
            "dipole": ai.get_dipole_moment(qc),
            "geo2": geo2,
            "charges": charges,
            "lxlylz_ket": lx_ket,
        }
        for k, v in res.items():
            out["%s__%s" % (name, k)] = numpy.asarray(v)
        print(name, "nao", S.shape[0], "max |S - 1| on the diagonal", numpy.abs(numpy.diag(S) - 1).max())
    numpy.savez_compressed(os.path.join(HERE, "overlap.npz"), **out)
    print("wrote", os.path.join(HERE, "overlap.npz"))


if __name__ == "__main__":
    main()
