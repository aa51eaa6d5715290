"""Generate the golden fixtures under tests/golden/ by running the reference itself.

Run in a container that has the reference tree (read-only) and Cython:

    python tests/golden/make_golden.py

It builds the reference's extensions from source (oracle/build_ref.py), imports
the unmodified reference package (oracle/refpkg.py) and stores, for small inputs,
the inputs in portable array form (orbkit_gb300.qcinfo.to_arrays) next to the
reference's outputs:

  h2o_molden.npz   the reference's own test case (test/grid_based/rho_compute.py:13-43):
                   molpro/h2o_rhf_sph.molden on the 5x9x7 grid of adjust_to_geo(extend=2,
                   step=1); keys zero..four are the reference's golden arrays
                   (test/grid_based/refdata_rho_compute.npz) plus rho/delta_rho for
                   drv x,y,z,xy computed by the reference.
  small_cart.npz   the seeded 'small' molecule (Cartesian) on a 6x5x4 regular grid:
                   AOs and MOs for drv 0..9, rho, delta_rho for x,y,z,xx,xy,yz, Laplacian.
  sph_fg_N.npz     a seeded 3-atom molecule with f and g shells, spherical basis and a
                   per-AO 'N' factor, on a vector grid that includes the nuclei:
                   AOs for drv 0..9, MOs, rho, delta_rho (x,y,z), Laplacian.
  normalized.npz   the 'small' molecule with pre-normalised contractions (pnum < 0):
                   AOs for drv 0..3, rho, delta_rho (x,y,z).
"""
import os
import sys

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)

import refpkg  # noqa: E402

from orbkit_gb300 import synthetic  # noqa: E402
from orbkit_gb300.qcinfo import to_arrays  # noqa: E402

DRV_ALL = [None, "x", "y", "z", "xx", "yy", "zz", "xy", "xz", "yz"]


def ref_qc(ok, qc_mine):
    return refpkg.to_reference_qc(ok, qc_mine)


def regular(ok, x, y, z):
    g = ok.grid
    g.x, g.y, g.z = x.copy(), y.copy(), z.copy()
    g.is_initialized = True
    g.is_vector = False
    g.is_regular = True


def vector(ok, x, y, z):
    g = ok.grid
    g.x, g.y, g.z = x.copy(), y.copy(), z.copy()
    g.is_initialized = True
    g.is_vector = True
    g.is_regular = False


def outputs(ok, qc, drv_rho, drv_ao=DRV_ALL):
    core = ok.core
    out = {}
    out["ao"] = numpy.array([core.rho_compute(qc, calc_ao=True, drv=[d], slice_length=0)[0] for d in drv_ao])
    out["mo"] = core.rho_compute(qc, calc_mo=True, drv=drv_ao, slice_length=0)
    out["rho"], out["delta_rho"] = core.rho_compute(qc, drv=drv_rho, slice_length=0)
    out["laplacian"] = core.rho_compute(qc, laplacian=True, slice_length=0)[-1]
    return out


def main():
    ok = refpkg.load()
    if ok is None:
        raise SystemExit("reference not available")
    from orbkit import read

    # 1) the reference's own H2O test case
    qc = read.main_read(os.path.join(refpkg.REF_ROOT, "orbkit/test/outputs_for_testing/molpro/h2o_rhf_sph.molden"),
                        all_mo=True)
    ok.grid.delta_ = numpy.zeros(3)
    ok.grid.adjust_to_geo(qc, extend=2.0, step=1)
    ok.grid.grid_init(is_vector=False, force=True)
    x, y, z = ok.grid.x.copy(), ok.grid.y.copy(), ok.grid.z.copy()
    gold = numpy.load(os.path.join(refpkg.REF_ROOT, "orbkit/test/grid_based/refdata_rho_compute.npz"))
    rho, drho = ok.core.rho_compute(qc, drv=["x", "y", "z", "xy"], slice_length=0)
    arrs = to_arrays(qc)
    arrs.update({"x": x, "y": y, "z": z, "rho_xyz": rho, "delta_rho_xyzxy": drho})
    for k in ("zero", "one", "two", "three", "four"):
        arrs[k] = gold[k]
    numpy.savez_compressed(os.path.join(HERE, "h2o_molden.npz"), **arrs)

    # 2) the seeded small molecule, Cartesian, regular 6x5x4 grid
    d = synthetic.small()
    q = ref_qc(ok, d["qc"])
    x = numpy.linspace(-3.0, 2.5, 6)
    y = numpy.linspace(-2.0, 2.0, 5)
    z = numpy.linspace(-1.5, 2.7, 4)
    regular(ok, x, y, z)
    out = outputs(ok, q, ["x", "y", "z", "xx", "xy", "yz"])
    arrs = to_arrays(d["qc"])
    arrs.update({"x": x, "y": y, "z": z})
    arrs.update(out)
    numpy.savez_compressed(os.path.join(HERE, "small_cart.npz"), **arrs)

    # 3) spherical f/g basis with a per-AO 'N' factor on a vector grid through the nuclei
    rng = numpy.random.default_rng(11)
    geo = numpy.array([[0.0, 0.0, 0.0], [0.0, 1.4, 1.1], [1.2, -0.9, 0.3]])
    shells = []
    for ia, kinds in enumerate([["s", "p", "d", "f", "g"], ["s", "p"], ["s", "d", "f"]]):
        for lt in kinds:
            n = 2 if lt in "sp" else 1
            shells.append({"atom": ia, "type": lt, "pnum": n, "coeffs": synthetic._contraction(rng, lt, n)})
    from orbkit_gb300.orbitals import AOClass
    ao = AOClass(shells)
    ao.set_lm_dict(p=[1, 0])
    ao.update()
    ncart = len(ao.get_lxlylz())
    ao[0]["N"] = rng.uniform(0.8, 1.2, (ncart, 1))
    ao.update()
    mo = synthetic.build_mos(rng, geo, ao, 6)
    qsph = synthetic.make_qc(geo, ["O", "H", "C"], ao, mo)
    q = ref_qc(ok, qsph)
    pts = numpy.concatenate([geo, rng.uniform(-3, 3, (37, 3)), [[9.0, -8.0, 7.5]]]).T.copy()
    vector(ok, pts[0], pts[1], pts[2])
    out = outputs(ok, q, ["x", "y", "z"])
    arrs = to_arrays(qsph)
    arrs.update({"points": pts})
    arrs.update(out)
    numpy.savez_compressed(os.path.join(HERE, "sph_fg_N.npz"), **arrs)

    # 4) pre-normalised contractions (pnum < 0)
    d = synthetic.small()
    for s in d["qc"].ao_spec.data:
        s["pnum"] = -abs(s["pnum"])
    d["qc"].ao_spec.update()
    q = ref_qc(ok, d["qc"])
    x = numpy.linspace(-2.0, 2.0, 5)
    regular(ok, x, x + 0.1, x - 0.2)
    out = outputs(ok, q, ["x", "y", "z"], drv_ao=[None, "x", "y", "z"])
    arrs = to_arrays(d["qc"])
    arrs.update({"x": x, "y": x + 0.1, "z": x - 0.2})
    arrs.update(out)
    numpy.savez_compressed(os.path.join(HERE, "normalized.npz"), **arrs)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
