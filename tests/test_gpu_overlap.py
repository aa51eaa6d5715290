"""Analytic AO overlap on the GPU (okg_ao_overlap behind
orbkit_gb300.analytical_integrals, the counterpart of orbkit/analytical_integrals.py):
against the reference's own outputs for four molecules (tests/golden/overlap.npz:
overlap, ket derivatives, a second ket geometry, a ket exponent override, dipole
matrices, MO overlap matrices, dipole moment), and the raw Cartesian matrix against
the oracle's restatement of cy_overlap.aooverlap on the 200-atom basis."""
import numpy
import pytest

from helpers import GOLDEN, assert_fp64_close, load_golden

pytestmark = pytest.mark.gpu

FIXTURES = ("h2o_molden", "small_cart", "sph_fg_N", "normalized")


@pytest.fixture(scope="module")
def ai():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from orbkit_gb300 import build
    build.build()
    from orbkit_gb300 import analytical_integrals
    return analytical_integrals


@pytest.mark.parametrize("name", FIXTURES)
def test_against_reference_outputs(ai, name):
    qc, _ = load_golden(name + ".npz")
    g = numpy.load(GOLDEN + "/overlap.npz")
    G = {k.split("__", 1)[1]: g[k] for k in g.files if k.startswith(name + "__")}
    geo = numpy.asarray(qc.geo_spec)
    S = ai.get_ao_overlap(geo, geo, qc.ao_spec)
    assert_fp64_close(S, G["S"], name + " S")
    assert_fp64_close(numpy.array(ai.get_ao_overlap(geo, geo, qc.ao_spec, drv=["x", "y", "z"])), G["Sd"],
                      name + " dS")
    S2 = ai.get_ao_overlap(geo, G["geo2"], qc.ao_spec)
    assert_fp64_close(S2, G["S2"], name + " S(geo, geo2)")
    for k, d in enumerate("xyz"):
        assert_fp64_close(ai.get_ao_overlap(geo, G["geo2"], qc.ao_spec, drv=d), G["S2d"][k], name + " dS/d" + d)
    assert_fp64_close(ai.get_ao_overlap(geo, geo, qc.ao_spec, lxlylz_b=G["lxlylz_ket"]), G["Sket"],
                      name + " ket exponents")
    # the plan's ket exponents are restored for the next plain call
    assert_fp64_close(ai.get_ao_overlap(geo, geo, qc.ao_spec), G["S"], name + " S again")
    mo = qc.mo_spec.get_coeffs()
    assert_fp64_close(ai.get_mo_overlap_matrix(mo, mo, S), G["moom"], name + " MO overlap")
    assert_fp64_close(ai.get_mo_overlap_matrix(qc.mo_spec, qc.mo_spec, S2), G["moom2"], name + " MO overlap geo2")
    assert abs(ai.get_mo_overlap(mo[0], mo[0], S) - G["moom"][0, 0]) <= 1e-12 * abs(G["moom"][0, 0])
    assert_fp64_close(numpy.array(ai.get_ao_dipole_matrix(qc, component=["x", "y", "z"])), G["dip"],
                      name + " dipole matrices")
    qc.geo_info = [["X", str(i + 1), "%d" % z] for i, z in enumerate(G["charges"])]
    assert_fp64_close(ai.get_dipole_moment(qc), G["dipole"], name + " dipole moment")


def test_raw_cartesian_and_tensor_io(ai):
    """okg_ao_overlap raw = 1 is cy_overlap.aooverlap (no 'N', Cartesian) and CUDA
    tensors stay on the device."""
    import torch
    import okref
    qc, _ = load_golden("sph_fg_N.npz")
    geo = numpy.asarray(qc.geo_spec)
    lx = qc.ao_spec.get_lxlylz()
    plan = ai.overlap_plan(qc.ao_spec)
    gd = torch.tensor(geo, device="cuda")
    shifted = geo + numpy.array([0.3, -0.2, 0.1])
    for drv in range(4):
        raw = plan.run(gd, torch.tensor(shifted, device="cuda"), drv, raw=True).cpu().numpy()
        assert_fp64_close(raw, okref.aooverlap(geo, shifted, lx, lx, qc.ao_spec, drv), "raw drv=%d" % drv)
    t = ai.get_ao_overlap(gd, gd, qc.ao_spec)
    assert isinstance(t, torch.Tensor) and t.is_cuda
    assert_fp64_close(t.cpu().numpy(), okref.ao_overlap(geo, geo, qc.ao_spec), "tensor path")


def test_large_basis_against_oracle(ai):
    """200 atoms, 2420 Cartesian AOs (spherical output): every element of the raw
    matrix and its x derivative against the oracle."""
    import torch
    import okref
    from orbkit_gb300 import synthetic
    qc = synthetic.large()["qc"]
    geo = numpy.asarray(qc.geo_spec)
    lx = qc.ao_spec.get_lxlylz()
    plan = ai.overlap_plan(qc.ao_spec)
    gd = torch.tensor(geo, device="cuda")
    S0 = None
    for drv in (0, 1):
        raw = plan.run(gd, gd, drv, raw=True).cpu().numpy()
        ref = okref.aooverlap(geo, geo, lx, lx, qc.ao_spec, drv)
        assert_fp64_close(raw, ref, "large raw drv=%d" % drv)
        S0 = ref if drv == 0 else S0
    # spherical output: T S T^T of the oracle's Cartesian matrix (T as orbkit builds it)
    from orbkit_gb300.overlap import spherical_transform
    T = spherical_transform(qc.ao_spec)
    assert_fp64_close(ai.get_ao_overlap(geo, geo, qc.ao_spec), T @ S0 @ T.T, "large spherical")


def test_argument_errors(ai):
    qc, _ = load_golden("small_cart.npz")
    geo = numpy.asarray(qc.geo_spec)
    with pytest.raises(ValueError):
        ai.get_ao_overlap(geo, geo, qc.ao_spec, drv=4)  # second derivatives are not supported
    # as in orbkit, a string of several letters is a list of components
    two = ai.get_ao_overlap(geo, geo, qc.ao_spec, drv="xz")
    assert len(two) == 2
    assert_fp64_close(two[1], ai.get_ao_overlap(geo, geo, qc.ao_spec, drv="z"), "drv='xz'")
    with pytest.raises(ValueError):
        ai.get_ao_overlap(geo, geo, qc.ao_spec, lxlylz_b=numpy.zeros((3, 3), dtype=int))
    with pytest.raises(ValueError):
        ai.get_ao_overlap(geo[:1], geo, qc.ao_spec)
    with pytest.raises(TypeError):
        ai.get_ao_overlap(geo, geo, list(qc.ao_spec))


def test_analytic_property_kats(ai):
    """The reference's analytic-property tests on the GPU path (test/analytical_properties/
    analytical_integral_norm.py, dipole.py; tests/golden/h2o_analytic.npz): H2O RHF/UHF,
    Cartesian/spherical, read from molden, Gaussian log/fchk and aomix files -- AO and MO
    overlaps and dipole moments against the reference's values (FP64 bar), MOs orthonormal
    and dipoles equal to the quantum-chemistry programs' own values (those tests' tolerances)."""
    from helpers import analytic_cases, cube_close
    for name, qc, a in analytic_cases():
        geo = numpy.asarray(qc.geo_spec)
        S = ai.get_ao_overlap(geo, geo, qc.ao_spec)
        assert_fp64_close(S, a["aoom"], name + " AO overlap")
        C = qc.mo_spec.get_coeffs()
        for spin in ("alpha", "beta"):
            idx = a["idx_" + spin]
            if len(idx) == 0:
                continue
            moom = ai.get_mo_overlap_matrix(C[idx], C[idx], S)
            assert_fp64_close(moom, a["moom_" + spin], name + " MO overlap " + spin)
            if not name.endswith("moved"):  # moving one atom leaves the MOs non-orthogonal
                cube_close(moom, numpy.eye(len(idx)), 1e-4)
        dip = ai.get_dipole_moment(qc)
        assert numpy.abs(dip - a["dipole"]).max() <= 1e-12 * max(1.0, numpy.abs(a["dipole"]).max()), name
        cube_close(dip, a["kat_dip"], 1e-5)
