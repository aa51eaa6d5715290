"""The oracle pinned against the reference's golden vectors and (where the
reference tree is present) against the reference extension itself.  CPU only."""
import numpy
import pytest

import okref
from helpers import GOLDEN, cube_case, cube_close, is_x86, load_golden

DRV_ALL = [None, "x", "y", "z", "xx", "yy", "zz", "xy", "xz", "yz"]


def _same(a, b, what):
    """Bit-identical on x86-64 (the fixtures were made there); 1e-13 elsewhere (other libm)."""
    if is_x86():
        numpy.testing.assert_array_equal(a, b, err_msg=what)
    else:
        numpy.testing.assert_allclose(a, b, rtol=1e-13, atol=1e-13 * numpy.abs(b).max(), err_msg=what)


def test_reference_golden_h2o():
    """test/grid_based/rho_compute.py:13-43 of the reference: rho, Laplacian and the
    10-drv MO grids of H2O (molden, Cartesian) on the adjust_to_geo(2, 1) grid."""
    qc, d = load_golden("h2o_molden.npz")
    x, y, z = d["x"], d["y"], d["z"]
    drv = [None, "x", "y", "z", "xx", "xy", "xz", "yy", "yz", "zz"]
    _same(okref.rho_compute(qc, slice_length=0, x=x, y=y, z=z, is_vector=False), d["zero"], "rho")
    _same(okref.rho_compute(qc, slice_length=11, x=x, y=y, z=z, is_vector=False), d["one"], "rho sliced")
    _same(okref.rho_compute(qc, laplacian=True, slice_length=0, x=x, y=y, z=z, is_vector=False)[-1], d["two"],
          "laplacian")
    _same(okref.rho_compute_no_slice(qc, laplacian=True, x=x, y=y, z=z, is_vector=False)[-1], d["three"],
          "laplacian no_slice")
    _same(okref.rho_compute(qc, calc_mo=True, drv=drv, slice_length=0, x=x, y=y, z=z, is_vector=False), d["four"],
          "drv MOs")
    r, dr = okref.rho_compute(qc, drv=["x", "y", "z", "xy"], slice_length=0, x=x, y=y, z=z, is_vector=False)
    _same(r, d["rho_xyz"], "rho")
    _same(dr, d["delta_rho_xyzxy"], "delta_rho x,y,z,xy")


@pytest.mark.parametrize("name,drv_rho", [("small_cart.npz", ["x", "y", "z", "xx", "xy", "yz"]),
                                          ("normalized.npz", ["x", "y", "z"])])
def test_golden_regular(name, drv_rho):
    qc, d = load_golden(name)
    x, y, z = d["x"], d["y"], d["z"]
    drv_ao = DRV_ALL[:d["ao"].shape[0]]
    for k, dv in enumerate(drv_ao):
        _same(okref.rho_compute(qc, calc_ao=True, drv=[dv], x=x, y=y, z=z, is_vector=False)[0], d["ao"][k],
              "ao drv=%s" % dv)
    _same(okref.rho_compute(qc, calc_mo=True, drv=drv_ao, x=x, y=y, z=z, is_vector=False), d["mo"], "mo")
    r, dr = okref.rho_compute(qc, drv=drv_rho, x=x, y=y, z=z, is_vector=False)
    _same(r, d["rho"], "rho")
    _same(dr, d["delta_rho"], "delta_rho")
    _same(okref.rho_compute(qc, laplacian=True, x=x, y=y, z=z, is_vector=False)[-1], d["laplacian"], "laplacian")


def test_golden_spherical_fg_renorm():
    """Spherical basis with f and g shells and a per-AO 'N' factor, vector grid through the nuclei."""
    qc, d = load_golden("sph_fg_N.npz")
    x, y, z = d["points"]
    for k, dv in enumerate(DRV_ALL):
        _same(okref.rho_compute(qc, calc_ao=True, drv=[dv], x=x, y=y, z=z)[0], d["ao"][k], "ao drv=%s" % dv)
    _same(okref.rho_compute(qc, calc_mo=True, drv=DRV_ALL, x=x, y=y, z=z), d["mo"], "mo")
    r, dr = okref.rho_compute(qc, drv=["x", "y", "z"], x=x, y=y, z=z)
    _same(r, d["rho"], "rho")
    _same(dr, d["delta_rho"], "delta_rho")
    _same(okref.rho_compute(qc, laplacian=True, x=x, y=y, z=z)[-1], d["laplacian"], "laplacian")


def test_threaded_driver_matches_sliced():
    qc, d = load_golden("small_cart.npz")
    pts = okref.grid2vector(d["x"], d["y"], d["z"])
    r, dr = okref.rho_threads(qc, *pts, drv=["x", "y", "z", "xx", "xy", "yz"], slice_length=7, nthreads=3)
    _same(r, d["rho"].reshape(-1), "threads rho")
    _same(dr, d["delta_rho"].reshape(6, -1), "threads delta_rho")


def test_mixed_derivative_formula_is_the_references():
    """drv 7..9 reproduce orbkit's formula (c_support.c:121-168), not the exact
    mixed derivative: for p_x, d2/dxdy differs from a finite difference of d/dx."""
    a, X, Y, Z = 0.7, 0.3, -0.4, 0.2
    ref = okref.lib().okref_get_ao_xyz(X, Y, Z, 1, 0, 0, a, 7)
    assert ref == pytest.approx(4 * a * a * X * X * Y + 1.0, rel=1e-15)
    exact = (1 - 2 * a * X * X) * (-2 * a * Y)
    assert abs(ref - exact) > 0.1


def _reference():
    import refpkg
    return refpkg.load()


@pytest.fixture(scope="module")
def ref():
    ok = _reference()
    if ok is None:
        pytest.skip("reference tree not available")
    return ok


def test_oracle_vs_reference_extension(ref):
    """Bit-identical AO / MO / density against the reference's compiled cy_core on
    the seeded mid-size molecule (random points)."""
    from orbkit_gb300 import synthetic
    from refpkg import to_reference_qc as ref_qc
    d = synthetic.mid()
    q = ref_qc(ref, d["qc"])
    rng = numpy.random.default_rng(5)
    x, y, z = rng.uniform(-10, 10, (3, 300))
    for dv in DRV_ALL:
        a = ref.core.ao_creator(q.geo_spec, q.ao_spec, drv=dv, x=x, y=y, z=z, is_vector=True)
        b = okref.ao_creator(d["qc"].geo_spec, d["qc"].ao_spec, drv=dv, x=x, y=y, z=z)
        numpy.testing.assert_array_equal(a, b, err_msg="ao drv=%s" % dv)
    R = ref.core.rho_compute_no_slice(q, drv=["x", "y", "z", "xy", "zz"], x=x, y=y, z=z, is_vector=True)
    O = okref.rho_compute_no_slice(d["qc"], drv=["x", "y", "z", "xy", "zz"], x=x, y=y, z=z)
    numpy.testing.assert_array_equal(R[0], O[0])
    numpy.testing.assert_array_equal(R[1], O[1])
    t = okref.rho_threads(d["qc"], x, y, z, drv=["x", "y", "z", "xy", "zz"], slice_length=64, nthreads=2)
    numpy.testing.assert_array_equal(R[0], t[0])
    numpy.testing.assert_array_equal(R[1], t[1])


def test_tables_and_flattening_vs_reference(ref):
    from orbkit import tools as rtools
    from orbkit.orbitals import AOClass as RAO
    from orbkit_gb300 import synthetic, tools
    for l in range(5):
        assert [tuple(c) for c in rtools.exp[l]] == [tuple(c) for c in tools.cartesian_order[l]]
        for m in range(-l, l + 1):
            a = rtools.get_cart2sph(l, m)
            b = tools.get_cart2sph(l, m)
            assert [tuple(c) for c in a[0]] == [tuple(c) for c in b[0]]
            numpy.testing.assert_array_equal(numpy.array(a[1]) * a[2], numpy.array(b[1]) * b[2])
    assert rtools.lquant == tools.lquant
    d = synthetic.mid()
    rao = RAO(seq=[dict(s) for s in d["qc"].ao_spec.data])
    rao.update()
    for g in ("get_lxlylz", "get_nlxlylz_per_cont", "get_prim_coeffs", "get_nprim_per_cont",
              "get_assign_cont_to_atoms", "get_normalized", "get_assign_lxlylz_to_cont"):
        numpy.testing.assert_array_equal(getattr(d["qc"].ao_spec, g)(), getattr(rao, g)(), err_msg=g)


def test_overlap_vs_reference(ref):
    from orbkit import analytical_integrals as ai
    from orbkit_gb300 import overlap, synthetic
    from refpkg import to_reference_qc as ref_qc
    for d in (synthetic.small(), synthetic.mid()):
        q = ref_qc(ref, d["qc"])
        S_ref = ai.get_ao_overlap(q.geo_spec, q.geo_spec, q.ao_spec)
        S = overlap.ao_overlap(d["qc"].geo_spec, d["qc"].ao_spec)
        numpy.testing.assert_allclose(S, S_ref, atol=1e-13)


def test_detci_golden():
    """CI transition densities, flux densities and their divergence of the reference's
    H3+ FCI test (test/detci/h3+.py): MO grids from the oracle, the detCI loops
    restated, against the reference's golden file (refdata_h3+.npz)."""
    import okref
    from helpers import detci_terms
    qc, d = load_golden("h3p_detci.npz")
    x, y, z = d["x"], d["y"], d["z"]
    mo = okref.rho_compute_no_slice(qc, calc_mo=True, drv=[None, "x", "y", "z", "xx", "yy", "zz"], x=x, y=y, z=z,
                                    is_vector=False)
    # the reference test runs its drivers with slice_length=1e2 on 51 x 51 = 2601 points:
    # its slicing leaves the last point at 0 (orbkit/detci/ci_core.py:120-125)
    assert okref.ci_covered(51 * 51, 1e2) == 2600
    for k in range(int(d["npairs"])):
        zero, sing = detci_terms(d, k)
        r = okref.ci_driver(okref.ci_rho, zero, sing, mo[0], slice_length=1e2)
        j = okref.ci_driver(okref.ci_jab, zero, sing, mo[0], mo[1:4], slice_length=1e2)
        nj = -okref.ci_driver(okref.ci_jab, zero, sing, mo[0], mo[4:7], slice_length=1e2).sum(axis=0)
        for name, a, b in (("rho", r, d["rho_01"][k]), ("j", j, d["j_01"][k]), ("nabla j", nj, d["nabla_j_01"][k])):
            assert numpy.abs(a - b).max() <= 1e-14 * numpy.abs(b).max(), (k, name, numpy.abs(a - b).max())
        assert d["rho_01"][k].reshape(-1)[-1] == 0.0 and okref.ci_rho(zero, sing, mo[0]).reshape(-1)[-1] != 0.0


OVERLAP_FIXTURES = ("h2o_molden", "small_cart", "sph_fg_N", "normalized")


@pytest.mark.parametrize("name", OVERLAP_FIXTURES)
def test_overlap_golden(name):
    """Analytic AO overlap, its ket derivatives, a second ket geometry, a ket exponent
    override, dipole matrices, MO overlap matrices and the dipole moment: the oracle
    against the reference's outputs (tests/golden/overlap.npz)."""
    qc, _ = load_golden(name + ".npz")
    g = numpy.load(GOLDEN + "/overlap.npz")
    G = {k.split("__", 1)[1]: g[k] for k in g.files if k.startswith(name + "__")}
    geo = qc.geo_spec
    S = okref.ao_overlap(geo, geo, qc.ao_spec)
    _same(S, G["S"], "S")
    _same(numpy.array(okref.ao_overlap(geo, geo, qc.ao_spec, drv=["x", "y", "z"])), G["Sd"], "dS")
    S2 = okref.ao_overlap(geo, G["geo2"], qc.ao_spec)
    _same(S2, G["S2"], "S(geo, geo2)")
    _same(numpy.array(okref.ao_overlap(geo, G["geo2"], qc.ao_spec, drv=["x", "y", "z"])), G["S2d"], "dS(geo, geo2)")
    _same(okref.ao_overlap(geo, geo, qc.ao_spec, lxlylz_b=G["lxlylz_ket"]), G["Sket"], "S ket exponents")
    mo = qc.mo_spec.get_coeffs()
    _same(okref.mo_overlap_matrix(mo, mo, S), G["moom"], "MO overlap")
    _same(okref.mo_overlap_matrix(mo, mo, S2), G["moom2"], "MO overlap (geo, geo2)")
    D = numpy.array([okref.ao_dipole_matrix(qc, c) for c in "xyz"])
    _same(D, G["dip"], "dipole matrices")
    _same(okref.dipole_moment(qc, G["charges"]), G["dipole"], "dipole moment")


def test_gaussian_cube_golden():
    """The reference's test/grid_based/cube_files.py: H2O with a spherical basis from
    Gaussian's fchk on a 3x3x3 grid through the O nucleus, against Gaussian's own cube
    values (cubegen: rho, grad rho, Laplacian, valence density, HOMO) with that test's
    tolerances, and against the reference's outputs bit for bit."""
    qc, qv, qh, d = cube_case()
    kw = dict(x=d["x"], y=d["y"], z=d["z"], is_vector=False)
    rho, drho = okref.rho_compute(qc, drv=["x", "y", "z"], slice_length=0, **kw)
    lapl = okref.rho_compute(qc, laplacian=True, slice_length=0, **kw)[-1]
    val = okref.rho_compute(qv, slice_length=0, **kw)
    mo = okref.rho_compute(qh, calc_mo=True, slice_length=0, **kw)
    for name, a, tol in (("rho", rho, 1e-5), ("drho", drho, 1e-3), ("lapl", lapl, 1e-5),
                         ("rho_valence", val, 1e-5), ("homo", mo, 1e-5)):
        cube_close(a, d["cube_" + name], tol)
        _same(a, d["ref_" + name], name)


def test_detci_matrix_folding_matches_term_sums():
    """Host side of the detCI quadratic forms (orbkit_gb300.detci.density_matrix /
    flux_matrix and the matrices handed to okg_ci_rho_matrix / okg_ci_flux_matrix),
    evaluated with numpy as the kernels define them, against the oracle's term-order
    sums of orbkit's loops: the three state pairs of the H3+ test on seeded MO grids."""
    from helpers import detci_terms
    from orbkit_gb300 import detci
    d = numpy.load(GOLDEN + "/h3p_detci.npz")
    rng = numpy.random.default_rng(3)
    nmo = 42
    mo = rng.standard_normal((nmo, 300))
    dr = rng.standard_normal((3, nmo, 300))
    for k in range(int(d["npairs"])):
        zero, sing = detci_terms(d, k)
        M = detci.density_matrix(zero, sing, nmo)
        S = M + M.T
        S[numpy.diag_indices(nmo)] = numpy.diag(M)
        qt = numpy.tril(S)  # row b: coefficients of MO_a, a <= b
        rho = numpy.einsum("bp,ba,ap->p", mo, qt, mo)
        r0 = okref.ci_rho(zero, sing, mo)
        assert numpy.abs(rho - r0).max() <= 1e-12 * numpy.abs(r0).max()
        C = detci.flux_matrix(sing, nmo)
        for Q, scale, fn in ((C - C.T, -0.5, okref.ci_jab), (C, 1.0, okref.ci_a_nabla_b)):
            j = scale * numpy.einsum("dbp,ba,ap->dp", dr, Q.T, mo)
            j0 = fn(zero, sing, mo, dr)
            assert numpy.abs(j - j0).max() <= 1e-12 * numpy.abs(j0).max()
    # index checks happen on the host
    with pytest.raises(IndexError):
        detci.density_matrix([[[1.0]], [[nmo]]], [[], []], nmo)


def test_atom2mo_and_lc_match_reference(ref):
    """get_atom2mo / get_lc of orbkit_gb300.analytical_integrals against the reference's
    (orbkit/analytical_integrals.py:442-505) for Cartesian and spherical fixtures."""
    from orbkit import analytical_integrals as ai_ref
    from orbkit_gb300 import analytical_integrals as ai
    from refpkg import to_reference_qc
    from orbkit.tools import exp, lquant
    for name in ("small_cart.npz", "h2o_molden.npz", "sph_fg_N.npz"):
        qc, _ = load_golden(name)
        q = to_reference_qc(ref, qc)
        for s in q.ao_spec:
            if "lxlylz" in s and [tuple(r) for r in s["lxlylz"]] == list(exp[lquant[s["type"]]]):
                del s["lxlylz"]
        q.ao_spec.update()
        a_ref = ai_ref.get_atom2mo(q)
        numpy.testing.assert_array_equal(ai.get_atom2mo(qc), a_ref)
        for atoms in (0, [0, 2], [1]):
            numpy.testing.assert_array_equal(ai.get_lc(atoms, a_ref), ai_ref.get_lc(atoms, a_ref))
            numpy.testing.assert_array_equal(ai.get_lc(atoms, a_ref, strict=True),
                                             ai_ref.get_lc(atoms, a_ref, strict=True))


def test_analytic_integral_kats():
    """The reference's analytic-property tests (test/analytical_properties/
    analytical_integral_norm.py, dipole.py): H2O RHF/UHF, Cartesian/spherical, from
    molden, Gaussian log/fchk and aomix files.  The oracle reproduces the reference's AO
    overlap, MO overlap matrices and dipole moments (tests/golden/h2o_analytic.npz), the MOs
    are orthonormal and the dipoles match the quantum-chemistry programs' own values,
    with the tolerances of those tests."""
    from helpers import analytic_cases
    for name, qc, a in analytic_cases():
        geo = qc.geo_spec
        S = okref.ao_overlap(geo, geo, qc.ao_spec)
        _same(S, a["aoom"], name + " AO overlap")
        C = qc.mo_spec.get_coeffs()
        for spin in ("alpha", "beta"):
            idx = a["idx_" + spin]
            if len(idx) == 0:
                continue
            moom = okref.mo_overlap_matrix(C[idx], C[idx], S)
            _same(moom, a["moom_" + spin], name + " MO overlap " + spin)
            if not name.endswith("moved"):  # moving one atom leaves the MOs non-orthogonal
                cube_close(moom, numpy.eye(len(idx)), 1e-4)
        dip = okref.dipole_moment(qc, a["charges"])
        _same(dip, a["dipole"], name + " dipole")
        cube_close(dip, a["kat_dip"], 1e-5)


def test_install_routes_and_restores(ref):
    """orbkit_gb300.install swaps the reference package's grid, detCI, extras and
    analytic-integral functions (module and package level) and restores them."""
    import orbkit_gb300
    from orbkit_gb300 import analytical_integrals, core, detci, extras
    import orbkit.analytical_integrals as ai_ref
    import orbkit.detci.ci_core as ci_ref
    originals = {
        (ref.core, "rho_compute"): ref.core.rho_compute,
        (ref, "rho_compute"): ref.rho_compute,
        (ref.extras, "calc_jmo"): ref.extras.calc_jmo,
        (ref, "calc_jmo"): ref.calc_jmo,
        (ci_ref, "jab"): ci_ref.jab,
        (ai_ref, "get_ao_overlap"): ai_ref.get_ao_overlap,
        (ai_ref, "get_dipole_moment"): ai_ref.get_dipole_moment,
        (ref, "get_dipole_moment"): ref.get_dipole_moment,
    }
    restore = orbkit_gb300.install(ref)
    try:
        assert ref.core.rho_compute is core.rho_compute and ref.rho_compute is core.rho_compute
        assert ref.extras.calc_jmo is extras.calc_jmo and ref.calc_jmo is extras.calc_jmo
        assert ci_ref.rho is detci.rho and ci_ref.jab is detci.jab and ci_ref.a_nabla_b is detci.a_nabla_b
        assert ai_ref.get_ao_overlap is analytical_integrals.get_ao_overlap
        assert ref.get_dipole_moment is analytical_integrals.get_dipole_moment
        assert core.grid is ref.grid
    finally:
        restore()
    for (obj, name), f in originals.items():
        assert getattr(obj, name) is f, name


@pytest.mark.parametrize("name", ["small_cart.npz", "sph_fg_N.npz", "normalized.npz", "h2o_gaussian_cube.npz"])
def test_oracle_vs_reference_extension_fixtures(ref, name):
    """Bit-identical AOs (all drv codes), MOs and rho / grad rho / Laplacian against the
    reference's compiled cy_core on the fixture molecules (Cartesian, spherical f/g with
    'N', pre-normalised, Gaussian fchk) at seeded random points."""
    from refpkg import to_reference_qc as ref_qc
    qc, _ = load_golden(name)
    q = ref_qc(ref, qc)
    rng = numpy.random.default_rng(len(name))
    x, y, z = rng.uniform(-4, 4, (3, 257))
    for dv in DRV_ALL:
        a = ref.core.ao_creator(q.geo_spec, q.ao_spec, drv=dv, x=x, y=y, z=z, is_vector=True)
        b = okref.ao_creator(qc.geo_spec, qc.ao_spec, drv=dv, x=x, y=y, z=z)
        _same(b, a, "%s ao drv=%s" % (name, dv))
    R = ref.core.rho_compute_no_slice(q, drv=["x", "y", "z", "xx", "yz"], laplacian=True, x=x, y=y, z=z,
                                      is_vector=True)
    O = okref.rho_compute_no_slice(qc, drv=["x", "y", "z", "xx", "yz"], laplacian=True, x=x, y=y, z=z)
    for k in range(len(R)):
        _same(O[k], R[k], "%s rho_compute_no_slice output %d" % (name, k))


def test_detci_oracle_vs_reference_extension(ref):
    """The oracle's detCI loops against the reference's compiled cy_ci (get_rho, get_jab,
    get_a_nabla_b) on the H3+ terms with seeded MO grids: bit for bit."""
    from helpers import detci_terms
    from orbkit.detci import cy_ci
    d = numpy.load(GOLDEN + "/h3p_detci.npz")
    rng = numpy.random.default_rng(9)
    mo = numpy.ascontiguousarray(rng.standard_normal((42, 211)))
    dr = numpy.ascontiguousarray(rng.standard_normal((3, 42, 211)))
    for k in range(int(d["npairs"])):
        zero, sing = detci_terms(d, k)
        _same(okref.ci_rho(zero, sing, mo), cy_ci.get_rho(0, 211, zero, sing, mo), "rho %d" % k)
        _same(okref.ci_jab(zero, sing, mo, dr), cy_ci.get_jab(0, 211, zero, sing, mo, dr), "jab %d" % k)
        _same(okref.ci_a_nabla_b(zero, sing, mo, dr), cy_ci.get_a_nabla_b(0, 211, zero, sing, mo, dr),
              "a_nabla_b %d" % k)


def test_overlap_oracle_vs_reference_extension(ref):
    """okref_aooverlap against the reference's compiled cy_overlap.aooverlap on the
    mid-size molecule: plain, the three ket derivatives and a second ket geometry."""
    from orbkit import cy_overlap
    from orbkit_gb300 import synthetic
    qc = synthetic.mid()["qc"]
    ao = qc.ao_spec
    geo = numpy.ascontiguousarray(qc.geo_spec, dtype=numpy.float64)
    geo2 = numpy.ascontiguousarray(geo + numpy.random.default_rng(1).uniform(-0.3, 0.3, geo.shape))
    lx = numpy.ascontiguousarray(ao.get_lxlylz(), dtype=numpy.intc)
    args = (numpy.ascontiguousarray(ao.get_nlxlylz_per_cont(), dtype=numpy.intc),
            numpy.ascontiguousarray(ao.get_prim_coeffs(), dtype=numpy.float64),
            numpy.ascontiguousarray(ao.get_nprim_per_cont(), dtype=numpy.intc),
            numpy.ascontiguousarray(ao.get_assign_cont_to_atoms(), dtype=numpy.intc))
    for gb in (geo, geo2):
        for drv in range(4):
            r = cy_overlap.aooverlap(geo, gb, lx, lx, *args, drv, int(ao.get_normalized()))
            _same(okref.aooverlap(geo, gb, lx, lx, ao, drv), r, "aooverlap drv=%d" % drv)


def test_argument_errors_match_reference(ref):
    """Invalid derivative selectors and mismatched grid vectors raise the reference's
    exception types and messages, before any device work (orbkit/tools.py:225-239,
    orbkit/core.py:79-80)."""
    from orbkit_gb300 import core
    from refpkg import to_reference_qc
    qc, _ = load_golden("small_cart.npz")
    q = to_reference_qc(ref, qc)
    x = numpy.linspace(-1, 1, 3)
    cases = [dict(drv="q", x=x, y=x, z=x), dict(drv=11, x=x, y=x, z=x), dict(drv=None, x=x, y=x[:2], z=x)]
    for kw in cases:
        with pytest.raises(Exception) as e_ref:
            ref.core.ao_creator(q.geo_spec, q.ao_spec, is_vector=True, **kw)
        with pytest.raises(Exception) as e_ours:
            core.ao_creator(qc.geo_spec, qc.ao_spec, is_vector=True, **kw)
        assert type(e_ours.value) is type(e_ref.value), kw
        assert str(e_ours.value) == str(e_ref.value), kw


def test_overlap_argument_errors_match_reference(ref):
    """get_ao_overlap's argument checks raise the reference's exceptions and messages
    before any device work (orbkit/analytical_integrals.py:66-97)."""
    from orbkit import analytical_integrals as ai_ref
    from orbkit_gb300 import analytical_integrals as ai
    from refpkg import to_reference_qc
    qc, _ = load_golden("small_cart.npz")
    q = to_reference_qc(ref, qc)
    geo = numpy.asarray(qc.geo_spec)
    cases = [dict(drv=4), dict(lxlylz_b=numpy.zeros((3, 3), dtype=int)), dict(drv="q")]
    for kw in cases:
        with pytest.raises(Exception) as e_ref:
            ai_ref.get_ao_overlap(geo, geo, q.ao_spec, **kw)
        with pytest.raises(Exception) as e_ours:
            ai.get_ao_overlap(geo, geo, qc.ao_spec, **kw)
        assert type(e_ours.value) is type(e_ref.value), kw
        assert str(e_ours.value) == str(e_ref.value), kw
    with pytest.raises(TypeError):
        ai.get_ao_overlap(geo, geo, list(qc.ao_spec))
