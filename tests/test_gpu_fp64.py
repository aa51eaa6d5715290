"""FP64 GPU path against the reference's golden outputs and the CPU oracle.

Parity bar: |gpu - ref| <= 1e-12 |ref| + 1e-13 max|ref| elementwise (helpers.FP64_*).
"""
import ctypes

import numpy
import pytest

from helpers import assert_fp64_close, cube_case, cube_close, load_golden

pytestmark = pytest.mark.gpu

DRV_ALL = [None, "x", "y", "z", "xx", "yy", "zz", "xy", "xz", "yz"]


@pytest.fixture(scope="module")
def core():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from orbkit_gb300 import build
    build.build()
    from orbkit_gb300 import core as c
    return c


def _check_outputs(core, qc, d, x, y, z, is_vector, drv_rho, tag):
    drv_ao = DRV_ALL[:d["ao"].shape[0]]
    for k, dv in enumerate(drv_ao):
        a = core.ao_creator(qc.geo_spec, qc.ao_spec, drv=dv, x=x, y=y, z=z, is_vector=is_vector)
        assert_fp64_close(a, d["ao"][k], "%s ao drv=%s" % (tag, dv))
    mo = core.rho_compute_no_slice(qc, calc_mo=True, drv=drv_ao, x=x, y=y, z=z, is_vector=is_vector)
    assert_fp64_close(mo, d["mo"], tag + " mo")
    r, dr = core.rho_compute_no_slice(qc, drv=drv_rho, x=x, y=y, z=z, is_vector=is_vector)
    assert_fp64_close(r, d["rho"], tag + " rho")
    assert_fp64_close(dr, d["delta_rho"], tag + " delta_rho")
    lap = core.rho_compute_no_slice(qc, laplacian=True, x=x, y=y, z=z, is_vector=is_vector)[-1]
    assert_fp64_close(lap, d["laplacian"], tag + " laplacian")


def test_golden_small_cartesian(core):
    qc, d = load_golden("small_cart.npz")
    _check_outputs(core, qc, d, d["x"], d["y"], d["z"], False, ["x", "y", "z", "xx", "xy", "yz"], "small")


def test_golden_spherical_fg_renorm(core):
    qc, d = load_golden("sph_fg_N.npz")
    x, y, z = d["points"]
    _check_outputs(core, qc, d, x, y, z, True, ["x", "y", "z"], "sph")


def test_golden_normalized(core):
    qc, d = load_golden("normalized.npz")
    _check_outputs(core, qc, d, d["x"], d["y"], d["z"], False, ["x", "y", "z"], "normalized")


def test_golden_reference_h2o(core):
    """The reference's own test (test/grid_based/rho_compute.py) through the module-global grid."""
    from orbkit_gb300 import grid
    qc, d = load_golden("h2o_molden.npz")
    grid.set_grid(d["x"], d["y"], d["z"], is_vector=False)
    drv = [None, "x", "y", "z", "xx", "xy", "xz", "yy", "yz", "zz"]
    assert_fp64_close(core.rho_compute(qc, slice_length=0), d["zero"], "rho")
    assert_fp64_close(core.rho_compute(qc, numproc=2), d["one"], "rho numproc")
    assert_fp64_close(core.rho_compute(qc, laplacian=True, slice_length=0)[-1], d["two"], "laplacian")
    assert_fp64_close(core.rho_compute(qc, laplacian=True, numproc=0)[-1], d["three"], "laplacian no_slice")
    assert_fp64_close(core.rho_compute(qc, calc_mo=True, drv=drv, slice_length=0), d["four"], "drv MOs")
    r, dr = core.rho_compute(qc, drv=["x", "y", "z", "xy"])
    assert_fp64_close(r, d["rho_xyz"], "rho")
    assert_fp64_close(dr, d["delta_rho_xyzxy"], "delta_rho")
    # vector form of the same grid
    grid.grid2vector()
    r2 = core.rho_compute(qc)
    assert_fp64_close(r2, d["zero"].reshape(-1), "rho vector grid")
    grid.reset_grid()


def test_golden_gaussian_cube(core):
    """The reference's test/grid_based/cube_files.py: H2O, spherical basis from Gaussian's
    fchk, 3x3x3 grid through the O nucleus -- against the reference's outputs (FP64 bar)
    and Gaussian's own cube values (that test's tolerances)."""
    qc, qv, qh, d = cube_case()
    kw = dict(x=d["x"], y=d["y"], z=d["z"], is_vector=False)
    rho, drho = core.rho_compute_no_slice(qc, drv=["x", "y", "z"], **kw)
    lapl = core.rho_compute_no_slice(qc, laplacian=True, **kw)[-1]
    val = core.rho_compute_no_slice(qv, **kw)
    mo = core.rho_compute_no_slice(qh, calc_mo=True, **kw)
    for name, a, tol in (("rho", rho, 1e-5), ("drho", drho, 1e-3), ("lapl", lapl, 1e-5),
                         ("rho_valence", val, 1e-5), ("homo", mo, 1e-5)):
        assert_fp64_close(a, d["ref_" + name], "cube case " + name)
        cube_close(a, d["cube_" + name], tol)


def test_small_full_grid_vs_oracle(core):
    """The 3-atom workload on its full 80^3 grid: rho and grad rho."""
    import okref
    from orbkit_gb300 import synthetic
    w = synthetic.small()
    qc = w["qc"]
    x, y, z = w["grid"]
    r, dr = core.rho_compute_no_slice(qc, drv=["x", "y", "z"], x=x, y=y, z=z, is_vector=False)
    pts = okref.grid2vector(x, y, z)
    ro, dro = okref.rho_threads(qc, *pts, drv=["x", "y", "z"], slice_length=4096)
    assert_fp64_close(r.reshape(-1), ro, "rho")
    assert_fp64_close(dr.reshape(3, -1), dro, "grad rho")


def test_mid_subgrid_vs_oracle(core):
    """The 20-atom workload (180 AOs, 40 MOs): a 24x20x16 block of its 160^3 grid, and
    a ragged run of flattened points through the regular-grid offset path."""
    import okref
    from orbkit_gb300 import synthetic
    w = synthetic.mid()
    qc = w["qc"]
    gx, gy, gz = w["grid"]
    x, y, z = gx[60:84], gy[70:90], gz[50:66]
    r, dr = core.rho_compute_no_slice(qc, drv=["x", "y", "z"], x=x, y=y, z=z, is_vector=False)
    pts = okref.grid2vector(x, y, z)
    ro, dro = okref.rho_threads(qc, *pts, drv=["x", "y", "z"], slice_length=512)
    assert_fp64_close(r.reshape(-1), ro, "rho")
    assert_fp64_close(dr.reshape(3, -1), dro, "grad rho")


def test_edge_sizes(core):
    """1, 63, 64, 65 and 1000 points, a point on a nucleus and far-field points."""
    import okref
    from orbkit_gb300 import synthetic
    w = synthetic.small()
    qc = w["qc"]
    rng = numpy.random.default_rng(3)
    for n in (1, 63, 64, 65, 1000):
        p = rng.uniform(-6, 6, (3, n))
        p[:, 0] = qc.geo_spec[1]
        if n > 2:
            p[:, 1] = [40.0, -35.0, 50.0]
        r, dr = core.rho_compute_no_slice(qc, drv=["x", "y", "z", "xy"], x=p[0], y=p[1], z=p[2], is_vector=True)
        ro, dro = okref.rho_threads(qc, *p, drv=["x", "y", "z", "xy"], slice_length=64, nthreads=2)
        assert_fp64_close(r, ro, "rho n=%d" % n)
        assert_fp64_close(dr, dro, "drho n=%d" % n)
        a = core.ao_creator(qc.geo_spec, qc.ao_spec, drv="yz", x=p[0], y=p[1], z=p[2], is_vector=True)
        assert_fp64_close(a, okref.ao_creator(qc.geo_spec, qc.ao_spec, drv="yz", x=p[0], y=p[1], z=p[2]), "ao yz")


def test_many_mos_multiple_passes(core):
    """More MOs than one pass of the fused kernel holds (40 per pass for rho+grad)."""
    import okref
    from orbkit_gb300 import synthetic
    rng = numpy.random.default_rng(7)
    geo = synthetic.random_geometry(rng, 8, 9.0)
    el = ["C", "O", "C", "H", "N", "H", "C", "H"]
    ao = synthetic.build_basis(rng, el)  # 5 heavy x 15 + 3 H x 5 = 90 AOs
    mo = synthetic.build_mos(rng, geo, ao, 70)
    qc = synthetic.make_qc(geo, el, ao, mo)
    p = rng.uniform(-5, 5, (3, 777))
    r, dr = core.rho_compute_no_slice(qc, drv=["x", "y", "z"], x=p[0], y=p[1], z=p[2], is_vector=True)
    ro, dro = okref.rho_threads(qc, *p, drv=["x", "y", "z"], slice_length=128, nthreads=2)
    assert_fp64_close(r, ro, "rho")
    assert_fp64_close(dr, dro, "drho")
    m = core.rho_compute_no_slice(qc, calc_mo=True, drv=["x", "xx"], x=p[0], y=p[1], z=p[2], is_vector=True)
    mref = okref.rho_compute_no_slice(qc, calc_mo=True, drv=["x", "xx"], x=p[0], y=p[1], z=p[2])
    assert_fp64_close(m, mref, "mo")


def test_few_points_kernel(core):
    """Small point sets (one CTA per point): 260 MOs (up to three MOs per thread), a
    spherical basis with f shells (267 AOs), rho alone, rho with one derivative and with
    x, y, z."""
    import okref
    from orbkit_gb300 import synthetic
    rng = numpy.random.default_rng(17)
    el = ["C", "O", "N", "H", "C", "H", "O", "C", "H", "N", "C", "C", "O", "N", "C"]
    geo = synthetic.random_geometry(rng, len(el), 11.0)
    ao = synthetic.build_basis(rng, el, with_f=True, spherical=True)
    mo = synthetic.build_mos(rng, geo, ao, 260)
    qc = synthetic.make_qc(geo, el, ao, mo)
    p = rng.uniform(-6, 6, (3, 300))
    p[:, :3] = numpy.asarray(qc.geo_spec)[:3].T
    for drv in (None, ["y"], ["x", "y", "z"]):
        out = core.rho_compute_no_slice(qc, drv=drv, x=p[0], y=p[1], z=p[2], is_vector=True)
        ref = okref.rho_threads(qc, *p, drv=drv, slice_length=64, nthreads=4)
        if drv is None:
            assert_fp64_close(out, ref if not isinstance(ref, tuple) else ref[0], "rho")
        else:
            assert_fp64_close(out[0], ref[0], "rho %s" % drv)
            assert_fp64_close(out[1], ref[1], "drho %s" % drv)


def test_exact_mixed_derivatives(core):
    """exact_mixed=True gives the true d2/dxdy (checked by central differences of d/dx)."""
    from orbkit_gb300 import synthetic
    qc = synthetic.small()["qc"]
    rng = numpy.random.default_rng(9)
    p = rng.uniform(-2, 2, (3, 50))
    h = 1e-5
    dxy = core.ao_creator(qc.geo_spec, qc.ao_spec, drv="xy", x=p[0], y=p[1], z=p[2], is_vector=True,
                          exact_mixed=True)
    fp = core.ao_creator(qc.geo_spec, qc.ao_spec, drv="x", x=p[0], y=p[1] + h, z=p[2], is_vector=True)
    fm = core.ao_creator(qc.geo_spec, qc.ao_spec, drv="x", x=p[0], y=p[1] - h, z=p[2], is_vector=True)
    fd = (fp - fm) / (2 * h)
    assert numpy.abs(dxy - fd).max() <= 1e-5 * numpy.abs(fd).max()


def test_c_abi_errors(core):
    """Bad derivative codes and leading dimensions are rejected with status codes."""
    import torch
    from orbkit_gb300 import _lib
    from orbkit_gb300.basis import get_basis
    from orbkit_gb300 import synthetic
    qc = synthetic.small()["qc"]
    L = _lib.load()
    b = get_basis(qc.geo_spec, qc.ao_spec, torch.device("cuda"))
    x = torch.zeros(10, dtype=torch.float64, device="cuda")
    g = _lib.OkgGrid(x.data_ptr(), x.data_ptr(), x.data_ptr(), 10, 0, 0, 0, 0, 0)
    out = torch.empty((1, b.nao, 10), dtype=torch.float64, device="cuda")
    assert L.okg_eval_ao(b.handle, ctypes.byref(g), 1, _lib.int_array([12]), 0, _lib.ptr(out), 10, None) == -3
    assert L.okg_eval_ao(b.handle, ctypes.byref(g), 1, _lib.int_array([1]), 0, _lib.ptr(out), 5, None) == -1
    g0 = _lib.OkgGrid(x.data_ptr(), x.data_ptr(), x.data_ptr(), 0, 0, 0, 0, 0, 0)
    assert L.okg_eval_ao(b.handle, ctypes.byref(g0), 1, _lib.int_array([1]), 0, _lib.ptr(out), 0, None) == 0
    gr = _lib.OkgGrid(x.data_ptr(), x.data_ptr(), x.data_ptr(), 10, 995, 10, 10, 10, 1)
    assert L.okg_eval_ao(b.handle, ctypes.byref(gr), 1, _lib.int_array([0]), 0, _lib.ptr(out), 10, None) == -1
    torch.cuda.synchronize()


def test_regular_grid_ranges_ao(core):
    """okg_eval_ao on point ranges of a regular grid that start and end inside grid
    lines (offset, npts) -- the slices a large call is cut into -- equal the same
    points of the whole-grid evaluation bit for bit, for Cartesian and spherical
    bases and value / first / second derivative channels; the whole grid is at the
    FP64 bar of the oracle."""
    import torch
    import okref
    from orbkit_gb300 import _lib
    from orbkit_gb300.basis import DeviceBasis
    from orbkit_gb300.core import _DeviceGrid
    L = _lib.load()
    x = numpy.linspace(-3.0, 3.2, 13)
    y = numpy.linspace(-2.5, 2.0, 11)
    z = numpy.linspace(-4.0, 3.5, 37)
    n = len(x) * len(y) * len(z)
    for name in ("small_cart.npz", "sph_fg_N.npz"):
        qc, d = load_golden(name)
        b = DeviceBasis(qc.geo_spec, qc.ao_spec)
        g = _DeviceGrid(x, y, z, False, b.device)
        codes = [0, 1, 6, 8]
        ca = _lib.int_array(codes)
        full = torch.empty((len(codes), b.nao, n), dtype=torch.float64, device=b.device)
        gd, keep = g.slice(0, n)
        _lib.check(L.okg_eval_ao(b.handle, gd, len(codes), ca, 0, _lib.ptr(full), n, _lib.stream_handle()))
        full = full.cpu().numpy()
        pts = okref.grid2vector(x, y, z)
        for k, c in enumerate(codes):
            assert_fp64_close(full[k], okref.ao_creator(qc.geo_spec, qc.ao_spec, drv=c, x=pts[0], y=pts[1], z=pts[2]),
                              "%s drv %d" % (name, c))
        for (i, j) in ((1234, 4234), (0, 37), (37 * 11 - 5, 37 * 11 + 300), (n - 777, n)):
            part = torch.empty((len(codes), b.nao, j - i), dtype=torch.float64, device=b.device)
            gd, keep = g.slice(i, j)
            _lib.check(L.okg_eval_ao(b.handle, gd, len(codes), ca, 0, _lib.ptr(part), j - i, _lib.stream_handle()))
            numpy.testing.assert_array_equal(part.cpu().numpy(), full[:, :, i:j])


def test_mo_matrix_and_transition_flux(core):
    """core.calc_mo_matrix (MO_a x dMO_b products, orbkit/core.py:841-941) and
    extras.calc_jmo (orbkit/extras.py:441-492) on the module grid, against the
    oracle's MO grids."""
    import okref
    from orbkit_gb300 import extras, grid, synthetic
    qc = synthetic.small()["qc"]
    x = numpy.linspace(-3.0, 3.0, 7)
    y = numpy.linspace(-2.5, 2.5, 6)
    z = numpy.linspace(-2.0, 2.0, 5)
    grid.set_grid(x, y, z, is_vector=False)
    drv = ["x", "y", "z"]
    mm = core.calc_mo_matrix(qc, drv=drv)
    mo = okref.rho_compute_no_slice(qc, calc_mo=True, drv=[None] + drv, x=x, y=y, z=z, is_vector=False)
    nmo = mo.shape[1]
    assert mm.shape == (3, nmo, nmo) + (7, 6, 5)
    ref = numpy.einsum("aigkl,dbgkl->daibgkl", mo[:1], mo[1:])[:, 0]
    assert_fp64_close(mm, ref, "mo matrix")
    pairs = [(0, 1), (2, 1), (3, 3)]
    jmo = extras.calc_jmo(qc, pairs, drv=drv)
    assert jmo.shape == (3, 3, 7, 6, 5)
    for n, (i, j) in enumerate(pairs):
        expect = -0.5 * (mo[0, i] * mo[1:, j] - mo[0, j] * mo[1:, i])
        assert_fp64_close(jmo[:, n], expect, "jmo %d %d" % (i, j))
    assert numpy.abs(jmo[:, 2]).max() == 0.0
    # the product kernels round as numpy does: bit for bit on the GPU's own MO grids
    mg = core.rho_compute(qc, calc_mo=True, drv=[None] + drv)
    numpy.testing.assert_array_equal(mm, mg[0][None, :, None] * mg[1:][:, None, :])
    for n, (i, j) in enumerate(pairs):
        numpy.testing.assert_array_equal(jmo[:, n], -0.5 * (mg[0, i] * mg[1:, j] - mg[0, j] * mg[1:, i]))
    # two molecules (bra from qc, ket from a second MO set on the same basis)
    # (the bra MOs then come from a values-only evaluation, as rho_compute(calc_mo=True)
    # gives them; the kernel with derivative channels may round the radial sums
    # differently in the last bit)
    qc2 = synthetic.small(seed=5)["qc"]
    mm2 = core.calc_mo_matrix(qc, qc2, drv="y")
    mb = core.rho_compute(qc, calc_mo=True)
    mg2 = core.rho_compute(qc2, calc_mo=True, drv=["y"])
    assert mm2.shape == (1, nmo, qc2.mo_spec.get_coeffs().shape[0], 7, 6, 5)
    numpy.testing.assert_array_equal(mm2, mb[None, :, None] * mg2[:, None, :])
    assert_fp64_close(mm2[0], numpy.einsum("agkl,bgkl->abgkl", mo[0], mg2[0]), "two-molecule mo matrix")
    grid.reset_grid()
