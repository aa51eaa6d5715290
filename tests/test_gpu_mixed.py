"""Mixed-precision (tensor-core) rho and grad rho against the FP64 oracle.

Error bar: max relative rho error <= 1e-6 over points with rho > 1e-10
(orbkit_gb300.mixed.MIXED_RHO_RTOL / MIXED_RHO_FLOOR).  The gradient error,
|grad - grad_ref| / (|grad_ref| + 1e-10), is bounded at GRAD_BAR = 5e-5 (the
benchmark measures 1.5e-5 over the whole mid grid).
"""
import numpy
import pytest

from helpers import load_golden

pytestmark = pytest.mark.gpu

GRAD_BAR = 5e-5


@pytest.fixture(scope="module")
def mixed():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from orbkit_gb300 import build
    build.build()
    from orbkit_gb300 import mixed as m
    return m


def _check(mixed, r, g, ro, go, what):
    rep = mixed.error_report(r, g, ro, go)
    assert rep["rho_max_rel"] <= mixed.MIXED_RHO_RTOL, (what, rep)
    assert rep["grad_max_rel"] <= GRAD_BAR, (what, rep)
    return rep


def test_mixed_small_full_grid(mixed):
    import okref
    from orbkit_gb300 import synthetic
    w = synthetic.small()
    qc = w["qc"]
    x, y, z = w["grid"]
    r, g = mixed.rho_grad(qc, x, y, z, False)
    pts = okref.grid2vector(x, y, z)
    ro, go = okref.rho_threads(qc, *pts, drv=["x", "y", "z"], slice_length=4096)
    _check(mixed, r, g, ro, go, "small 80^3")


def test_mixed_mid_subgrid(mixed):
    import okref
    from orbkit_gb300 import synthetic
    w = synthetic.mid()
    qc = w["qc"]
    gx, gy, gz = w["grid"]
    x, y, z = gx[40:72], gy[70:90], gz[50:70]
    r, g = mixed.rho_grad(qc, x, y, z, False)
    ro, go = okref.rho_threads(qc, *okref.grid2vector(x, y, z), drv=["x", "y", "z"], slice_length=512)
    _check(mixed, r, g, ro, go, "mid block")


def test_mixed_mid_full_grid_sampled(mixed):
    """The mid workload as the benchmark runs it -- the whole 160^3 grid in one call
    (brick tiles, per-tile screening) with the FP64 cusp points -- compared with the
    oracle on 200 000 seeded random grid points plus every point within the cusp
    radius of a nucleus."""
    import okref
    from orbkit_gb300 import synthetic
    w = synthetic.mid()
    qc = w["qc"]
    gx, gy, gz = w["grid"]
    r, g = mixed.rho_grad(qc, gx, gy, gz, False)
    n = len(gx) * len(gy) * len(gz)
    near = mixed.cusp_points_regular(qc.geo_spec, gx, gy, gz, mixed.CUSP_RADIUS)
    assert len(near) > 0
    idx = numpy.unique(numpy.concatenate([numpy.random.default_rng(11).integers(0, n, 200000), near]))
    nyz = len(gy) * len(gz)
    px, py, pz = gx[idx // nyz], gy[(idx // len(gz)) % len(gy)], gz[idx % len(gz)]
    ro, go = okref.rho_threads(qc, px, py, pz, drv=["x", "y", "z"], slice_length=2048)
    rep = _check(mixed, r.reshape(-1)[idx], g.reshape(3, -1)[:, idx], ro, go, "mid full grid")
    print("mid full grid, %d sampled points: %s" % (len(idx), rep))


def test_mixed_kernel_deterministic(mixed):
    """The tensor-core kernel gives the same bits on repeated launches over the whole
    mid grid (tiles are handed out dynamically, so CTAs see different tiles each time;
    every point's arithmetic must not depend on that)."""
    import torch
    from orbkit_gb300 import synthetic
    from orbkit_gb300.core import _DeviceGrid
    w = synthetic.mid()
    ev = mixed.MixedEvaluator(w["qc"], cusp_radius=0.0)
    g = _DeviceGrid(*w["grid"], False, ev.device)
    n = g.npts
    gd, keep = g.slice(0, n)
    outs = []
    for _ in range(3):
        r = torch.full((n,), float("nan"), dtype=torch.float64, device=ev.device)
        gr = torch.full((3, n), float("nan"), dtype=torch.float64, device=ev.device)
        ev.plan.rho(gd, r, gr, n)
        torch.cuda.synchronize()
        ev.check()
        outs.append((r.cpu().numpy(), gr.cpu().numpy()))
    for r, gr in outs[1:]:
        numpy.testing.assert_array_equal(r, outs[0][0])
        numpy.testing.assert_array_equal(gr, outs[0][1])


def test_mixed_spherical_fg(mixed):
    """Spherical basis with f and g shells and an 'N' factor (golden data of the reference)."""
    qc, d = load_golden("sph_fg_N.npz")
    x, y, z = d["points"]
    r, g = mixed.rho_grad(qc, x, y, z, True)
    _check(mixed, r, g, d["rho"], d["delta_rho"], "spherical")


def test_mixed_many_mos_and_ragged(mixed):
    """70 MOs (two MO passes of the kernel) on 1, 127, 128, 129 and 1000 points."""
    import okref
    from orbkit_gb300 import synthetic
    rng = numpy.random.default_rng(7)
    geo = synthetic.random_geometry(rng, 8, 9.0)
    el = ["C", "O", "C", "H", "N", "H", "C", "H"]
    ao = synthetic.build_basis(rng, el)
    mo = synthetic.build_mos(rng, geo, ao, 70)
    qc = synthetic.make_qc(geo, el, ao, mo)
    for n in (1, 127, 128, 129, 1000):
        p = rng.uniform(-5, 5, (3, n))
        r, g = mixed.rho_grad(qc, p[0], p[1], p[2], True)
        ro, go = okref.rho_threads(qc, *p, drv=["x", "y", "z"], slice_length=128, nthreads=2)
        _check(mixed, r, g, ro, go, "n=%d" % n)


def test_mixed_cusp_points_use_fp64(mixed):
    """Points within the cusp radius of a nucleus carry FP64 values."""
    import okref
    from orbkit_gb300 import synthetic
    qc = synthetic.small()["qc"]
    p = numpy.array(qc.geo_spec).T.copy()
    p = numpy.concatenate([p, p + 0.05], axis=1)
    r, g = mixed.rho_grad(qc, p[0], p[1], p[2], True)
    ro, go = okref.rho_threads(qc, *p, drv=["x", "y", "z"], slice_length=8, nthreads=1)
    numpy.testing.assert_allclose(r, ro, rtol=1e-12)
    numpy.testing.assert_allclose(g, go, rtol=1e-11, atol=1e-12 * numpy.abs(go).max())


def test_mixed_spherical_f_many_mos(mixed):
    """Spherical basis with f shells and 100 MOs (two MO passes) on the mixed path."""
    import okref
    from orbkit_gb300 import synthetic
    rng = numpy.random.default_rng(21)
    el = ["C", "N", "O", "H", "C", "H", "C", "O", "H", "C"]
    geo = synthetic.random_geometry(rng, len(el), 10.0)
    ao = synthetic.build_basis(rng, el, with_f=True, spherical=True)
    mo = synthetic.build_mos(rng, geo, ao, 100)
    qc = synthetic.make_qc(geo, el, ao, mo)
    p = rng.uniform(-6, 6, (3, 3000))
    r, g = mixed.rho_grad(qc, p[0], p[1], p[2], True)
    ro, go = okref.rho_threads(qc, *p, drv=["x", "y", "z"], slice_length=128, nthreads=4)
    _check(mixed, r, g, ro, go, "spherical f, 100 MOs")


@pytest.mark.parametrize("layout", [(256, 1), (512, 1), (256, 2), (384, 2)])
def test_mixed_generation_layouts(mixed, layout):
    """Every generation layout (threads per CTA, points per thread) on a spherical f basis,
    a brick-tiled full grid and ragged vector point sets."""
    import okref
    from orbkit_gb300 import synthetic
    rng = numpy.random.default_rng(31)
    el = ["C", "O", "H", "N", "H", "C"]
    geo = synthetic.random_geometry(rng, len(el), 7.0)
    ao = synthetic.build_basis(rng, el, with_f=True, spherical=True)
    mo = synthetic.build_mos(rng, geo, ao, 30)
    qc = synthetic.make_qc(geo, el, ao, mo)
    ev = mixed.MixedEvaluator(qc)
    ev.plan.set_generation(*layout)
    g = numpy.linspace(-4.0, 4.0, 21)
    r, gr = ev.evaluate(g, g[:13], g[:9], False)
    ro, go = okref.rho_threads(qc, *okref.grid2vector(g, g[:13], g[:9]), drv=["x", "y", "z"], slice_length=256)
    _check(mixed, r, gr, ro, go, "grid %s" % (layout,))
    for n in (1, 129, 700):
        p = rng.uniform(-5, 5, (3, n))
        r, gr = ev.evaluate(p[0], p[1], p[2], True)
        ro, go = okref.rho_threads(qc, *p, drv=["x", "y", "z"], slice_length=128, nthreads=2)
        _check(mixed, r, gr, ro, go, "n=%d %s" % (n, layout))


def test_mixed_column_order(mixed):
    """okg_basis_set_mixed_order: the basis order, the exponent-class order the package
    chooses and a reversed order all give the oracle's results; a non-permutation is
    refused, and so is any reordering once a plan uses the basis."""
    import ctypes
    import torch
    import okref
    from orbkit_gb300 import synthetic, basis as bmod, _lib
    from orbkit_gb300.core import _DeviceGrid
    from orbkit_gb300.qcinfo import unpack
    rng = numpy.random.default_rng(5)
    w = synthetic.small()
    qc = w["qc"]
    geo, ao_spec, mo_spec = unpack(qc)
    occ = numpy.array([m["occ_num"] for m in mo_spec], dtype=numpy.float64)
    p = rng.uniform(-4, 4, (3, 3000))
    ro, go = okref.rho_threads(qc, *p, drv=["x", "y", "z"], slice_length=1000, nthreads=2)
    ip = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    for name in ("basis", "package", "reversed"):
        b = bmod.DeviceBasis(geo, ao_spec)
        if name != "package":
            order = numpy.arange(b.nshell, dtype=numpy.int32)
            if name == "reversed":
                order = order[::-1].copy()
            _lib.check(b._L.okg_basis_set_mixed_order(b.handle, ip(order)))
        bad = numpy.zeros(b.nshell, dtype=numpy.int32)
        with pytest.raises(_lib.OkgError):
            _lib.check(b._L.okg_basis_set_mixed_order(b.handle, ip(bad)))
        plan = mixed.MixedPlan(b, mo_spec.get_coeffs(), occ)
        with pytest.raises(_lib.OkgError):
            _lib.check(b._L.okg_basis_set_mixed_order(b.handle, ip(b.mixed_order)))
        g = _DeviceGrid(p[0], p[1], p[2], True, b.device)
        gd, keep = g.slice(0, g.npts)
        r = torch.empty(g.npts, dtype=torch.float64, device=b.device)
        gr = torch.empty((3, g.npts), dtype=torch.float64, device=b.device)
        plan.rho(gd, r, gr, g.npts)
        torch.cuda.synchronize()
        _check(mixed, r.cpu().numpy(), gr.cpu().numpy(), ro, go, "order " + name)


def test_mixed_through_drop_in_api(mixed):
    """core.rho_compute(..., precision='mixed') routes rho / grad rho to the tensor-core path."""
    from helpers import load_golden
    from orbkit_gb300 import core, grid
    qc, d = load_golden("h2o_molden.npz")
    grid.set_grid(d["x"], d["y"], d["z"], is_vector=False)
    r, dr = core.rho_compute(qc, drv=["x", "y", "z"], precision="mixed")
    r64, dr64 = core.rho_compute(qc, drv=["x", "y", "z"])
    _check(mixed, r.reshape(-1), dr.reshape(3, -1), r64.reshape(-1), dr64.reshape(3, -1), "drop-in")
    assert core.rho_compute(qc, precision="mixed").shape == r64.shape
    grid.reset_grid()


def test_mixed_gaussian_cube(mixed):
    """Tensor-core path on the Gaussian cube case (spherical basis from an fchk file, a
    grid point on the O nucleus): within the mixed bar of the FP64 path and within the
    reference test's tolerances of Gaussian's cube values."""
    from helpers import cube_case, cube_close
    from orbkit_gb300 import core
    qc, _, _, d = cube_case()
    kw = dict(x=d["x"], y=d["y"], z=d["z"], is_vector=False)
    r, dr = core.rho_compute_no_slice(qc, drv=["x", "y", "z"], precision="mixed", **kw)
    r64, dr64 = core.rho_compute_no_slice(qc, drv=["x", "y", "z"], **kw)
    _check(mixed, r.reshape(-1), dr.reshape(3, -1), r64.reshape(-1), dr64.reshape(3, -1), "cube case")
    cube_close(r, d["cube_rho"], 1e-5)
    cube_close(dr, d["cube_drho"], 1e-3)
