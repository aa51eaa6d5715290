"""Batched persistent launch (okg_batch_run) over molecules with atom-centred
point sets: equal to the per-molecule mixed path, within the mixed error bar of
the FP64 path and the oracle, and unchanged when replayed from a CUDA graph; the
in-kernel FP64 cusp points (the default) within the bar at every point near a
nucleus."""
import numpy
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from orbkit_gb300 import build, synthetic
    build.build()
    d = synthetic.batch(seed=11, nmol=6, min_atoms=3, max_atoms=14)
    rng = numpy.random.default_rng(2)
    mols = []
    for m in d["molecules"]:
        pts = m["points"]
        keep = rng.choice(pts.shape[1], size=min(pts.shape[1], 20000 + int(rng.integers(0, 5000))), replace=False)
        mols.append((m["qc"], pts[:, numpy.sort(keep)].copy()))
    return torch, mols


def test_batch_matches_single_molecule_mixed_and_fp64(setup, tmp_path, monkeypatch):
    torch, mols = setup
    monkeypatch.setenv("ORBKIT_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    from orbkit_gb300 import mixed
    from orbkit_gb300.batch import BatchEvaluator
    ev = BatchEvaluator(mols, cusp_radius=0.0, tune=True)
    assert ev.schedule["n_max"] in (32, 64)
    ev.run()
    torch.cuda.synchronize()
    ev.check()
    res = ev.results()
    for (qc, pts), (r, g) in zip(mols, res):
        r1, g1 = mixed.rho_grad(qc, pts[0], pts[1], pts[2], True, cusp_radius=0.0)
        if ev.schedule["n_max"] == 64:
            numpy.testing.assert_array_equal(r, r1)
            numpy.testing.assert_array_equal(g, g1)
        from orbkit_gb300 import core
        r64, g64 = core.rho_compute_no_slice(qc, drv=["x", "y", "z"], x=pts[0], y=pts[1], z=pts[2], is_vector=True)
        rep = mixed.error_report(r, g, r64, g64)
        assert rep["rho_max_rel"] <= mixed.MIXED_RHO_RTOL, rep
        assert rep["grad_max_rel"] <= 1e-3, rep


def test_batch_oracle_subsample_and_graph_replay(setup):
    torch, mols = setup
    import okref
    from orbkit_gb300 import mixed
    from orbkit_gb300.batch import BatchEvaluator
    ev = BatchEvaluator(mols, cusp_radius=mixed.CUSP_RADIUS, tune=False,
                        schedule={"n_max": 32, "grab": 2, "order": "largest_first"})
    ev.run()
    torch.cuda.synchronize()
    first = ev.results()
    for m in ev.mols:
        m["rho"].fill_(float("nan"))
        m["grad"].fill_(float("nan"))
    g = ev.capture()
    for m in ev.mols:
        m["rho"].fill_(float("nan"))
    g.replay()
    torch.cuda.synchronize()
    ev.check()
    again = ev.results()
    for (a, b), (c, d) in zip(first, again):
        numpy.testing.assert_array_equal(a, c)
        numpy.testing.assert_array_equal(b, d)
    rng = numpy.random.default_rng(4)
    for (qc, pts), (r, gr) in zip(mols, first):
        sel = rng.choice(pts.shape[1], size=600, replace=False)
        ro, go = okref.rho_threads(qc, *pts[:, sel], drv=["x", "y", "z"], slice_length=64, nthreads=4)
        rep = mixed.error_report(r[sel], gr[:, sel], ro, go)
        assert rep["rho_max_rel"] <= mixed.MIXED_RHO_RTOL, rep


def test_batch_kernel_cusp_points(setup):
    """Every point within the cusp radius of a nucleus, with the cusp atom's steep
    primitives in FP64 inside the persistent launch (cusp_mode='kernel', the default),
    against the oracle: within the mixed bar; the same points from the tensor cores
    alone are reported beside it."""
    torch, mols = setup
    import okref
    from orbkit_gb300 import mixed
    from orbkit_gb300.batch import BatchEvaluator
    sch = {"n_max": 64, "grab": 1, "order": "given", "layout": (384, 1)}
    ev = BatchEvaluator(mols, tune=False, schedule=sch)
    assert ev.kernel_cusp
    ev.run()
    torch.cuda.synchronize()
    ev.check()
    res = ev.results()
    ev0 = BatchEvaluator(mols, cusp_radius=0.0, tune=False, schedule=sch)
    ev0.run()
    torch.cuda.synchronize()
    res0 = ev0.results()
    for m, (qc, pts), (r, g), (r0, g0) in zip(ev.mols, mols, res, res0):
        sel = numpy.nonzero(m["near"].cpu().numpy() >= 0)[0]
        assert len(sel) > 0
        sel = sel[:: max(1, len(sel) // 1500)]
        ro, go = okref.rho_threads(qc, *pts[:, sel], drv=["x", "y", "z"], slice_length=64, nthreads=4)
        rep = mixed.error_report(r[sel], g[:, sel], ro, go)
        rep0 = mixed.error_report(r0[sel], g0[:, sel], ro, go)
        print("cusp points %d: FP64 steep part %s | tensor cores alone %s" % (len(sel), rep, rep0))
        assert rep["rho_max_rel"] <= mixed.MIXED_RHO_RTOL, rep
        assert rep["grad_max_rel"] <= 5e-5, rep


def test_single_molecule_kernel_cusp_mode(setup):
    """MixedEvaluator(cusp_mode='kernel') on points near and on the nuclei (vector grid)
    and on a regular block through a nucleus: within the mixed bar of the oracle."""
    torch, mols = setup
    import okref
    from orbkit_gb300 import mixed, synthetic
    qc = synthetic.small()["qc"]
    ev = mixed.MixedEvaluator(qc, cusp_mode="kernel")
    p = numpy.array(qc.geo_spec).T.copy()
    p = numpy.concatenate([p, p + 0.05, p - 0.11, p + 0.29], axis=1)
    r, g = ev.evaluate(p[0], p[1], p[2], True)
    ev.check()
    ro, go = okref.rho_threads(qc, *p, drv=["x", "y", "z"], slice_length=8, nthreads=1)
    rep = mixed.error_report(r, g, ro, go)
    print("near nuclei, in-kernel FP64 cusp:", rep)
    assert rep["rho_max_rel"] <= mixed.MIXED_RHO_RTOL, rep
    x = numpy.linspace(-0.6, 0.6, 9)
    r, g = ev.evaluate(x, x, x, False)
    ev.check()
    ro, go = okref.rho_threads(qc, *okref.grid2vector(x, x, x), drv=["x", "y", "z"], slice_length=64, nthreads=2)
    rep = mixed.error_report(r, g, ro, go)
    print("block through the O nucleus, in-kernel FP64 cusp:", rep)
    assert rep["rho_max_rel"] <= mixed.MIXED_RHO_RTOL, rep
