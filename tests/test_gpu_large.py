"""The large workload's basis on the GPU: 200 atoms in a 40-bohr box, a spherical
basis with one f shell per heavy atom (2136 spherical / 2420 Cartesian AOs), 400
occupied MOs (synthetic.large()), rho and grad rho on both paths against the
oracle (a C restatement of orbkit's cy_core / c_grid-based path, itself bit for bit
the reference).

Points: a 16^3 block of the 256^3 grid around the box centre (a whole regular grid
of its own, so the mixed kernel tiles it in bricks), 4096 seeded random points of
the full grid, and 512 points within 0.3 bohr of 64 seeded nuclei.

Bars: FP64 path |gpu - ref| <= 1e-12 |ref| + 1e-13 max|ref| (helpers.FP64_*); mixed
path max relative rho error <= 1e-6 over rho > 1e-10 and gradient error
|g - g_ref| / (|g_ref| + 1e-10) <= 5e-5, with and without the FP64 recomputation of
the points near nuclei.
"""
import numpy
import pytest

from helpers import assert_fp64_close

pytestmark = pytest.mark.gpu

GRAD_BAR = 5e-5


@pytest.fixture(scope="module")
def case():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from orbkit_gb300 import build
    build.build()
    import okref
    from orbkit_gb300 import synthetic
    w = synthetic.large()
    qc = w["qc"]
    gx, gy, gz = w["grid"]
    assert qc.ao_spec.get_ao_num() == 2136 and len(qc.ao_spec.get_lxlylz()) == 2420
    assert len(qc.mo_spec) == 400
    rng = numpy.random.default_rng(44)
    c = len(gx) // 2
    block = (gx[c - 8:c + 8], gy[c - 8:c + 8], gz[c - 8:c + 8])
    n = len(gx) * len(gy) * len(gz)
    idx = rng.integers(0, n, 4096)
    nyz = len(gy) * len(gz)
    rand = numpy.stack([gx[idx // nyz], gy[(idx // len(gz)) % len(gy)], gz[idx % len(gz)]])
    geo = numpy.asarray(qc.geo_spec)
    at = rng.choice(len(geo), 64, replace=False)
    d = rng.standard_normal((512, 3))
    d *= (rng.uniform(0.0, 0.3, 512) / numpy.linalg.norm(d, axis=1))[:, None]
    near = (geo[at[numpy.arange(512) % 64]] + d).T.copy()
    ref = {}
    ref["block"] = okref.rho_threads(qc, *okref.grid2vector(*block), drv=["x", "y", "z"], slice_length=128)
    ref["rand"] = okref.rho_threads(qc, *rand, drv=["x", "y", "z"], slice_length=128)
    ref["near"] = okref.rho_threads(qc, *near, drv=["x", "y", "z"], slice_length=64)
    return qc, block, rand, near, ref


def test_large_fp64_path(case):
    from orbkit_gb300 import core
    qc, block, rand, near, ref = case
    r, dr = core.rho_compute_no_slice(qc, drv=["x", "y", "z"], x=block[0], y=block[1], z=block[2], is_vector=False)
    assert_fp64_close(r.reshape(-1), ref["block"][0], "large block rho")
    assert_fp64_close(dr.reshape(3, -1), ref["block"][1], "large block grad")
    for key, p in (("rand", rand), ("near", near)):
        r, dr = core.rho_compute_no_slice(qc, drv=["x", "y", "z"], x=p[0], y=p[1], z=p[2], is_vector=True)
        assert_fp64_close(r, ref[key][0], "large %s rho" % key)
        assert_fp64_close(dr, ref[key][1], "large %s grad" % key)


@pytest.mark.parametrize("cusp", [True, False])
def test_large_mixed_path(case, cusp):
    """With the FP64 cusp points (the default), and the tensor-core kernel alone."""
    from orbkit_gb300 import mixed
    qc, block, rand, near, ref = case
    radius = mixed.CUSP_RADIUS if cusp else 0.0
    ev = mixed.MixedEvaluator(qc, cusp_radius=radius)
    for key, (p, vec) in (("block", (block, False)), ("rand", (rand, True)), ("near", (near, True))):
        r, g = ev.evaluate(p[0], p[1], p[2], vec)
        ev.check()
        rep = mixed.error_report(r, g, *ref[key])
        print("large mixed %s cusp=%s: %s" % (key, cusp, rep))
        assert rep["rho_max_rel"] <= mixed.MIXED_RHO_RTOL, (key, rep)
        assert rep["grad_max_rel"] <= GRAD_BAR, (key, rep)
