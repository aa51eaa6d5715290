"""The standalone grid operations on given AO values: core.mo_creator
(orbkit/core.py:107-132, cy_core.mocreator at orbkit/cy_core.pyx:82-101) and
core.cartesian2spherical (orbkit/core.py:135-176), each one hand-written kernel
(okg_mo_from_ao, okg_cart2sph), against the oracle and the reference's golden
AO / MO arrays.

Bars: mo_creator at the FP64 bar (|gpu - ref| <= 1e-12 |ref| + 1e-13 max|ref|, FMA
accumulation); cartesian2spherical bit for bit against the oracle's restatement of
orbkit's term-by-term numpy arithmetic.
"""
import numpy
import pytest

from helpers import assert_fp64_close, load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def core():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from orbkit_gb300 import build
    build.build()
    from orbkit_gb300 import core as c
    return c


def test_mo_creator_golden_cartesian(core):
    """Every drv slot of the reference's AO arrays (small Cartesian molecule) through
    mo_creator gives the reference's MO arrays."""
    qc, d = load_golden("small_cart.npz")
    for k in range(d["ao"].shape[0]):
        mo = core.mo_creator(d["ao"][k], qc.mo_spec)
        assert mo.shape == d["mo"][k].shape
        assert_fp64_close(mo, d["mo"][k], "mo_creator drv slot %d" % k)


def test_mo_creator_golden_spherical(core):
    """Spherical f/g basis with 'N' on a vector grid (reference's arrays)."""
    qc, d = load_golden("sph_fg_N.npz")
    for k in range(d["ao"].shape[0]):
        assert_fp64_close(core.mo_creator(d["ao"][k], qc.mo_spec), d["mo"][k], "spherical slot %d" % k)


@pytest.mark.parametrize("nmo,nao,npts", [(1, 7, 1), (5, 25, 63), (17, 33, 1000), (70, 300, 4099), (130, 64, 257)])
def test_mo_creator_vs_oracle_sizes(core, nmo, nao, npts):
    """Every MO-block width of the kernel (1, 2, 4, 8, 16 MOs per group), AO counts not a
    multiple of the 32-AO chunk, ragged point counts, against the oracle's mocreator."""
    import okref
    from orbkit_gb300.orbitals import MOClass
    rng = numpy.random.default_rng(nmo * 1000 + nao)
    ao = rng.standard_normal((nao, npts))
    C = rng.standard_normal((nmo, nao))
    mo_spec = MOClass([{"coeffs": C[i], "occ_num": 2.0, "energy": 0.0, "sym": "%d.1" % i} for i in range(nmo)])
    mo_spec.update()
    assert_fp64_close(core.mo_creator(ao, mo_spec), okref.mocreator(ao, C), "mo_creator %d x %d x %d" % (nmo, nao, npts))


def test_mo_creator_keeps_grid_shape_and_checks_columns(core):
    qc, d = load_golden("small_cart.npz")
    ao = d["ao"][0]  # (25, 6, 5, 4)
    assert core.mo_creator(ao, qc.mo_spec).shape == (5, 6, 5, 4)
    with pytest.raises(ValueError):
        core.mo_creator(ao[:20], qc.mo_spec)


def test_cartesian2spherical_bitwise(core):
    """Cartesian AOs (oracle, with the basis' 'N' factor as ao_creator applies it) ->
    spherical rows: bit for bit the oracle's restatement of orbkit's numpy loop, and
    the reference's spherical AO arrays within the FP64 bar."""
    import okref
    qc, d = load_golden("sph_fg_N.npz")
    x, y, z = d["points"]
    for k in range(d["ao"].shape[0]):
        cart = okref.aocreator(qc.geo_spec, qc.ao_spec, x, y, z, k)
        cart *= qc.ao_spec[0]["N"]
        sph = core.cartesian2spherical(cart, qc.ao_spec)
        numpy.testing.assert_array_equal(sph, okref.cartesian2spherical(cart, qc.ao_spec))
        assert_fp64_close(sph, d["ao"][k], "cartesian2spherical drv %d" % k)


def test_cartesian2spherical_large_basis_regular_shape(core):
    """The 2420-Cartesian-AO basis with f shells on a small regular block: shapes kept,
    bit for bit against the oracle."""
    import okref
    from orbkit_gb300 import synthetic
    qc = synthetic.large()["qc"]
    rng = numpy.random.default_rng(3)
    cart = rng.standard_normal((len(qc.ao_spec.get_lxlylz()), 3, 4, 5))
    sph = core.cartesian2spherical(cart, qc.ao_spec)
    assert sph.shape == (qc.ao_spec.get_ao_num(), 3, 4, 5)
    numpy.testing.assert_array_equal(sph.reshape(sph.shape[0], -1),
                                     okref.cartesian2spherical(cart.reshape(cart.shape[0], -1), qc.ao_spec))
