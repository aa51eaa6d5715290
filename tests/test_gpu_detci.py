"""detCI grid loops (orbkit/detci/cy_ci.pyx, ci_core.py) on the GPU: the kernels fed
the oracle's MO grids against the oracle restatement (bit for bit), and the whole
GPU pipeline (FP64 MO grids, then the CI kernels) against the reference's own test
data for H3+ FCI/cc-pVTZ (test/detci/refdata_h3+.npz, via tests/golden/h3p_detci.npz)."""
import numpy
import pytest

from helpers import assert_fp64_close, detci_terms, load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from orbkit_gb300 import build
    build.build()
    import okref
    from orbkit_gb300 import core, detci
    qc, d = load_golden("h3p_detci.npz")
    drv = [None, "x", "y", "z", "xx", "yy", "zz"]
    mo_oracle = okref.rho_compute_no_slice(qc, calc_mo=True, drv=drv, x=d["x"], y=d["y"], z=d["z"], is_vector=False)
    mo_gpu = core.rho_compute_no_slice(qc, calc_mo=True, drv=drv, x=d["x"], y=d["y"], z=d["z"], is_vector=False)
    return detci, okref, d, mo_oracle, mo_gpu


def test_ci_kernels_bitwise_on_oracle_mos(env):
    detci, okref, d, mo, _ = env
    for k in range(int(d["npairs"])):
        zero, sing = detci_terms(d, k)
        for sl, rs in ((1e2, True), (1e4, False)):
            r = detci.rho(zero, sing, mo[0], slice_length=sl, reference_slicing=rs, exact=True)
            j = detci.jab(zero, sing, mo[0], mo[1:4], slice_length=sl, reference_slicing=rs, exact=True)
            a = detci.a_nabla_b(zero, sing, mo[0], mo[1:4], slice_length=sl, reference_slicing=rs, exact=True)
            if rs:
                r0 = okref.ci_driver(okref.ci_rho, zero, sing, mo[0], slice_length=sl)
                j0 = okref.ci_driver(okref.ci_jab, zero, sing, mo[0], mo[1:4], slice_length=sl)
                a0 = okref.ci_driver(okref.ci_a_nabla_b, zero, sing, mo[0], mo[1:4], slice_length=sl)
            else:
                r0 = okref.ci_rho(zero, sing, mo[0])
                j0 = okref.ci_jab(zero, sing, mo[0], mo[1:4])
                a0 = okref.ci_a_nabla_b(zero, sing, mo[0], mo[1:4])
            numpy.testing.assert_array_equal(r, r0)
            numpy.testing.assert_array_equal(j, j0)
            numpy.testing.assert_array_equal(a, a0)


def test_ci_quadratic_forms_on_oracle_mos(env):
    """Default evaluation (terms folded into NMO x NMO matrices) against the oracle's
    term-order sums, on the fixture's MO grids and on seeded grids of 3000 points
    that cover several 128-point blocks and a ragged tail."""
    import torch
    detci, okref, d, mo, _ = env
    rng = numpy.random.default_rng(5)
    rand = rng.standard_normal((4, 42, 3001))
    for k in range(int(d["npairs"])):
        zero, sing = detci_terms(d, k)
        for m0, md in ((mo[0], mo[1:4]), (rand[0], rand[1:4])):
            assert_fp64_close(detci.rho(zero, sing, m0, reference_slicing=False), okref.ci_rho(zero, sing, m0),
                              "rho pair %d" % k)
            assert_fp64_close(detci.jab(zero, sing, m0, md, reference_slicing=False),
                              okref.ci_jab(zero, sing, m0, md), "jab pair %d" % k)
            assert_fp64_close(detci.a_nabla_b(zero, sing, m0, md, reference_slicing=False),
                              okref.ci_a_nabla_b(zero, sing, m0, md), "a_nabla_b pair %d" % k)
    # device tensors in, device tensors out; odd MO counts (row padding of the matrices)
    zero, sing = [[[0.5, -0.25]], [[0, 4]]], [[0.3, -0.7, 1.1], [[0, 1], [4, 2], [3, 3]]]
    m = torch.tensor(rand[0][:5, :777], device="cuda")
    dm = torch.tensor(rand[1:4][:, :5, :777], device="cuda")
    r = detci.rho(zero, sing, m, reference_slicing=False)
    assert r.is_cuda
    assert_fp64_close(r.cpu().numpy(), okref.ci_rho(zero, sing, rand[0][:5, :777]), "rho nmo=5")
    assert_fp64_close(detci.jab(zero, sing, m, dm, reference_slicing=False).cpu().numpy(),
                      okref.ci_jab(zero, sing, rand[0][:5, :777], rand[1:4][:, :5, :777]), "jab nmo=5")


def test_ci_pipeline_against_reference_data(env):
    detci, _, d, _, mo = env
    for k in range(int(d["npairs"])):
        zero, sing = detci_terms(d, k)
        r = detci.rho(zero, sing, mo[0], slice_length=1e2)
        j = detci.jab(zero, sing, mo[0], mo[1:4], slice_length=1e2)
        nj = -detci.jab(zero, sing, mo[0], mo[4:7], slice_length=1e2).sum(axis=0)
        # sums of thousands of MO products with cancellation: normwise FP64 bar
        for name, a, b in (("rho", r, d["rho_01"][k]), ("j", j, d["j_01"][k]), ("nabla j", nj, d["nabla_j_01"][k])):
            err = numpy.abs(a - b).max() / numpy.abs(b).max()
            assert err <= 1e-11, (k, name, err)


def test_ci_device_tensors_and_errors(env):
    import torch
    detci, _, d, mo, _ = env
    zero, sing = detci_terms(d, 1)
    t = torch.as_tensor(mo[0], device="cuda")
    r = detci.rho(zero, sing, t, reference_slicing=False)
    assert isinstance(r, torch.Tensor) and tuple(r.shape) == mo.shape[2:]
    assert_fp64_close(r.cpu().numpy(), detci.rho(zero, sing, mo[0], reference_slicing=False), "tensor input")
    bad = [list(sing[0][:1]), [[0, mo.shape[1]]]]
    with pytest.raises(IndexError):
        detci.rho([[], []], bad, mo[0])
    with pytest.raises(ValueError):
        detci.jab(zero, sing, mo[0], mo[1:3])
