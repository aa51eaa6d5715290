"""Shared test helpers: golden fixtures, parity metrics, library build."""
import os
import platform

import numpy

from orbkit_gb300.qcinfo import from_arrays

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# Parity bar of the FP64 GPU path against the oracle / the reference's outputs:
# every element satisfies |gpu - ref| <= FP64_RTOL * |ref| + FP64_ATOL_REL * max|ref|
# (max over the compared array).  The second term covers elements that are
# themselves cancellation residues (near nodes and sign changes), whose
# absolute error is set by the size of the terms that cancel, not by their
# own value.
FP64_RTOL = 1e-12
FP64_ATOL_REL = 1e-13


def load_golden(name):
    d = dict(numpy.load(os.path.join(GOLDEN, name), allow_pickle=False))
    return from_arrays(d), d


def is_x86():
    return platform.machine() in ("x86_64", "AMD64")


def rel_errors(a, b):
    """(max normwise error max|a-b|/max|b|, max elementwise error over |b| > 1e-6 max|b|)."""
    a = numpy.asarray(a, dtype=numpy.float64)
    b = numpy.asarray(b, dtype=numpy.float64)
    scale = numpy.abs(b).max() if b.size else 0.0
    if scale == 0.0:
        return float(numpy.abs(a - b).max() if a.size else 0.0), 0.0
    d = numpy.abs(a - b)
    m = numpy.abs(b) > 1e-6 * scale
    elem = float((d[m] / numpy.abs(b[m])).max()) if m.any() else 0.0
    return float(d.max() / scale), elem


def assert_fp64_close(a, b, what="", rtol=FP64_RTOL, atol_rel=FP64_ATOL_REL):
    a = numpy.asarray(a, dtype=numpy.float64)
    b = numpy.asarray(b, dtype=numpy.float64)
    assert a.shape == b.shape, "%s: shape %s != %s" % (what, a.shape, b.shape)
    scale = numpy.abs(b).max() if b.size else 0.0
    assert numpy.isfinite(b).all(), "%s: reference holds non-finite values" % what
    bound = rtol * numpy.abs(b) + atol_rel * scale
    bad = ~(numpy.abs(a - b) <= bound)  # NaN in a counts as a mismatch
    if bad.any():
        i = numpy.unravel_index(numpy.argmax(numpy.abs(a - b) - bound), a.shape)
        raise AssertionError("%s: %d elements outside |d| <= %g|ref| + %g max|ref|; worst at %s: %r vs %r "
                             "(errors %s)" % (what, bad.sum(), rtol, atol_rel, i, a[i], b[i], rel_errors(a, b)))


def detci_terms(d, k):
    """(zero, sing) of state pair k of the detCI fixture, in orbkit's nested-list form."""
    zc, zo, zl = d["zero_coef_%d" % k], d["zero_orb_%d" % k], d["zero_len_%d" % k]
    zero = [[], []]
    o = 0
    for n in zl:
        zero[0].append([float(v) for v in zc[o:o + n]])
        zero[1].append([int(v) for v in zo[o:o + n]])
        o += n
    sing = [[float(v) for v in d["sing_coef_%d" % k]], [[int(a), int(b)] for a, b in d["sing_pair_%d" % k]]]
    return zero, sing


def cube_case():
    """The Gaussian cube case (h2o_gaussian_cube.npz): the molecule with all MOs,
    without the core MO (Gaussian's "Total SCF Density"), and the HOMO alone."""
    qc, d = load_golden("h2o_gaussian_cube.npz")
    dv = dict(d)
    dv["mo_coeffs"], dv["mo_occ"] = d["mo_coeffs"][1:], d["mo_occ"][1:]
    dh = dict(d)
    dh["mo_coeffs"], dh["mo_occ"] = d["homo_coeffs"].reshape(1, -1), d["mo_occ"][:1]
    return qc, from_arrays(dv), from_arrays(dh), d


def cube_close(a, b, tol):
    """The reference's test/tools.py equal(): allclose(a, b, rtol=100 tol, atol=tol)."""
    numpy.testing.assert_allclose(a, b, rtol=tol * 1e2, atol=tol)


def analytic_cases():
    """The cases of h2o_analytic.npz: (name, qc, dict of the case's arrays)."""
    d = numpy.load(os.path.join(GOLDEN, "h2o_analytic.npz"), allow_pickle=False)
    out = []
    for k, name in enumerate(d["names"]):
        pre = "c%d__" % k
        arrs = {key[len(pre):]: d[key] for key in d.files if key.startswith(pre)}
        qc = from_arrays(arrs)
        qc.geo_info = [["X", str(i + 1), repr(float(z))] for i, z in enumerate(arrs["charges"])]
        out.append((str(name), qc, arrs))
    return out
