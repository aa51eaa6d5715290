"""The allocation-free mixed-path entry point (okg_rho_mixed_noalloc) through the C ABI.

It exists for callers that cannot allocate device memory where they evaluate the
density (a framework owning all device memory through its own pool, or a loop
that cannot take cudaMalloc's implicit synchronisation).  Its results must equal
those of the plan-based entry point (okg_rho_mixed) within the mixed-path error
bar, on two calls in a row that share the static scratch array.  This file is
collected last so that a run stopping at the first failure has run every other
test; it also passes on its own in a fresh process.
"""
import ctypes

import numpy
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from orbkit_gb300 import build
    build.build()
    from orbkit_gb300 import _lib
    L = _lib.load()
    f = L.okg_rho_mixed_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.POINTER(_lib.OkgGrid), ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]
    return torch, L, _lib


def _rel(a, b, floor):
    m = b > floor
    return float((numpy.abs(a - b)[m] / b[m]).max())


def _plan_result(mixed, b, C, occ, gd, n, torch, dev):
    """rho and grad from the plan-based entry point for coefficients C (host, nmo x nao)."""
    plan = mixed.MixedPlan(b, C, occ)
    r = torch.empty(n, dtype=torch.float64, device=dev)
    g = torch.empty((3, n), dtype=torch.float64, device=dev)
    plan.rho(gd, r, g, n)
    torch.cuda.synchronize()
    plan.check()
    return plan, r.cpu().numpy(), g.cpu().numpy()


def test_noalloc_matches_plan_entry_point_twice(env):
    """Two calls in a row with different inputs -- 40 MOs, then 31 MOs with scaled and
    permuted coefficients and other occupations -- each against the plan entry point
    fed the same inputs, so the second call cannot pass on what the first one left in
    the shared scratch array."""
    torch, L, _lib = env
    from orbkit_gb300 import mixed, synthetic
    from orbkit_gb300.basis import DeviceBasis
    from orbkit_gb300.core import _DeviceGrid
    w = synthetic.mid()
    qc = w["qc"]
    gx, gy, gz = w["grid"]
    x, y, z = gx[40:72], gy[60:92], gz[50:82]
    dev = torch.device("cuda")
    b = DeviceBasis(qc.geo_spec, qc.ao_spec, dev)
    g = _DeviceGrid(x, y, z, False, dev)
    n = g.npts
    gd, keep = g.slice(0, n)
    C0 = qc.mo_spec.get_coeffs()
    occ0 = numpy.array([m["occ_num"] for m in qc.mo_spec])
    rng = numpy.random.default_rng(5)
    perm = rng.permutation(C0.shape[0])[:31]
    cases = [(C0, occ0), (0.9 * C0[perm], rng.uniform(0.5, 2.0, 31))]

    status = torch.ones(1, dtype=torch.int32, device=dev)
    for call, (C, occ) in enumerate(cases):
        plan, r_ref, g_ref = _plan_result(mixed, b, C, occ, gd, n, torch, dev)
        r = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
        gr = torch.full((3, n), float("nan"), dtype=torch.float64, device=dev)
        st = L.okg_rho_mixed_noalloc(b.handle, ctypes.byref(gd), plan.nmo, _lib.ptr(plan.C), _lib.ptr(plan.occ), 1,
                                     _lib.ptr(r), _lib.ptr(gr), n, _lib.ptr(status), _lib.stream_handle())
        assert st == 0, L.okg_last_error()
        torch.cuda.synchronize()
        assert int(status.item()) == 0, "tensor-core wait timed out"
        r, gr = r.cpu().numpy(), gr.cpu().numpy()
        assert numpy.isfinite(r).all() and numpy.isfinite(gr).all()
        assert _rel(r, r_ref, mixed.MIXED_RHO_FLOOR) <= mixed.MIXED_RHO_RTOL, "call %d" % call
        rep = mixed.error_report(r, gr, r_ref, g_ref)
        assert rep["grad_max_rel"] <= 1e-6, (call, rep)


def _small_case(torch, _lib, nao_atoms, nmo):
    from orbkit_gb300 import synthetic
    from orbkit_gb300.basis import DeviceBasis
    rng = numpy.random.default_rng(1)
    geo = synthetic.random_geometry(rng, nao_atoms, 30.0)
    ao = synthetic.build_basis(rng, ["C"] * nao_atoms)
    dev = torch.device("cuda")
    b = DeviceBasis(geo, ao, dev)
    C = torch.zeros((nmo, b.ncart), dtype=torch.float64, device=dev)
    occ = torch.full((nmo,), 2.0, dtype=torch.float64, device=dev)
    x = torch.zeros(4, dtype=torch.float64, device=dev)
    gd = _lib.OkgGrid(x.data_ptr(), x.data_ptr(), x.data_ptr(), 4, 0, 0, 0, 0, 0)
    r = torch.empty(4, dtype=torch.float64, device=dev)
    gr = torch.empty((3, 4), dtype=torch.float64, device=dev)
    return b, C, occ, x, gd, r, gr


def test_noalloc_rejects_oversized_scratch(env):
    torch, L, _lib = env
    # 40 carbon atoms: 600 Cartesian AOs in whole-shell column chunks of at most 32
    # columns, so at least 19 chunks; 600 MOs: 10 passes of 64 MO columns.  The split
    # coefficients take passes x chunks x 3 parts x 64 rows x 64 bytes (one 32-column
    # BF16 row is 64 bytes): at least 2.3 MB, above the 2 MiB of static scratch.
    b, C, occ, x, gd, r, gr = _small_case(torch, _lib, 40, 600)
    chunks_at_least = -(-b.ncart // 32)
    need = 10 * chunks_at_least * 3 * 64 * 64
    assert need > 2 << 20, need
    status = torch.zeros(1, dtype=torch.int32, device=b.device)
    st = L.okg_rho_mixed_noalloc(b.handle, ctypes.byref(gd), 600, _lib.ptr(C), _lib.ptr(occ), 1, _lib.ptr(r),
                                 _lib.ptr(gr), 4, _lib.ptr(status), _lib.stream_handle())
    assert st == -7
    assert b"2 MiB" in L.okg_last_error()


def test_noalloc_requires_status_word(env):
    """Without a status word an expired wait could not be reported: rejected."""
    torch, L, _lib = env
    b, C, occ, x, gd, r, gr = _small_case(torch, _lib, 2, 4)
    st = L.okg_rho_mixed_noalloc(b.handle, ctypes.byref(gd), 4, _lib.ptr(C), _lib.ptr(occ), 1, _lib.ptr(r),
                                 _lib.ptr(gr), 4, None, _lib.stream_handle())
    assert st == -1
    assert b"d_status" in L.okg_last_error()
