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


def test_noalloc_matches_plan_entry_point_twice(env):
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
    occ = numpy.array([m["occ_num"] for m in qc.mo_spec])
    plan = mixed.MixedPlan(b, qc.mo_spec.get_coeffs(), occ)
    g = _DeviceGrid(x, y, z, False, dev)
    n = g.npts
    gd, keep = g.slice(0, n)
    r_ref = torch.empty(n, dtype=torch.float64, device=dev)
    g_ref = torch.empty((3, n), dtype=torch.float64, device=dev)
    plan.rho(gd, r_ref, g_ref, n)
    torch.cuda.synchronize()
    plan.check()
    r_ref, g_ref = r_ref.cpu().numpy(), g_ref.cpu().numpy()

    status = torch.ones(1, dtype=torch.int32, device=dev)
    for call in range(2):
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


def test_noalloc_rejects_oversized_scratch(env):
    torch, L, _lib = env
    from orbkit_gb300 import synthetic
    from orbkit_gb300.basis import DeviceBasis
    rng = numpy.random.default_rng(1)
    el = ["C"] * 40
    geo = synthetic.random_geometry(rng, 40, 30.0)
    ao = synthetic.build_basis(rng, el)  # 600 Cartesian AOs -> 10 column chunks
    dev = torch.device("cuda")
    b = DeviceBasis(geo, ao, dev)
    nmo = 600  # 10 MO passes x 10 chunks x 3 parts x 64 x 128 B = 2.4 MB > 2 MiB
    C = torch.zeros((nmo, b.ncart), dtype=torch.float64, device=dev)
    occ = torch.full((nmo,), 2.0, dtype=torch.float64, device=dev)
    x = torch.zeros(4, dtype=torch.float64, device=dev)
    gd = _lib.OkgGrid(x.data_ptr(), x.data_ptr(), x.data_ptr(), 4, 0, 0, 0, 0, 0)
    r = torch.empty(4, dtype=torch.float64, device=dev)
    gr = torch.empty((3, 4), dtype=torch.float64, device=dev)
    st = L.okg_rho_mixed_noalloc(b.handle, ctypes.byref(gd), nmo, _lib.ptr(C), _lib.ptr(occ), 1, _lib.ptr(r),
                                 _lib.ptr(gr), 4, None, _lib.stream_handle())
    assert st == -7
    assert b"2 MiB" in L.okg_last_error()
