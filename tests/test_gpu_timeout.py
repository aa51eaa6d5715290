"""Failure detection of the tensor-core kernel, without a GPU fault: every wait in
the kernel is bounded; here the plan's wait limit is set to one poll so that the
waits expire on purpose.  The kernel must then raise its status word, drain its
own bulk copies and MMAs in flight, free its tensor memory and return; the host
reads OKG_ERR_TIMEOUT; and the next launch on the same plan, with the default
limit, must give the normal results bit for bit.
"""
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
    from orbkit_gb300 import _lib, mixed
    return torch, _lib, mixed


def test_expired_wait_reports_timeout_and_next_launch_is_correct(env):
    torch, _lib, mixed = env
    from orbkit_gb300 import synthetic
    from orbkit_gb300.core import _DeviceGrid
    w = synthetic.mid()
    qc = w["qc"]
    gx, gy, gz = w["grid"]
    ev = mixed.MixedEvaluator(qc, cusp_radius=0.0)
    g = _DeviceGrid(gx[40:88], gy[40:88], gz[40:88], False, ev.device)
    n = g.npts
    gd, keep = g.slice(0, n)
    r0 = torch.empty(n, dtype=torch.float64, device=ev.device)
    g0 = torch.empty((3, n), dtype=torch.float64, device=ev.device)
    ev.plan.rho(gd, r0, g0, n)
    torch.cuda.synchronize()
    ev.check()
    for attempt in range(3):
        ev.plan.set_wait_limit(1)
        r = torch.zeros(n, dtype=torch.float64, device=ev.device)
        gr = torch.zeros((3, n), dtype=torch.float64, device=ev.device)
        ev.plan.rho(gd, r, gr, n)
        torch.cuda.synchronize()  # the kernel returned: no hang
        with pytest.raises(_lib.OkgError) as e:
            ev.check()
        assert e.value.status == -6, e.value
        ev.plan.set_wait_limit(1 << 24)
        ev.check()  # the status word was cleared by the first check
        ev.plan.rho(gd, r, gr, n)
        torch.cuda.synchronize()
        ev.check()
        numpy.testing.assert_array_equal(r.cpu().numpy(), r0.cpu().numpy())
        numpy.testing.assert_array_equal(gr.cpu().numpy(), g0.cpu().numpy())


def test_wait_limit_argument_checked(env):
    torch, _lib, mixed = env
    from orbkit_gb300 import synthetic
    ev = mixed.MixedEvaluator(synthetic.small()["qc"], cusp_radius=0.0)
    with pytest.raises(_lib.OkgError):
        ev.plan.set_wait_limit(0)
