"""The hand-written adjoint (okg_rho_backward behind a torch.autograd.Function)
against a float64 PyTorch reference gradient, central finite differences, and its
FP32 variant against FP64.

Bars: FP64 adjoint vs the float64 reference: normwise relative 1e-10 per parameter
block; vs central differences of the FP64 loss (h = 1e-6, FP64 GPU forward, 64^3
points of the differentiation workload): |adj - fd| <= 1e-5 (|fd| + 1e-3 max|adj|) for
the FP64 adjoint and <= 1e-4 (|fd| + 1e-3 max|adj|) for the FP32 variant (FP32
arithmetic, forward on the mixed path); FP32 variant vs FP64: normwise relative 2e-3.
"""
import numpy
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    from orbkit_gb300 import build
    build.build()
    return t


def _params(torch, qc, dev):
    prim = qc.ao_spec.get_prim_coeffs()
    C = torch.tensor(qc.mo_spec.get_coeffs(), dtype=torch.float64, device=dev, requires_grad=True)
    alpha = torch.tensor(prim[:, 0], dtype=torch.float64, device=dev, requires_grad=True)
    coef = torch.tensor(prim[:, 1], dtype=torch.float64, device=dev, requires_grad=True)
    geo = torch.tensor(numpy.asarray(qc.geo_spec), dtype=torch.float64, device=dev, requires_grad=True)
    return C, alpha, coef, geo


def _nrel(a, b):
    a = a.detach().cpu().numpy()
    b = b.detach().cpu().numpy()
    return float(numpy.abs(a - b).max() / max(numpy.abs(b).max(), 1e-300))


def _molecule(seed, spherical=False):
    from orbkit_gb300 import synthetic
    rng = numpy.random.default_rng(seed)
    el = ["O", "H", "C", "H"]
    geo = synthetic.random_geometry(rng, 4, 5.0)
    ao = synthetic.build_basis(rng, el, with_f=spherical, spherical=spherical)
    mo = synthetic.build_mos(rng, geo, ao, 7)
    return synthetic.make_qc(geo, el, ao, mo), rng


@pytest.mark.parametrize("spherical", [False, True])
def test_adjoint_matches_float64_reference(torch, spherical):
    import torch_ref
    from orbkit_gb300.adjoint import DensityModel
    qc, rng = _molecule(3 if not spherical else 4, spherical)
    dev = torch.device("cuda")
    pts = rng.uniform(-3.5, 3.5, (3, 300))
    pts[:, 0] = qc.geo_spec[0] + 0.05
    model = DensityModel(qc, pts[0], pts[1], pts[2], True, "fp64")
    u = torch.tensor(rng.uniform(-1, 1, 300), dtype=torch.float64, device=dev)
    v = torch.tensor(rng.uniform(-1, 1, (3, 300)), dtype=torch.float64, device=dev)

    C, alpha, coef, geo = _params(torch, qc, dev)
    rho, grad = model(C, alpha, coef, geo)
    ((u * rho).sum() + (v * grad).sum()).backward()

    C2, alpha2, coef2, geo2 = _params(torch, qc, dev)
    st = torch_ref.Structure(qc.ao_spec, model.basis.T)
    occ = model.occ
    r_ref, g_ref = torch_ref.rho_grad(C2, alpha2, coef2, geo2, st, occ, torch.tensor(pts, device=dev))
    ((u * r_ref).sum() + (v * g_ref).sum()).backward()

    assert _nrel(rho, r_ref) < 1e-12 and _nrel(grad, g_ref) < 1e-11
    for name, a, b in (("C", C.grad, C2.grad), ("alpha", alpha.grad, alpha2.grad), ("c", coef.grad, coef2.grad),
                       ("R", geo.grad, geo2.grad)):
        assert _nrel(a, b) < 1e-10, (name, _nrel(a, b))


@pytest.mark.parametrize("prec,bar", [("fp64", 1e-5), ("fp32", 1e-4)])
def test_adjoint_central_differences(torch, prec, bar):
    """Density-fitting loss of the differentiation workload (12 atoms, 40 MOs) on a
    64^3 grid against central differences with step 1e-6 of the FP64 loss."""
    from orbkit_gb300 import synthetic
    from orbkit_gb300.adjoint import DensityModel, density_fit_loss
    w = synthetic.grad(npts=64)
    qc = w["qc"]
    x, y, z = w["grid"]
    dev = torch.device("cuda")
    model = DensityModel(qc, x, y, z, False, "fp64")
    assert model.npts == 64 ** 3
    t = w["target"]
    prim = qc.ao_spec.get_prim_coeffs()
    with torch.no_grad():
        Ct = torch.tensor(t["coeffs"], device=dev)
        at = torch.tensor(t["alpha"], device=dev)
        ct = torch.tensor(prim[:, 1], device=dev)
        gt = torch.tensor(t["geo"], device=dev)
        rho_t, grad_t = model(Ct, at, ct, gt)
        rho_t, grad_t = rho_t.clone(), grad_t.clone()
    wts = torch.tensor(numpy.random.default_rng(w["weight_seed"]).uniform(1e-12, 1.0, model.npts), device=dev)

    amodel = model if prec == "fp64" else DensityModel(qc, x, y, z, False, prec)
    C, alpha, coef, geo = _params(torch, qc, dev)
    loss = density_fit_loss(*amodel(C, alpha, coef, geo), rho_t, grad_t, wts)
    loss.backward()

    def L(Cv, av, cv, gv):
        with torch.no_grad():
            return float(density_fit_loss(*model(Cv, av, cv, gv), rho_t, grad_t, wts))

    h = 1e-6
    rng = numpy.random.default_rng(0)
    base = [C.detach(), alpha.detach(), coef.detach(), geo.detach()]
    grads = [C.grad, alpha.grad, coef.grad, geo.grad]
    for which in range(4):
        g = grads[which].detach().cpu().numpy().reshape(-1)
        idx = list(rng.choice(g.size, size=min(6, g.size), replace=False)) + [int(numpy.argmax(numpy.abs(g)))]
        for i in idx:
            plus = [b.clone() for b in base]
            minus = [b.clone() for b in base]
            plus[which].view(-1)[i] += h
            minus[which].view(-1)[i] -= h
            fd = (L(*plus) - L(*minus)) / (2 * h)
            assert abs(g[i] - fd) <= bar * (abs(fd) + 1e-3 * numpy.abs(g).max()), (prec, which, i, g[i], fd)


def test_adjoint_many_mos(torch):
    """110 MOs (three blocks of the adjoint's MO pass, W and V in the workspace) on a
    spherical f basis: FP64 adjoint against the float64 reference, FP32 against FP64."""
    import torch_ref
    from orbkit_gb300 import synthetic
    from orbkit_gb300.adjoint import DensityModel
    rng = numpy.random.default_rng(17)
    el = ["C", "N", "O", "H", "C", "H", "C", "O", "H"]
    geo = synthetic.random_geometry(rng, len(el), 7.0)
    ao = synthetic.build_basis(rng, el, with_f=True, spherical=True)
    mo = synthetic.build_mos(rng, geo, ao, 110)
    qc = synthetic.make_qc(geo, el, ao, mo)
    dev = torch.device("cuda")
    pts = rng.uniform(-4.0, 4.0, (3, 400))
    u = torch.tensor(rng.uniform(-1, 1, 400), dtype=torch.float64, device=dev)
    v = torch.tensor(rng.uniform(-1, 1, (3, 400)), dtype=torch.float64, device=dev)
    out = {}
    for prec in ("fp64", "fp32"):
        model = DensityModel(qc, pts[0], pts[1], pts[2], True, prec)
        assert model.nmo == 110
        C, alpha, coef, geo_t = _params(torch, qc, dev)
        rho, grad = model(C, alpha, coef, geo_t)
        ((u * rho).sum() + (v * grad).sum()).backward()
        out[prec] = (C.grad, alpha.grad, coef.grad, geo_t.grad)
    C2, alpha2, coef2, geo2 = _params(torch, qc, dev)
    st = torch_ref.Structure(qc.ao_spec, DensityModel(qc, pts[0], pts[1], pts[2], True, "fp64").basis.T)
    occ = torch.tensor([m["occ_num"] for m in qc.mo_spec], dtype=torch.float64, device=dev)
    r_ref, g_ref = torch_ref.rho_grad(C2, alpha2, coef2, geo2, st, occ, torch.tensor(pts, device=dev))
    ((u * r_ref).sum() + (v * g_ref).sum()).backward()
    for name, a, b in zip(("C", "alpha", "c", "R"), out["fp64"], (C2.grad, alpha2.grad, coef2.grad, geo2.grad)):
        assert _nrel(a, b) < 1e-10, (name, _nrel(a, b))
    for name, a, b in zip(("C", "alpha", "c", "R"), out["fp32"], out["fp64"]):
        assert _nrel(a, b) < 2e-3, (name, _nrel(a, b))


def test_adjoint_fp32_variant(torch):
    from orbkit_gb300 import synthetic
    from orbkit_gb300.adjoint import DensityModel
    w = synthetic.grad(npts=24)
    qc = w["qc"]
    x, y, z = w["grid"]
    dev = torch.device("cuda")
    rng = numpy.random.default_rng(5)
    out = {}
    for prec in ("fp64", "fp32"):
        model = DensityModel(qc, x, y, z, False, prec)
        C, alpha, coef, geo = _params(torch, qc, dev)
        rho, grad = model(C, alpha, coef, geo)
        u = torch.tensor(rng.uniform(0, 1, model.npts), device=dev) if prec == "fp64" else out["u"]
        v = torch.tensor(rng.uniform(-1, 1, (3, model.npts)), device=dev) if prec == "fp64" else out["v"]
        out["u"], out["v"] = u, v
        ((u * rho).sum() + (v * grad).sum()).backward()
        out[prec] = (C.grad, alpha.grad, coef.grad, geo.grad)
    for a, b, name in zip(out["fp32"], out["fp64"], ("C", "alpha", "c", "R")):
        assert _nrel(a, b) < 2e-3, (name, _nrel(a, b))
