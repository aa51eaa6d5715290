"""Seeded synthetic workloads (molecules, bases, MOs and grids).

orbkit ships no benchmark inputs for the grid path, so every measurement and
parity test runs on seeded synthetic molecules with the shapes below.

  small   3-atom water-like molecule, Cartesian basis (25 AOs), 5 occupied MOs,
          regular 80^3 grid over +-5 bohr.
  mid     20 atoms (C/N/O/H drawn 6:1:1:12) in a 16-bohr box, min. separation
          1.9 bohr, heavy 3s2p1d / H 2s1p (~180 Cartesian AOs), 40 occupied MOs,
          regular 160^3 grid at 0.15 bohr.
  grad    the same family with 12 atoms (box edge 16*(12/20)^(1/3) bohr), 40 MOs,
          regular 128^3 grid at 0.15 bohr, plus seeded perturbed parameters
          (C + 0.01 N(0,1), exponents * exp(0.05 N(0,1)), nuclei + 0.05 N(0,1) bohr)
          for the density-fitting loss.
  batch   256 molecules of 3-60 atoms of the same family (20-600 Cartesian AOs,
          l <= 2), nocc = NAO // 5; atom-centred point sets: radial count 50-200
          on r = R (1+x)/(1-x), R = 1 bohr, x = cos(i pi/(n+1)) (Chebyshev nodes
          of the second kind), times a Fibonacci-spiral unit-sphere set of
          110-302 points.
  large   200 atoms in a 40-bohr box, spherical basis with one f shell per heavy
          atom (~2280 spherical / ~2600 Cartesian AOs), 400 occupied MOs,
          regular 256^3 grid at 0.16 bohr.

Shell recipe (all sizes): heavy atom s(6), s(3), s(1), p(3), p(1), d(1)
[+ f(1) in 'large']; H s(3), s(1), p(1).  Exponents log-uniform in [0.1, 1e4]
(s) and [0.1, 50] (p, d, f); contraction coefficients uniform in [0.1, 1] then
normalised so that the contracted x^l component has unit norm.  MO coefficients
are seeded Gaussian and Loewdin (symmetrically) orthonormalised with the analytic
AO overlap: C <- (C0 S C0^T)^(-1/2) C0, so C S C^T = 1.  Occupation 2.0.
"""
import numpy

from .orbitals import AOClass, MOClass
from .overlap import ao_overlap
from .qcinfo import QCinfo

HEAVY_SHELLS = [("s", 6), ("s", 3), ("s", 1), ("p", 3), ("p", 1), ("d", 1)]
H_SHELLS = [("s", 3), ("s", 1), ("p", 1)]
ELEMENTS = ["C", "N", "O", "H"]
ELEMENT_P = numpy.array([6, 1, 1, 12], dtype=float) / 20.0
_L = {"s": 0, "p": 1, "d": 2, "f": 3, "g": 4}

CONFIG_NAMES = ["small", "mid", "grad", "batch", "large"]


def _contraction(rng, ltype, nprim):
    lo, hi = (0.1, 1e4) if ltype == "s" else (0.1, 50.0)
    alpha = numpy.exp(rng.uniform(numpy.log(lo), numpy.log(hi), nprim))
    c = rng.uniform(0.1, 1.0, nprim)
    L = _L[ltype]
    # norm of the contracted x^L component built from unit-norm primitives
    aa = alpha[:, None]
    bb = alpha[None, :]
    s = (2.0 * numpy.sqrt(aa * bb) / (aa + bb)) ** (L + 1.5)
    c = c / numpy.sqrt(c @ s @ c)
    return numpy.stack([alpha, c], axis=1)


def build_basis(rng, elements, with_f=False, spherical=False):
    ao = []
    for ia, el in enumerate(elements):
        shells = HEAVY_SHELLS + ([("f", 1)] if with_f else []) if el != "H" else H_SHELLS
        for lt, n in shells:
            ao.append({"atom": ia, "type": lt, "pnum": n, "coeffs": _contraction(rng, lt, n)})
    spec = AOClass(ao)
    if spherical:
        spec.set_lm_dict(p=[1, 0])
    spec.update()
    return spec


def build_mos(rng, geo, ao_spec, nmo, occ=2.0, S=None):
    if S is None:
        S = ao_overlap(geo, ao_spec)
    nao = S.shape[0]
    C0 = rng.standard_normal((nmo, nao))
    M = C0 @ S @ C0.T
    w, V = numpy.linalg.eigh(M)
    C = (V * (1.0 / numpy.sqrt(w))) @ V.T @ C0
    mo = MOClass([{"coeffs": C[i].copy(), "occ_num": occ, "energy": -1.0 + 0.01 * i, "sym": "%d.1" % (i + 1)}
                  for i in range(nmo)])
    mo.update()
    return mo


def random_geometry(rng, natom, box, min_sep=1.9, max_tries=200000):
    pos = []
    tries = 0
    while len(pos) < natom:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("could not place %d atoms in a %.1f-bohr box" % (natom, box))
        p = rng.uniform(-box / 2, box / 2, 3)
        if all(numpy.linalg.norm(p - q) >= min_sep for q in pos):
            pos.append(p)
    return numpy.array(pos)


def draw_elements(rng, natom, min_heavy=1):
    el = list(rng.choice(ELEMENTS, size=natom, p=ELEMENT_P))
    nh = sum(e != "H" for e in el)
    i = 0
    while nh < min(min_heavy, natom):
        if el[i] == "H":
            el[i] = "C"
            nh += 1
        i += 1
    return el


def make_qc(geo, elements, ao_spec, mo_spec):
    qc = QCinfo()
    qc.geo_spec = numpy.asarray(geo, dtype=numpy.float64)
    qc.geo_info = [[e, str(i + 1), "0"] for i, e in enumerate(elements)]
    qc.ao_spec = ao_spec
    qc.mo_spec = mo_spec
    return qc


def small(seed=0):
    """3-atom water-like molecule, Cartesian basis, 5 occupied MOs, 80^3 grid over +-5 bohr."""
    rng = numpy.random.default_rng(seed)
    th = numpy.deg2rad(104.5) / 2.0
    R = 1.81
    geo = numpy.array([[0.0, 0.0, 0.0],
                       [0.0, R * numpy.sin(th), R * numpy.cos(th)],
                       [0.0, -R * numpy.sin(th), R * numpy.cos(th)]])
    el = ["O", "H", "H"]
    ao = build_basis(rng, el)
    mo = build_mos(rng, geo, ao, 5)
    g = numpy.linspace(-5.0, 5.0, 80)
    return {"name": "small", "qc": make_qc(geo, el, ao, mo), "grid": (g.copy(), g.copy(), g.copy())}


def _family(seed, natom, box, nmo, npts, spacing, with_f=False, spherical=False):
    rng = numpy.random.default_rng(seed)
    el = draw_elements(rng, natom)
    geo = random_geometry(rng, natom, box)
    ao = build_basis(rng, el, with_f=with_f, spherical=spherical)
    mo = build_mos(rng, geo, ao, nmo)
    g = (numpy.arange(npts) - (npts - 1) / 2.0) * spacing
    return rng, {"qc": make_qc(geo, el, ao, mo), "grid": (g.copy(), g.copy(), g.copy())}


def mid(seed=1, npts=160):
    """20 atoms, ~180 Cartesian AOs, 40 occupied MOs, 160^3 grid at 0.15 bohr."""
    _, d = _family(seed, 20, 16.0, 40, npts, 0.15)
    d["name"] = "mid"
    return d


def grad(seed=2, npts=128):
    """12 atoms, 40 MOs, 128^3 grid, plus the perturbed target parameters and weights."""
    natom = 12
    rng, d = _family(seed, natom, 16.0 * (natom / 20.0) ** (1.0 / 3.0), 40, npts, 0.15)
    qc = d["qc"]
    C = qc.mo_spec.get_coeffs()
    prim = qc.ao_spec.get_prim_coeffs()
    d["target"] = {
        "coeffs": C + 0.01 * rng.standard_normal(C.shape),
        "alpha": prim[:, 0] * numpy.exp(0.05 * rng.standard_normal(len(prim))),
        "geo": qc.geo_spec + 0.05 * rng.standard_normal(qc.geo_spec.shape),
    }
    d["weight_seed"] = seed + 1000
    d["name"] = "grad"
    return d


def fibonacci_sphere(n):
    """n quasi-uniform unit vectors on a golden-angle spiral."""
    i = numpy.arange(n) + 0.5
    zc = 1.0 - 2.0 * i / n
    r = numpy.sqrt(numpy.maximum(0.0, 1.0 - zc * zc))
    phi = numpy.pi * (3.0 - numpy.sqrt(5.0)) * i
    return numpy.stack([r * numpy.cos(phi), r * numpy.sin(phi), zc], axis=1)


def becke_radial(n, R=1.0):
    """Radii r = R (1+x)/(1-x) at the Chebyshev nodes of the second kind x_i = cos(i pi/(n+1))."""
    x = numpy.cos(numpy.arange(1, n + 1) * numpy.pi / (n + 1))
    return R * (1.0 + x) / (1.0 - x)


def atom_point_set(rng, center):
    nr = int(rng.integers(50, 201))
    na = int(rng.integers(110, 303))
    r = becke_radial(nr)
    u = fibonacci_sphere(na)
    pts = center[None, None, :] + r[:, None, None] * u[None, :, :]
    return pts.reshape(-1, 3)


def batch(seed=3, nmol=256, min_atoms=3, max_atoms=60):
    """Many molecules with atom-centred point sets of uneven sizes."""
    rng = numpy.random.default_rng(seed)
    mols = []
    for m in range(nmol):
        natom = int(rng.integers(min_atoms, max_atoms + 1))
        el = draw_elements(rng, natom)
        geo = random_geometry(rng, natom, 16.0 * (natom / 20.0) ** (1.0 / 3.0))
        ao = build_basis(rng, el)
        nao = ao.get_ao_num()
        mo = build_mos(rng, geo, ao, max(1, nao // 5))
        pts = numpy.concatenate([atom_point_set(rng, geo[a]) for a in range(natom)], axis=0)
        mols.append({"qc": make_qc(geo, el, ao, mo), "points": numpy.ascontiguousarray(pts.T)})
    return {"name": "batch", "molecules": mols}


def large(seed=4, npts=256):
    """200 atoms, spherical basis with f, ~2280 AOs, 400 MOs, 256^3 grid at 0.16 bohr."""
    _, d = _family(seed, 200, 40.0, 400, npts, 0.16, with_f=True, spherical=True)
    d["name"] = "large"
    return d


def make(name, **kw):
    return {"small": small, "mid": mid, "grad": grad, "batch": batch, "large": large}[name](**kw)
