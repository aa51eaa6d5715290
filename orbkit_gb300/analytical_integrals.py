"""Analytic one-electron integrals over the AO basis on the GPU: the functions of
orbkit/analytical_integrals.py with the same names, arguments and return values.

The AO overlap (and its first ket derivative, and the ket-exponent override used
for dipole integrals) is computed by the okg_ao_overlap kernel (replacing
cy_overlap.aooverlap, orbkit/cy_overlap.pyx:78-163); the 'N' factor and the
transform to real spherical harmonics are applied by the same call.  MO overlaps
(C_a S C_b^T, replacing the loops of cy_overlap.mooverlap / mooverlapmatrix,
orbkit/cy_overlap.pyx:167-205) are FP64 matrix products on the device.

Inputs may be numpy arrays (results are numpy arrays, as orbkit returns) or CUDA
tensors (results stay on the device).  There is no CPU path: without the built
library and a GPU the calls raise.
"""
import ctypes

import numpy

from . import _lib
from .basis import flatten, fingerprint
from .orbitals import AOClass, MOClass
from .tools import validate_drv

_SIGS = {
    "okg_overlap_plan_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 4 +
                                [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int] +
                                [ctypes.c_void_p] * 3 + [ctypes.POINTER(ctypes.c_void_p)]),
    "okg_overlap_plan_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "okg_overlap_plan_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int),
                                             ctypes.POINTER(ctypes.c_int)]),
    "okg_overlap_plan_set_ket": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "okg_ao_overlap": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]),
}


def _L():
    L = _lib.load()
    for n, (r, a) in _SIGS.items():
        f = getattr(L, n)
        f.restype = r
        f.argtypes = a
    return L


def _np_ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


class OverlapPlan:
    """okg_overlap_plan for one AO basis (tables on the current device)."""

    def __init__(self, ao_spec):
        L = _L()
        f = flatten(ao_spec)
        self.flat = f
        self.ncart = len(f["lxlylz"])
        natom = int(f["atoms"].max()) + 1
        nsph = len(f["sph_ptr"]) - 1 if f["spherical"] else 0
        h = ctypes.c_void_p()
        _lib.check(L.okg_overlap_plan_create(natom, len(f["ncart"]), _np_ptr(f["atoms"]), _np_ptr(f["ncart"]),
                                             _np_ptr(f["nprim"]), _np_ptr(f["lxlylz"]), f["normalized"],
                                             _np_ptr(f["prim"]), _np_ptr(f["renorm"]), nsph,
                                             _np_ptr(f.get("sph_ptr")), _np_ptr(f.get("sph_idx")),
                                             _np_ptr(f.get("sph_coef")), ctypes.byref(h)))
        self._h = h
        self._L = L
        self.natom_min = natom
        self.nao = nsph if nsph else self.ncart
        self._ket = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._L.okg_overlap_plan_destroy(h)
            except Exception:
                pass
            self._h = None

    def set_ket(self, lxlylz_b):
        key = None if lxlylz_b is None else numpy.require(lxlylz_b, dtype=numpy.intc, requirements="CA")
        same = (key is None and self._ket is None) or (key is not None and self._ket is not None and
                                                       numpy.array_equal(key, self._ket))
        if not same:
            _lib.check(self._L.okg_overlap_plan_set_ket(self._h, _np_ptr(key)))
            self._ket = None if key is None else key.copy()

    def run(self, geo_a, geo_b, drv, raw=False, stream=None):
        """(nao, nao) float64 CUDA tensor."""
        import torch
        n = self.ncart if raw else self.nao
        out = torch.empty((n, n), dtype=torch.float64, device=geo_a.device)
        _lib.check(self._L.okg_ao_overlap(self._h, _lib.ptr(geo_a), _lib.ptr(geo_b), int(drv), int(bool(raw)),
                                          _lib.ptr(out), n, _lib.stream_handle(stream)))
        return out


_plans = {}


def overlap_plan(ao_spec):
    """Cached OverlapPlan for this basis (keyed by its flattened tables)."""
    key = fingerprint(numpy.zeros((0, 3)), flatten(ao_spec))
    p = _plans.get(key)
    if p is None:
        if len(_plans) >= 16:
            _plans.pop(next(iter(_plans)))
        p = _plans[key] = OverlapPlan(ao_spec)
    return p


def _dev():
    import torch
    return torch.device("cuda", torch.cuda.current_device())


def _geo_tensor(coord, natom_min):
    import torch
    t = torch.as_tensor(coord, dtype=torch.float64)
    t = t.to(_dev()).reshape(-1, 3).contiguous()
    if t.shape[0] < natom_min:
        raise ValueError("geometry has %d atoms, the basis refers to atom %d" % (t.shape[0], natom_min - 1))
    return t


def _is_tensor(a):
    try:
        import torch
        return isinstance(a, torch.Tensor)
    except ImportError:
        return False


def get_ao_overlap(coord_a, coord_b, ao_spec, lxlylz_b=None, drv=None):
    """Overlap matrix <bra at coord_a | ket at coord_b> of the basis set
    (orbkit/analytical_integrals.py:37-116): lxlylz_b replaces the ket's Cartesian
    exponents (the primitive norms still use ao_spec's), drv = 'x', 'y', 'z' (or
    1..3) differentiates the ket, a list of drv returns a list of matrices."""
    if not (isinstance(ao_spec, AOClass) or hasattr(ao_spec, "get_lxlylz")):
        raise TypeError('ao_spec must be an instance of the AOClass')  # orbkit's own AOClass is accepted too
    if isinstance(drv, list) or (isinstance(drv, str) and len(drv) > 1):
        return [get_ao_overlap(coord_a, coord_b, ao_spec, lxlylz_b=lxlylz_b, drv=d) for d in drv]
    lxlylz_a = ao_spec.get_lxlylz()
    if lxlylz_b is not None:
        try:
            lxlylz_b = numpy.array(lxlylz_b, dtype=numpy.intc)
        except ValueError:
            raise ValueError('The keyword argument `lxlylz` has to be convertable into a numpy integer array.')
        if lxlylz_a.shape != lxlylz_b.shape:
            raise ValueError('The exponents lxlylz for basis set a and basis set b have to have the same shape.')
    drv = validate_drv(drv)
    if drv > 3:
        raise ValueError('Only first derivatives are currently supported for analytical integrals.')
    plan = overlap_plan(ao_spec)
    ga = _geo_tensor(coord_a, plan.natom_min)
    gb = _geo_tensor(coord_b, plan.natom_min)
    plan.set_ket(lxlylz_b)
    out = plan.run(ga, gb, drv)
    return out if _is_tensor(coord_a) else out.cpu().numpy()


def cartesian2spherical_aoom(ao_overlap_matrix, ao_spec):
    """Cartesian -> real spherical harmonic AO matrix, T S T^T with orbkit's
    Schlegel-Frisch combinations (orbkit/analytical_integrals.py:118-182)."""
    import torch
    from .basis import spherical_csr
    ptr, idx, coef = spherical_csr(ao_spec)
    ncart = len(ao_spec.get_lxlylz())
    S = torch.as_tensor(ao_overlap_matrix, dtype=torch.float64).to(_dev())
    if tuple(S.shape) != (ncart, ncart):
        raise IOError('No contraction is currently not supported for a spherical harmonics.')
    T = numpy.zeros((len(ptr) - 1, ncart))
    for r in range(len(ptr) - 1):
        for t in range(ptr[r], ptr[r + 1]):
            T[r, idx[t]] += coef[t]
    Td = torch.from_numpy(T).to(S.device)
    out = Td @ S @ Td.T
    return out if _is_tensor(ao_overlap_matrix) else out.cpu().numpy()


def _coeffs(mo):
    if isinstance(mo, MOClass) or hasattr(mo, "get_coeffs"):  # this package's MOClass or orbkit's
        return mo.get_coeffs()
    if isinstance(mo, dict):
        return numpy.array(mo['coeffs'])
    return mo


def _mat(a):
    import torch
    return torch.as_tensor(a, dtype=torch.float64).to(_dev())


def get_mo_overlap(mo_a, mo_b, ao_overlap_matrix):
    """<mo_a|mo_b> = a S b^T for two coefficient vectors (orbkit/analytical_integrals.py:184-214)."""
    shape = tuple(ao_overlap_matrix.shape)
    mo_a = _coeffs(mo_a)
    mo_b = _coeffs(mo_b)
    if mo_a.ndim != 1 or len(mo_a) != shape[0]:
        raise ValueError('The coefficients of mo_a have to be a vector of the length of the ao_overlap_matrix.')
    if mo_b.ndim != 1 or len(mo_b) != shape[1]:
        raise ValueError('The coefficients of mo_b have to be a vector of the length of the ao_overlap_matrix.')
    return float(_mat(mo_a) @ _mat(ao_overlap_matrix) @ _mat(mo_b))


def get_mo_overlap_matrix(mo_a, mo_b, ao_overlap_matrix, numproc=1):
    """(NMO_a, NMO_b) overlaps C_a S C_b^T (orbkit/analytical_integrals.py:224-287);
    numproc is accepted for compatibility (one device call)."""
    mo_a = _coeffs(mo_a)
    mo_b = _coeffs(mo_b)
    if mo_a.shape[1] != ao_overlap_matrix.shape[0] or mo_b.shape[1] != ao_overlap_matrix.shape[1]:
        raise ValueError('mo_a and mo_b have to correspond to the same basis set, i.e., shape_a[1] != shape_b[1]')
    out = _mat(mo_a) @ _mat(ao_overlap_matrix) @ _mat(mo_b).T
    return out if _is_tensor(ao_overlap_matrix) else out.cpu().numpy()


def get_atom2mo(qc):
    """Atom index of every output AO (orbkit/analytical_integrals.py:442-469).  The
    AOs per shell are counted in the output basis (spherical functions of a
    spherical basis), which is orbkit's count for shells without an explicit
    'lxlylz' list."""
    ao = qc.ao_spec
    if getattr(ao, "spherical", False):
        per = numpy.bincount(ao.get_assign_lm_to_cont(), minlength=len(ao))
    else:
        per = ao.get_nlxlylz_per_cont()
    return numpy.repeat(numpy.array([s['atom'] for s in ao], dtype=int), per)


def get_lc(atoms, atom2mo, strict=False):
    """Indices of the AOs of the selected atoms (orbkit/analytical_integrals.py:471-505)."""
    if isinstance(atoms, int):
        atoms = [atoms]
    if not strict:
        lc = numpy.zeros(len(atom2mo), dtype=bool)
        for i in atoms:
            lc = numpy.logical_or(atom2mo == i, lc)
        return numpy.nonzero(lc)[0]
    return numpy.array([k for i in atoms for k, j in enumerate(atom2mo) if i == j], dtype=numpy.intc)


def get_moom_atoms(atoms, qc, mo_a, mo_b, ao_overlap_matrix, numproc=1):
    """MO overlap matrix restricted to the ket AOs of the selected atoms
    (orbkit/analytical_integrals.py:289-316)."""
    mo_a = mo_a.get_coeffs()
    mo_b = mo_b.get_coeffs()
    indices = get_lc(atoms, get_atom2mo(qc), strict=True)
    aoom = numpy.asarray(ao_overlap_matrix)[:, indices]
    return get_mo_overlap_matrix(numpy.ascontiguousarray(mo_a), numpy.ascontiguousarray(mo_b[:, indices]),
                                 numpy.ascontiguousarray(aoom), numproc=numproc)


def check_mo_norm(qc):
    """|| C S C^T - 1 || of qc's MOs (orbkit/analytical_integrals.py:318-326)."""
    aoom = get_ao_overlap(qc.geo_spec, qc.geo_spec, qc.ao_spec)
    moom = get_mo_overlap_matrix(qc.mo_spec, qc.mo_spec, aoom)
    return numpy.linalg.norm(moom - numpy.eye(len(moom)))


def get_ao_dipole_matrix(qc, component='x'):
    """<AO_i | r_c | AO_j> (orbkit/analytical_integrals.py:363-414): the overlap with
    the ket exponent along c raised by one, plus the ket atom's coordinate times the
    overlap."""
    import torch
    if isinstance(component, list):
        return [get_ao_dipole_matrix(qc, component=c) for c in component]
    if not isinstance(component, int):
        component = 'xyz'.find(component)
    if component == -1:
        raise ValueError("The selection of the component was not valid! (component = 'x' or 'y' or 'z')")
    lxlylz_b = numpy.array(qc.ao_spec.get_lxlylz(), dtype=numpy.intc)
    lxlylz_b[:, component] += 1
    geo = torch.as_tensor(numpy.asarray(qc.geo_spec, dtype=numpy.float64)).to(_dev())
    part_1 = get_ao_overlap(geo, geo, qc.ao_spec, lxlylz_b=lxlylz_b)
    part_2 = get_ao_overlap(geo, geo, qc.ao_spec)
    col = geo[torch.as_tensor(get_atom2mo(qc), device=geo.device), component]
    return (part_1 + part_2 * col[None, :]).cpu().numpy()


def get_nuclear_dipole_moment(qc, component='x'):
    """sum_nuc Z r_c (orbkit/analytical_integrals.py:416-440); Z from geo_info[:, 2]."""
    if not isinstance(component, int):
        component = 'xyz'.find(component)
    if component == -1:
        raise ValueError("The selection of the component was not valid! (component = 'x' or 'y' or 'z')")
    out = 0.0
    for i in range(len(qc.geo_spec)):
        out += float(qc.geo_info[i][2]) * qc.geo_spec[i][component]
    return out


def get_dipole_moment(qc, component=['x', 'y', 'z']):
    """Electronic plus nuclear dipole moment (orbkit/analytical_integrals.py:328-361):
    -sum_i occ_i c_i D c_i^T + sum Z r."""
    try:
        component = list(component)
    except TypeError:
        component = [component]
    coeffs = _mat(qc.mo_spec.get_coeffs())
    occ = _mat(qc.mo_spec.get_occ())
    out = numpy.zeros((len(component),))
    for i, c in enumerate(component):
        D = _mat(get_ao_dipole_matrix(qc, component=c))
        out[i] = -float((occ * ((coeffs @ D) * coeffs).sum(1)).sum())
        out[i] += get_nuclear_dipole_moment(qc, component=c)
    return out
