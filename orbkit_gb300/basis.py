"""Device-resident basis: orbkit's AO description packed for the GPU kernels.

``DeviceBasis`` takes the arrays that orbkit's AOClass getters produce
(orbkit/orbitals.py:336-385 -- the same ones orbkit/core.py:89-97 hands to
cy_core.aocreator), creates the C-ABI basis handle (okg_basis_create) and keeps
the nuclear positions and primitive exponents/coefficients as device tensors
(okg_basis_set_params).  Spherical bases are evaluated in the Cartesian basis
and transformed: AO outputs go through the per-shell transform of
orbkit/core.py:135-176, and MO coefficients are folded into the Cartesian basis,
C_eff = C_sph . T, so the fused kernels only see Cartesian shells.
"""
import ctypes
import hashlib

import numpy

from . import _lib
from .tools import get_cart2sph


def spherical_csr(ao_spec):
    """CSR (ptr, listed Cartesian row, coefficient) of the spherical transform,
    following orbkit's cartesian2spherical: for each listed (lx,ly,lz) of the
    Schlegel-Frisch combination the last matching row of the shell is used and
    the coefficient is coef * global factor."""
    lxlylz = ao_spec.get_lxlylz()
    assign = ao_spec.get_assign_lxlylz_to_cont()
    rows = {}
    for i, j in enumerate(assign):
        rows.setdefault(int(j), []).append(i)
    ptr, idx, coef = [0], [], []
    for (j0, k0) in ao_spec.get_old_ao_spherical():
        comps, cf, fac = get_cart2sph(*k0)
        for c, f in zip(comps, cf):
            hit = None
            for i in rows[int(j0)]:
                if tuple(int(v) for v in lxlylz[i]) == tuple(c):
                    hit = i
            if hit is None:
                raise ValueError("spherical component %s missing from shell %d" % (c, j0))
            idx.append(hit)
            coef.append(f * fac)
        ptr.append(len(idx))
    return (numpy.array(ptr, dtype=numpy.intc), numpy.array(idx, dtype=numpy.intc),
            numpy.array(coef, dtype=numpy.float64))


def flatten(ao_spec):
    """The AOClass getter arrays used by the kernels."""
    d = {
        "lxlylz": numpy.require(ao_spec.get_lxlylz(), dtype=numpy.intc, requirements="CA"),
        "ncart": numpy.require(ao_spec.get_nlxlylz_per_cont(), dtype=numpy.intc, requirements="CA"),
        "prim": numpy.require(ao_spec.get_prim_coeffs(), dtype=numpy.float64, requirements="CA"),
        "nprim": numpy.require(ao_spec.get_nprim_per_cont(), dtype=numpy.intc, requirements="CA"),
        "atoms": numpy.require(ao_spec.get_assign_cont_to_atoms(), dtype=numpy.intc, requirements="CA"),
        "normalized": int(ao_spec.get_normalized()),
        "spherical": bool(getattr(ao_spec, "spherical", False)),
    }
    d["renorm"] = (numpy.require(numpy.asarray(ao_spec[0]["N"], dtype=numpy.float64).reshape(-1), requirements="CA")
                   if "N" in ao_spec[0] else None)
    if d["spherical"]:
        d["sph_ptr"], d["sph_idx"], d["sph_coef"] = spherical_csr(ao_spec)
    return d


def fingerprint(geo, flat):
    h = hashlib.sha1()
    h.update(numpy.ascontiguousarray(geo, dtype=numpy.float64).tobytes())
    for k in ("lxlylz", "ncart", "prim", "nprim", "atoms", "renorm", "sph_ptr", "sph_idx", "sph_coef"):
        v = flat.get(k)
        if v is not None:
            h.update(k.encode())
            h.update(numpy.ascontiguousarray(v).tobytes())
    h.update(bytes([flat["normalized"], int(flat["spherical"])]))
    return h.hexdigest()


def mixed_order(geo, flat):
    """Shell order of the tensor-core path's columns (okg_basis_set_mixed_order).

    A grid tile keeps a primitive while alpha log2(e) d^2 <= 64 (d: distance from its
    atom to the tile), so the most diffuse shells are kept by nearly every tile and
    the steep ones only near their atom.  Shells whose smallest exponents lie in the
    same factor-4 class go together, most diffuse first, and inside a class atoms
    follow a Morton curve: a tile's kept shells then fill few 16-column K-steps (on
    the 20-atom, 180-AO molecule 4.1 instead of 8.1 K-steps per 128-point tile)."""
    nprim = numpy.asarray(flat["nprim"], dtype=numpy.int64)
    off = numpy.concatenate(([0], numpy.cumsum(nprim)))
    alpha = numpy.asarray(flat["prim"], dtype=numpy.float64)[:, 0]
    amin = numpy.array([alpha[off[s]:off[s + 1]].min() for s in range(len(nprim))])
    cls = numpy.floor(numpy.log(numpy.maximum(amin, 1e-300)) / numpy.log(4.0))
    atoms = numpy.asarray(flat["atoms"], dtype=numpy.int64)
    geo = numpy.asarray(geo, dtype=numpy.float64).reshape(-1, 3)
    lo = geo.min(0)
    q = ((geo - lo) / numpy.maximum(geo.max(0) - lo, 1e-9) * 1023).astype(numpy.int64)
    code = numpy.zeros(len(geo), dtype=numpy.int64)
    for b in range(10):
        for d in range(3):
            code |= ((q[:, d] >> b) & 1) << (3 * b + d)
    order = sorted(range(len(nprim)), key=lambda s: (cls[s], code[atoms[s]], atoms[s], amin[s], s))
    return numpy.asarray(order, dtype=numpy.int32)


class DeviceBasis:
    """A packed basis on the current CUDA device."""

    def __init__(self, geo_spec, ao_spec, device="cuda"):
        import torch
        L = _lib.load()
        self.flat = f = flatten(ao_spec)
        geo = numpy.require(numpy.asarray(geo_spec, dtype=numpy.float64).reshape(-1, 3), requirements="CA")
        self.natom = geo.shape[0]
        self.ncart = len(f["lxlylz"])
        self.nshell = len(f["ncart"])
        self.nprim = len(f["prim"])
        self.spherical = f["spherical"]
        self.nao = len(f["sph_ptr"]) - 1 if self.spherical else self.ncart
        self.device = torch.device(device)
        if self.spherical:
            T = numpy.zeros((self.nao, self.ncart))
            for r in range(self.nao):
                for t in range(f["sph_ptr"][r], f["sph_ptr"][r + 1]):
                    T[r, f["sph_idx"][t]] += f["sph_coef"][t]
            self.T = T
            self.T_dev = torch.from_numpy(T).to(self.device)
        else:
            self.T = None
            self.T_dev = None
        h = ctypes.c_void_p()
        ip = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int)) if a is not None else None
        dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if a is not None else None
        nsph = self.nao if self.spherical else 0
        _lib.check(L.okg_basis_create(self.natom, self.nshell, ip(f["atoms"]), ip(f["ncart"]), ip(f["nprim"]),
                                      ip(f["lxlylz"]), f["normalized"], dp(f["renorm"]), nsph,
                                      ip(f.get("sph_ptr")), ip(f.get("sph_idx")), dp(f.get("sph_coef")),
                                      ctypes.byref(h)))
        self._h = h
        self._L = L
        self.mixed_order = mixed_order(geo, f)
        _lib.check(L.okg_basis_set_mixed_order(h, ip(self.mixed_order)))
        self.geo = torch.from_numpy(geo.copy()).to(self.device)
        self.prim = torch.from_numpy(f["prim"].copy()).to(self.device)
        self.set_params()

    @property
    def handle(self):
        return self._h

    def set_params(self, geo=None, prim=None, stream=None):
        """Upload new nuclear positions (natom, 3) and/or primitive [alpha, c] (nprim, 2)."""
        import torch
        if geo is not None:
            self.geo = torch.as_tensor(geo, dtype=torch.float64, device=self.device).reshape(self.natom, 3).contiguous()
        if prim is not None:
            self.prim = torch.as_tensor(prim, dtype=torch.float64, device=self.device).reshape(self.nprim, 2).contiguous()
        _lib.check(self._L.okg_basis_set_params(self._h, _lib.ptr(self.geo), _lib.ptr(self.prim),
                                                _lib.stream_handle(stream)))

    def c_eff(self, coeffs):
        """MO coefficients (nmo, nao) -> Cartesian-basis coefficients (nmo, ncart) on the device."""
        import torch
        C = torch.as_tensor(coeffs, dtype=torch.float64, device=self.device)
        if C.dim() == 1:
            C = C[None, :]
        if C.shape[1] != self.nao:
            raise ValueError("MO coefficients have %d columns, the basis has %d AOs" % (C.shape[1], self.nao))
        if self.spherical:
            # C_eff = C_sph . T by the FP64 contraction kernel (T's Cartesian columns
            # play the role of grid points)
            C = C.contiguous()
            out = torch.empty((C.shape[0], self.ncart), dtype=torch.float64, device=self.device)
            _lib.check(self._L.okg_mo_from_ao(C.shape[0], self.nao, _lib.ptr(C), _lib.ptr(self.T_dev), self.ncart,
                                              self.ncart, _lib.ptr(out), self.ncart, _lib.stream_handle()))
            return out
        return C.contiguous()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._L.okg_basis_destroy(h)
            except Exception:
                pass
            self._h = None


_cache = {}


def get_basis(geo_spec, ao_spec, device="cuda"):
    """Cached DeviceBasis for (geometry, basis); rebuilt when either changes."""
    flat = flatten(ao_spec)
    key = (fingerprint(geo_spec, flat), str(device))
    b = _cache.get(key)
    if b is None:
        if len(_cache) > 8:
            _cache.clear()
        b = DeviceBasis(geo_spec, ao_spec, device)
        _cache[key] = b
    return b
