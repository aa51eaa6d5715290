"""Basis-set and orbital containers with orbkit's interface.

``AOClass`` and ``MOClass`` follow orbkit's classes of the same names
(orbkit/orbitals.py:25-409 and :411-1210) for everything the grid path reads:
the list-of-dicts form of ``ao_spec`` / ``mo_spec`` and the flattened numpy
getters (``get_lxlylz``, ``get_nlxlylz_per_cont``, ``get_prim_coeffs``,
``get_nprim_per_cont``, ``get_assign_cont_to_atoms``, ``get_normalized``,
``get_lm``, ``get_assign_lm_to_cont``, ``get_coeffs``, ``get_occ`` ...).
orbkit's own objects work unchanged with this package; these classes exist so
the package needs no orbkit installation.  MO selection by label strings,
spin handling and file restarts are out of scope.
"""
from collections import UserList
from copy import copy

import numpy

from .tools import cartesian_order, lquant, require


class AOClass(UserList):
    """Contracted Gaussian shells.  Each item is a dict with keys
    'atom', 'type', 'pnum', 'coeffs' ((nprim, 2) [exponent, coefficient]) and
    optionally 'lxlylz', 'lm' (spherical), 'N' (per-Cartesian-AO renormalisation,
    only read from item 0 as orbkit does at core.py:98-100)."""

    def __init__(self, data=None, seq=()):
        if isinstance(data, (list, tuple)):
            seq = data
        UserList.__init__(self, list(seq))
        self._up_to_date = False
        self.normalized = False
        self.spherical = False

    # list mutations invalidate the flattened arrays
    def __setitem__(self, i, item):
        self.data[i] = item
        self._up_to_date = False

    def __delitem__(self, i):
        del self.data[i]
        self._up_to_date = False

    def append(self, item):
        UserList.append(self, item)
        self._up_to_date = False

    def extend(self, item):
        UserList.extend(self, item)
        self._up_to_date = False

    def update(self):
        """Flatten the dict list into arrays (orbitals.py:198-209)."""
        if not self.data:
            raise ValueError("ao_spec not initialized")
        for i, j in enumerate(self.data):
            if not isinstance(j, dict):
                raise ValueError("ao_spec[{0}] has to be a dictionary".format(i))
            missing = [k for k in ("atom", "type", "pnum", "coeffs") if k not in j]
            if self.spherical and "lm" not in j:
                missing.append("lm")
            if missing:
                raise ValueError("ao_spec[{0}] misses {1}".format(i, missing))
        atoms, types, nprim, coeffs, p2c = [], [], [], [], []
        for i, cont in enumerate(self.data):
            c = numpy.asarray(cont["coeffs"], dtype=numpy.float64).reshape(-1, 2)
            atoms.append(cont["atom"])
            types.append(cont["type"])
            nprim.append(len(c))
            coeffs.append(c)
            p2c.extend([i] * len(c))
        self._assign_cont_to_atoms = require(atoms, "i")
        self._cont_types = types
        self._nprim_per_cont = require(nprim, "i")
        self._prim_coeffs = require(numpy.concatenate(coeffs, axis=0) if coeffs else numpy.zeros((0, 2)), "f")
        self._assign_prim_to_cont = require(p2c, "i")

        lxlylz, assign = [], []
        for i, cont in enumerate(self.data):
            if "lxlylz" in cont:
                ll = [tuple(int(v) for v in row) for row in cont["lxlylz"]]
            else:
                ll = cartesian_order[lquant[cont["type"]]]
            lxlylz.extend(ll)
            assign.extend([i] * len(ll))
        self._lxlylz = require(numpy.array(lxlylz, dtype=numpy.intc).reshape(-1, 3), "i")
        self._assign_lxlylz_to_cont = require(assign, "i")
        self._nlxlylz_per_cont = require(numpy.bincount(self._assign_lxlylz_to_cont, minlength=len(self.data)), "i")

        if self.spherical:
            lm, alm = [], []
            for i, cont in enumerate(self.data):
                for v in cont["lm"]:
                    lm.append(tuple(int(t) for t in v))
                    alm.append(i)
            self._lm = require(numpy.array(lm, dtype=numpy.intc).reshape(-1, 2), "i")
            self._assign_lm_to_cont = require(alm, "i")
        else:
            self._lm = None
            self._assign_lm_to_cont = None

        flags = [cont["pnum"] < 0 for cont in self.data]
        if all(flags) != any(flags):
            raise ValueError("Either all or none of the atomic orbitals have to be normalized!")
        self.normalized = all(flags)
        self._up_to_date = True

    def set_lm_dict(self, p=(1, 0)):
        """Real solid harmonics per shell, p in the order given by ``p`` (orbitals.py:303-316)."""
        for cont in self.data:
            l = lquant[cont["type"]]
            cont["lm"] = []
            for m in (range(0, l + 1) if l != 1 else p):
                cont["lm"].append((l, m))
                if m != 0:
                    cont["lm"].append((l, -m))
        self.spherical = True
        self._up_to_date = False

    def _get(self, name):
        if not self._up_to_date:
            self.update()
        return copy(getattr(self, name))

    def get_assign_cont_to_atoms(self):
        return self._get("_assign_cont_to_atoms")

    def get_cont_types(self):
        return self._get("_cont_types")

    def get_nprim_per_cont(self):
        return self._get("_nprim_per_cont")

    def get_prim_coeffs(self):
        return self._get("_prim_coeffs")

    def get_assign_prim_to_cont(self):
        return self._get("_assign_prim_to_cont")

    def get_lxlylz(self):
        return self._get("_lxlylz")

    def get_assign_lxlylz_to_cont(self):
        return self._get("_assign_lxlylz_to_cont")

    def get_nlxlylz_per_cont(self):
        return self._get("_nlxlylz_per_cont")

    def get_lm(self):
        return self._get("_lm")

    def get_assign_lm_to_cont(self):
        return self._get("_assign_lm_to_cont")

    def get_normalized(self):
        if not self._up_to_date:
            self.update()
        return int(self.normalized)

    def get_old_ao_spherical(self):
        if not self._up_to_date:
            self.update()
        return list(zip(self.get_assign_lm_to_cont(), [tuple(v) for v in self.get_lm()])) if self.spherical else []

    def get_ao_num(self):
        if not self._up_to_date:
            self.update()
        return len(self._lm) if self.spherical else len(self._lxlylz)

    def get_labels(self):
        if not self._up_to_date:
            self.update()
        atoms = self._assign_cont_to_atoms
        if self.spherical:
            return ["l,m=%s,atom=%d" % (tuple(self._lm[i]), atoms[j]) for i, j in enumerate(self._assign_lm_to_cont)]
        return ["lxlylz=%s,atom=%d" % (tuple(self._lxlylz[i]), atoms[j]) for i, j in enumerate(self._assign_lxlylz_to_cont)]


class MOClass(UserList):
    """Molecular orbitals: dicts with 'coeffs' (NAO,), 'occ_num', 'energy', 'sym'."""

    def __init__(self, data=None, seq=()):
        if isinstance(data, (list, tuple)):
            seq = data
        UserList.__init__(self, list(seq))
        self._up_to_date = False
        self.coeffs = None
        self.occ = None
        self.eig = None
        self.sym = None

    def __getitem__(self, item):
        if isinstance(item, (int, numpy.integer)):
            return self.data[item]
        if isinstance(item, slice):
            return MOClass(self.data[item])
        idx = numpy.asarray(item)
        if idx.dtype == bool:
            idx = numpy.nonzero(idx)[0]
        return MOClass([self.data[int(i)] for i in idx])

    def __setitem__(self, i, item):
        self.data[i] = item
        self._up_to_date = False

    def append(self, item):
        UserList.append(self, item)
        self._up_to_date = False

    def update(self):
        self.coeffs = require(numpy.array([m["coeffs"] for m in self.data], dtype=numpy.float64), "f")
        self.occ = require([m["occ_num"] for m in self.data], "f")
        self.eig = require([m.get("energy", 0.0) for m in self.data], "f")
        self.sym = numpy.array([str(m.get("sym", "%d.1" % (i + 1))) for i, m in enumerate(self.data)])
        self._up_to_date = True

    def get_coeffs(self):
        if not self._up_to_date:
            self.update()
        return copy(self.coeffs)

    def get_occ(self):
        if not self._up_to_date:
            self.update()
        return copy(self.occ)

    def get_eig(self):
        if not self._up_to_date:
            self.update()
        return copy(self.eig)

    def get_labels(self, format="default"):
        if format == "print":
            return ["%s (Occ = %.2f, E = %+.4f E_h)" % (m.get("sym", "?"), m["occ_num"], m.get("energy", 0.0))
                    for m in self.data]
        return ["%s, Occ=%.2f, E=%+.4f E_h" % (m.get("sym", "?"), m["occ_num"], m.get("energy", 0.0)) for m in self.data]
