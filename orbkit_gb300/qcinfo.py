"""``QCinfo``: geometry plus basis and orbitals, as orbkit's container of the same
name (orbkit/qcinfo.py:35-63) exposes them to the grid path.

``geo_spec`` is (NATOMS, 3) in bohr, ``ao_spec`` an ``AOClass`` and ``mo_spec`` a
``MOClass``.  orbkit's own ``QCinfo`` objects (or dicts with the same keys) work
with this package directly.
"""
import numpy

from .orbitals import AOClass, MOClass


class QCinfo:
    def __init__(self, data=None):
        self.geo_info = []
        self.geo_spec = []
        self.ao_spec = AOClass()
        self.mo_spec = MOClass()
        if data:
            self.geo_spec = numpy.asarray(data["geo_spec"], dtype=numpy.float64)
            self.geo_info = data.get("geo_info", [])
            self.ao_spec = data["ao_spec"] if isinstance(data["ao_spec"], AOClass) else AOClass(list(data["ao_spec"]))
            self.mo_spec = data["mo_spec"] if isinstance(data["mo_spec"], MOClass) else MOClass(list(data["mo_spec"]))

    def update(self):
        self.ao_spec.update()
        self.mo_spec.update()


def unpack(qc):
    """(geo_spec, ao_spec, mo_spec) of a QCinfo-like object or dict."""
    if isinstance(qc, dict):
        return numpy.asarray(qc["geo_spec"], dtype=numpy.float64), qc["ao_spec"], qc["mo_spec"]
    return numpy.asarray(qc.geo_spec, dtype=numpy.float64), qc.ao_spec, qc.mo_spec


def to_arrays(qc):
    """Flat numpy form of a QCinfo-like object (portable, e.g. for .npz files)."""
    geo, ao, mo = unpack(qc)
    ao.update() if hasattr(ao, "update") else None
    d = {
        "geo_spec": numpy.asarray(geo, dtype=numpy.float64),
        "shell_atom": numpy.array([s["atom"] for s in ao], dtype=numpy.intc),
        "shell_type": numpy.array([s["type"] for s in ao]),
        "shell_pnum": numpy.array([s["pnum"] for s in ao], dtype=numpy.intc),
        "shell_nprim": numpy.array([len(s["coeffs"]) for s in ao], dtype=numpy.intc),
        "prim_coeffs": numpy.concatenate([numpy.asarray(s["coeffs"], dtype=numpy.float64).reshape(-1, 2) for s in ao]),
        "lxlylz": numpy.asarray(ao.get_lxlylz(), dtype=numpy.intc),
        "ncart": numpy.asarray(ao.get_nlxlylz_per_cont(), dtype=numpy.intc),
        "spherical": numpy.array(bool(getattr(ao, "spherical", False))),
        "mo_coeffs": numpy.asarray(mo.get_coeffs(), dtype=numpy.float64),
        "mo_occ": numpy.array([m["occ_num"] for m in mo], dtype=numpy.float64),
    }
    if d["spherical"]:
        d["lm"] = numpy.asarray(ao.get_lm(), dtype=numpy.intc)
        d["nlm"] = numpy.bincount(ao.get_assign_lm_to_cont(), minlength=len(ao)).astype(numpy.intc)
    if "N" in ao[0]:
        d["renorm"] = numpy.asarray(ao[0]["N"], dtype=numpy.float64)
    return d


def from_arrays(d):
    """Inverse of ``to_arrays``: a QCinfo with this package's AOClass/MOClass."""
    off = numpy.concatenate([[0], numpy.cumsum(d["shell_nprim"])])
    coff = numpy.concatenate([[0], numpy.cumsum(d["ncart"])])
    shells = []
    for i in range(len(d["shell_atom"])):
        s = {"atom": int(d["shell_atom"][i]), "type": str(d["shell_type"][i]), "pnum": int(d["shell_pnum"][i]),
             "coeffs": numpy.array(d["prim_coeffs"][off[i]:off[i + 1]]),
             "lxlylz": [tuple(int(v) for v in r) for r in d["lxlylz"][coff[i]:coff[i + 1]]]}
        shells.append(s)
    if "renorm" in d:
        shells[0]["N"] = numpy.array(d["renorm"])
    if bool(d["spherical"]):
        loff = numpy.concatenate([[0], numpy.cumsum(d["nlm"])])
        for i, s in enumerate(shells):
            s["lm"] = [tuple(int(v) for v in r) for r in d["lm"][loff[i]:loff[i + 1]]]
    ao = AOClass(shells)
    ao.spherical = bool(d["spherical"])
    ao.update()
    mo = MOClass([{"coeffs": numpy.array(d["mo_coeffs"][i]), "occ_num": float(d["mo_occ"][i]), "energy": 0.0,
                   "sym": "%d.1" % (i + 1)} for i in range(len(d["mo_occ"]))])
    mo.update()
    qc = QCinfo()
    qc.geo_spec = numpy.array(d["geo_spec"], dtype=numpy.float64)
    qc.ao_spec = ao
    qc.mo_spec = mo
    return qc
