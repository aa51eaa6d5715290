"""CPU oracle for orbkit's grid path -- TEST INFRASTRUCTURE, never the product.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module, and only as the checker.  It restates the
reference algorithm on the CPU:

  * numerical kernels in plain C (``oracle/okref.c``; bit-identical to the
    reference's extension when both are built without FMA contraction),
  * the Python drivers of orbkit/core.py restated with numpy:
      ao_creator            core.py:38-105
      mo_creator            core.py:107-132
      cartesian2spherical   core.py:135-176
      rho_compute           core.py:314-605  (sliced; in-process, or POSIX threads
                                              over slices instead of a process pool)
      rho_compute_no_slice  core.py:607-839

Parity pins: against the reference's own golden file
(test/grid_based/refdata_rho_compute.npz, committed here as tests/golden/h2o_molden.npz
with the generating script) and, in the development container, against the
reference extension itself (tests/test_oracle.py).
"""
import ctypes
import os
import subprocess

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "okref.c")
LIB = os.path.join(BUILD, "libokref.so")

_lib = None


def build(force=False):
    """Compile okref.c (gcc, -O2, no FMA contraction) into oracle/_build/libokref.so."""
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + ".tmp%d" % os.getpid()
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", tmp, SRC, "-lm",
                               "-lpthread"])
        os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        L.okref_aocreator.argtypes = [dp, ip, ip, dp, ip, dp, ip, ctypes.c_int, dp, dp, dp, ctypes.c_long,
                                      ctypes.c_int, ctypes.c_int]
        L.okref_mocreator.argtypes = [dp, dp, dp, ctypes.c_int, ctypes.c_int, ctypes.c_long]
        L.okref_get_ao_xyz.argtypes = [ctypes.c_double] * 3 + [ctypes.c_int] * 3 + [ctypes.c_double, ctypes.c_int]
        L.okref_get_ao_xyz.restype = ctypes.c_double
        L.okref_ao_norm.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double, ctypes.c_int]
        L.okref_ao_norm.restype = ctypes.c_double
        L.okref_slice_rho.restype = ctypes.c_int
        L.okref_rho_threads.restype = ctypes.c_int
        L.okref_aooverlap.argtypes = [dp, dp, dp, ip, ip, ip, dp, ip, ip, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.okref_mooverlapmatrix.argtypes = [dp, dp, dp, dp] + [ctypes.c_int] * 4
        _lib = L
    return _lib


def _p(a, t=ctypes.c_double):
    return a.ctypes.data_as(ctypes.POINTER(t))


def _f(a):
    return numpy.require(a, dtype=numpy.float64, requirements="CA")


def _i(a):
    return numpy.require(a, dtype=numpy.intc, requirements="CA")


DRV = {None: 0, "None": 0, "": 0, "x": 1, "y": 2, "z": 3, "xx": 4, "x2": 4, "yy": 5, "y2": 5, "zz": 6, "z2": 6,
       "xy": 7, "yx": 7, "xz": 8, "zx": 8, "yz": 9, "zy": 9}


def validate_drv(drv):
    """orbkit/tools.py:225-239."""
    if isinstance(drv, str) or drv is None:
        if drv in DRV:
            return DRV[drv]
        raise ValueError("The selection `drv=%s` is not valid!" % drv)
    if isinstance(drv, (int, numpy.integer)) and 0 <= drv <= 9:
        return int(drv)
    raise ValueError("The selection `drv=%s` is not valid!" % drv)


def grid2vector(x, y, z):
    """orbkit/cy_grid.pyx:14-30 (x slowest, z fastest)."""
    out = numpy.zeros((3, len(x) * len(y) * len(z)))
    out[0] = numpy.repeat(x, len(y) * len(z))
    out[1] = numpy.tile(numpy.repeat(y, len(z)), len(x))
    out[2] = numpy.tile(z, len(x) * len(y))
    return out


def aocreator(geo_spec, ao_spec, x, y, z, drv):
    """cy_core.aocreator -> (NAOcart, npts) float64."""
    L = lib()
    lxlylz = _i(ao_spec.get_lxlylz())
    assign = _i(ao_spec.get_nlxlylz_per_cont())
    coeffs = _f(ao_spec.get_prim_coeffs())
    pnum = _i(ao_spec.get_nprim_per_cont())
    atoms = _i(ao_spec.get_assign_cont_to_atoms())
    geo = _f(geo_spec)
    x, y, z = _f(x), _f(y), _f(z)
    out = numpy.zeros((len(lxlylz), len(x)))
    L.okref_aocreator(_p(out), _p(lxlylz, ctypes.c_int), _p(assign, ctypes.c_int), _p(coeffs), _p(pnum, ctypes.c_int),
                      _p(geo), _p(atoms, ctypes.c_int), len(assign), _p(x), _p(y), _p(z), len(x), int(drv),
                      int(ao_spec.get_normalized()))
    return out


def mocreator(ao_list, coeffs):
    """cy_core.mocreator: naive (i, j, k) triple loop."""
    ao_list = _f(ao_list)
    coeffs = _f(coeffs)
    out = numpy.zeros((coeffs.shape[0], ao_list.shape[1]))
    lib().okref_mocreator(_p(out), _p(ao_list), _p(coeffs), ao_list.shape[0], coeffs.shape[0], ao_list.shape[1])
    return out


def cartesian2spherical(ao_list, ao_spec):
    """core.py:135-176, evaluated in the same order."""
    from_tab = _cart2sph_lookup()
    lxlylz = ao_spec.get_lxlylz()
    assign = ao_spec.get_assign_lxlylz_to_cont()
    sph = ao_spec.get_old_ao_spherical()
    l = [[] for _ in range(len(ao_spec))]
    for i, j in enumerate(assign):
        l[j].append(i)
    shape = list(ao_list.shape)
    shape[0] = len(sph)
    out = numpy.zeros(shape)
    for i0, (j0, k0) in enumerate(sph):
        comps, coefs, fac = from_tab(*k0)
        index0 = None
        for c0 in range(len(comps)):
            for i, j in enumerate(l[j0]):
                if tuple(lxlylz[j]) == comps[c0]:
                    index0 = i + l[j0][0]
            out[i0, :] += coefs[c0] * fac * ao_list[index0, :]
    return out


_tab = None


def _cart2sph_lookup():
    """The Schlegel-Frisch table in orbkit's form (orbkit/tools.py:155-191)."""
    global _tab
    if _tab is None:
        s = numpy.sqrt
        t = [
            [[[(0, 0, 0)], [1.], 1.]],
            [[[(0, 1, 0)], [1.], 1.], [[(0, 0, 1)], [1.], 1.], [[(1, 0, 0)], [1.], 1.]],
            [[[(1, 1, 0)], [1.], 1.], [[(0, 1, 1)], [1.], 1.],
             [[(0, 0, 2), (2, 0, 0), (0, 2, 0)], [1., -1 / 2., -1 / 2.], 1.],
             [[(1, 0, 1)], [1.], 1.], [[(2, 0, 0), (0, 2, 0)], [1., -1.], s(3) / 2.]],
            [[[(0, 3, 0), (2, 1, 0)], [-s(5), 3.], 1 / (2. * s(2))], [[(1, 1, 1)], [1.], 1.],
             [[(0, 1, 2), (0, 3, 0), (2, 1, 0)], [s(3 / 5.), -s(3) / 4., -s(3) / (4. * s(5))], s(2)],
             [[(0, 0, 3), (2, 0, 1), (0, 2, 1)], [1., -3 / (2 * s(5)), -3 / (2 * s(5))], 1.],
             [[(1, 0, 2), (3, 0, 0), (1, 2, 0)], [s(3 / 5.), -s(3) / 4., -s(3) / (4. * s(5))], s(2)],
             [[(2, 0, 1), (0, 2, 1)], [1., -1.], s(3) / 2.],
             [[(3, 0, 0), (1, 2, 0)], [s(5), -3.], 1 / (2. * s(2))]],
            [[[(3, 1, 0), (1, 3, 0)], [1., -1.], s(2) * s(5 / 8.)],
             [[(0, 3, 1), (2, 1, 1)], [-s(5) / 4., 3 / 4.], s(2)],
             [[(1, 1, 2), (3, 1, 0), (1, 3, 0)], [3 / s(14), -s(5) / (2 * s(14)), -s(5) / (2 * s(14))], s(2)],
             [[(0, 3, 1), (0, 3, 1), (2, 1, 1)], [s(5 / 7.), -3 * s(5) / (4. * s(7)), -3 / (4. * s(7))], s(2)],
             [[(0, 0, 4), (4, 0, 0), (0, 4, 0), (2, 0, 2), (0, 2, 2), (2, 2, 0)],
              [1., 3 / 8., 3 / 8., -3 * s(3) / s(35), -3 * s(3) / s(35), -1 / 4.], s(2)],
             [[(1, 0, 3), (3, 0, 1), (1, 2, 1)], [s(5 / 7.), -3 * s(5) / (4. * s(7)), -3 / (4. * s(7))], s(2)],
             [[(2, 0, 2), (0, 2, 2), (4, 0, 0), (0, 4, 0)],
              [3 * s(3) / (2. * s(14)), -3 * s(3) / (2. * s(14)), -s(5) / (4. * s(2)), s(5) / (4. * s(2))], s(2)],
             [[(3, 0, 1), (1, 2, 1)], [s(5) / 4., -3 / 4.], s(2)],
             [[(4, 0, 0), (0, 4, 0), (2, 2, 0)], [s(35) / (8. * s(2)), s(35) / (8. * s(2)), -3 * s(3) / (4. * s(2))],
              s(2)]],
        ]
        _tab = lambda l, m: t[int(l)][int(l) + int(m)]
    return _tab


def ao_creator(geo_spec, ao_spec, drv=None, x=None, y=None, z=None, is_vector=True):
    """core.py:38-105 with an explicit grid."""
    if not is_vector:
        N = (len(x), len(y), len(z))
        x, y, z = grid2vector(x, y, z)
    else:
        if len(x) != len(y) or len(x) != len(z):
            raise ValueError("Dimensions of x-, y-, and z- coordinate differ!")
        N = (len(x),)
    ao_list = aocreator(geo_spec, ao_spec, x, y, z, validate_drv(drv))
    if "N" in ao_spec[0]:
        ao_list *= ao_spec[0]["N"]
    if ao_spec.spherical:
        ao_list = cartesian2spherical(ao_list, ao_spec)
    if not is_vector:
        return ao_list.reshape((len(ao_list),) + N, order="C")
    return ao_list


def mo_creator(ao_list, mo_spec):
    """core.py:107-132."""
    ao_list = _f(ao_list)
    shape = ao_list.shape
    coeffs = mo_spec.get_coeffs()
    return mocreator(ao_list.reshape(shape[0], -1), coeffs).reshape((len(coeffs),) + shape[1:], order="C")


def _unpack(qc):
    if isinstance(qc, dict):
        return qc["geo_spec"], qc["ao_spec"], qc["mo_spec"]
    return qc.geo_spec, qc.ao_spec, qc.mo_spec


def _normalise_drv(drv, laplacian):
    if laplacian:
        drv = ["xx", "yy", "zz"]
    if drv is None:
        return None
    if isinstance(drv, str):
        return [drv] if drv in DRV else list(drv)
    try:
        return list(drv)
    except TypeError:
        return [drv]


def slice_rho(qc, x, y, z, calc_ao=False, calc_mo=False, drv=None):
    """core.py:179-308 for one slice of a vector grid."""
    geo_spec, ao_spec, mo_spec = _unpack(qc)
    _mo = (lambda a, m: a) if calc_ao else mo_creator
    if drv is not None and calc_mo:
        return numpy.array([_mo(ao_creator(geo_spec, ao_spec, drv=d, x=x, y=y, z=z), mo_spec) for d in drv])
    mo_list = _mo(ao_creator(geo_spec, ao_spec, x=x, y=y, z=z), mo_spec)
    if calc_mo:
        return numpy.array(mo_list)
    occ = [m["occ_num"] for m in mo_spec]
    rho = numpy.zeros(len(x))
    mo_norm = numpy.zeros(len(mo_list))
    for i in range(len(mo_list)):
        mo_norm[i] = numpy.sum(numpy.square(mo_list[i]))
        rho += occ[i] * numpy.square(numpy.abs(mo_list[i]))
    if drv is None:
        return rho, mo_norm
    delta_rho = numpy.zeros((len(drv), len(x)))
    for i, d in enumerate(drv):
        dmo = mo_creator(ao_creator(geo_spec, ao_spec, drv=d, x=x, y=y, z=z), mo_spec)
        if isinstance(d, str) and len(d) == 2:
            a0 = mo_creator(ao_creator(geo_spec, ao_spec, drv=d[0], x=x, y=y, z=z), mo_spec)
            if "2" in d or d[0] == d[1]:
                d2 = numpy.array(a0) ** 2
            else:
                d2 = numpy.array(a0) * numpy.array(mo_creator(ao_creator(geo_spec, ao_spec, drv=d[1], x=x, y=y, z=z),
                                                              mo_spec))
        for k in range(len(mo_list)):
            delta_rho[i] += occ[k] * 2 * dmo[k] * mo_list[k]
            if isinstance(d, str) and len(d) == 2:
                delta_rho[i] += occ[k] * 2 * d2[k]
    return rho, mo_norm, delta_rho


def rho_compute(qc, calc_ao=False, calc_mo=False, drv=None, laplacian=False, slice_length=1e4, x=None, y=None,
                z=None, is_vector=True):
    """core.py:314-605 (numproc=1, in-RAM) with an explicit grid."""
    if calc_ao and calc_mo:
        raise ValueError("Choose either calc_ao=True or calc_mo=True")
    elif calc_ao:
        calc_mo = True
    geo_spec, ao_spec, mo_spec = _unpack(qc)
    drv = _normalise_drv(drv, laplacian)
    N = (len(x),) if is_vector else (len(x), len(y), len(z))
    if not is_vector:
        x, y, z = grid2vector(x, y, z)
    npts = len(x)
    mo_num = ao_spec.get_ao_num() if calc_ao else len(mo_spec)
    if slice_length <= 0:
        slice_length = npts + 1
    slice_length = int(slice_length)
    bounds = [(i, min(i + slice_length, npts)) for i in range(0, npts, slice_length)]
    if calc_mo:
        out = numpy.zeros((mo_num, npts) if drv is None else (len(drv), mo_num, npts))
    else:
        rho = numpy.zeros(npts)
        delta_rho = numpy.zeros((len(drv), npts)) if drv is not None else None
    for (i, j) in bounds:
        r = slice_rho(qc, x[i:j], y[i:j], z[i:j], calc_ao=calc_ao, calc_mo=calc_mo, drv=drv)
        if calc_mo:
            if drv is None:
                out[:, i:j] = r
            else:
                out[:, :, i:j] = r
        else:
            rho[i:j] = r[0]
            if drv is not None:
                delta_rho[:, i:j] = r[2]
    if calc_mo:
        return out.reshape(((mo_num,) if drv is None else (len(drv), mo_num)) + N)
    rho = rho.reshape(N)
    if drv is None:
        return rho
    delta_rho = delta_rho.reshape((len(drv),) + N)
    if laplacian:
        return rho, delta_rho, delta_rho.sum(axis=0)
    return rho, delta_rho


def rho_compute_no_slice(qc, calc_ao=False, calc_mo=False, drv=None, laplacian=False, return_components=False,
                         x=None, y=None, z=None, is_vector=True):
    """core.py:607-839 with an explicit grid."""
    if calc_ao and calc_mo:
        raise ValueError("calc_ao and calc_mo are mutually exclusive arguments.")
    geo_spec, ao_spec, mo_spec = _unpack(qc)
    was_vector = is_vector
    if not is_vector:
        N = (len(x), len(y), len(z))
        x, y, z = grid2vector(x, y, z)
    else:
        N = (len(x),)

    def conv(d):
        d = numpy.array(d, order="C")
        return d if was_vector else d.reshape(d.shape[:-1] + N, order="C")

    drv = _normalise_drv(drv, laplacian)
    if drv is not None:
        dao = [ao_creator(geo_spec, ao_spec, drv=d, x=x, y=y, z=z) for d in drv]
        dmo = [None] * len(drv) if calc_ao else [mo_creator(a, mo_spec) for a in dao]
        dao = conv(dao)
        if calc_ao:
            return dao
        dmo = conv(dmo)
        if calc_mo:
            return (dao, dmo) if return_components else dmo
        d2 = [None] * len(drv)
        for i, d in enumerate(drv):
            if isinstance(d, str) and len(d) == 2:
                a0 = ao_creator(geo_spec, ao_spec, drv=d[0], x=x, y=y, z=z)
                if "2" in d or d in ("xx", "yy", "zz"):
                    d2[i] = mo_creator(a0, mo_spec) ** 2
                else:
                    a1 = ao_creator(geo_spec, ao_spec, drv=d[1], x=x, y=y, z=z)
                    d2[i] = mo_creator(a0, mo_spec) * mo_creator(a1, mo_spec)
                d2[i] = conv(d2[i])
    ao_list = ao_creator(geo_spec, ao_spec, x=x, y=y, z=z)
    if not calc_ao:
        mo_list = conv(mo_creator(ao_list, mo_spec))
    ao_list = conv(ao_list)
    if calc_ao:
        return ao_list
    if calc_mo:
        return (ao_list, mo_list) if return_components else mo_list
    occ = [m["occ_num"] for m in mo_spec]
    rho = numpy.zeros(N)
    for i in range(len(mo_list)):
        rho += numpy.square(numpy.abs(mo_list[i])) * occ[i]
    if drv is None:
        return (ao_list, mo_list, rho) if return_components else rho
    delta_rho = numpy.zeros((len(drv),) + N)
    for i, d in enumerate(drv):
        for k in range(len(mo_list)):
            delta_rho[i] += occ[k] * 2 * dmo[i, k] * mo_list[k]
            if isinstance(d, str) and len(d) == 2:
                delta_rho[i] += occ[k] * 2 * d2[i][k]
    delta = (delta_rho, delta_rho.sum(axis=0)) if laplacian else (delta_rho,)
    return ((ao_list, mo_list, rho, dao, dmo) + delta) if return_components else (rho,) + delta


class Basis:
    """Flattened basis + MOs for the threaded C driver (keeps the arrays alive)."""

    def __init__(self, qc):
        geo_spec, ao_spec, mo_spec = _unpack(qc)
        self.lxlylz = _i(ao_spec.get_lxlylz())
        self.assign = _i(ao_spec.get_nlxlylz_per_cont())
        self.coeffs = _f(ao_spec.get_prim_coeffs())
        self.pnum = _i(ao_spec.get_nprim_per_cont())
        self.geo = _f(geo_spec)
        self.atoms = _i(ao_spec.get_assign_cont_to_atoms())
        self.renorm = _f(numpy.asarray(ao_spec[0]["N"]).reshape(-1)) if "N" in ao_spec[0] else None
        self.C = _f(mo_spec.get_coeffs())
        self.occ = _f([m["occ_num"] for m in mo_spec])
        ptr, idx, coef = [0], [], []
        if ao_spec.spherical:
            tab = _cart2sph_lookup()
            lxl = ao_spec.get_lxlylz()
            l = [[] for _ in range(len(ao_spec))]
            for i, j in enumerate(ao_spec.get_assign_lxlylz_to_cont()):
                l[j].append(i)
            for (j0, k0) in ao_spec.get_old_ao_spherical():
                comps, cf, fac = tab(*k0)
                index0 = None
                for c0 in range(len(comps)):
                    for i, j in enumerate(l[j0]):
                        if tuple(lxl[j]) == comps[c0]:
                            index0 = i + l[j0][0]
                    idx.append(index0)
                    coef.append(cf[c0] * fac)
                ptr.append(len(idx))
        self.nsph = len(ptr) - 1
        self.sph_ptr = _i(ptr)
        self.sph_idx = _i(idx if idx else [0])
        self.sph_coef = _f(coef if coef else [0.0])

        class S(ctypes.Structure):
            _fields_ = [("lxlylz", ctypes.c_void_p), ("assign", ctypes.c_void_p), ("coeffs", ctypes.c_void_p),
                        ("pnum", ctypes.c_void_p), ("geo", ctypes.c_void_p), ("atom_idx", ctypes.c_void_p),
                        ("nshell", ctypes.c_int), ("ncart", ctypes.c_int), ("is_normalized", ctypes.c_int),
                        ("renorm", ctypes.c_void_p), ("nsph", ctypes.c_int), ("sph_ptr", ctypes.c_void_p),
                        ("sph_idx", ctypes.c_void_p), ("sph_coef", ctypes.c_void_p), ("C", ctypes.c_void_p),
                        ("occ", ctypes.c_void_p), ("nmo", ctypes.c_int)]

        self.s = S(self.lxlylz.ctypes.data, self.assign.ctypes.data, self.coeffs.ctypes.data, self.pnum.ctypes.data,
                   self.geo.ctypes.data, self.atoms.ctypes.data, len(self.assign), len(self.lxlylz),
                   int(ao_spec.get_normalized()), self.renorm.ctypes.data if self.renorm is not None else None,
                   self.nsph, self.sph_ptr.ctypes.data, self.sph_idx.ctypes.data, self.sph_coef.ctypes.data,
                   self.C.ctypes.data, self.occ.ctypes.data, len(self.occ))


def rho_threads(qc, x, y, z, drv=("x", "y", "z"), slice_length=10000, nthreads=None):
    """rho and delta_rho on a vector grid, slices spread over POSIX threads.

    Same per-slice algorithm and results as ``rho_compute(qc, drv=drv)``; used as
    the timed CPU baseline.  Returns (rho, delta_rho)."""
    b = Basis(qc)
    x, y, z = _f(x), _f(y), _f(z)
    drv = list(drv) if drv is not None else []
    codes = _i([validate_drv(d) for d in drv] or [0])
    a = _i([validate_drv(d[0]) if isinstance(d, str) and len(d) == 2 else 0 for d in drv] or [0])
    bb = _i([validate_drv(d[1]) if isinstance(d, str) and len(d) == 2 and d[1] in "xyz" else 0 for d in drv] or [0])
    sq = _i([1 if isinstance(d, str) and len(d) == 2 and ("2" in d or d[0] == d[1]) else 0 for d in drv] or [0])
    rho = numpy.zeros(len(x))
    drho = numpy.zeros((max(len(drv), 1), len(x)))
    if nthreads is None:
        nthreads = len(os.sched_getaffinity(0))
    L = lib()
    vp = ctypes.c_void_p
    L.okref_rho_threads.argtypes = [ctypes.POINTER(type(b.s)), vp, vp, vp, ctypes.c_long, ctypes.c_int, vp, vp, vp,
                                    vp, vp, vp, ctypes.c_long, ctypes.c_int]
    err = L.okref_rho_threads(ctypes.byref(b.s), x.ctypes.data, y.ctypes.data, z.ctypes.data, len(x), len(drv),
                              codes.ctypes.data, a.ctypes.data, bb.ctypes.data, sq.ctypes.data, rho.ctypes.data,
                              drho.ctypes.data, int(slice_length), int(nthreads))
    if err:
        raise MemoryError("oracle slice allocation failed")
    return rho, drho[:len(drv)]


# ------------------------------------------------------------------- detCI
# CI (transition) density and flux density on a grid from MO grids, restating the
# loops of orbkit/detci/cy_ci.pyx: terms in the given order, every product and sum
# rounded as written there (numpy float64 elementwise operations, no FMA).
# zero = [coefficient lists, orbital lists], sing = [coefficients, orbital pairs]
# as produced by orbkit/detci/occ_check.py.

def ci_rho(zero, sing, molist):
    """orbkit/detci/cy_ci.pyx:70-96 (get_rho) over all points."""
    mo = numpy.asarray(molist, dtype=numpy.float64).reshape(len(molist), -1)
    rho = numpy.zeros(mo.shape[1])
    for cs, js in zip(zero[0], zero[1]):
        for c, j in zip(cs, js):
            rho += (c * mo[j]) * mo[j]
    for c, (a, b) in zip(sing[0], sing[1]):
        rho += (c * mo[a]) * mo[b]
    return rho.reshape(numpy.shape(molist)[1:])


def ci_jab(zero, sing, molist, molistdrv):
    """orbkit/detci/cy_ci.pyx:152-178 (get_jab): -sum 0.5 c (MO_a dMO_b - MO_b dMO_a)."""
    mo = numpy.asarray(molist, dtype=numpy.float64).reshape(len(molist), -1)
    dr = numpy.asarray(molistdrv, dtype=numpy.float64).reshape(3, len(molist), -1)
    j = numpy.zeros((3, mo.shape[1]))
    for c, (a, b) in zip(sing[0], sing[1]):
        for d in range(3):
            j[d] -= 0.5 * (c * (mo[a] * dr[d, b] - mo[b] * dr[d, a]))
    return j.reshape((3,) + numpy.shape(molist)[1:])


def ci_a_nabla_b(zero, sing, molist, molistdrv):
    """orbkit/detci/cy_ci.pyx:203-229 (get_a_nabla_b): sum c MO_a dMO_b."""
    mo = numpy.asarray(molist, dtype=numpy.float64).reshape(len(molist), -1)
    dr = numpy.asarray(molistdrv, dtype=numpy.float64).reshape(3, len(molist), -1)
    j = numpy.zeros((3, mo.shape[1]))
    for c, (a, b) in zip(sing[0], sing[1]):
        for d in range(3):
            j[d] += c * (mo[a] * dr[d, b])
    return j.reshape((3,) + numpy.shape(molist)[1:])


def ci_covered(npts, slice_length):
    """Points orbkit's detCI drivers evaluate (orbkit/detci/ci_core.py:120-125): the
    slices come from arange(0, npts + 1, s) with s = min(npts, slice_length), so the
    trailing npts % s points are never evaluated and stay 0."""
    s = int(min(npts, abs(int(slice_length))))
    return (npts // s) * s if s > 0 else 0


def ci_driver(fn, zero, sing, molist, *rest, slice_length=1e4):
    """orbkit/detci/ci_core.py rho/jab/a_nabla_b: fn over all points, then the
    driver's slicing (points beyond the last full slice left 0)."""
    out = fn(zero, sing, molist, *rest)
    shape = out.shape
    flat = out.reshape(shape[:-len(numpy.shape(molist)[1:])] + (-1,)) if len(shape) > len(numpy.shape(molist)[1:]) \
        else out.reshape(-1)
    n = flat.shape[-1]
    flat[..., ci_covered(n, slice_length):] = 0.0
    return flat.reshape(shape)


# ------------------------------------------------------------------ AO overlap
def aooverlap(coord_a, coord_b, lxlylz_a, lxlylz_b, ao_spec, drv):
    """cy_overlap.aooverlap (orbkit/cy_overlap.pyx:78-163) -> (NAOcart, NAOcart)."""
    lxa = _i(lxlylz_a)
    lxb = _i(lxlylz_b)
    assign = _i(ao_spec.get_nlxlylz_per_cont())
    coeffs = _f(ao_spec.get_prim_coeffs())
    pnum = _i(ao_spec.get_nprim_per_cont())
    atoms = _i(ao_spec.get_assign_cont_to_atoms())
    out = numpy.zeros((len(lxa), len(lxa)))
    lib().okref_aooverlap(_p(out), _p(_f(coord_a)), _p(_f(coord_b)), _p(lxa, ctypes.c_int), _p(lxb, ctypes.c_int),
                          _p(assign, ctypes.c_int), _p(coeffs), _p(pnum, ctypes.c_int), _p(atoms, ctypes.c_int),
                          len(assign), int(drv), int(ao_spec.get_normalized()))
    return out


def cartesian2spherical_aoom(aoom, ao_spec):
    """orbkit/analytical_integrals.py:118-182, evaluated in the same order: for every
    output pair (i0, i1) the terms are added component of i0 outer, of i1 inner, each
    (coef0 fac0 coef1 fac1) S[row0, row1]."""
    tab = _cart2sph_lookup()
    lxlylz = ao_spec.get_lxlylz()
    assign = ao_spec.get_assign_lxlylz_to_cont()
    sph = ao_spec.get_old_ao_spherical()
    rows = [[] for _ in range(len(ao_spec))]
    for i, j in enumerate(assign):
        rows[j].append(i)
    terms = []  # per spherical row: list of (coef, fac, Cartesian row)
    for (j0, k0) in sph:
        comps, coefs, fac = tab(*k0)
        t = []
        for c0, comp in enumerate(comps):
            for i, j in enumerate(rows[j0]):
                if tuple(lxlylz[j]) == comp:
                    t.append((coefs[c0], fac, i + rows[j0][0]))
        terms.append(t)
    n = len(sph)
    out = numpy.zeros((n, n))
    for i0 in range(n):
        for (a0, f0, r0) in terms[i0]:
            for i1 in range(n):
                for (a1, f1, r1) in terms[i1]:
                    out[i0, i1] += a0 * f0 * a1 * f1 * aoom[r0, r1]
    return out


def ao_overlap(coord_a, coord_b, ao_spec, lxlylz_b=None, drv=None):
    """get_ao_overlap (orbkit/analytical_integrals.py:37-116): aooverlap, then the
    'N' factor on rows and columns, then the spherical transform."""
    if isinstance(drv, list) or (isinstance(drv, str) and len(drv) > 1):
        return [ao_overlap(coord_a, coord_b, ao_spec, lxlylz_b=lxlylz_b, drv=d) for d in drv]
    lxa = ao_spec.get_lxlylz()
    lxb = numpy.array(lxa, copy=True) if lxlylz_b is None else numpy.array(lxlylz_b, dtype=numpy.intc)
    drv = validate_drv(drv)
    if drv > 3:
        raise ValueError("Only first derivatives are supported for analytical integrals.")
    S = aooverlap(coord_a, coord_b, lxa, lxb, ao_spec, drv)
    if "N" in ao_spec[0]:
        N = numpy.asarray(ao_spec[0]["N"], dtype=numpy.float64)
        for i in range(len(S)):
            S[i, :] *= N[i] * N[:, 0]
    if getattr(ao_spec, "spherical", False):
        S = cartesian2spherical_aoom(S, ao_spec)
    return S


def mo_overlap_matrix(mo_a, mo_b, aoom):
    """cy_overlap.mooverlapmatrix over all rows (orbkit/cy_overlap.pyx:184-205)."""
    A, B, S = _f(mo_a), _f(mo_b), _f(aoom)
    out = numpy.zeros((A.shape[0], B.shape[0]))
    lib().okref_mooverlapmatrix(_p(out), _p(A), _p(B), _p(S), A.shape[0], B.shape[0], S.shape[0], S.shape[1])
    return out


def ao_dipole_matrix(qc, component):
    """get_ao_dipole_matrix (orbkit/analytical_integrals.py:363-414): overlap with the
    ket exponent along `component` raised by one, plus the overlap with column i
    scaled by the coordinate of AO i's atom."""
    c = "xyz".find(component) if isinstance(component, str) else int(component)
    lxb = numpy.array(qc.ao_spec.get_lxlylz(), dtype=numpy.intc)
    lxb[:, c] += 1
    part1 = ao_overlap(qc.geo_spec, qc.geo_spec, qc.ao_spec, lxlylz_b=lxb)
    part2 = ao_overlap(qc.geo_spec, qc.geo_spec, qc.ao_spec)
    sph = getattr(qc.ao_spec, "spherical", False)
    per = (numpy.bincount(qc.ao_spec.get_assign_lm_to_cont(), minlength=len(qc.ao_spec)) if sph
           else qc.ao_spec.get_nlxlylz_per_cont())
    i = 0
    for s, n in zip(qc.ao_spec, per):
        for _ in range(n):
            part2[:, i] *= qc.geo_spec[s["atom"], c]
            i += 1
    return part1 + part2


def dipole_moment(qc, charges, component=("x", "y", "z")):
    """get_dipole_moment (orbkit/analytical_integrals.py:328-361) with the nuclear
    charges given explicitly (orbkit reads them from geo_info[:, 2])."""
    coeffs = qc.mo_spec.get_coeffs()
    occ = qc.mo_spec.get_occ()
    out = numpy.zeros(len(component))
    for k, c in enumerate(component):
        D = ao_dipole_matrix(qc, c)
        for i in range(len(coeffs)):
            out[k] -= occ[i] * mo_overlap_matrix(coeffs[i:i + 1], coeffs[i:i + 1], D)[0, 0]
        ci = "xyz".find(c)
        nuc = 0.0
        for a in range(len(qc.geo_spec)):
            nuc += float(charges[a]) * qc.geo_spec[a][ci]
        out[k] += nuc
    return out
