"""Drop-in replacement for the grid path of orbkit.core, running on the GPU.

Same names, arguments, return shapes and errors as orbkit/core.py:
  ao_creator            core.py:38-105
  mo_creator            core.py:107-132
  cartesian2spherical   core.py:135-176
  rho_compute           core.py:314-605
  rho_compute_no_slice  core.py:607-839
  calc_mo_matrix        core.py:841-941
Inputs are orbkit objects (QCinfo or dict with geo_spec / ao_spec / mo_spec) or
this package's equivalents; the grid comes from the module ``core.grid``
(orbkit_gb300.grid by default, orbkit.grid after ``orbkit_gb300.install(orbkit)``)
or from explicit x, y, z.  Results are float64 numpy arrays in orbkit's layouts.

Work runs on the current CUDA device through liborbkit_gb300.so; there is no
CPU path.  ``numproc`` and ``slice_length`` are accepted for compatibility: the
GPU evaluates the grid in device-sized slices of its own.  Mixed second
derivatives (drv 'xy', 'xz', 'yz') use orbkit's formula (orbkit/c_support.c:121-168)
unless ``exact_mixed=True`` is given.
"""
import numpy

from . import _lib
from . import grid as _default_grid
from .basis import get_basis
from .qcinfo import unpack
from .tools import require, validate_drv

grid = _default_grid

# points per device slice (bounded so that slice outputs stay a few GB)
MAX_SLICE_BYTES = 4 << 30

# orbkit's terminal output (orbkit/display.py: display); install() routes it to
# orbkit's own display, which honours orbkit.options.quiet and the .oklog file
quiet = False
# orbkit's options module once install(orbkit) routed display to orbkit's own
_orbkit_options = None


def display(msg):
    if not quiet:
        print(msg)


def _displaying():
    """Whether a message would be shown or logged (the norms and the electron count are
    only summed when it would)."""
    if _orbkit_options is not None:
        return not (getattr(_orbkit_options, "quiet", False) and getattr(_orbkit_options, "no_log", False))
    return not quiet


def _report(rho, mo_norm, mo_spec, d3r, was_vector, drv, calc_ao=False):
    """The MO norms (regular grid, no derivatives) and the electron count (regular
    grid) that orbkit's rho_compute prints (orbkit/core.py:572-592)."""
    if was_vector or not _displaying():
        return
    if drv is None and mo_norm is not None:
        display("\nNorm of the MOs:")
        labels = mo_spec.get_labels(format="print")
        for i in range(len(mo_norm)):
            display("\t%(m).6f\t%(t)s %(n)s" % {"m": mo_norm[i] * d3r, "n": labels[i], "t": "AO" if calc_ao else "MO"})
    display("We have " + str(numpy.sum(rho) * d3r) + " electrons.")


def _report_norms_no_slice(norms, mo_spec, d3r):
    """The MO norms rho_compute_no_slice prints (orbkit/core.py:797-802)."""
    display("\nNorm of the MOs:")
    for i in range(len(norms)):
        display("\t%(m).6f\tMO %(n)s" % {"m": norms[i] * d3r, "n": mo_spec[i].get("sym", "?")})


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise _lib.OkgError(-8, "no CUDA device visible")
    return torch


def _grid_arrays(x, y, z, is_vector, use_module=True):
    """Resolve the grid like orbkit: explicit arrays or the grid module."""
    if use_module and all(v is None for v in (x, y, z, is_vector)) and not grid.is_initialized:
        grid.grid_init(is_vector=True)
    if x is None:
        x = grid.x
    if y is None:
        y = grid.y
    if z is None:
        z = grid.z
    if is_vector is None:
        is_vector = grid.is_vector
    x, y, z = require(x, "f"), require(y, "f"), require(z, "f")
    if is_vector:
        if len(x) != len(y) or len(x) != len(z):
            raise ValueError("Dimensions of x-, y-, and z- coordinate differ!")
        return x, y, z, True, (len(x),)
    return x, y, z, False, (len(x), len(y), len(z))


class _DeviceGrid:
    """Coordinates on the device, sliced into okg_grid descriptors."""

    def __init__(self, x, y, z, is_vector, device):
        torch = _torch()
        self.regular = not is_vector
        self.npts = len(x) if is_vector else len(x) * len(y) * len(z)
        self.shape = (len(x), len(y), len(z))
        self.host = (x, y, z)
        self.dev = None
        if self.regular:
            self.dev = tuple(torch.from_numpy(numpy.ascontiguousarray(v)).to(device) for v in (x, y, z))
        self.device = device

    def slice(self, i, j):
        """okg_grid for points [i, j) and the device tensors that keep it alive."""
        torch = _torch()
        g = _lib.OkgGrid()
        if self.regular:
            xs = self.dev
            g.offset, g.npts = i, j - i
            g.nx, g.ny, g.nz = self.shape
            g.regular = 1
        else:
            xs = tuple(torch.from_numpy(numpy.ascontiguousarray(v[i:j])).to(self.device, non_blocking=False)
                       for v in self.host)
            g.offset, g.npts = 0, j - i
            g.nx = g.ny = g.nz = 0
            g.regular = 0
        g.d_x, g.d_y, g.d_z = xs[0].data_ptr(), xs[1].data_ptr(), xs[2].data_ptr()
        return g, xs


def _slices(npts, bytes_per_point):
    step = max(1, min(npts, MAX_SLICE_BYTES // max(1, bytes_per_point)))
    return [(i, min(i + step, npts)) for i in range(0, npts, step)] or [(0, 0)]


def _drv_list(drv):
    if drv is None:
        return None
    if isinstance(drv, str):
        try:
            validate_drv(drv)
            return [drv]
        except ValueError:
            return list(drv)
    try:
        return list(drv)
    except TypeError:
        return [drv]


def _eval(qc_geo, ao_spec, mo_spec, x, y, z, is_vector, what, drv_codes, exact_mixed=False, occ=None,
          mo_norm=False):
    """Evaluate on the GPU.  what: 'ao' -> (ndrv, nao, npts); 'mo' -> (ndrv, nmo, npts);
    'rho' -> (rho (npts,), drho (ndrv, npts)), plus the MO norms sum_i MO_m(i)^2
    (nmo,) when mo_norm is true."""
    torch = _torch()
    L = _lib.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    b = get_basis(qc_geo, ao_spec, dev)
    g = _DeviceGrid(x, y, z, is_vector, dev)
    npts = g.npts
    nd = len(drv_codes)
    codes = _lib.int_array(drv_codes)
    em = 1 if exact_mixed else 0
    st = _lib.stream_handle()
    if what == "ao":
        out = numpy.empty((nd, b.nao, npts))
        for (i, j) in _slices(npts, 8 * nd * b.nao):
            if j <= i:
                continue
            gd, keep = g.slice(i, j)
            o = torch.empty((nd, b.nao, j - i), dtype=torch.float64, device=dev)
            _lib.check(L.okg_eval_ao(b.handle, gd, nd, codes, em, _lib.ptr(o), j - i, st))
            out[:, :, i:j] = o.cpu().numpy()
        return out
    C = b.c_eff(mo_spec.get_coeffs())
    nmo = C.shape[0]
    if what == "mo":
        out = numpy.empty((nd, nmo, npts))
        for (i, j) in _slices(npts, 8 * nd * nmo):
            if j <= i:
                continue
            gd, keep = g.slice(i, j)
            o = torch.empty((nd, nmo, j - i), dtype=torch.float64, device=dev)
            _lib.check(L.okg_eval_mo(b.handle, gd, nmo, _lib.ptr(C), nd, codes, em, _lib.ptr(o), j - i, st))
            out[:, :, i:j] = o.cpu().numpy()
        return out
    if occ is None:
        occ = numpy.array([m["occ_num"] for m in mo_spec], dtype=numpy.float64)
    occ_d = torch.as_tensor(numpy.asarray(occ, dtype=numpy.float64), device=dev).contiguous()
    norm_d = torch.zeros(nmo, dtype=torch.float64, device=dev) if mo_norm else None
    rho = numpy.empty(npts)
    drho = numpy.empty((nd, npts))
    for (i, j) in _slices(npts, 8 * (1 + nd)):
        if j <= i:
            continue
        gd, keep = g.slice(i, j)
        r = torch.empty(j - i, dtype=torch.float64, device=dev)
        dr = torch.empty((max(nd, 1), j - i), dtype=torch.float64, device=dev)
        _lib.check(L.okg_rho(b.handle, gd, nmo, _lib.ptr(C), _lib.ptr(occ_d), nd, codes, em, _lib.ptr(r),
                             _lib.ptr(dr), j - i, _lib.ptr(norm_d), st))
        rho[i:j] = r.cpu().numpy()
        if nd:
            drho[:, i:j] = dr[:nd].cpu().numpy()
    if mo_norm:
        return rho, drho, norm_d.cpu().numpy()
    return rho, drho


def ao_creator(geo_spec, ao_spec, drv=None, x=None, y=None, z=None, is_vector=None, exact_mixed=False):
    """AOs or AO derivatives on the grid: (NAO,) + N float64 (orbkit/core.py:38-105)."""
    x, y, z, vec, N = _grid_arrays(x, y, z, is_vector)
    code = validate_drv(drv)
    out = _eval(geo_spec, ao_spec, None, x, y, z, vec, "ao", [code], exact_mixed)[0]
    return out.reshape((out.shape[0],) + N) if not vec else out


def _point_steps(npts, bytes_per_point):
    """Point ranges of at most MAX_SLICE_BYTES of device buffers each."""
    return [(i, j) for (i, j) in _slices(npts, bytes_per_point) if j > i]


def mo_creator(ao_list, mo_spec):
    """MOs from given AO values, MO = C . AO (orbkit/core.py:107-132; cy_core.pyx:82-101),
    as the hand-written FP64 contraction okg_mo_from_ao on the device (points sliced
    so that device buffers stay bounded).  The fused paths never materialise AOs."""
    torch = _torch()
    L = _lib.load()
    ao_list = require(ao_list, "f")
    shape = ao_list.shape
    coeffs = require(mo_spec.get_coeffs(), "f")
    if coeffs.ndim != 2 or coeffs.shape[1] != shape[0]:
        raise ValueError("MO coefficients of shape %s do not match %d AOs" % (coeffs.shape, shape[0]))
    A = ao_list.reshape(shape[0], -1)
    npts = A.shape[1]
    nmo, nao = coeffs.shape
    dev = torch.device("cuda", torch.cuda.current_device())
    C = torch.from_numpy(coeffs).to(dev)
    out = numpy.empty((nmo, npts))
    st = _lib.stream_handle()
    for (i, j) in _point_steps(npts, 8 * (nao + nmo)):
        a = torch.from_numpy(numpy.ascontiguousarray(A[:, i:j])).to(dev)
        o = torch.empty((nmo, j - i), dtype=torch.float64, device=dev)
        _lib.check(L.okg_mo_from_ao(nmo, nao, _lib.ptr(C), _lib.ptr(a), j - i, j - i, _lib.ptr(o), j - i, st))
        out[:, i:j] = o.cpu().numpy()
    return out.reshape((nmo,) + shape[1:])


def cartesian2spherical(ao_list, ao_spec):
    """Cartesian -> real spherical AOs (orbkit/core.py:135-176): the kernel okg_cart2sph
    applies orbkit's cart2sph combinations (Schlegel-Frisch table, last matching
    Cartesian row, coefficient x global factor) term by term in orbkit's order, so
    the result equals orbkit's bit for bit."""
    torch = _torch()
    L = _lib.load()
    from .basis import spherical_csr
    ptr, idx, coef = spherical_csr(ao_spec)
    ao_list = require(ao_list, "f")
    shape = ao_list.shape
    ncart = shape[0]
    if len(idx) and int(idx.max()) >= ncart:
        raise ValueError("ao_list has %d rows, the basis lists %d Cartesian AOs" % (ncart, int(idx.max()) + 1))
    nsph = len(ptr) - 1
    A = ao_list.reshape(ncart, -1)
    npts = A.shape[1]
    dev = torch.device("cuda", torch.cuda.current_device())
    d_ptr, d_idx, d_coef = (torch.from_numpy(numpy.ascontiguousarray(v)).to(dev) for v in (ptr, idx, coef))
    out = numpy.empty((nsph, npts))
    st = _lib.stream_handle()
    for (i, j) in _point_steps(npts, 8 * (ncart + nsph)):
        a = torch.from_numpy(numpy.ascontiguousarray(A[:, i:j])).to(dev)
        o = torch.empty((nsph, j - i), dtype=torch.float64, device=dev)
        _lib.check(L.okg_cart2sph(nsph, ncart, _lib.ptr(d_ptr), _lib.ptr(d_idx), _lib.ptr(d_coef), _lib.ptr(a), j - i,
                                  j - i, _lib.ptr(o), j - i, st))
        out[:, i:j] = o.cpu().numpy()
    return out.reshape((nsph,) + shape[1:])


class _MoGrids:
    """MO grids of one molecule on the device, one point range at a time (the
    fused okg_eval_mo; AO values stay on chip)."""

    def __init__(self, qc, x, y, z, vec, exact_mixed=False, mo_index=None):
        torch = _torch()
        self.L = _lib.load()
        self.dev = torch.device("cuda", torch.cuda.current_device())
        geo, ao_spec, mo_spec = unpack(qc)
        self.b = get_basis(geo, ao_spec, self.dev)
        coeffs = mo_spec.get_coeffs()
        if mo_index is not None:
            coeffs = coeffs[numpy.asarray(mo_index)]
        self.C = self.b.c_eff(coeffs)
        self.nmo = self.C.shape[0]
        self.g = _DeviceGrid(x, y, z, vec, self.dev)
        self.em = 1 if exact_mixed else 0

    def __call__(self, codes, i, j):
        """(len(codes), nmo, j - i) device tensor of the MOs' derivatives `codes`."""
        torch = _torch()
        gd, keep = self.g.slice(i, j)
        o = torch.empty((len(codes), self.nmo, j - i), dtype=torch.float64, device=self.dev)
        _lib.check(self.L.okg_eval_mo(self.b.handle, gd, self.nmo, _lib.ptr(self.C), len(codes),
                                      _lib.int_array(codes), self.em, _lib.ptr(o), j - i, _lib.stream_handle()))
        return o


def _mixed_rho(qc, x, y, z, vec, N, drv):
    """rho (and grad rho) through the tensor-core mixed path."""
    from .mixed import rho_grad
    rho, grad = rho_grad(qc, x, y, z, vec)
    rho = rho.reshape(N)
    if drv is None:
        return rho
    return rho, grad.reshape((3,) + N)


def _mixed_ok(calc_mo, drv, laplacian):
    if calc_mo or laplacian:
        return False
    return drv is None or [validate_drv(d) for d in drv] == [1, 2, 3]


def rho_compute(qc, calc_ao=False, calc_mo=False, drv=None, laplacian=False, numproc=1, slice_length=1e4,
                vector=None, save_hdf5=False, exact_mixed=False, precision="fp64", **kwargs):
    """Density, MOs, AOs or their derivatives on the grid module's grid (orbkit/core.py:314-605).

    precision="mixed" evaluates rho (drv=None) or rho and grad rho (drv=['x','y','z'])
    on the tensor cores (orbkit_gb300.mixed, max relative rho error <= 1e-6); other
    requests always run the FP64 path."""
    if calc_ao and calc_mo:
        raise ValueError("Choose either calc_ao=True or calc_mo=True")
    elif calc_ao:
        calc_mo = True
    if numproc <= 0:
        return rho_compute_no_slice(qc, calc_ao=calc_ao, calc_mo=calc_mo, drv=drv, laplacian=laplacian,
                                    exact_mixed=exact_mixed, **kwargs)
    if save_hdf5:
        raise NotImplementedError("save_hdf5 is not supported by the GPU path")
    if laplacian:
        drv = ["xx", "yy", "zz"]
    drv = _drv_list(drv)
    geo, ao_spec, mo_spec = unpack(qc)
    if not grid.is_initialized:
        grid.grid_init()
    vec = grid.is_vector
    x, y, z, vec, N = _grid_arrays(grid.x, grid.y, grid.z, vec, use_module=False)
    if precision == "mixed" and _mixed_ok(calc_mo, drv, laplacian):
        out = _mixed_rho(qc, x, y, z, vec, N, drv)
        # (the tensor-core kernel forms no MO norms: only the electron count is reported)
        _report(out if drv is None else out[0], None, mo_spec, grid.d3r, vec, drv)
        return out
    codes = [0] if drv is None else [validate_drv(d) for d in drv]
    if calc_mo:
        what = "ao" if calc_ao else "mo"
        out = _eval(geo, ao_spec, mo_spec, x, y, z, vec, what, codes, exact_mixed)
        if drv is None:
            out = out[0]
            return out.reshape((out.shape[0],) + N)
        return out.reshape(out.shape[:2] + N)
    rcodes = [] if drv is None else codes
    want_norm = drv is None and not vec
    res = _eval(geo, ao_spec, mo_spec, x, y, z, vec, "rho", rcodes, exact_mixed, mo_norm=want_norm)
    rho, drho = res[0], res[1]
    _report(rho, res[2] if want_norm else None, mo_spec, grid.d3r, vec, drv)
    rho = rho.reshape(N)
    if drv is None:
        return rho
    drho = drho.reshape((len(drv),) + N)
    if laplacian:
        return rho, drho, drho.sum(axis=0)
    return rho, drho


def rho_compute_no_slice(qc, calc_ao=False, calc_mo=False, drv=None, laplacian=False, return_components=False,
                         x=None, y=None, z=None, is_vector=None, exact_mixed=False, precision="fp64", **kwargs):
    """Unsliced variant with optional components (orbkit/core.py:607-839); precision as rho_compute."""
    if calc_ao and calc_mo:
        raise ValueError("calc_ao and calc_mo are mutually exclusive arguments."
                         "Use calc_mo and return_components instead!")
    x, y, z, vec, N = _grid_arrays(x, y, z, is_vector)
    geo, ao_spec, mo_spec = unpack(qc)
    if laplacian:
        drv = ["xx", "yy", "zz"]
    drv = _drv_list(drv)
    if precision == "mixed" and not return_components and not calc_ao and _mixed_ok(calc_mo, drv, laplacian):
        return _mixed_rho(qc, x, y, z, vec, N, drv)
    conv = lambda a: a if vec else a.reshape(a.shape[:-1] + N)
    if drv is not None:
        codes = [validate_drv(d) for d in drv]
        dao = conv(_eval(geo, ao_spec, mo_spec, x, y, z, vec, "ao", codes, exact_mixed))
        if calc_ao:
            return dao
        dmo = conv(_eval(geo, ao_spec, mo_spec, x, y, z, vec, "mo", codes, exact_mixed))
        if calc_mo:
            return (dao, dmo) if return_components else dmo
    ao_list = conv(_eval(geo, ao_spec, mo_spec, x, y, z, vec, "ao", [0])[0]) if (calc_ao or return_components) else None
    if calc_ao:
        return ao_list
    mo_list = conv(_eval(geo, ao_spec, mo_spec, x, y, z, vec, "mo", [0])[0]) if (calc_mo or return_components) else None
    d3r = 1.0
    for v in (x, y, z):
        if len(v) > 1:
            d3r *= v[1] - v[0]
    if mo_list is not None and not vec and _displaying():
        _report_norms_no_slice(numpy.array([numpy.sum(m ** 2) for m in mo_list]), mo_spec, d3r)
    if calc_mo:
        return (ao_list, mo_list) if return_components else mo_list
    rcodes = [] if drv is None else codes
    res = _eval(geo, ao_spec, mo_spec, x, y, z, vec, "rho", rcodes, exact_mixed, mo_norm=mo_list is None and not vec)
    rho, drho = res[0], res[1]
    if not vec and _displaying():
        if mo_list is None:
            _report_norms_no_slice(res[2], mo_spec, d3r)
        display("We have " + str(numpy.sum(rho) * d3r) + " electrons.")
    rho = conv(rho)
    if drv is None:
        return (ao_list, mo_list, rho) if return_components else rho
    drho = conv(drho)
    delta = (drho, drho.sum(axis=0)) if laplacian else (drho,)
    return ((ao_list, mo_list, rho, dao, dmo) + delta) if return_components else (rho,) + delta


def calc_mo_matrix(qc_a, qc_b=None, drv=None, numproc=1, slice_length=1e4, save_hdf5=False, exact_mixed=False,
                   **kwargs):
    """Products MO_a(r) * dMO_b(r) on the grid module's grid (orbkit/core.py:841-941):
    shape (NDRV, NMO_a, NMO_b) + grid shape.  The MO grids are evaluated and
    multiplied on the device (okg_eval_mo, okg_mo_products); only the products come
    back to the host."""
    if save_hdf5:
        raise NotImplementedError("save_hdf5 is not supported by the GPU path")
    ibra = [0]
    if drv is None:
        drv = [None]
        iket = [0]
    elif not isinstance(drv, list):
        drv = [None, drv]
        iket = [1]
    else:
        drv = [None] + drv
        iket = list(range(1, len(drv)))
    codes = [validate_drv(d) for d in drv]
    if not grid.is_initialized:
        grid.grid_init()
    x, y, z, vec, N = _grid_arrays(grid.x, grid.y, grid.z, grid.is_vector, use_module=False)
    same = qc_b is None or qc_a is qc_b
    mo_a = _MoGrids(qc_a, x, y, z, vec, exact_mixed)
    mo_b = mo_a if same else _MoGrids(qc_b, x, y, z, vec, exact_mixed)
    na, nb, nk = mo_a.nmo, mo_b.nmo, len(iket)
    npts = mo_a.g.npts
    out = numpy.empty((nk, na, nb, npts))
    L = _lib.load()
    torch = _torch()
    for (i, j) in _point_steps(npts, 8 * (nk * na * nb + (len(drv) + 1) * max(na, nb))):
        if same:
            m = mo_a(codes, i, j)
            bra, ket = m[ibra[0]], m[iket].contiguous()
        else:
            bra = mo_a([codes[k] for k in ibra], i, j)[0]
            ket = mo_b([codes[k] for k in iket], i, j)
        o = torch.empty((nk, na, nb, j - i), dtype=torch.float64, device=mo_a.dev)
        _lib.check(L.okg_mo_products(nk, na, nb, _lib.ptr(bra), j - i, _lib.ptr(ket), j - i, j - i, _lib.ptr(o),
                                     j - i, _lib.stream_handle()))
        out[..., i:j] = o.cpu().numpy()
    return out.reshape((nk, na, nb) + N)
