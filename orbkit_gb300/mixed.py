"""Mixed-precision rho and grad rho on the tensor cores.

The C.AO contraction runs in BF16 on tcgen05 tensor cores with every operand
split into three BF16 parts (six MMAs per product, FP32 accumulation); the
exponent arguments and the final density accumulation stay FP64.  Points
within ``cusp_radius`` bohr of a nucleus are recomputed with the FP64 path
(the cusp region stays FP64).

Error bar (measured by tests/test_gpu_mixed.py against the FP64 path, which itself
matches the oracle to 1e-12): max relative rho error <= MIXED_RHO_RTOL over
points with rho > MIXED_RHO_FLOOR.
"""
import ctypes

import numpy

from . import _lib
from .basis import get_basis
from .qcinfo import unpack

MIXED_RHO_RTOL = 1e-6
MIXED_RHO_FLOOR = 1e-10
CUSP_RADIUS = 0.3


def cusp_alpha(radius):
    """Default exponent threshold of the in-kernel FP64 cusp treatment: primitives with
    alpha > 24 ln 2 / r_c^2 fall below 2^-24 of their peak within the cusp radius r_c,
    i.e. they vary on a scale finer than the cusp region."""
    return 24.0 * numpy.log(2.0) / (radius * radius)


def near_atoms(geo, pts, radius, device):
    """int16 tensor (npts,) on the device: the atom within `radius` of each point
    (3, npts) -- atoms are further apart than 2 radius -- or -1."""
    import torch
    if isinstance(pts, torch.Tensor):
        P = pts.to(device=device, dtype=torch.float64)
    else:
        P = torch.as_tensor(numpy.asarray(pts, dtype=numpy.float64), device=device)
    G = torch.as_tensor(numpy.asarray(geo, dtype=numpy.float64).reshape(-1, 3), device=device)
    near = torch.full((P.shape[1],), -1, dtype=torch.int16, device=device)
    for a in range(G.shape[0]):
        near[((P - G[a][:, None]) ** 2).sum(0) <= radius * radius] = a
    return near

_SIGS = {
    "okg_mixed_plan_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "okg_mixed_plan_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "okg_mixed_set_coeffs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "okg_rho_mixed": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(_lib.OkgGrid), ctypes.c_int, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]),
    "okg_mixed_status": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "okg_mixed_plan_set_threads": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "okg_mixed_plan_set_generation": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "okg_mixed_plan_set_wait_limit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_longlong]),
    "okg_mixed_plan_set_cusp": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double]),
}


def _L():
    L = _lib.load()
    for n, (r, a) in _SIGS.items():
        f = getattr(L, n)
        f.restype = r
        f.argtypes = a
    return L


class MixedPlan:
    """Tensor-core operand form of a set of MO coefficients for one DeviceBasis."""

    def __init__(self, basis, coeffs, occ, stream=None, threads=None):
        import torch
        self.basis = basis
        self._L = _L()
        C = basis.c_eff(coeffs)
        self.nmo = C.shape[0]
        self.occ = torch.as_tensor(numpy.asarray(occ, dtype=numpy.float64), device=basis.device).contiguous()
        h = ctypes.c_void_p()
        _lib.check(self._L.okg_mixed_plan_create(basis.handle, self.nmo, ctypes.byref(h)))
        self._h = h
        self.C = C
        _lib.check(self._L.okg_mixed_set_coeffs(h, _lib.ptr(C), _lib.ptr(self.occ), _lib.stream_handle(stream)))
        if threads is None:
            import os
            threads = int(os.environ.get("ORBKIT_GB300_MIXED_THREADS", "0")) or None
        if threads:
            self.set_threads(threads)

    def set_threads(self, threads):
        """AO-generation threads per CTA of the mixed kernel: 256, 384 or 512 (one point each)."""
        _lib.check(self._L.okg_mixed_plan_set_threads(self._h, int(threads)))

    def set_generation(self, threads, points_per_thread):
        """Generation threads per CTA and grid points per generation thread:
        (256|384|512, 1) or (256|384, 2)."""
        _lib.check(self._L.okg_mixed_plan_set_generation(self._h, int(threads), int(points_per_thread)))

    def set_cusp(self, near, alpha_c):
        """FP64 cusp points inside the tensor-core kernel: near (int16 device tensor, one
        entry per point of the grids this plan evaluates, -1 = none) names each point's
        cusp atom; that atom's primitives with alpha > alpha_c are evaluated in FP64 in
        the epilogue.  near=None switches it off."""
        self._near = near
        _lib.check(self._L.okg_mixed_plan_set_cusp(self._h, _lib.ptr(near), float(alpha_c)))

    def set_wait_limit(self, polls):
        """Polls per bounded device wait (default 2^24); an expired wait makes check() raise."""
        _lib.check(self._L.okg_mixed_plan_set_wait_limit(self._h, int(polls)))

    @property
    def handle(self):
        return self._h

    def rho(self, grid_desc, rho, grad, ld, stream=None):
        """Launch on an okg_grid; rho (npts) and grad (3, ld) are device tensors."""
        _lib.check(self._L.okg_rho_mixed(self._h, grid_desc, 1 if grad is not None else 0, _lib.ptr(rho),
                                         _lib.ptr(grad), ld, _lib.stream_handle(stream)))

    def check(self):
        st = ctypes.c_int(0)
        _lib.check(self._L.okg_mixed_status(self._h, ctypes.byref(st)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self._L.okg_mixed_plan_destroy(h)
            except Exception:
                pass
            self._h = None


def cusp_points_regular(geo, x, y, z, radius):
    """Flattened indices of regular-grid points within `radius` of any nucleus."""
    out = []
    nyz = len(y) * len(z)
    for A in numpy.asarray(geo, dtype=numpy.float64).reshape(-1, 3):
        ix = numpy.nonzero(numpy.abs(x - A[0]) <= radius)[0]
        iy = numpy.nonzero(numpy.abs(y - A[1]) <= radius)[0]
        iz = numpy.nonzero(numpy.abs(z - A[2]) <= radius)[0]
        if not (len(ix) and len(iy) and len(iz)):
            continue
        I, J, K = numpy.meshgrid(ix, iy, iz, indexing="ij")
        d2 = (x[I] - A[0]) ** 2 + (y[J] - A[1]) ** 2 + (z[K] - A[2]) ** 2
        m = d2 <= radius * radius
        out.append((I[m] * nyz + J[m] * len(z) + K[m]).astype(numpy.int64))
    if not out:
        return numpy.zeros(0, dtype=numpy.int64)
    return numpy.unique(numpy.concatenate(out))


class _Slab:
    """x slab [a, b) of a regular grid already on the device: a regular grid of its own
    whose x axis starts at element a of the device x axis (no upload)."""

    def __init__(self, full, x, y, z, a, b):
        self.full = full
        self.regular = True
        self.host = (x[a:b], y, z)
        self.shape = (b - a, len(y), len(z))
        self.npts = (b - a) * len(y) * len(z)
        self.a = a

    def grid(self):
        xd, yd, zd = self.full.dev
        g = _lib.OkgGrid()
        g.d_x, g.d_y, g.d_z = xd.data_ptr() + 8 * self.a, yd.data_ptr(), zd.data_ptr()
        g.npts, g.offset = self.npts, 0
        g.nx, g.ny, g.nz = self.shape
        g.regular = 1
        return g


class MixedEvaluator:
    """Device resources for repeated mixed-precision rho / grad rho evaluation of
    one molecule: the packed basis, the tensor-core coefficient plan and output
    buffers.  ``update`` uploads new parameters from host arrays; ``evaluate``
    takes a host grid and writes host outputs."""

    def __init__(self, qc, cusp_radius=CUSP_RADIUS, device=None, cusp_mode="recompute", cusp_alpha_c=None):
        """cusp_mode 'recompute' (default): the points within cusp_radius of a nucleus are
        recomputed whole by the FP64 path after the tensor-core launch (exact FP64);
        'kernel': the tensor-core kernel evaluates those points' steep primitives (alpha >
        cusp_alpha_c, default cusp_alpha(cusp_radius)) in FP64 itself."""
        import torch
        geo, ao_spec, mo_spec = unpack(qc)
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        self.basis = get_basis(geo, ao_spec, self.device)
        occ = numpy.array([m["occ_num"] for m in mo_spec], dtype=numpy.float64)
        self.plan = MixedPlan(self.basis, mo_spec.get_coeffs(), occ)
        self.geo = numpy.asarray(geo, dtype=numpy.float64)
        self.cusp_radius = cusp_radius
        if cusp_mode not in ("kernel", "recompute"):
            raise ValueError("cusp_mode must be 'kernel' or 'recompute'")
        self.cusp_mode = cusp_mode
        self.cusp_alpha_c = cusp_alpha(cusp_radius) if (cusp_alpha_c is None and cusp_radius) else (cusp_alpha_c or 0.0)
        self._near_key = None
        self._bufs = None

    def update(self, geo=None, prim=None, coeffs=None, occ=None, stream=None):
        """New nuclear positions / primitives / MO coefficients / occupations (host or device)."""
        import torch
        if geo is not None or prim is not None:
            self.basis.set_params(geo=geo, prim=prim, stream=stream)
            if geo is not None:
                self.geo = (geo.cpu().numpy() if hasattr(geo, "cpu") else numpy.asarray(geo)).reshape(-1, 3)
        if coeffs is not None or occ is not None:
            p = self.plan
            if coeffs is not None:
                p.C = self.basis.c_eff(torch.as_tensor(coeffs, dtype=torch.float64).to(self.device, non_blocking=True))
            if occ is not None:
                p.occ = torch.as_tensor(occ, dtype=torch.float64).to(self.device, non_blocking=True).contiguous()
            _lib.check(p._L.okg_mixed_set_coeffs(p.handle, _lib.ptr(p.C), _lib.ptr(p.occ), _lib.stream_handle(stream)))

    def evaluate_device(self, g, rho=None, grad=None):
        """Run on a _DeviceGrid; returns device tensors (rho, grad).  The points
        within the cusp radius of a nucleus are then recomputed by the FP64 path
        (its small-point CTA shape) and scattered into the outputs, on the same
        stream."""
        import torch
        n = g.npts
        if rho is None:
            rho = torch.empty(n, dtype=torch.float64, device=self.device)
            grad = torch.empty((3, n), dtype=torch.float64, device=self.device)
        gd, keep = g.slice(0, n)
        kernel_cusp = self.cusp_mode == "kernel" and self.cusp_radius and self.cusp_radius > 0
        if kernel_cusp:
            self._set_near(g)
        self.plan.rho(gd, rho, grad, n)
        if self.cusp_radius and self.cusp_radius > 0 and not kernel_cusp:
            self._cusp_fix(g, rho, grad)
        return rho, grad

    def _set_near(self, g):
        """Cusp atom of every point of g for the in-kernel FP64 cusp treatment (cached per grid)."""
        import torch
        key = (self.cusp_radius, self.geo.tobytes(),
               tuple(numpy.ascontiguousarray(v).tobytes() for v in g.host) if g.regular else id(g))
        if self._near_key != key:
            self._near_grid = g
            self._near_key = key
            if g.regular:
                near = torch.full((g.npts,), -1, dtype=torch.int16, device=self.device)
                gx, gy, gz = g.host
                nyz = len(gy) * len(gz)
                for a, A in enumerate(self.geo):
                    idx = cusp_points_regular(A[None, :], gx, gy, gz, self.cusp_radius)
                    if len(idx):
                        near[torch.from_numpy(idx).to(self.device)] = a
            else:
                near = near_atoms(self.geo, numpy.stack(g.host), self.cusp_radius, self.device)
            self.plan.set_cusp(near, self.cusp_alpha_c)

    def _cusp_fix(self, g, rho, grad):
        import torch
        # cached per regular grid (its axes) or per vector-grid object (held here, so
        # its identity is not reused), and per geometry and radius; a few grids are
        # kept (the x slabs of a pipelined evaluation are grids of their own)
        key = (self.cusp_radius, self.geo.tobytes(),
               tuple(numpy.ascontiguousarray(v).tobytes() for v in g.host) if g.regular else id(g))
        cache = self.__dict__.setdefault("_cusp_cache", {})
        if key not in cache:
            if len(cache) >= 16:
                cache.pop(next(iter(cache)))
            idx, pts = cusp_points(self.geo, g, self.cusp_radius, self.device)
            m = len(idx)
            r = torch.empty(m, dtype=torch.float64, device=self.device)
            dr = torch.empty((3, m), dtype=torch.float64, device=self.device)
            gd = _lib.OkgGrid(pts[0].data_ptr(), pts[1].data_ptr(), pts[2].data_ptr(), m, 0, 0, 0, 0, 0)
            cache[key] = (idx, pts, r, dr, gd, _lib.int_array([1, 2, 3]), None if g.regular else g)
        idx, pts, r, dr, gd, codes, _ = cache[key]
        self._cusp = cache[key]
        m = len(idx)
        if m == 0:
            return
        p = self.plan
        _lib.check(_lib.load().okg_rho(p.basis.handle, gd, p.nmo, _lib.ptr(p.C), _lib.ptr(p.occ), 3, codes, 1,
                                       _lib.ptr(r), _lib.ptr(dr), m, None, _lib.stream_handle()))
        rho.index_copy_(0, idx, r)
        grad.index_copy_(1, idx, dr)

    SLABS = 2  # x slabs of a pipelined regular-grid evaluation

    def _evaluate_slabs(self, x, y, z, out):
        """Regular grid in x slabs (each a regular grid of its own, brick-tiled), the
        read-back of one slab on a second stream while the next slab's kernel runs."""
        import torch
        from .core import _DeviceGrid
        nx, nyz = len(x), len(y) * len(z)
        n = nx * nyz
        cuts = sorted({min(nx, 4 * round(nx * i / (4 * self.SLABS))) for i in range(self.SLABS + 1)} | {0, nx})
        bufs = getattr(self, "_slab_bufs", None)
        if bufs is None or bufs[0].numel() != n:
            bufs = (torch.empty(n, dtype=torch.float64, device=self.device),
                    torch.empty((3, n), dtype=torch.float64, device=self.device))
            self._slab_bufs = bufs
        rho, grad = bufs
        if getattr(self, "_copy_stream", None) is None:
            self._copy_stream = torch.cuda.Stream(device=self.device)
        comp, copy = torch.cuda.current_stream(), self._copy_stream
        full = _DeviceGrid(x, y, z, False, self.device)  # the three axes, uploaded once
        for a, b in zip(cuts[:-1], cuts[1:]):
            if b <= a:
                continue
            g = _Slab(full, x, y, z, a, b)
            s0, s1 = a * nyz, b * nyz
            gd = g.grid()
            rv, gv = rho[s0:s1], grad[:, s0:s1]
            self.plan.rho(gd, rv, gv, n)
            if self.cusp_radius and self.cusp_radius > 0:
                self._cusp_fix(g, rv, gv)
            done = torch.cuda.Event()
            done.record(comp)
            copy.wait_event(done)
            with torch.cuda.stream(copy):
                out[0][s0:s1].copy_(rv, non_blocking=True)
                for c in range(3):
                    out[1][c, s0:s1].copy_(grad[c, s0:s1], non_blocking=True)
        copy.synchronize()
        # the next call's kernels must not overwrite the buffers before these copies end
        comp.wait_stream(copy)
        return out

    def evaluate(self, x, y, z, is_vector, out=None):
        """Host grid in, host (rho, grad) out.  `out` may hold preallocated (pinned)
        host tensors (rho (npts,), grad (3, npts)) that receive the results.  A regular
        grid with the FP64 recomputation of its cusp points is evaluated in x slabs whose
        read-backs overlap the following slabs' kernels."""
        import torch
        from .core import _DeviceGrid
        x = numpy.asarray(x, dtype=numpy.float64)
        y = numpy.asarray(y, dtype=numpy.float64)
        z = numpy.asarray(z, dtype=numpy.float64)
        if not is_vector and self.cusp_mode == "recompute" and len(x) >= 8 * self.SLABS:
            npts = len(x) * len(y) * len(z)
            if out is None:
                out = (torch.empty(npts, dtype=torch.float64, pin_memory=True),
                       torch.empty((3, npts), dtype=torch.float64, pin_memory=True))
                self._evaluate_slabs(x, y, z, out)
                return out[0].numpy(), out[1].numpy()
            return self._evaluate_slabs(x, y, z, out)
        g = _DeviceGrid(x, y, z, is_vector, self.device)
        rho, grad = self.evaluate_device(g)
        if out is None:
            # page-locked host arrays from torch's caching host allocator (reused
            # after the first call): the read-back runs at pinned-copy bandwidth; the
            # numpy arrays keep their tensors, and so the memory, alive
            out = (torch.empty(rho.shape, dtype=torch.float64, pin_memory=True),
                   torch.empty(grad.shape, dtype=torch.float64, pin_memory=True))
            out[0].copy_(rho, non_blocking=True)
            out[1].copy_(grad, non_blocking=True)
            torch.cuda.current_stream().synchronize()
            return out[0].numpy(), out[1].numpy()
        out[0].copy_(rho, non_blocking=True)
        out[1].copy_(grad, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        return out

    def check(self):
        self.plan.check()


_evaluators = {}


def evaluator_for(qc, cusp_radius=CUSP_RADIUS, device=None):
    """A MixedEvaluator for this molecule, reused across calls: keyed by the basis and
    geometry (the DeviceBasis fingerprint), the MO coefficients and occupations, the
    cusp radius and the device, so that repeated drop-in calls (core.rho_compute with
    precision='mixed') skip the plan set-up and the cusp-point search of a grid they
    have seen (a few evaluators are kept)."""
    import hashlib
    import torch
    from .basis import fingerprint, flatten
    geo, ao_spec, mo_spec = unpack(qc)
    dev = device or torch.device("cuda", torch.cuda.current_device())
    h = hashlib.sha1(numpy.ascontiguousarray(mo_spec.get_coeffs(), dtype=numpy.float64).tobytes())
    h.update(numpy.array([m["occ_num"] for m in mo_spec], dtype=numpy.float64).tobytes())
    key = (fingerprint(geo, flatten(ao_spec)), h.hexdigest(), float(cusp_radius), str(dev))
    ev = _evaluators.get(key)
    if ev is None:
        if len(_evaluators) >= 4:
            _evaluators.pop(next(iter(_evaluators)))
        ev = MixedEvaluator(qc, cusp_radius, dev)
        _evaluators[key] = ev
    return ev


def rho_grad(qc, x, y, z, is_vector, cusp_radius=CUSP_RADIUS, return_device=False):
    """rho and grad rho (3, npts) on the GPU mixed path, with the cusp region in FP64
    (evaluator and cusp points reused across calls on the same molecule and grid)."""
    from .core import _DeviceGrid
    ev = evaluator_for(qc, cusp_radius)
    if return_device:
        g = _DeviceGrid(numpy.asarray(x, dtype=numpy.float64), numpy.asarray(y, dtype=numpy.float64),
                        numpy.asarray(z, dtype=numpy.float64), is_vector, ev.device)
        out = ev.evaluate_device(g)
        ev.check()
        return out
    out = ev.evaluate(x, y, z, is_vector)
    ev.check()
    return out


def cusp_points(geo, g, radius, device):
    """(flattened indices, (3, m) coordinates) of the grid points within `radius` of a nucleus."""
    import torch
    if g.regular:
        idx = cusp_points_regular(geo, *g.host, radius)
        gx, gy, gz = g.host
        nyz = len(gy) * len(gz)
        pts = numpy.stack([gx[idx // nyz], gy[(idx // len(gz)) % len(gy)], gz[idx % len(gz)]])
        return torch.from_numpy(idx).to(device), torch.from_numpy(pts).to(device)
    pts_all = torch.stack([torch.from_numpy(numpy.ascontiguousarray(v)).to(device) for v in g.host])
    G = torch.as_tensor(numpy.asarray(geo, dtype=numpy.float64), device=device)
    near = torch.zeros(pts_all.shape[1], dtype=torch.bool, device=device)
    for a in range(G.shape[0]):
        near |= ((pts_all - G[a][:, None]) ** 2).sum(0) <= radius * radius
    it = torch.nonzero(near).flatten()
    return it, pts_all[:, it].contiguous()


def fix_cusp(plan, geo, g, rho, grad, radius):
    """Recompute the points within `radius` of a nucleus with the FP64 kernel."""
    import torch
    L = _lib.load()
    dev = rho.device
    if g.regular:
        idx = cusp_points_regular(geo, *g.host, radius)
        if len(idx) == 0:
            return
        gx, gy, gz = g.host
        nyz = len(gy) * len(gz)
        px = gx[idx // nyz]
        py = gy[(idx // len(gz)) % len(gy)]
        pz = gz[idx % len(gz)]
        pts = torch.from_numpy(numpy.stack([px, py, pz])).to(dev)
        it = torch.from_numpy(idx).to(dev)
    else:
        pts_all = torch.stack([torch.from_numpy(numpy.ascontiguousarray(v)).to(dev) for v in g.host])
        G = torch.as_tensor(numpy.asarray(geo, dtype=numpy.float64), device=dev)
        near = torch.zeros(pts_all.shape[1], dtype=torch.bool, device=dev)
        for a in range(G.shape[0]):
            near |= ((pts_all - G[a][:, None]) ** 2).sum(0) <= radius * radius
        it = torch.nonzero(near).flatten()
        if it.numel() == 0:
            return
        pts = pts_all[:, it].contiguous()
    m = pts.shape[1]
    gd = _lib.OkgGrid(pts[0].data_ptr(), pts[1].data_ptr(), pts[2].data_ptr(), m, 0, 0, 0, 0, 0)
    r = torch.empty(m, dtype=torch.float64, device=dev)
    dr = torch.empty((3, m), dtype=torch.float64, device=dev)
    b = plan.basis
    _lib.check(L.okg_rho(b.handle, gd, plan.nmo, _lib.ptr(plan.C), _lib.ptr(plan.occ), 3, _lib.int_array([1, 2, 3]),
                         1, _lib.ptr(r), _lib.ptr(dr), m, None, _lib.stream_handle()))
    rho.index_copy_(0, it, r)
    grad.index_copy_(1, it, dr)


def error_report(rho, grad, rho_ref, grad_ref, floor=MIXED_RHO_FLOOR):
    """Max relative rho error over rho_ref > floor, max abs rho error, and the grad error
    normalised by |grad_ref| + floor."""
    rho = numpy.asarray(rho).reshape(-1)
    rho_ref = numpy.asarray(rho_ref).reshape(-1)
    m = rho_ref > floor
    rel = numpy.abs(rho - rho_ref)[m] / rho_ref[m]
    gr = numpy.asarray(grad).reshape(3, -1)
    gref = numpy.asarray(grad_ref).reshape(3, -1)
    gn = numpy.linalg.norm(gref, axis=0)
    gerr = numpy.linalg.norm(gr - gref, axis=0) / (gn + floor)
    return {
        "rho_max_rel": float(rel.max()) if rel.size else 0.0,
        "rho_p999_rel": float(numpy.percentile(rel, 99.9)) if rel.size else 0.0,
        "rho_max_abs": float(numpy.abs(rho - rho_ref).max()),
        "grad_max_rel": float(gerr.max()),
        "floor": floor,
        "points_above_floor": int(m.sum()),
    }


def smoke_check(qc, x, y, z, rho_ref, grad_ref):
    r, g = rho_grad(qc, x, y, z, False)
    rep = error_report(r, g, rho_ref, grad_ref)
    assert rep["rho_max_rel"] <= MIXED_RHO_RTOL, rep
    print("smoke mixed: rho max rel err %.2e (rho > %g), grad max rel err %.2e" % (
        rep["rho_max_rel"], rep["floor"], rep["grad_max_rel"]))
