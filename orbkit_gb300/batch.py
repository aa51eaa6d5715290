"""Batched evaluation: many molecules with uneven point sets in one persistent launch.

``BatchEvaluator(molecules)`` packs every molecule's basis and MO coefficients
(tensor-core operand form), uploads its point set (3, n) and output buffers,
and builds one okg_batch: all 128-point tiles of all molecules, handed out by a
device counter to one persistent CTA per SM.  ``run()`` is a counter reset plus
one kernel launch; ``capture()`` records it in a CUDA graph; the schedule
(MMA N tile per MO pass, tiles per counter grab, molecule order, generation
threads and points per thread) comes from the autotuner (orbkit_gb300.autotune),
measured once per size bucket.

The cusp region near nuclei stays FP64: by default (``cusp_mode='kernel'``) every
point within ``cusp_radius`` of a nucleus has that atom's steep primitives (alpha >
``cusp_alpha``, default mixed.cusp_alpha(cusp_radius)) evaluated, contracted with the
MO coefficients and squared in FP64 inside the same persistent launch;
``cusp_mode='recompute'`` instead recomputes those points whole with the FP64 path
(exact FP64, but a third of an atom-centred grid lies in the cusp region);
``cusp_radius=0`` evaluates every point on the tensor cores alone.
"""
import ctypes

import numpy

from . import _lib, autotune
from .basis import DeviceBasis
from .qcinfo import unpack

_SIGS = {
    "okg_mixed_plan_create_tiled": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                                   ctypes.POINTER(ctypes.c_void_p)]),
    "okg_mixed_plan_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "okg_mixed_set_coeffs": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "okg_batch_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(_lib.OkgGrid),
                                        ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                                        ctypes.POINTER(ctypes.c_int64), ctypes.c_int,
                                        ctypes.POINTER(ctypes.c_void_p)]),
    "okg_batch_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "okg_batch_set_schedule": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "okg_batch_set_generation": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "okg_batch_tiles": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_longlong)]),
    "okg_batch_run": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "okg_batch_status": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "okg_mixed_plan_set_cusp": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double]),
}

N_TILES = (32, 64)
GRABS = (1, 4)
ORDERS = ("given", "largest_first")
# (generation threads per CTA, grid points per generation thread)
LAYOUTS = ((256, 1), (384, 1), (512, 1), (256, 2))


def _L():
    L = _lib.load()
    for n, (r, a) in _SIGS.items():
        f = getattr(L, n)
        f.restype = r
        f.argtypes = a
    return L


class _Plan:
    def __init__(self, L, basis, C, occ, n_max):
        self._L = L
        h = ctypes.c_void_p()
        _lib.check(L.okg_mixed_plan_create_tiled(basis.handle, C.shape[0], n_max, ctypes.byref(h)))
        self.h = h
        _lib.check(L.okg_mixed_set_coeffs(h, _lib.ptr(C), _lib.ptr(occ), _lib.stream_handle()))

    def __del__(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self._L.okg_mixed_plan_destroy(self.h)
            self.h = None


class BatchEvaluator:
    """molecules: sequence of (qc, points) with points a (3, n) float64 array."""

    def __init__(self, molecules, want_grad=True, cusp_radius=None, tune=True, schedule=None, device=None,
                 cusp_mode="kernel", cusp_alpha=None):
        import torch
        from . import mixed
        self._L = _L()
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        self.want_grad = want_grad
        self.cusp_radius = mixed.CUSP_RADIUS if cusp_radius is None else cusp_radius
        if cusp_mode not in ("kernel", "recompute"):
            raise ValueError("cusp_mode must be 'kernel' or 'recompute'")
        self.cusp_mode = cusp_mode
        self.cusp_alpha = (mixed.cusp_alpha(self.cusp_radius) if self.cusp_radius > 0 else 0.0) \
            if cusp_alpha is None else cusp_alpha
        self.mols = []
        for qc, pts in molecules:
            geo, ao_spec, mo_spec = unpack(qc)
            b = DeviceBasis(geo, ao_spec, self.device)
            C = b.c_eff(mo_spec.get_coeffs())
            occ = torch.as_tensor(numpy.array([m["occ_num"] for m in mo_spec], dtype=numpy.float64),
                                  device=self.device)
            P = torch.as_tensor(numpy.ascontiguousarray(pts, dtype=numpy.float64), device=self.device)
            n = P.shape[1]
            m = {"basis": b, "C": C, "occ": occ, "pts": P, "n": n, "geo": numpy.asarray(geo, dtype=numpy.float64),
                 "rho": torch.empty(n, dtype=torch.float64, device=self.device),
                 "grad": torch.empty((3, n), dtype=torch.float64, device=self.device), "plans": {}}
            m["near"] = mixed.near_atoms(m["geo"], P, self.cusp_radius, self.device) \
                if self.kernel_cusp else None
            self.mols.append(m)
        self.npts = sum(m["n"] for m in self.mols)
        self._batch = None
        self._cusp = None
        if schedule is None:
            schedule = self.autotune() if tune else {"n_max": 64, "grab": 1, "order": "given", "layout": (384, 1)}
        self.set_schedule(schedule)

    @property
    def kernel_cusp(self):
        return self.cusp_mode == "kernel" and self.cusp_radius > 0

    # ------------------------------------------------------------- schedule
    def _plan(self, m, n_max):
        if n_max not in m["plans"]:
            p = _Plan(self._L, m["basis"], m["C"], m["occ"], n_max)
            if m["near"] is not None:
                _lib.check(self._L.okg_mixed_plan_set_cusp(p.h, _lib.ptr(m["near"]), float(self.cusp_alpha)))
            m["plans"][n_max] = p
        return m["plans"][n_max]

    def _order(self, order):
        idx = list(range(len(self.mols)))
        if order == "largest_first":
            idx.sort(key=lambda i: -(self.mols[i]["n"] * self.mols[i]["basis"].ncart * max(1, len(self.mols[i]["occ"]))))
        return idx

    def set_schedule(self, sch):
        if self._batch is not None:
            self._L.okg_batch_destroy(self._batch)
            self._batch = None
        order = self._order(sch["order"])
        nm = len(order)
        plans = (ctypes.c_void_p * nm)()
        grids = (_lib.OkgGrid * nm)()
        rhos = (ctypes.c_void_p * nm)()
        grads = (ctypes.c_void_p * nm)()
        lds = (ctypes.c_int64 * nm)()
        for j, i in enumerate(order):
            m = self.mols[i]
            plans[j] = self._plan(m, sch["n_max"]).h.value
            P = m["pts"]
            grids[j] = _lib.OkgGrid(P[0].data_ptr(), P[1].data_ptr(), P[2].data_ptr(), m["n"], 0, 0, 0, 0, 0)
            rhos[j] = m["rho"].data_ptr()
            grads[j] = m["grad"].data_ptr()
            lds[j] = m["n"]
        h = ctypes.c_void_p()
        _lib.check(self._L.okg_batch_create(nm, plans, grids, rhos, grads, lds, 1 if self.want_grad else 0,
                                            ctypes.byref(h)))
        self._batch = h
        sms = __import__("torch").cuda.get_device_properties(self.device).multi_processor_count
        threads, points = sch.get("layout", (sch.get("threads", 384), 1))
        if self.kernel_cusp and points != 1:
            raise ValueError("the in-kernel FP64 cusp points need one point per generation thread")
        _lib.check(self._L.okg_batch_set_schedule(h, sch["grab"], sms, 384))
        _lib.check(self._L.okg_batch_set_generation(h, int(threads), int(points)))
        self.schedule = dict(sch)

    def tiles(self):
        t = ctypes.c_longlong(0)
        _lib.check(self._L.okg_batch_tiles(self._batch, ctypes.byref(t)))
        return t.value

    def autotune(self, use_cache=True):
        import torch
        key = "batch-" + autotune.bucket(nmol=len(self.mols), pts=self.npts,
                                         nao=max(m["basis"].ncart for m in self.mols),
                                         nmo=max(len(m["occ"]) for m in self.mols))
        # (the FP64 cusp variant of the kernel has one point per generation thread)
        layouts = [lt for lt in LAYOUTS if lt[1] == 1 or not self.kernel_cusp]
        key += "-cusp" if self.kernel_cusp else ""
        cands = [{"n_max": n, "grab": g, "order": o, "layout": lt}
                 for n in N_TILES for g in GRABS for o in ORDERS for lt in layouts]

        def measure(c):
            self.set_schedule(c)
            self.run(cusp=False)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            self.run(cusp=False)
            e1.record()
            torch.cuda.synchronize()
            self.check()
            return e0.elapsed_time(e1)

        best, self.tune_report = autotune.tune(key, cands, measure, repeats=1, use_cache=use_cache)
        return best

    # ------------------------------------------------------------------ run
    def run(self, stream=None, cusp=True):
        _lib.check(self._L.okg_batch_run(self._batch, _lib.stream_handle(stream)))
        if cusp and self.cusp_radius > 0 and self.cusp_mode == "recompute":
            self._fix_cusp()

    def _fix_cusp(self):
        import torch
        if self._cusp is None:
            self._cusp = []
            for m in self.mols:
                G = torch.as_tensor(m["geo"], device=self.device)
                near = torch.zeros(m["n"], dtype=torch.bool, device=self.device)
                for a in range(G.shape[0]):
                    near |= ((m["pts"] - G[a][:, None]) ** 2).sum(0) <= self.cusp_radius ** 2
                idx = torch.nonzero(near).flatten()
                sub = m["pts"][:, idx].contiguous()
                self._cusp.append((idx, sub, torch.empty(len(idx), dtype=torch.float64, device=self.device),
                                   torch.empty((3, len(idx)), dtype=torch.float64, device=self.device)))
        codes = _lib.int_array([1, 2, 3])
        for m, (idx, sub, r, dr) in zip(self.mols, self._cusp):
            k = len(idx)
            if k == 0:
                continue
            gd = _lib.OkgGrid(sub[0].data_ptr(), sub[1].data_ptr(), sub[2].data_ptr(), k, 0, 0, 0, 0, 0)
            _lib.check(self._L.okg_rho(m["basis"].handle, gd, len(m["occ"]), _lib.ptr(m["C"]), _lib.ptr(m["occ"]), 3,
                                       codes, 1, _lib.ptr(r), _lib.ptr(dr), k, None, _lib.stream_handle()))
            m["rho"].index_copy_(0, idx, r)
            m["grad"].index_copy_(1, idx, dr)

    def capture(self):
        """CUDA graph of one run (counter reset + persistent launch [+ cusp recomputation])."""
        import torch
        self.run()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                self.run()
        torch.cuda.current_stream().wait_stream(s)
        return g

    def check(self):
        st = ctypes.c_int(0)
        _lib.check(self._L.okg_batch_status(self._batch, ctypes.byref(st)))

    def results(self):
        return [(m["rho"].cpu().numpy(), m["grad"].cpu().numpy()) for m in self.mols]

    def __del__(self):
        if getattr(self, "_batch", None) is not None and self._batch.value:
            try:
                self._L.okg_batch_destroy(self._batch)
            except Exception:
                pass
            self._batch = None
