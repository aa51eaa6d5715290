#!/usr/bin/env python
"""Benchmark: grid points/s for rho + grad rho on one GB300, mixed vs FP64 GPU path.

Workload (default): the mid-size molecule -- 20 atoms (C/N/O/H 6:1:1:12) in a
16-bohr box, 180 Cartesian AOs, 40 occupied MOs, regular 160^3 grid at 0.15 bohr
(4 096 000 points) -- seeded synthetic data (orbkit_gb300.synthetic.mid).

  value      points/s of the mixed-precision path (tensor-core contraction, FP64
             exponent arguments and density accumulation, FP64 cusp region), inputs
             resident in HBM, L2 flushed (256 MB write) between timed steps.
  e2e        the same through orbkit's drop-in call core.rho_compute(qc,
             drv=['x','y','z'], precision='mixed') on the grid module's axes: grid
             axes uploaded, rho + grad rho returned as numpy arrays every step (the
             evaluator is reused from the first call on the molecule and grid); the
             evaluator path that uploads every parameter each step from pinned host
             memory is reported beside it.
  roofline   of the dominant kernel (the fused mixed kernel), achieved = algorithmic
             contraction FLOPs (8 NMO NAO per point) / its CUDA-event launch time.
  cpu_baseline  the CPU oracle (a C restatement of orbkit's cy_core/c_grid-based
             path) on the host cores, on a bounded random sample of the grid.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun every rank evaluates its own copy of the workload (weak scaling).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "grid points/s for rho+grad rho, mixed vs FP64 GPU path at stated max rel err"
UNIT = "grid points/s"
WORKLOAD = ("mid: 20 atoms (C/N/O/H 6:1:1:12, 16-bohr box), 180 Cartesian AOs (3s2p1d / 2s1p), "
            "40 occupied MOs, regular 160^3 grid at 0.15 bohr, rho + grad rho")


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def profile_traffic(kernel_key):
    """DRAM bytes per launch of a kernel from the committed ncu summary, or None."""
    p = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            parts = line.split()
            if len(parts) >= 2 and parts[0] == kernel_key:
                try:
                    return float(parts[1])
                except ValueError:
                    return None
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 50 ms in the background."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.samples = []
        self.proc = None
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-lms", "50", "-i", str(self.gpu)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.time(), line.strip()))

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.t is not None:
                self.t.join(timeout=2)

    def summary(self, t0, t1):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        window = [s for (t, s) in self.samples if t0 - 0.06 <= t <= t1 + 0.06] or [s for (_, s) in self.samples]
        for s in window:
            f = [v.strip() for v in s.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(numpy.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_rate(qc, gx, gy, gz, target_s=12.0, seed=0, max_pts=2_000_000, nthreads=None):
    """Oracle points/s on a random sample of the regular grid (all host threads, or
    nthreads)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import okref
    okref.build()
    cores = nthreads or len(os.sched_getaffinity(0))
    rng = numpy.random.default_rng(seed)

    def sample(n):
        idx = rng.integers(0, len(gx) * len(gy) * len(gz), n)
        nyz = len(gy) * len(gz)
        return gx[idx // nyz], gy[(idx // len(gz)) % len(gy)], gz[idx % len(gz)]

    n0 = 64 * cores
    x, y, z = sample(n0)
    t = time.perf_counter()
    okref.rho_threads(qc, x, y, z, drv=["x", "y", "z"], slice_length=64, nthreads=cores)
    dt = time.perf_counter() - t
    n = int(min(max_pts, max(n0, n0 / max(dt, 1e-6) * target_s)))
    x, y, z = sample(n)
    t = time.perf_counter()
    okref.rho_threads(qc, x, y, z, drv=["x", "y", "z"], slice_length=max(64, n // (8 * cores)), nthreads=cores)
    dt = time.perf_counter() - t
    return n / dt, cores, n, dt


def dist_setup(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def run_reference(args):
    """The reference's CPU path for this workload: the C restatement of orbkit's
    cy_core / c_grid-based grid path (rho + grad rho per slice, slices over all
    host threads), bounded random samples of the same grid."""
    rank, world, local = dist_setup(args)
    if rank != 0:
        return
    from orbkit_gb300 import synthetic
    w = synthetic.mid()
    qc = w["qc"]
    gx, gy, gz = w["grid"]
    rates = []
    cores = n = None
    for i in range(args.warmup + args.steps):
        r, cores, n, dt = cpu_rate(qc, gx, gy, gz, target_s=args.ref_step_s, seed=i)
        if i >= args.warmup:
            rates.append((n, dt))
    tot_n = sum(a for a, _ in rates)
    tot_t = sum(b for _, b in rates)
    value = tot_n / tot_t
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / len(rates),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "npts_per_step": n, "sample": "random grid points"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "%d random points of the 160^3 grid per step, rho + grad rho" % n},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def run_ours(args):
    import torch
    rank, world, local = dist_setup(args)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    from orbkit_gb300 import _lib, mixed, synthetic
    from orbkit_gb300.core import _DeviceGrid

    L = _lib.load()
    w = synthetic.mid()
    qc = w["qc"]
    gx, gy, gz = w["grid"]
    npts = len(gx) * len(gy) * len(gz)
    ev = mixed.MixedEvaluator(qc, device=dev)
    b, plan = ev.basis, ev.plan
    g = _DeviceGrid(gx, gy, gz, False, dev)
    gd, keep = g.slice(0, npts)
    rho = torch.empty(npts, dtype=torch.float64, device=dev)
    grad = torch.empty((3, npts), dtype=torch.float64, device=dev)
    r64 = torch.empty_like(rho)
    g64 = torch.empty_like(grad)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    codes = _lib.int_array([1, 2, 3])
    st = _lib.stream_handle()

    def step_mixed():
        ev.evaluate_device(g, rho, grad)

    def step_fp64():
        _lib.check(L.okg_rho(b.handle, gd, plan.nmo, _lib.ptr(plan.C), _lib.ptr(plan.occ), 3, codes, 0,
                             _lib.ptr(r64), _lib.ptr(g64), npts, None, st))

    def sync_all():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    def timed(fn, k, w_):
        for _ in range(w_):
            fn()
        sync_all()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k)]
        t0 = time.time()
        for e0, e1 in evs:
            flush.fill_(1)
            e0.record()
            fn()
            e1.record()
        sync_all()
        t1 = time.time()
        return sum(e0.elapsed_time(e1) for e0, e1 in evs) / k, t0, t1

    # accuracy of the mixed path against the FP64 path (itself at 1e-12 of the oracle)
    step_fp64()
    step_mixed()
    torch.cuda.synchronize()
    ev.check()
    err = mixed.error_report(rho.cpu().numpy(), grad.cpu().numpy(), r64.cpu().numpy(), g64.cpu().numpy())
    # the tensor-core kernel alone at the points the FP64 recomputation replaces
    near = mixed.cusp_points_regular(qc.geo_spec, gx, gy, gz, ev.cusp_radius)
    plan.rho(gd, rho, grad, npts)
    torch.cuda.synchronize()
    err_near = mixed.error_report(rho.cpu().numpy()[near], grad.cpu().numpy()[:, near], r64.cpu().numpy()[near],
                                  g64.cpu().numpy()[:, near]) if len(near) else None

    fp64_ms, _, _ = timed(step_fp64, 2, 1)

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    ms, t0, t1 = timed(step_mixed, args.steps, args.warmup)
    clocks.stop()
    ev.check()
    clk = clocks.summary(t0, t1)

    # the dominant kernel alone (same stream as its launch: torch's current stream)
    def kernel_only():
        plan.rho(gd, rho, grad, npts)
    kms, _, _ = timed(kernel_only, max(3, args.steps), 1)

    # end to end through orbkit's drop-in call, as an orbkit user makes it: the grid
    # module holds the 160^3 axes (numpy), core.rho_compute(qc, drv=['x','y','z'],
    # precision='mixed') uploads them, evaluates (tensor-core kernel + FP64 cusp
    # points; the evaluator, its plan and the cusp points are reused from the first
    # call on this molecule and grid) and returns numpy rho and grad rho
    from orbkit_gb300 import core as okcore, grid as okgrid
    okgrid.set_grid(gx, gy, gz, is_vector=False)
    okcore.quiet = True

    def step_dropin():
        okcore.rho_compute(qc, drv=["x", "y", "z"], precision="mixed")

    for _ in range(args.warmup):
        step_dropin()
    sync_all()
    te = time.perf_counter()
    for _ in range(args.steps):
        step_dropin()
    sync_all()
    dropin_ms = (time.perf_counter() - te) * 1e3 / args.steps
    dropin_h2d = 8 * (len(gx) + len(gy) + len(gz))

    # end to end through the evaluator with pinned host buffers, every parameter
    # (geometry, primitives, MO coefficients, occupations) uploaded every step
    prim_h = torch.from_numpy(b.flat["prim"].copy()).pin_memory()
    geo_h = torch.from_numpy(numpy.asarray(qc.geo_spec, dtype=numpy.float64).copy()).pin_memory()
    C_h = torch.from_numpy(qc.mo_spec.get_coeffs()).pin_memory()
    occ_h = torch.from_numpy(numpy.array([m["occ_num"] for m in qc.mo_spec])).pin_memory()
    out_h = (torch.empty(npts, dtype=torch.float64).pin_memory(), torch.empty((3, npts), dtype=torch.float64).pin_memory())
    gvec = [numpy.ascontiguousarray(v) for v in (gx, gy, gz)]

    def step_e2e():
        ev.update(geo=geo_h, prim=prim_h, coeffs=C_h, occ=occ_h)
        ev.evaluate(*gvec, False, out=out_h)

    for _ in range(args.warmup):
        step_e2e()
    sync_all()
    te = time.perf_counter()
    for _ in range(args.steps):
        step_e2e()
    sync_all()
    e2e_ms = (time.perf_counter() - te) * 1e3 / args.steps
    h2d = (geo_h.numel() + prim_h.numel() + C_h.numel() + occ_h.numel() + sum(len(v) for v in gvec)) * 8
    d2h = 4 * npts * 8

    times = torch.tensor([ms, kms, e2e_ms, fp64_ms, dropin_ms], dtype=torch.float64, device=dev)
    if world > 1:
        torch.distributed.all_reduce(times, op=torch.distributed.ReduceOp.MAX)
    ms, kms, e2e_ms, fp64_ms, dropin_ms = [float(v) for v in times.cpu()]
    if rank != 0:
        return

    pk, pk_kind = peaks()
    ncart, nmo = b.ncart, plan.nmo
    flops = 8.0 * nmo * b.nao * npts
    achieved = flops / (kms * 1e-3) / 1e12
    fma = ctypes_fp64_rate(L)
    fp64_path_fma_rate = 4.0 * nmo * ncart * npts / (fp64_ms * 1e-3)
    n_fix = len(mixed.cusp_points_regular(qc.geo_spec, gx, gy, gz, ev.cusp_radius))
    out = {
        "metric": METRIC,
        "value": world * npts / (ms * 1e-3),
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "bf16",
        "data": "synthetic",
        "config": {
            "workload": WORKLOAD, "npts": npts, "nao": b.nao, "nmo": nmo, "path": "mixed",
            "precision": "C.AO on tcgen05 with BF16x3 operand splits (6 MMAs), FP32 accumulation in TMEM; "
                         "FP64 exponent arguments and density accumulation; points within %.2f bohr of a nucleus "
                         "(%d points) recomputed in FP64" % (ev.cusp_radius, n_fix),
            "max_rel_err": {"rho_max_rel": err["rho_max_rel"], "rho_floor": err["floor"],
                            "rho_max_abs": err["rho_max_abs"], "grad_max_rel": err["grad_max_rel"],
                            "against": "FP64 GPU path (1e-12 of the oracle)"},
            "near_nuclei_tensor_core_err": None if err_near is None else {
                "points": int(len(near)), "rho_max_rel": err_near["rho_max_rel"],
                "grad_max_rel": err_near["grad_max_rel"],
                "note": "the tensor-core kernel alone at the points recomputed in FP64"},
            "fp64_path": {"value": world * npts / (fp64_ms * 1e-3), "ms_per_step": fp64_ms,
                          "fp64_fma_per_s_contraction": fp64_path_fma_rate},
            "mixed_over_fp64": fp64_ms / ms,
            "l2": "flushed between timed steps (256 MB device write)",
            "parallelism": "weak: every GPU evaluates its own copy of the workload",
        },
        "roofline": {
            "bound": "tensor", "achieved": achieved, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
            "frac": achieved / pk["bf16_tflops"], "traffic": profile_traffic("rho_mixed_kernel"),
            "peak_source": "bf16 burst, %s (MEASURED_PEAKS.json)" % pk_kind if pk_kind == "measured" else pk_kind,
            "kernel": "rho_mixed_kernel", "kernel_ms": kms,
            "algorithmic": "8*NMO*NAO FLOP per point (value + 3 derivatives of C.AO)",
            "hbm_bytes_per_point": 32, "hbm_gbs": 32.0 * npts / (kms * 1e-3) / 1e9, "hbm_peak_gbs": pk["hbm_gbs"],
            "fp64_fma_peak_per_s": fp64_fma_peak(), "fp64_fma_diag_per_s": fma,
        },
        "clocks": clk,
        "e2e": {"value": world * npts / (dropin_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": int(dropin_h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": dropin_ms,
                "api": "orbkit_gb300.core.rho_compute(qc, drv=['x','y','z'], precision='mixed') on the grid "
                       "module's 160^3 axes, numpy results",
                "evaluator_all_parameters_uploaded": {
                    "value": world * npts / (e2e_ms * 1e-3), "ms_per_step": e2e_ms, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h),
                    "api": "mixed.MixedEvaluator.update + evaluate, pinned host buffers"}},
        "gpu_launches": args.steps * (1 + (1 if n_fix else 0)),
    }
    if world == 1 and not args.no_cpu_baseline:
        rate, cores, n, dt = cpu_rate(qc, gx, gy, gz)
        rate1, _, n1, dt1 = cpu_rate(qc, gx, gy, gz, target_s=4.0, seed=1, nthreads=1)
        out["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                               "sample": "%d random points of the 160^3 grid, rho + grad rho, %.1f s" % (n, dt),
                               "single_core": {"value": rate1, "cores": 1,
                                               "sample": "%d random points, one thread (numproc=1), %.1f s"
                                                         % (n1, dt1)}}
    print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


def run_profile(args):
    """Minimal launch sequence for ncu: each kernel of the path once as warm-up, then
    once more (mixed kernel, FP64 fused kernel) on the full workload.  With --workload
    detci / overlap: the kernels of that row twice on a smaller case."""
    if args.workload == "detci":
        return _profile_detci()
    if args.workload == "overlap":
        return _profile_overlap()
    if args.workload == "large":
        return _profile_large()
    if args.workload == "ao":
        return _profile_ao()
    if args.workload == "batch":
        return _profile_batch()
    import torch
    from orbkit_gb300 import _lib, mixed, synthetic
    from orbkit_gb300.core import _DeviceGrid
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    L = _lib.load()
    w = synthetic.mid()
    qc = w["qc"]
    gx, gy, gz = w["grid"]
    npts = len(gx) * len(gy) * len(gz)
    ev = mixed.MixedEvaluator(qc, device=dev)
    g = _DeviceGrid(gx, gy, gz, False, dev)
    gd, keep = g.slice(0, npts)
    rho = torch.empty(npts, dtype=torch.float64, device=dev)
    grad = torch.empty((3, npts), dtype=torch.float64, device=dev)
    codes = _lib.int_array([1, 2, 3])
    for _ in range(2):
        ev.plan.rho(gd, rho, grad, npts)
        _lib.check(L.okg_rho(ev.basis.handle, gd, ev.plan.nmo, _lib.ptr(ev.plan.C), _lib.ptr(ev.plan.occ), 3, codes,
                             0, _lib.ptr(rho), _lib.ptr(grad), npts, None, _lib.stream_handle()))
    torch.cuda.synchronize()
    ev.check()
    print("profile run done: %d points" % npts)


def _profile_large():
    """The large basis (2420 Cartesian AOs, 400 MOs) on a 128 x 128 x 64 block of its
    grid (2^20 points, brick tiles) on the mixed path, and the FP64 fused kernel on
    2^16 of those points; each twice."""
    import torch
    from orbkit_gb300 import _lib, mixed, synthetic
    from orbkit_gb300.core import _DeviceGrid
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    L = _lib.load()
    w = synthetic.large()
    qc = w["qc"]
    gx, gy, gz = w["grid"]
    bx, by, bz = gx[64:192], gy[64:192], gz[96:160]
    ev = mixed.MixedEvaluator(qc, device=dev, cusp_radius=0.0)
    g = _DeviceGrid(bx, by, bz, False, dev)
    n = g.npts
    gd, keep = g.slice(0, n)
    rho = torch.empty(n, dtype=torch.float64, device=dev)
    grad = torch.empty((3, n), dtype=torch.float64, device=dev)
    n64 = 1 << 16
    gd64, keep64 = g.slice(n // 2, n // 2 + n64)
    codes = _lib.int_array([1, 2, 3])
    for _ in range(2):
        ev.plan.rho(gd, rho, grad, n)
        _lib.check(L.okg_rho(ev.basis.handle, gd64, ev.plan.nmo, _lib.ptr(ev.plan.C), _lib.ptr(ev.plan.occ), 3, codes,
                             0, _lib.ptr(rho), _lib.ptr(grad), n64, None, _lib.stream_handle()))
    torch.cuda.synchronize()
    ev.check()
    print("profile run done: large, %d points mixed, %d FP64" % (n, n64))


def _profile_batch():
    """A 12-molecule batch (10-30 atoms each, atom-centred point sets, 6.1 M points) on
    the persistent batch kernel, three launches with the FP64 cusp region in the launch
    and three from the tensor cores alone (schedule fixed: 384 x 1, 64 MO columns)."""
    import torch
    from orbkit_gb300 import synthetic
    from orbkit_gb300.batch import BatchEvaluator
    torch.cuda.set_device(0)
    d = synthetic.batch(nmol=12, min_atoms=10, max_atoms=30)
    mols = [(m["qc"], m["points"]) for m in d["molecules"]]
    npts = sum(pp.shape[1] for _, pp in mols)
    sch = {"n_max": 64, "grab": 1, "order": "largest_first", "layout": (384, 1)}
    for radius in (None, 0.0):
        ev = BatchEvaluator(mols, tune=False, cusp_radius=radius, schedule=sch)
        for _ in range(3):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            ev.run()
            e1.record()
            torch.cuda.synchronize()
            print("batch %s: %d points, %.3f ms" % ("FP64 cusp region" if radius is None else "tensor cores alone",
                                                   npts, e0.elapsed_time(e1)))
        ev.check()
    print("profile run done: batch")


def _profile_ao():
    """okg_eval_ao (drv 0) on the mid molecule: 40 x 160 x 160 points of its grid
    (1 024 000 points, 180 AOs: 1.47 GB written), twice."""
    import torch
    from orbkit_gb300 import _lib, synthetic
    from orbkit_gb300.basis import get_basis
    from orbkit_gb300.core import _DeviceGrid
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    L = _lib.load()
    w = synthetic.mid()
    qc = w["qc"]
    gx, gy, gz = w["grid"]
    b = get_basis(qc.geo_spec, qc.ao_spec, dev)
    g = _DeviceGrid(gx[60:100], gy, gz, False, dev)
    n = g.npts
    gd, keep = g.slice(0, n)
    out = torch.empty((b.nao, n), dtype=torch.float64, device=dev)
    for _ in range(2):
        _lib.check(L.okg_eval_ao(b.handle, gd, 1, _lib.int_array([0]), 0, _lib.ptr(out), n, _lib.stream_handle()))
    torch.cuda.synchronize()
    print("profile run done: ao, %d points x %d AOs" % (n, b.nao))


def _profile_detci():
    """detci kernels (quadratic forms and term order) twice each on 2^20 points of
    seeded MO grids (42 MOs, the first state pair's terms): 1.4 GB on the device."""
    import torch
    from orbkit_gb300 import detci
    d = numpy.load(os.path.join(ROOT, "tests", "golden", "h3p_detci.npz"))
    npts = 1 << 20
    zero = [[list(d["zero_coef_0"])], [list(int(v) for v in d["zero_orb_0"])]]
    sing = [list(d["sing_coef_0"]), [list(map(int, p)) for p in d["sing_pair_0"]]]
    g = torch.Generator(device="cuda").manual_seed(7)
    mo = torch.randn((42, npts), generator=g, dtype=torch.float64, device="cuda")
    drv = torch.randn((3, 42, npts), generator=g, dtype=torch.float64, device="cuda")
    for exact in (False, False, True, True):
        detci.rho(zero, sing, mo, reference_slicing=False, exact=exact)
        detci.jab(zero, sing, mo, drv, reference_slicing=False, exact=exact)
    torch.cuda.synchronize()
    print("profile run done: detci, %d points" % npts)


def _profile_overlap():
    """okg_ao_overlap on the 200-atom basis (2420 Cartesian AOs): S and dS/dx, twice."""
    import torch
    from orbkit_gb300 import analytical_integrals as ai, synthetic
    qc = synthetic.large()["qc"]
    geo = torch.tensor(numpy.asarray(qc.geo_spec), device="cuda")
    for _ in range(2):
        for d in (None, "x"):
            ai.get_ao_overlap(geo, geo, qc.ao_spec, drv=d)
    torch.cuda.synchronize()
    print("profile run done: overlap")


def _events():
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def _time_ms(fn, steps, warmup, flush=None):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    tot = 0.0
    for _ in range(steps):
        if flush is not None:
            flush.fill_(1)
        e0, e1 = _events()
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        tot += e0.elapsed_time(e1)
    return tot / steps


def run_workload(args):
    """Other workload shapes (one JSON line each; the default run is the mid workload)."""
    import torch
    from orbkit_gb300 import _lib, mixed, synthetic
    from orbkit_gb300.core import _DeviceGrid
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    L = _lib.load()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    name = args.workload
    out = {"metric": METRIC, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "data": "synthetic", "dtype": "bf16"}
    if name in ("small", "large"):
        out.update(_single_workload(args, name, flush, L))
    elif name == "grad":
        from orbkit_gb300.adjoint import DensityModel, density_fit_loss
        w = synthetic.grad()
        qc = w["qc"]
        x, y, z = w["grid"]
        prim = qc.ao_spec.get_prim_coeffs()
        res = {}
        for prec in ("fp64", "fp32"):
            model = DensityModel(qc, x, y, z, False, prec)
            t = w["target"]
            with torch.no_grad():
                rt, gt = model(torch.tensor(t["coeffs"], device=dev), torch.tensor(t["alpha"], device=dev),
                               torch.tensor(prim[:, 1], device=dev), torch.tensor(t["geo"], device=dev))
                rt, gt = rt.clone(), gt.clone()
            wts = torch.tensor(numpy.random.default_rng(w["weight_seed"]).uniform(1e-12, 1, model.npts), device=dev)
            C = torch.tensor(qc.mo_spec.get_coeffs(), device=dev, requires_grad=True)
            a = torch.tensor(prim[:, 0], device=dev, requires_grad=True)
            c = torch.tensor(prim[:, 1], device=dev, requires_grad=True)
            gg = torch.tensor(numpy.asarray(qc.geo_spec), device=dev, requires_grad=True)

            def step():
                for q in (C, a, c, gg):
                    q.grad = None
                density_fit_loss(*model(C, a, c, gg), rt, gt, wts).backward()
            res[prec] = (_time_ms(step, args.steps, args.warmup, flush), model.npts,
                         [q.grad.detach().clone() for q in (C, a, c, gg)])
        rel = [float((g32 - g64).abs().max() / g64.abs().max()) for g32, g64 in zip(res["fp32"][2], res["fp64"][2])]
        npts = res["fp64"][1]
        out.update({"metric": "grid points/s for loss + gradient (dL/dC, dL/dalpha, dL/dc, dL/dR), FP32 vs FP64",
                    "value": npts / (res["fp32"][0] * 1e-3), "ms_per_step": res["fp32"][0], "dtype": "f32",
                    "config": {"workload": "grad: 12 atoms, 128^3 grid, density-fitting loss, forward + adjoint",
                               "npts": npts, "fp64": {"value": npts / (res["fp64"][0] * 1e-3),
                                                      "ms_per_step": res["fp64"][0]},
                               "fp32_vs_fp64_gradient_rel_err": dict(zip(["C", "alpha", "c", "R"], rel))}})
    elif name == "batch":
        from orbkit_gb300.batch import BatchEvaluator
        d = synthetic.batch()
        mols = [(m["qc"], m["points"]) for m in d["molecules"]]
        npts = sum(pp.shape[1] for _, pp in mols)
        from orbkit_gb300 import mixed
        # default: the cusp region (points within CUSP_RADIUS of a nucleus, a third of
        # these atom-centred grids) keeps its steep primitives in FP64 inside the launch
        ev = BatchEvaluator(mols, tune=True)
        graph = ev.capture()
        ms = _time_ms(graph.replay, args.steps, args.warmup)
        ev.check()
        ncusp = int(sum(int((m["near"] >= 0).sum()) for m in ev.mols))
        # the same batch from the tensor cores alone (no FP64 cusp part)
        ev0 = BatchEvaluator(mols, cusp_radius=0.0, tune=True)
        graph0 = ev0.capture()
        ms0 = _time_ms(graph0.replay, args.steps, args.warmup)
        ev0.check()
        out.update({"value": npts / (ms * 1e-3), "ms_per_step": ms,
                    "config": {"workload": "batch: 256 molecules, 3-60 atoms, atom-centred point sets",
                               "npts": npts, "molecules": len(mols), "tiles": ev.tiles(), "schedule": ev.schedule,
                               "launch": "CUDA graph replay of one persistent kernel",
                               "cusp": {"radius": ev.cusp_radius, "alpha_c": ev.cusp_alpha, "points": ncusp,
                                        "mode": "steep primitives of the cusp atom in FP64 inside the launch"},
                               "tensor_cores_alone": {"value": npts / (ms0 * 1e-3), "ms_per_step": ms0,
                                                      "schedule": ev0.schedule},
                               "with_over_without_cusp": ms0 / ms}})
    elif name == "ao":
        out.update(_ao_workload(args, flush, L))
    elif name == "overlap":
        out.update(_overlap_workload(args, flush))
    elif name == "detci":
        out.update(_detci_workload(args, flush))
    print(json.dumps(out))


def _single_workload(args, name, flush, L):
    """The small or large molecule on its full regular grid: mixed path (value), its
    kernel alone (tensor roofline), and the FP64 path on a seeded random sample of the
    grid's points (whole grid for small; 2^18 points for large) with its FP64-pipe
    roofline; the mixed path's error against the FP64 path at those points."""
    import torch
    from orbkit_gb300 import _lib, mixed, synthetic
    from orbkit_gb300.core import _DeviceGrid
    dev = torch.device("cuda", 0)
    w = synthetic.small() if name == "small" else synthetic.large()
    qc = w["qc"]
    gx, gy, gz = w["grid"]
    npts = len(gx) * len(gy) * len(gz)
    ev = mixed.MixedEvaluator(qc, device=dev)
    b, p = ev.basis, ev.plan
    g = _DeviceGrid(gx, gy, gz, False, dev)
    gd, keep = g.slice(0, npts)
    rho = torch.empty(npts, dtype=torch.float64, device=dev)
    grad = torch.empty((3, npts), dtype=torch.float64, device=dev)
    ms = _time_ms(lambda: ev.evaluate_device(g, rho, grad), args.steps, args.warmup, flush)
    ev.check()
    kms = _time_ms(lambda: p.rho(gd, rho, grad, npts), max(3, args.steps), 1, flush)
    ev.evaluate_device(g, rho, grad)
    # FP64 path on a seeded random sample of the grid (a vector grid of those points)
    if name == "small":
        idx = numpy.arange(npts)
    else:
        idx = numpy.sort(numpy.random.default_rng(9).choice(npts, 1 << 18, replace=False))
    n64 = len(idx)
    nyz = len(gy) * len(gz)
    pts = [torch.from_numpy(numpy.ascontiguousarray(v)).to(dev)
           for v in (gx[idx // nyz], gy[(idx // len(gz)) % len(gy)], gz[idx % len(gz)])]
    gd64 = _lib.OkgGrid(pts[0].data_ptr(), pts[1].data_ptr(), pts[2].data_ptr(), n64, 0, 0, 0, 0, 0)
    r64 = torch.empty(n64, dtype=torch.float64, device=dev)
    g64 = torch.empty((3, n64), dtype=torch.float64, device=dev)
    codes = _lib.int_array([1, 2, 3])
    fp64_ms = _time_ms(lambda: _lib.check(L.okg_rho(b.handle, gd64, p.nmo, _lib.ptr(p.C), _lib.ptr(p.occ), 3, codes,
                                                    0, _lib.ptr(r64), _lib.ptr(g64), n64, None,
                                                    _lib.stream_handle())), 2, 1, flush)
    it = torch.from_numpy(idx).to(dev)
    err = mixed.error_report(rho[it].cpu().numpy(), grad[:, it].cpu().numpy(), r64.cpu().numpy(), g64.cpu().numpy())
    pk, pk_kind = peaks()
    tflops = 8.0 * p.nmo * b.nao * npts / (kms * 1e-3) / 1e12
    fma64 = 4.0 * p.nmo * b.ncart * n64 / (fp64_ms * 1e-3)
    fpk = fp64_fma_peak()
    res = {"value": npts / (ms * 1e-3), "ms_per_step": ms,
           "config": {"workload": name, "npts": npts, "nao": b.nao, "ncart": b.ncart, "nmo": p.nmo,
                      "spherical": b.spherical, "path": "mixed",
                      "fp64_path": {"value": n64 / (fp64_ms * 1e-3), "points_timed": n64,
                                    "sample": "all grid points" if n64 == npts else
                                    "seeded random sample of the grid's points (vector grid)"},
                      "mixed_over_fp64": (npts / ms) / (n64 / fp64_ms),
                      "max_rel_err": dict(err, against="FP64 GPU path at the %d points it timed" % n64)},
           "roofline": {"bound": "tensor", "achieved": tflops, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                        "frac": tflops / pk["bf16_tflops"], "traffic": profile_traffic("rho_mixed_kernel_" + name),
                        "kernel": "rho_mixed_kernel", "kernel_ms": kms,
                        "peak_source": "bf16 burst, %s (MEASURED_PEAKS.json)" % pk_kind,
                        "algorithmic": "8*NMO*NAO FLOP per point (value + 3 derivatives of C.AO)",
                        "fp64_path": {"bound": "fp64", "achieved": fma64, "peak": fpk, "unit": "FMA/s",
                                      "frac": fma64 / fpk, "kernel": "fused64_kernel", "kernel_ms": fp64_ms,
                                      "traffic": profile_traffic("fused64_kernel_" + name),
                                      "algorithmic": "4*NMO*NCART FMA per point (C.AO for value + 3 derivatives)",
                                      "peak_source": "2 DFMA/clk/SM x SMs x max SM clock"}},
           "gpu_launches": args.steps * 2}
    if not args.no_cpu_baseline:
        rate, cores, n, dt = cpu_rate(qc, gx, gy, gz, target_s=8.0)
        res["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                               "sample": "%d random grid points, %.1f s" % (n, dt)}
    return res


def _ao_workload(args, flush, L):
    """AO values (drv 0, and the three first derivatives) of the mid molecule on 40 x
    160 x 160 points of its grid through okg_eval_ao: the HBM roofline of the AO
    kernel (8 B written per (AO, point, drv); a regular grid reads no coordinates)."""
    import torch
    from orbkit_gb300 import _lib, synthetic
    from orbkit_gb300.basis import get_basis
    from orbkit_gb300.core import _DeviceGrid
    dev = torch.device("cuda", 0)
    w = synthetic.mid()
    qc = w["qc"]
    gx, gy, gz = w["grid"]
    b = get_basis(qc.geo_spec, qc.ao_spec, dev)
    g = _DeviceGrid(gx[60:100], gy, gz, False, dev)
    n = g.npts
    gd, keep = g.slice(0, n)
    res = {}
    for nd, codes in ((1, [0]), (4, [0, 1, 2, 3])):
        out = torch.empty((nd, b.nao, n), dtype=torch.float64, device=dev)
        ca = _lib.int_array(codes)
        ms = _time_ms(lambda: _lib.check(L.okg_eval_ao(b.handle, gd, nd, ca, 0, _lib.ptr(out), n,
                                                       _lib.stream_handle())), args.steps, args.warmup, flush)
        res[nd] = (ms, 8.0 * nd * b.nao * n)
        del out
    pk, pk_kind = peaks()
    ms, byt = res[1]
    gbs = byt / (ms * 1e-3) / 1e9
    gbs4 = res[4][1] / (res[4][0] * 1e-3) / 1e9
    return {"metric": "AO values written per second (okg_eval_ao), GB/s", "unit": "GB/s", "value": gbs,
            "ms_per_step": ms, "dtype": "f64",
            "config": {"workload": "ao: mid molecule (180 Cartesian AOs), 40 x 160 x 160 = %d grid points, drv 0" % n,
                       "with_first_derivatives": {"ndrv": 4, "ms_per_step": res[4][0], "GB/s": gbs4}},
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": pk["hbm_gbs"], "unit": "GB/s",
                         "frac": gbs / pk["hbm_gbs"], "traffic": profile_traffic("ao_eval_kernel"),
                         "kernel": "ao_eval_kernel", "kernel_ms": ms,
                         "algorithmic": "8 B written per (AO, point, drv)",
                         "peak_source": "HBM copy, %s (MEASURED_PEAKS.json)" % pk_kind},
            "gpu_launches": args.steps}


def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import okref
    okref.build()
    return okref


def _overlap_workload(args, flush):
    """get_ao_overlap on the 200-atom basis (2420 Cartesian AOs, spherical output):
    S and its three ket derivatives per step."""
    import torch
    from orbkit_gb300 import analytical_integrals as ai, synthetic
    qc = synthetic.large()["qc"]
    geo = numpy.asarray(qc.geo_spec)
    plan = ai.overlap_plan(qc.ao_spec)
    gd = torch.tensor(geo, device="cuda")
    outs = [torch.empty((plan.nao, plan.nao), dtype=torch.float64, device="cuda") for _ in range(4)]
    L, h = plan._L, plan._h
    from orbkit_gb300 import _lib

    def step():
        for d in range(4):
            _lib.check(L.okg_ao_overlap(h, _lib.ptr(gd), _lib.ptr(gd), d, 0, _lib.ptr(outs[d]), plan.nao,
                                        _lib.stream_handle()))
    ms = _time_ms(step, args.steps, args.warmup, flush)
    f = plan.flat
    nidx = int((f["ncart"] * f["nprim"]).sum())
    res = {"metric": "AO overlap matrices/s (S, dS/dx, dS/dy, dS/dz per step)", "unit": "matrices/s",
           "value": 4 / (ms * 1e-3), "ms_per_step": ms, "dtype": "f64",
           "config": {"workload": "overlap: 200 atoms, %d Cartesian AOs, %d spherical, %d (row, primitive) pairs"
                      % (plan.ncart, plan.nao, nidx), "api": "analytical_integrals.get_ao_overlap"}}
    # end to end through the public call (host geometry in, host matrix out)
    t = time.perf_counter()
    for d in (None, "x", "y", "z"):
        ai.get_ao_overlap(geo, geo, qc.ao_spec, drv=d)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t
    res["e2e"] = {"value": 4 / e2e_s, "unit": "matrices/s", "h2d_bytes_per_step": 2 * geo.nbytes * 4,
                  "d2h_bytes_per_step": 4 * plan.nao * plan.nao * 8}
    res["gpu_launches"] = 8
    if not args.no_cpu_baseline:
        okref = _oracle()
        lx = qc.ao_spec.get_lxlylz()
        t = time.perf_counter()
        okref.aooverlap(geo, geo, lx, lx, qc.ao_spec, 0)
        dt = time.perf_counter() - t
        res["cpu_baseline"] = {"value": 1 / dt, "unit": "matrices/s", "cores": 1, "kind": "port",
                               "sample": "one raw Cartesian overlap matrix (cy_overlap.aooverlap restated in C), "
                                         "%.2f s" % dt}
    return res


def _detci_workload(args, flush):
    """CI transition density and flux density (detci.rho + detci.jab) from MO grids:
    the determinant-comparison terms of the first state pair of the H3+ FCI test
    (436 zero terms, 7160 single-excitation terms over 42 MOs) on 2^21 points of
    seeded MO grids.  value: the default evaluation (terms folded into 42 x 42
    matrices, okg_ci_rho_matrix + okg_ci_flux_matrix); term_order: orbkit's term-order
    sums (okg_ci_rho + okg_ci_jab)."""
    import torch
    from orbkit_gb300 import _lib, detci
    d = numpy.load(os.path.join(ROOT, "tests", "golden", "h3p_detci.npz"))
    npts, nmo = 1 << 21, 42
    zc, zi = d["zero_coef_0"], d["zero_orb_0"]
    sc, sp = d["sing_coef_0"], d["sing_pair_0"]
    zero = [[list(zc)], [list(int(v) for v in zi)]]
    sing = [list(sc), [list(map(int, p)) for p in sp]]
    g = torch.Generator(device="cuda").manual_seed(7)
    mo = torch.randn((nmo, npts), generator=g, dtype=torch.float64, device="cuda")
    drv = torch.randn((3, nmo, npts), generator=g, dtype=torch.float64, device="cuda")
    rho = torch.empty(npts, dtype=torch.float64, device="cuda")
    j = torch.empty((3, npts), dtype=torch.float64, device="cuda")
    L = detci._L()
    keep = [torch.from_numpy(numpy.ascontiguousarray(a)).cuda() for a in (zc, zi.astype(numpy.int32), sc,
                                                                           sp.astype(numpy.int32))]
    M = detci.density_matrix(zero, sing, nmo)
    S = M + M.T
    S[numpy.diag_indices(nmo)] = numpy.diag(M)
    q_rho = detci._qt_device(numpy.tril(S), nmo)
    C = detci.flux_matrix(sing, nmo)
    q_jab = detci._qt_device((C - C.T).T, nmo)
    st = _lib.stream_handle()

    def step_terms():
        _lib.check(L.okg_ci_rho(npts, _lib.ptr(mo), npts, len(zc), _lib.ptr(keep[0]), _lib.ptr(keep[1]), len(sc),
                                _lib.ptr(keep[2]), _lib.ptr(keep[3]), _lib.ptr(rho), st))
        _lib.check(L.okg_ci_jab(npts, _lib.ptr(mo), _lib.ptr(drv), npts, nmo, len(sc), _lib.ptr(keep[2]),
                                _lib.ptr(keep[3]), _lib.ptr(j), st))

    def step_matrix():
        _lib.check(L.okg_ci_rho_matrix(npts, _lib.ptr(mo), npts, nmo, _lib.ptr(q_rho), _lib.ptr(rho), st))
        _lib.check(L.okg_ci_flux_matrix(npts, _lib.ptr(mo), _lib.ptr(drv), npts, nmo, _lib.ptr(q_jab), -0.5,
                                        _lib.ptr(j), st))
    ms = _time_ms(step_matrix, args.steps, args.warmup, flush)
    r_m, j_m = rho.clone(), j.clone()
    ms_terms = _time_ms(step_terms, max(2, args.steps // 2), 1, flush)
    err = max(float((r_m - rho).abs().max() / rho.abs().max()), float((j_m - j).abs().max() / j.abs().max()))
    # FMAs the quadratic forms issue per point: rho visits a <= b in chunks of 16, the
    # flux all (a, b) plus three accumulations per b
    ch = (nmo + 15) // 16
    fma_rho = sum(16 * (nmo - 16 * c) for c in range(ch)) + sum(nmo - 16 * c for c in range(ch))
    fma_jab = ch * nmo * (16 + 3)
    fma_rate = (fma_rho + fma_jab) * npts / (ms * 1e-3)
    peak = fp64_fma_peak()
    diag = ctypes_fp64_rate(_lib.load())
    res = {"metric": "grid points/s for the CI transition density + flux density from MO grids",
           "unit": "grid points/s", "value": npts / (ms * 1e-3), "ms_per_step": ms, "dtype": "f64",
           "config": {"workload": "detci: %d zero + %d single terms over %d MOs, %d points (rho then jab)"
                      % (len(zc), len(sc), nmo, npts),
                      "api": "okg_ci_rho_matrix + okg_ci_flux_matrix (detci.rho / detci.jab default)",
                      "term_order": {"value": npts / (ms_terms * 1e-3), "ms_per_step": ms_terms,
                                     "api": "okg_ci_rho + okg_ci_jab (exact=True)"},
                      "max_normwise_diff_vs_term_order": err},
           "roofline": {"bound": "fp64", "achieved": fma_rate, "peak": peak, "unit": "FMA/s",
                        "frac": fma_rate / peak, "traffic": None,
                        "note": "FMAs issued per point %d (rho) + %d (flux); peak = 2 DFMA/clk/SM x SMs x max "
                                "clock; the FMA-chain diagnostic reaches %.3g" % (fma_rho, fma_jab, diag or 0)},
           "gpu_launches": 2}
    if not args.no_cpu_baseline:
        okref = _oracle()
        n = 4096
        m = mo[:, :n].cpu().numpy()
        md = drv[:, :, :n].cpu().numpy()
        t = time.perf_counter()
        okref.ci_rho(zero, sing, m)
        okref.ci_jab(zero, sing, m, md)
        dt = time.perf_counter() - t
        res["cpu_baseline"] = {"value": n / dt, "unit": "grid points/s", "cores": 1, "kind": "port",
                               "sample": "%d points, the same terms (numpy restatement of cy_ci), %.2f s" % (n, dt)}
    return res


def fp64_fma_peak():
    """FP64 FMA peak of the device: 2 DFMA per clock per SM (the rate ncu shows for
    ci_quad_kernel at 98.6 % FP64-pipe activity) x SMs x the maximum SM clock."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    try:
        out = subprocess.run(["nvidia-smi", "-i", "0", "--query-gpu=clocks.max.sm", "--format=csv,noheader,nounits"],
                             capture_output=True, text=True, timeout=20).stdout.strip().splitlines()
        mhz = float(out[0])
    except Exception:
        mhz = 2070.0
    return 2.0 * sms * mhz * 1e6


def ctypes_fp64_rate(L):
    import ctypes
    v = ctypes.c_double(0)
    if L.okg_diag_fp64_fma_rate(4000, ctypes.byref(v)) != 0:
        return None
    return v.value


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-step-s", type=float, default=4.0)
    ap.add_argument("--profile", action="store_true", help="minimal launch sequence for ncu captures")
    ap.add_argument("--workload", default="mid",
                    choices=["mid", "small", "grad", "batch", "large", "overlap", "detci", "ao"])
    args = ap.parse_args()
    if args.profile:
        return run_profile(args)
    if args.workload != "mid" and args.impl == "ours":
        if args.warmup < 3:
            args.warmup = 3
        return run_workload(args)
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
