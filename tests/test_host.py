"""Host-side logic on the CPU: tables, grid, basis packing checks of the C ABI,
exported symbols, sharding (2 gloo ranks).  No GPU work."""
import ctypes
import os
import re

import numpy
import pytest

import okref
from helpers import load_golden

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from orbkit_gb300 import build
    build.build()
    return ctypes.CDLL(os.path.join(ROOT, "orbkit_gb300", "liborbkit_gb300.so"))


def header_functions():
    src = open(os.path.join(ROOT, "include", "orbkit_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(okg_\w+)\s*\(", src)))


def test_library_exports_every_header_symbol(lib):
    names = header_functions()
    assert len(names) >= 14
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings(lib):
    lib.okg_status_string.restype = ctypes.c_char_p
    assert lib.okg_status_string(0) == b"ok"
    assert lib.okg_status_string(-2) == b"unsupported angular momentum"
    assert lib.okg_version() >= 100


def _create(lib, lxlylz, ncart, nprim=None, atoms=None, natom=1, renorm=None):
    ip = lambda a: (ctypes.c_int * len(a))(*a)
    nshell = len(ncart)
    nprim = nprim or [1] * nshell
    atoms = atoms or [0] * nshell
    flat = [v for row in lxlylz for v in row]
    h = ctypes.c_void_p()
    lib.okg_basis_create.restype = ctypes.c_int
    st = lib.okg_basis_create(natom, nshell, ip(atoms), ip(ncart), ip(nprim), ip(flat), 0, None, 0, None, None,
                              None, ctypes.byref(h))
    return st


def test_basis_validation_errors(lib):
    """Rejected before any device work: L > 4, mixed L in a shell, repeated component,
    bad atom index, empty shells."""
    lib.okg_last_error.restype = ctypes.c_char_p
    assert _create(lib, [(5, 0, 0)], [1]) == -2
    assert b"above 4" in lib.okg_last_error()
    assert _create(lib, [(1, 0, 0), (0, 0, 0)], [2]) == -2
    assert _create(lib, [(1, 0, 0), (1, 0, 0)], [2]) == -2
    assert _create(lib, [(0, 0, 0)], [1], atoms=[3], natom=2) == -1
    assert _create(lib, [(0, 0, 0)], [0]) == -1


def test_compute_entry_points_reject_null(lib):
    g = (ctypes.c_byte * 64)()
    lib.okg_eval_ao.restype = ctypes.c_int
    assert lib.okg_eval_ao(None, ctypes.byref(g), 1, None, 0, None, ctypes.c_int64(1), None) == -1
    lib.okg_rho.restype = ctypes.c_int
    assert lib.okg_rho(None, ctypes.byref(g), 1, None, None, 0, None, 0, None, None, ctypes.c_int64(1), None,
                       None) == -1


def test_grid_operation_entry_points_validate_arguments(lib):
    """okg_mo_from_ao / okg_cart2sph / okg_mo_products / okg_mo_pair_flux reject NULL
    pointers, empty counts and leading dimensions below npts before touching a device;
    npts == 0 is a no-op."""
    i64 = ctypes.c_int64
    fake = ctypes.c_void_p(16)  # never dereferenced: rejected or zero-size before any device work
    for f in ("okg_mo_from_ao", "okg_cart2sph", "okg_mo_products", "okg_mo_pair_flux"):
        getattr(lib, f).restype = ctypes.c_int
    assert lib.okg_mo_from_ao(0, 4, fake, fake, i64(8), i64(8), fake, i64(8), None) == -1
    assert lib.okg_mo_from_ao(2, 4, None, fake, i64(8), i64(8), fake, i64(8), None) == -1
    assert lib.okg_mo_from_ao(2, 4, fake, fake, i64(4), i64(8), fake, i64(8), None) == -1
    assert lib.okg_mo_from_ao(2, 4, fake, fake, i64(8), i64(0), fake, i64(8), None) == 0
    assert lib.okg_cart2sph(3, 0, fake, fake, fake, fake, i64(8), i64(8), fake, i64(8), None) == -1
    assert lib.okg_cart2sph(3, 5, fake, fake, fake, fake, i64(8), i64(9), fake, i64(8), None) == -1
    assert lib.okg_mo_products(1, 2, 0, fake, i64(8), fake, i64(8), i64(8), fake, i64(8), None) == -1
    assert lib.okg_mo_products(1, 2, 2, fake, i64(8), None, i64(8), i64(8), fake, i64(8), None) == -1
    assert lib.okg_mo_pair_flux(3, 4, 1, None, fake, i64(8), fake, i64(8), i64(8), fake, i64(8), None) == -1
    assert lib.okg_mo_pair_flux(3, 4, 1, fake, fake, i64(8), fake, i64(2), i64(8), fake, i64(8), None) == -1
    assert lib.okg_mo_pair_flux(3, 4, 1, fake, fake, i64(8), fake, i64(8), i64(0), fake, i64(8), None) == 0


def test_mixed_order_entry_point_rejects_null(lib):
    """okg_basis_set_mixed_order checks its handle and order before any device work."""
    lib.okg_basis_set_mixed_order.restype = ctypes.c_int
    order = (ctypes.c_int * 2)(0, 1)
    assert lib.okg_basis_set_mixed_order(None, order) == -1
    assert lib.okg_basis_set_mixed_order(ctypes.c_void_p(16), None) == -1


def _mixed_layout(order, ncols):
    """Whole shells in `order` packed into 32-column chunks (the C builder's rule):
    shell -> (chunk, first column)."""
    col, chunk, pos = {}, 0, 0
    for s in order:
        if pos + ncols[s] > 32:
            chunk, pos = chunk + 1, 0
        col[s] = (chunk, pos)
        pos += ncols[s]
    return col, chunk + 1


def test_mixed_order_is_exponent_classes_then_morton():
    """The tensor-core column order: a permutation of the shells; factor-4 classes of the
    smallest exponent ascending; inside a class, atoms along a Morton curve."""
    from orbkit_gb300 import basis, synthetic
    qc = synthetic.mid()["qc"]
    f = basis.flatten(qc.ao_spec)
    order = basis.mixed_order(qc.geo_spec, f)
    assert sorted(order.tolist()) == list(range(len(f["nprim"])))
    off = numpy.concatenate(([0], numpy.cumsum(f["nprim"])))
    amin = numpy.array([f["prim"][off[s]:off[s + 1], 0].min() for s in range(len(f["nprim"]))])
    cls = numpy.floor(numpy.log(amin) / numpy.log(4.0))[order]
    assert numpy.all(numpy.diff(cls) >= 0)
    # inside a class, the atoms' Morton codes do not decrease
    geo = numpy.asarray(qc.geo_spec, dtype=float)
    q = ((geo - geo.min(0)) / (geo.max(0) - geo.min(0)) * 1023).astype(numpy.int64)
    code = numpy.zeros(len(geo), dtype=numpy.int64)
    for b in range(10):
        for d in range(3):
            code |= ((q[:, d] >> b) & 1) << (3 * b + d)
    at = numpy.asarray(f["atoms"])[order]
    for c in numpy.unique(cls):
        assert numpy.all(numpy.diff(code[at[cls == c]]) >= 0)
    assert numpy.array_equal(order, basis.mixed_order(qc.geo_spec, f))


def test_mixed_order_halves_issued_ksteps():
    """Replay of the tensor-core kernel's screening on every 4x4x8 brick of the mid grid
    (a primitive is kept while alpha log2(e) d^2 <= 64, d: distance from its atom to the
    brick): the K-steps (16 columns) holding a kept column, per brick, in basis order and
    in the package's order.  The GPU kernel counted 8.13 and 4.08."""
    from orbkit_gb300 import basis, synthetic
    w = synthetic.mid()
    qc = w["qc"]
    gx, gy, gz = w["grid"]
    f = basis.flatten(qc.ao_spec)
    geo = numpy.asarray(qc.geo_spec, dtype=float)
    ncols = [(L + 1) * (L + 2) // 2 for L in
             (numpy.asarray(f["lxlylz"])[numpy.concatenate(([0], numpy.cumsum(f["ncart"])))[:-1]].sum(1))]
    off = numpy.concatenate(([0], numpy.cumsum(f["nprim"])))
    amin = numpy.array([f["prim"][off[s]:off[s + 1], 0].min() for s in range(len(ncols))])

    def box(ax, n):
        return numpy.array([(ax[i], ax[min(i + n - 1, len(ax) - 1)]) for i in range(0, len(ax), n)])

    bx, by, bz = box(gx, 4), box(gy, 4), box(gz, 8)
    dist = lambda b, a: numpy.maximum(0.0, numpy.maximum(b[:, 0] - a, a - b[:, 1]))
    kept = numpy.zeros((len(bx) * len(by) * len(bz), len(ncols)), dtype=bool)
    for s in range(len(ncols)):
        a = geo[f["atoms"][s]]
        d2 = (dist(bx, a[0])[:, None, None] ** 2 + dist(by, a[1])[None, :, None] ** 2 +
              dist(bz, a[2])[None, None, :] ** 2).ravel()
        kept[:, s] = amin[s] * 1.4426950408889634 * d2 <= 64.0

    def ksteps(order):
        col, nchunk = _mixed_layout(order, ncols)
        M = numpy.zeros((len(ncols), 2 * nchunk), dtype=numpy.int32)
        for s, (c, p) in col.items():
            for k in range(p, p + ncols[s]):
                M[s, 2 * c + k // 16] = 1
        return ((kept.astype(numpy.int32) @ M) > 0).sum(1).mean()

    before = ksteps(list(range(len(ncols))))
    after = ksteps(basis.mixed_order(geo, f).tolist())
    assert abs(before - 8.13) < 0.02 and abs(after - 4.08) < 0.02, (before, after)


def _overlap_plan(lib, lxlylz, ncart, nprim=None, atoms=None, natom=1):
    ip = lambda a: (ctypes.c_int * len(a))(*a)
    nshell = len(ncart)
    nprim = nprim or [1] * nshell
    atoms = atoms or [0] * nshell
    flat = [v for row in lxlylz for v in row]
    prim = (ctypes.c_double * (2 * sum(nprim)))(*([1.0, 1.0] * sum(nprim)))
    h = ctypes.c_void_p()
    lib.okg_overlap_plan_create.restype = ctypes.c_int
    return lib.okg_overlap_plan_create(natom, nshell, ip(atoms), ip(ncart), ip(nprim), ip(flat), 0, prim, None, 0,
                                       None, None, None, ctypes.byref(h))


def test_overlap_and_ci_validation_errors(lib):
    """AO overlap plan and the detCI quadratic forms: bad arguments are rejected before
    any device work."""
    lib.okg_last_error.restype = ctypes.c_char_p
    assert _overlap_plan(lib, [(0, 0, 0)], [1], atoms=[2], natom=2) == -1
    assert _overlap_plan(lib, [(-1, 0, 0)], [1]) == -2
    assert _overlap_plan(lib, [(40, 0, 0)], [1]) == -2
    assert b"too large" in lib.okg_last_error()
    assert _overlap_plan(lib, [(0, 0, 0)], [0]) == -1
    lib.okg_ao_overlap.restype = ctypes.c_int
    assert lib.okg_ao_overlap(None, None, None, 0, 0, None, ctypes.c_int64(1), None) == -1
    lib.okg_overlap_plan_set_ket.restype = ctypes.c_int
    assert lib.okg_overlap_plan_set_ket(None, None) == -1
    lib.okg_ci_rho_matrix.restype = ctypes.c_int
    assert lib.okg_ci_rho_matrix(ctypes.c_int64(10), None, ctypes.c_int64(10), 4, None, None, None) == -1
    lib.okg_ci_flux_matrix.restype = ctypes.c_int
    assert lib.okg_ci_flux_matrix(ctypes.c_int64(10), None, None, ctypes.c_int64(10), 4, None, ctypes.c_double(1.0),
                                  None, None) == -1
    lib.okg_ci_rho.restype = ctypes.c_int
    assert lib.okg_ci_rho(ctypes.c_int64(-1), None, ctypes.c_int64(0), 0, None, None, 0, None, None, None, None) == -1


def test_validate_drv_and_tables():
    from orbkit_gb300 import tools
    assert [tools.validate_drv(d) for d in [None, "x", "y", "z", "xx", "yy", "zz", "xy", "xz", "yz"]] == list(range(10))
    assert tools.validate_drv("x2") == 4 and tools.validate_drv("zy") == 9 and tools.validate_drv(7) == 7
    for bad in ("q", 10, -1, "xyz"):
        with pytest.raises(ValueError):
            tools.validate_drv(bad)
    for l in range(5):
        assert len(tools.cartesian_order[l]) == (l + 1) * (l + 2) // 2
        for m in range(-l, l + 1):
            comps, coef, fac = tools.get_cart2sph(l, m)
            assert all(sum(c) == l for c in comps) and len(comps) == len(coef)


def test_grid_module_matches_orbkit_ordering():
    from orbkit_gb300 import grid
    x, y, z = numpy.linspace(-1, 1, 4), numpy.linspace(0, 2, 3), numpy.linspace(-3, -1, 5)
    numpy.testing.assert_array_equal(grid.regular_to_vector(x, y, z), okref.grid2vector(x, y, z))
    grid.set_grid(x, y, z, is_vector=False)
    grid.grid2vector()
    assert grid.is_vector and len(grid.x) == 60
    grid.vector2grid(4, 3, 5)
    numpy.testing.assert_array_equal(grid.x, x)
    numpy.testing.assert_array_equal(grid.z, z)
    grid.reset_grid()


def test_spherical_transform_matches_oracle():
    """The transform T folded into C_eff reproduces orbkit's cartesian2spherical."""
    from orbkit_gb300.basis import spherical_csr
    qc, d = load_golden("sph_fg_N.npz")
    ptr, idx, coef = spherical_csr(qc.ao_spec)
    ncart = len(qc.ao_spec.get_lxlylz())
    T = numpy.zeros((len(ptr) - 1, ncart))
    for r in range(len(ptr) - 1):
        for t in range(ptr[r], ptr[r + 1]):
            T[r, idx[t]] += coef[t]
    A = numpy.random.default_rng(0).standard_normal((ncart, 17))
    numpy.testing.assert_allclose(T @ A, okref.cartesian2spherical(A, qc.ao_spec), rtol=1e-14, atol=1e-14)


def test_synthetic_mos_orthonormal():
    from orbkit_gb300 import overlap, synthetic
    for d in (synthetic.small(), synthetic.grad(npts=8)):
        qc = d["qc"]
        C = qc.mo_spec.get_coeffs()
        S = overlap.ao_overlap(qc.geo_spec, qc.ao_spec)
        numpy.testing.assert_allclose(C @ S @ C.T, numpy.eye(len(C)), atol=1e-10)


def test_point_range_partition():
    from orbkit_gb300.shard import point_range
    for n in (0, 1, 7, 4096000):
        for w in (1, 2, 3, 8):
            ranges = [point_range(n, r, w) for r in range(w)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(ranges, ranges[1:]))
            assert max(e - s for s, e in ranges) - min(e - s for s, e in ranges) <= 1


def _shard_worker(rank, world, port, out):
    import torch.distributed as dist
    import okref as ok
    from orbkit_gb300.shard import gather_blocks, point_range
    from helpers import load_golden as lg
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    qc, d = lg("small_cart.npz")
    pts = ok.grid2vector(d["x"], d["y"], d["z"])
    s, e = point_range(pts.shape[1], rank, world)
    r, dr = ok.rho_threads(qc, *pts[:, s:e], drv=["x", "y", "z"], slice_length=16, nthreads=1)
    full = gather_blocks(numpy.concatenate([r[None], dr]))
    if rank == 0:
        numpy.save(out, full)
    dist.destroy_process_group()


def test_sharded_points_two_gloo_ranks(tmp_path):
    """Two ranks evaluate disjoint point blocks; the host-side concatenation equals
    the single-rank result (no data-path collective)."""
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = str(tmp_path / "full.npy")
    mp.start_processes(_shard_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    full = numpy.load(out)
    qc, d = load_golden("small_cart.npz")
    numpy.testing.assert_array_equal(full[0], d["rho"].reshape(-1))
    numpy.testing.assert_array_equal(full[1:], d["delta_rho"][:3].reshape(3, -1))
