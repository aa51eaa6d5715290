"""Module-global grid state with orbkit.grid's interface (orbkit/grid.py:31-243, 553-677).

A regular grid is three coordinate vectors ``x, y, z`` (``is_vector == False``);
flattened it becomes a vector grid with x running slowest and z fastest
(orbkit/cy_grid.pyx:14-30).  The GPU kernels never materialise the flattened
coordinates of a regular grid: they take the three short vectors and derive a
point's coordinates from its index, which gives the same float64 values as
the flattened arrays.

orbkit.grid can be used instead of this module: ``orbkit_gb300.core`` reads
whichever module ``core.grid`` points at (see ``orbkit_gb300.install``).
"""
import sys

import numpy

min_ = [-8.0, -8.0, -8.0]
max_ = [8.0, 8.0, 8.0]
N_ = [101, 101, 101]
x = numpy.array([0.0])
y = numpy.array([0.0])
z = numpy.array([0.0])
delta_ = numpy.zeros(3)
d3r = 0.0
is_initialized = False
is_vector = True
is_regular = False

_mod = sys.modules[__name__]


def grid_init(is_vector=False, force=False):
    """Build the regular grid from ``min_``, ``max_`` and ``delta_`` (or ``N_``)."""
    global x, y, z, d3r, delta_, N_, is_initialized, is_regular
    if is_initialized and not force:
        return 0
    delta_ = numpy.array(delta_, dtype=numpy.float64).reshape(-1)[:3] if numpy.size(delta_) >= 3 else numpy.zeros(3)
    g = [None, None, None]
    for i in range(3):
        if max_[i] == min_[i]:
            g[i] = numpy.array([min_[i]], dtype=numpy.float64)
            delta_[i] = 1
            N_[i] = 1
        elif delta_[i]:
            g[i] = numpy.arange(min_[i], max_[i] + delta_[i], delta_[i], dtype=numpy.float64)
            N_[i] = len(g[i])
        else:
            g[i] = numpy.array(numpy.linspace(min_[i], max_[i], N_[i]), dtype=numpy.float64)
            delta_[i] = g[i][1] - g[i][0]
    x, y, z = g
    d3r = float(numpy.prod(delta_))
    is_initialized = True
    is_regular = True
    if is_vector:
        grid2vector()
    else:
        setattr(_mod, "is_vector", False)


init = grid_init


def set_grid(xnew, ynew, znew, is_vector=None):
    """Set the coordinate vectors directly."""
    global x, y, z, is_initialized, is_regular, min_, max_, N_, delta_
    out = []
    for c in (xnew, ynew, znew):
        c = numpy.array(c, dtype=numpy.float64).reshape(-1) if not numpy.isscalar(c) else numpy.array([c], dtype=numpy.float64)
        out.append(c)
    x, y, z = out
    is_initialized = True
    if isinstance(is_vector, bool):
        setattr(_mod, "is_vector", is_vector)
    is_regular = is_vector is False
    min_ = [x.min(), y.min(), z.min()]
    max_ = [x.max(), y.max(), z.max()]
    N_ = [len(x), len(y), len(z)]
    if is_regular:
        f = lambda v: 1.0 if len(v) <= 1 else v[1] - v[0]
        delta_ = numpy.array([f(x), f(y), f(z)])


def regular_to_vector(xv, yv, zv):
    """(3, Nx*Ny*Nz) coordinates, x slowest and z fastest (cy_grid.pyx:14-30)."""
    xv, yv, zv = (numpy.asarray(v, dtype=numpy.float64) for v in (xv, yv, zv))
    out = numpy.empty((3, len(xv) * len(yv) * len(zv)), dtype=numpy.float64)
    out[0] = numpy.repeat(xv, len(yv) * len(zv))
    out[1] = numpy.tile(numpy.repeat(yv, len(zv)), len(xv))
    out[2] = numpy.tile(zv, len(xv) * len(yv))
    return out


def grid2vector():
    global x, y, z, is_regular
    if not is_initialized:
        raise ValueError("You have to initialize a grid before calling `grid.grid2vector`.")
    x, y, z = regular_to_vector(x, y, z)
    setattr(_mod, "is_vector", True)
    is_regular = True


def vector2grid(Nx, Ny, Nz):
    global x, y, z
    if not is_initialized:
        raise ValueError("You have to initialize a grid before calling `grid.vector2grid`.")
    if not (len(x) == len(y) == len(z)) or Nx * Ny * Nz != len(x):
        raise ValueError("It has to hold that `len(x) = (N_x * N_y * N_z)`")
    x, y, z = x[::Ny * Nz].copy(), y[:Ny * Nz:Nz].copy(), z[:Nz].copy()
    setattr(_mod, "is_vector", False)


def adjust_to_geo(qc, extend=5.0, step=0.1):
    """Grid boundaries around the molecule with spacing ``step`` (grid.py:553-581)."""
    global min_, max_, N_, delta_, is_initialized
    geo = numpy.asarray(qc.geo_spec if not isinstance(qc, dict) else qc["geo_spec"], dtype=numpy.float64)
    min_, max_, N_ = list(min_), list(max_), list(N_)
    delta_ = numpy.zeros(3)
    for i in range(3):
        min_[i] = min(geo[:, i]) - extend
        max_[i] = max(geo[:, i]) + extend
        dist = max_[i] - min_[i]
        N_[i] = int(numpy.ceil(dist / step)) + 1
        rest = (N_[i] - 1) * step - dist
        min_[i] -= rest / 2.0
        max_[i] += rest / 2.0
        delta_[i] = step
    setattr(_mod, "is_vector", False)
    is_initialized = False


def reset_grid():
    global is_initialized, is_regular, min_, max_, N_, delta_
    is_initialized = False
    setattr(_mod, "is_vector", True)
    is_regular = False
    min_ = [-8.0, -8.0, -8.0]
    max_ = [8.0, 8.0, 8.0]
    N_ = [101, 101, 101]
    delta_ = numpy.zeros(3)


def get_shape():
    if not is_initialized:
        raise ValueError("`grid.get_shape` requires the grid to be initialized.")
    return (len(x),) if is_vector else (len(x), len(y), len(z))


def tolist():
    return [numpy.copy(x), numpy.copy(y), numpy.copy(z)]


def todict():
    return {"x": x, "y": y, "z": z}


def get_grid(start="\t"):
    s = ""
    for c, v in zip("xyz", (x, y, z)):
        s += "%s%s[0] = %.2f %s[-1] = %.2f N%s = %d\n" % (start, c, v[0], c, v[-1], c, len(v))
    return s
