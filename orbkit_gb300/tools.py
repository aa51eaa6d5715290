"""Tables and small helpers shared by the grid-evaluation path.

Everything here is data or argument handling that must agree exactly with
orbkit for the drop-in to return identical results:

* ``lquant``            shell letter -> angular momentum      (orbkit/tools.py:88-90)
* ``cartesian_order``   Molden ordering of Cartesian components (orbkit/tools.py:117-135)
* ``cart2sph``          Schlegel-Frisch real solid-harmonic combinations
                        (orbkit/tools.py:155-191, Int. J. Quantum Chem. 54, 83 (1995))
* ``validate_drv``      derivative selector -> code 0..9          (orbkit/tools.py:225-239)
* ``require``           C-contiguous float64 / intc arrays        (orbkit/tools.py:290-295)
"""
import string

import numpy

# Shell letters: s, p, d, then the alphabet from 'f' on without 's' and 'p'.
_letters = "spd" + "".join(c for c in string.ascii_lowercase[5:] if c not in "sp")
lquant = {c: i for i, c in enumerate(_letters)}

# Molden order of the Cartesian components (lx, ly, lz) per angular momentum.
cartesian_order = [
    [(0, 0, 0)],
    [(1, 0, 0), (0, 1, 0), (0, 0, 1)],
    [(2, 0, 0), (0, 2, 0), (0, 0, 2), (1, 1, 0), (1, 0, 1), (0, 1, 1)],
    [(3, 0, 0), (0, 3, 0), (0, 0, 3), (1, 2, 0), (2, 1, 0), (2, 0, 1),
     (1, 0, 2), (0, 1, 2), (0, 2, 1), (1, 1, 1)],
    [(4, 0, 0), (0, 4, 0), (0, 0, 4), (3, 1, 0), (3, 0, 1), (1, 3, 0),
     (0, 3, 1), (1, 0, 3), (0, 1, 3), (2, 2, 0), (2, 0, 2), (0, 2, 2),
     (2, 1, 1), (1, 2, 1), (1, 1, 2)],
]
exp = cartesian_order  # orbkit's name for the same table

MAX_L = 4  # highest angular momentum with a Cartesian order and a spherical table

_r = numpy.sqrt


def _cart2sph_table():
    """(l, m) -> (list of (lx,ly,lz), list of coefficients, global factor).

    The entries are the Schlegel-Frisch transformation as orbkit tabulates it.
    orbkit's g(m=-1) row lists (0,3,1) twice and never (0,1,3); the drop-in has to
    reproduce orbkit's numbers, so that row is kept exactly as orbkit evaluates it.
    """
    t = {}
    t[(0, 0)] = ([(0, 0, 0)], [1.0], 1.0)
    # p: m = -1 -> y, 0 -> z, +1 -> x
    t[(1, -1)] = ([(0, 1, 0)], [1.0], 1.0)
    t[(1, 0)] = ([(0, 0, 1)], [1.0], 1.0)
    t[(1, 1)] = ([(1, 0, 0)], [1.0], 1.0)
    # d
    t[(2, -2)] = ([(1, 1, 0)], [1.0], 1.0)
    t[(2, -1)] = ([(0, 1, 1)], [1.0], 1.0)
    t[(2, 0)] = ([(0, 0, 2), (2, 0, 0), (0, 2, 0)], [1.0, -0.5, -0.5], 1.0)
    t[(2, 1)] = ([(1, 0, 1)], [1.0], 1.0)
    t[(2, 2)] = ([(2, 0, 0), (0, 2, 0)], [1.0, -1.0], _r(3) / 2.0)
    # f
    t[(3, -3)] = ([(0, 3, 0), (2, 1, 0)], [-_r(5), 3.0], 1 / (2.0 * _r(2)))
    t[(3, -2)] = ([(1, 1, 1)], [1.0], 1.0)
    t[(3, -1)] = ([(0, 1, 2), (0, 3, 0), (2, 1, 0)],
                  [_r(3 / 5.0), -_r(3) / 4.0, -_r(3) / (4.0 * _r(5))], _r(2))
    t[(3, 0)] = ([(0, 0, 3), (2, 0, 1), (0, 2, 1)],
                 [1.0, -3 / (2 * _r(5)), -3 / (2 * _r(5))], 1.0)
    t[(3, 1)] = ([(1, 0, 2), (3, 0, 0), (1, 2, 0)],
                 [_r(3 / 5.0), -_r(3) / 4.0, -_r(3) / (4.0 * _r(5))], _r(2))
    t[(3, 2)] = ([(2, 0, 1), (0, 2, 1)], [1.0, -1.0], _r(3) / 2.0)
    t[(3, 3)] = ([(3, 0, 0), (1, 2, 0)], [_r(5), -3.0], 1 / (2.0 * _r(2)))
    # g
    t[(4, -4)] = ([(3, 1, 0), (1, 3, 0)], [1.0, -1.0], _r(2) * _r(5 / 8.0))
    t[(4, -3)] = ([(0, 3, 1), (2, 1, 1)], [-_r(5) / 4.0, 3 / 4.0], _r(2))
    t[(4, -2)] = ([(1, 1, 2), (3, 1, 0), (1, 3, 0)],
                  [3 / _r(14), -_r(5) / (2 * _r(14)), -_r(5) / (2 * _r(14))], _r(2))
    t[(4, -1)] = ([(0, 3, 1), (0, 3, 1), (2, 1, 1)],
                  [_r(5 / 7.0), -3 * _r(5) / (4.0 * _r(7)), -3 / (4.0 * _r(7))], _r(2))
    t[(4, 0)] = ([(0, 0, 4), (4, 0, 0), (0, 4, 0), (2, 0, 2), (0, 2, 2), (2, 2, 0)],
                 [1.0, 3 / 8.0, 3 / 8.0, -3 * _r(3) / _r(35), -3 * _r(3) / _r(35), -1 / 4.0], _r(2))
    t[(4, 1)] = ([(1, 0, 3), (3, 0, 1), (1, 2, 1)],
                 [_r(5 / 7.0), -3 * _r(5) / (4.0 * _r(7)), -3 / (4.0 * _r(7))], _r(2))
    t[(4, 2)] = ([(2, 0, 2), (0, 2, 2), (4, 0, 0), (0, 4, 0)],
                 [3 * _r(3) / (2.0 * _r(14)), -3 * _r(3) / (2.0 * _r(14)),
                  -_r(5) / (4.0 * _r(2)), _r(5) / (4.0 * _r(2))], _r(2))
    t[(4, 3)] = ([(3, 0, 1), (1, 2, 1)], [_r(5) / 4.0, -3 / 4.0], _r(2))
    t[(4, 4)] = ([(4, 0, 0), (0, 4, 0), (2, 2, 0)],
                 [_r(35) / (8.0 * _r(2)), _r(35) / (8.0 * _r(2)), -3 * _r(3) / (4.0 * _r(2))], _r(2))
    return t


cart2sph = _cart2sph_table()


def get_cart2sph(l, m):
    """Components, coefficients and global factor of the real solid harmonic (l, m)."""
    return cart2sph[(int(l), int(m))]


_DRV_CODES = {
    "x": 1, "y": 2, "z": 3,
    "xx": 4, "x2": 4, "yy": 5, "y2": 5, "zz": 6, "z2": 6,
    "xy": 7, "yx": 7, "xz": 8, "zx": 8, "yz": 9, "zy": 9,
}
DRV_NAMES = [None, "x", "y", "z", "xx", "yy", "zz", "xy", "xz", "yz"]


def validate_drv(drv):
    """Map a derivative selector (None, 'x', ..., 'yz', or 0..9) to its code 0..9."""
    if drv is None or (isinstance(drv, str) and drv in ("None", "")):
        return 0
    if isinstance(drv, str):
        if drv in _DRV_CODES:
            return _DRV_CODES[drv]
        raise ValueError("The selection `drv=%s` is not valid!" % drv)
    if isinstance(drv, (int, numpy.integer)) and not isinstance(drv, bool) and 0 <= int(drv) <= 9:
        return int(drv)
    raise ValueError("The selection `drv=%s` is not valid!" % drv)


def require(data, dtype="f"):
    """C-contiguous, aligned copy/view as float64 ('f') or C int ('i')."""
    if dtype == "f":
        dtype = numpy.float64
    elif dtype == "i":
        dtype = numpy.intc
    return numpy.require(data, dtype=dtype, requirements="CA")


def doublefactorial(n):
    """n!! with (n <= 0) -> 1."""
    r = 1
    while n > 0:
        r *= n
        n -= 2
    return r
