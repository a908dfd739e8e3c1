"""Site orders of the reference's packed arrays.

The reference takes the caller's site order through two callbacks at init
(``getLinearSiteIndex`` / ``getSiteCoords``, include/sse_dslash.h:13-17).  The
QDP++ orders it was written for, and which this library runs without any
permutation, are:

* cb2 (4D):  ``lin = p*V/2 + ((t*Lz+z)*Ly+y)*(Lx/2) + x/2``, p = (x+y+z+t)&1
  (lib/shift_tables_scalar.c:99-123);
* cb3d (3D): ``lin = p*V/2 + t + Lt*(x/2 + (Lx/2)*(y+Ly*z))``, p = (x+y+z)&1
  (lib/shift_tables_scalar_3d.c:97-141).

Everything here is vectorised numpy over coordinate arrays.
"""
from __future__ import annotations

import numpy as np


def volume(dims) -> int:
    return int(np.prod(np.asarray(dims, dtype=np.int64)))


def cb2_linear(dims, x, y, z, t):
    Lx, Ly, Lz, Lt = (int(v) for v in dims)
    p = (x + y + z + t) & 1
    return p * (volume(dims) // 2) + ((t * Lz + z) * Ly + y) * (Lx // 2) + x // 2


def cb3d_linear(dims, x, y, z, t):
    Lx, Ly, Lz, Lt = (int(v) for v in dims)
    p = (x + y + z) & 1
    return p * (volume(dims) // 2) + t + Lt * (x // 2 + (Lx // 2) * (y + Ly * z))


def internal_coords(dims, nd: int):
    """(x, y, z, t) of internal site i = 0..V-1 (cb2 order for nd=4, cb3d for nd=3)."""
    Lx, Ly, Lz, Lt = (int(v) for v in dims)
    V = volume(dims)
    Vh = V // 2
    i = np.arange(V, dtype=np.int64)
    p, r = i // Vh, i % Vh
    if nd == 4:
        xh = r % (Lx // 2); r = r // (Lx // 2)
        y = r % Ly; r = r // Ly
        z = r % Lz; t = r // Lz
        x = 2 * xh + ((p + y + z + t) & 1)
    else:
        t = r % Lt; r = r // Lt
        xh = r % (Lx // 2); r = r // (Lx // 2)
        y = r % Ly; z = r // Ly
        x = 2 * xh + ((p + y + z) & 1)
    return x, y, z, t


def site_table(dims, nd: int, linear_of_coords) -> np.ndarray:
    """Caller linear index of every internal site, from a vectorised
    ``linear_of_coords(x, y, z, t)``; the argument of
    ``DslashOperator.set_layout``."""
    x, y, z, t = internal_coords(dims, nd)
    return np.asarray(linear_of_coords(x, y, z, t), dtype=np.int32)
