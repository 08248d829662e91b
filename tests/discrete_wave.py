"""Exact solution of the Yee scheme for one periodic plane-wave mode (test
helper).

One update_fields step (B/2, E, B/2; src/FDTD_kokkos/FDTD_kokkos.cpp:91-104)
maps the amplitudes (E, B) of the mode exp(i k x) (B on its staggered points
x + d/2) by the matrix
    [[1 + a^2/2, -a], [-a (1 + a^2/4), 1 + a^2/2]],  a = 2 i s sin(k d/2),
s = c dt / d.  Its eigenvalues are exp(+-i w dt) with
    sin(w dt / 2) = s sin(k d / 2)          (the Yee dispersion relation)
and its eigenvectors have B = +-cos(w dt / 2) E.  Initial data E = sin(k x),
B = sin(k (x + d/2)) is therefore the sum of a forward wave of amplitude
(1 + 1/cos(w dt/2)) / 2 and a backward wave of amplitude (1 - 1/cos(w dt/2)) / 2.
The exact wave numbers use math.pi, so that the mode is periodic on the grid.
"""
import math

import numpy as np

# (E component, B component) of a wave along x, y, z whose continuous
# solution moves in the +axis direction with B = E.
PAIRS = {0: (1, 5), 1: (2, 3), 2: (0, 4)}


def initial(params, axis, mode=1):
    """Flat E and B arrays of the mode along `axis` (cells i + j Ni + k Ni Nj)."""
    n = (params.Ni, params.Nj, params.Nk)[axis]
    u = np.arange(n, dtype=np.float64)
    k = 2.0 * math.pi * mode / n
    shape = (params.Nk, params.Nj, params.Ni)
    bshape = [1, 1, 1]
    bshape[2 - axis] = n
    e = np.broadcast_to(np.sin(k * u).reshape(bshape), shape).reshape(-1).copy()
    b = np.broadcast_to(np.sin(k * (u + 0.5)).reshape(bshape), shape).reshape(-1).copy()
    return e, b


def exact(params, axis, s, steps, mode=1):
    """E and B along the axis (one line of cells) after `steps` steps."""
    n = (params.Ni, params.Nj, params.Nk)[axis]
    u = np.arange(n, dtype=np.float64)
    k = 2.0 * math.pi * mode / n
    w = 2.0 * math.asin(s * math.sin(k / 2.0))
    c = math.cos(w / 2.0)
    fwd, bwd = (1.0 + 1.0 / c) / 2.0, (1.0 - 1.0 / c) / 2.0
    e = fwd * np.sin(k * u - w * steps) + bwd * np.sin(k * u + w * steps)
    b = c * (fwd * np.sin(k * (u + 0.5) - w * steps) - bwd * np.sin(k * (u + 0.5) + w * steps))
    return e, b


def line(flat, params, axis):
    """The cells (0, 0, 0) .. along `axis` of a flat field."""
    a = flat.reshape(params.Nk, params.Nj, params.Ni)
    return a[0, 0, :] if axis == 0 else a[0, :, 0] if axis == 1 else a[:, 0, 0]
