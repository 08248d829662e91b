"""Field-slice files for the reference's plotting script
(python_script_legend/visualization.py:10-45).

The script reads OutFiles_<n>/<iteration>.csv for component n = 1..6
(Ex, Ey, Ez, Bx, By, Bz), ';'-separated, with a decimal comma and a header
row (pandas.read_csv's default), and shows each file as a 2-D image.
``write_slice_csv`` writes one such file: the plane of constant z (or x, y)
of one component, rows along the second in-plane axis.
"""
import os

import numpy as np

from .fdtd import Component

COMPONENT_NUMBER = {Component.EX: 1, Component.EY: 2, Component.EZ: 3,
                    Component.BX: 4, Component.BY: 5, Component.BZ: 6}


def field_plane(values, params, axis=2, index=None):
    """The plane of a flat field (index i + j*Ni + k*Ni*Nj) at `index` along
    `axis` (default: the middle plane) as a 2-D array: (j, i) for z, (k, i)
    for y, (k, j) for x."""
    cube = np.asarray(values).reshape(params.Nk, params.Nj, params.Ni)
    n = (params.Ni, params.Nj, params.Nk)[axis]
    idx = n // 2 if index is None else int(index)
    if not 0 <= idx < n:
        raise ValueError("plane index %d outside 0..%d" % (idx, n - 1))
    if axis == 2:
        return cube[idx, :, :]
    if axis == 1:
        return cube[:, idx, :]
    return cube[:, :, idx]


def write_slice_csv(sim, comp, iteration, root=".", axis=2, index=None, digits=8):
    """Writes root/OutFiles_<n>/<iteration>.csv for E/B component `comp` of
    solver `sim` (any precision form; values copied to the host).  Returns
    the path."""
    comp = Component(comp)
    if comp not in COMPONENT_NUMBER:
        raise ValueError("only E and B components are plotted")
    plane = field_plane(sim.get_field(comp).numpy(), sim.parameters, axis, index)
    folder = os.path.join(root, "OutFiles_%d" % COMPONENT_NUMBER[comp])
    os.makedirs(folder, exist_ok=True)
    path = os.path.join(folder, "%d.csv" % int(iteration))
    fmt = "%%.%de" % digits
    with open(path, "w") as f:
        f.write(";".join(str(c) for c in range(plane.shape[1])) + "\n")
        for row in plane:
            f.write(";".join((fmt % v).replace(".", ",") for v in row) + "\n")
    return path
