"""Restatement of the reference's test harness, written against any solver
that offers set(comp, values) / run(steps) / get(comp).

  Test_FDTD::initial_filling     src/FDTD_kokkos/test_FDTD_kokkos.cpp:7-66
  Test_FDTD::set_sign/set_axis   src/FDTD_kokkos/test_FDTD_kokkos.cpp:68-102
  Test_FDTD::get_shift           src/FDTD_kokkos/test_FDTD_kokkos.cpp:103-111
  Test_FDTD::get_max_abs_error   src/FDTD_kokkos/test_FDTD_kokkos.cpp:113-161
  run_test_kokkos + 12 TESTs     unit-tests/test_FDTD_method_kokkos.cpp:7-201

Floating-point expressions keep the reference's association so that a solver
that is bit-identical to the reference reproduces its error ratios exactly.
"""
import math

import numpy as np

from fdtd_method_gb300.fdtd import Component as Cp, Const, Parameters

DEFAULT_TIME = 5e-13  # unit-tests/test_FDTD_method_kokkos.cpp:7

# (test name, test field, (selected E, selected B), grid) — the 12 Kokkos tests
CONVERGENCE_CASES = [
    ("x_axis_EY", Cp.EY, (Cp.EY, Cp.BZ), (16, 8, 4)),
    ("x_axis_BZ", Cp.BZ, (Cp.EY, Cp.BZ), (16, 8, 4)),
    ("x_axis_EZ", Cp.EZ, (Cp.EZ, Cp.BY), (16, 8, 4)),
    ("x_axis_BY", Cp.BY, (Cp.EZ, Cp.BY), (16, 8, 4)),
    ("y_axis_EX", Cp.EX, (Cp.EX, Cp.BZ), (8, 16, 4)),
    ("y_axis_BZ", Cp.BZ, (Cp.EX, Cp.BZ), (8, 16, 4)),
    ("y_axis_EZ", Cp.EZ, (Cp.EZ, Cp.BX), (8, 16, 4)),
    ("y_axis_BX", Cp.BX, (Cp.EZ, Cp.BX), (8, 16, 4)),
    ("z_axis_EX", Cp.EX, (Cp.EX, Cp.BY), (4, 8, 16)),
    ("z_axis_BY", Cp.BY, (Cp.EX, Cp.BY), (4, 8, 16)),
    ("z_axis_EY", Cp.EY, (Cp.EY, Cp.BX), (4, 8, 16)),
    ("z_axis_BX", Cp.BX, (Cp.EY, Cp.BX), (4, 8, 16)),
]


def initial_func(x, size):
    return math.sin(2.0 * Const.PI * (x - size[0]) / (size[1] - size[0]))


def true_func(x, t, size):
    return math.sin(2.0 * Const.PI * (x - size[0] - Const.C * t) / (size[1] - size[0]))


def select_sign(e, b):
    if (e, b) in ((Cp.EX, Cp.BZ), (Cp.EZ, Cp.BY), (Cp.EY, Cp.BX)):
        return -1.0
    if (e, b) in ((Cp.EY, Cp.BZ), (Cp.EZ, Cp.BX), (Cp.EX, Cp.BY)):
        return 1.0
    raise RuntimeError("ERROR: invalid selected fields")


def select_axis(e, b):
    if (e, b) in ((Cp.EY, Cp.BZ), (Cp.EZ, Cp.BY)):
        return 0
    if (e, b) in ((Cp.EX, Cp.BZ), (Cp.EZ, Cp.BX)):
        return 1
    if (e, b) in ((Cp.EX, Cp.BY), (Cp.EY, Cp.BX)):
        return 2
    raise RuntimeError("ERROR: invalid selected fields")


def unit_test_params(Ni, Nj, Nk):
    """Parameters of run_test_kokkos (unit-tests/test_FDTD_method_kokkos.cpp:21-29)."""
    return Parameters(Ni, Nj, Nk, 0.0, 1.0, 0.0, 2.0, 0.0, 3.0,
                      (1 - 0) / float(Ni), (2 - 0) / float(Nj), (3 - 0) / float(Nk))


def initial_filling(p, sel):
    """Returns {comp: flat array} for the selected (E, B) pair."""
    e, b = sel
    axis = select_axis(e, b)
    sign = select_sign(e, b)
    n = (p.Ni, p.Nj, p.Nk)[axis]
    d = (p.dx, p.dy, p.dz)[axis]
    size = ((p.ax, p.bx), (p.ay, p.by), (p.az, p.bz))[axis]
    d_b = d / 2.0
    ev = np.empty(n)
    bv = np.empty(n)
    for q in range(n):
        u = float(q) * d
        ev[q] = sign * initial_func(u, size)
        bv[q] = initial_func(d_b + u, size)
    shape = [1, 1, 1]
    shape[2 - axis] = n
    full = (p.Nk, p.Nj, p.Ni)
    return {e: np.broadcast_to(ev.reshape(shape), full).reshape(-1).copy(),
            b: np.broadcast_to(bv.reshape(shape), full).reshape(-1).copy()}


def max_abs_error(p, sel, field_values, comp, time):
    e, b = sel
    axis = select_axis(e, b)
    sign = select_sign(e, b)
    d = (p.dx, p.dy, p.dz)[axis]
    size = ((p.ax, p.bx), (p.ay, p.by), (p.az, p.bz))[axis]
    n = (p.Ni, p.Nj, p.Nk)[axis]
    u = 0.0
    if int(comp) > int(Cp.EZ):
        sign = 1.0
        u = d / 2.0
    stride = (1, p.Ni, p.Ni * p.Nj)[axis]
    worst = 0.0
    for q in range(n):
        err = abs(sign * field_values[q * stride] - true_func(u, time, size))
        if err > worst:
            worst = err
        u += d
    return worst


def run_convergence(make_solver, test_field, sel, Ni, Nj, Nk):
    """run_test_kokkos: error ratio between (N, dt) and (2N, dt/2).
    make_solver(params, dt) -> object with set(comp, v), run(steps), get(comp)."""
    errs = []
    for scale in (1, 2):
        p = unit_test_params(Ni * scale, Nj * scale, Nk * scale)
        iters = 16 * scale
        dt = DEFAULT_TIME / float(iters)
        s = make_solver(p, dt)
        for comp, v in initial_filling(p, sel).items():
            s.set(comp, v)
        s.run(iters)
        errs.append(max_abs_error(p, sel, s.get(test_field), test_field, DEFAULT_TIME))
    return errs[0] / errs[1], errs
