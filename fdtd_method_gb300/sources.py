"""Builders of separable current sources and seeded synthetic workloads.

A source is J_c(i,j,k,s) += amp[s] * gx[di] * gy[dj] * gz[dk] over a periodic
box (see ``fdtd_source`` in include/fdtd_gb300.h).  Two families:

* ``sample_box_source`` — the reference sample's box current
  sin(2 pi t/T) cos^2(2 pi x/Tx) cos^2(2 pi y/Ty) cos^2(2 pi z/Tz), set in
  Jx, Jy and Jz for the first period/dt steps, t = (step+1) dt
  (perf-tests/kokkos_sample/kokkos_sample.cpp:16-129).
* ``gaussian_pulse`` — A sin(2 pi t/T + phi) exp(-((t-t0)/tau)^2) times a
  Gaussian spatial envelope exp(-r^2 / (2 sigma^2)), t in steps, evaluated at
  t = step + 1 like the sample.

Normalised units: dx = dy = dz = C and dt = 0.5/sqrt(3), so C dt/dx =
0.5/sqrt(3) and the reference's coefficients are those of c = 1, dx = 1 (the
mapping perf-tests/kokkos_sample/kokkos_sample.cpp:38-53 uses).
"""
import math

import numpy as np

from .fdtd import Const, CurrentParameters, Parameters, SeparableSource

COURANT_DT = 0.5 / math.sqrt(3.0)


def normalised_parameters(Ni, Nj, Nk):
    """Periodic grid with dx = dy = dz = C, centred on the origin."""
    d = Const.C
    return Parameters(Ni, Nj, Nk, -Ni / 2.0 * d, Ni / 2.0 * d, -Nj / 2.0 * d, Nj / 2.0 * d,
                      -Nk / 2.0 * d, Nk / 2.0 * d, d, d, d)


class SplitMix64:
    """splitmix64 (Steele, Lea, Flood 2014): a tiny, portable seeded generator."""

    MASK = (1 << 64) - 1

    def __init__(self, seed):
        self.state = int(seed) & self.MASK

    def next_u64(self):
        self.state = (self.state + 0x9E3779B97F4A7C15) & self.MASK
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & self.MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & self.MASK
        return z ^ (z >> 31)

    def uniform(self, lo=0.0, hi=1.0):
        return lo + (hi - lo) * ((self.next_u64() >> 11) * (1.0 / (1 << 53)))

    def integer(self, lo, hi):
        """Uniform integer in [lo, hi]."""
        return lo + self.next_u64() % (hi - lo + 1)


def sample_box_source(params, cur_param=None, iterations=None):
    """The reference sample's SetCurrent box (kokkos_sample.cpp:17-28, 58-108).

    Returns (source, cur_time): cur_time = min(period/dt, iterations) steps
    carry current, as in the sample's first loop; the source is silent after."""
    if cur_param is None:
        cur_param = CurrentParameters(8, 4, 0.2)
    cur_param.iterations = int(float(cur_param.period) / cur_param.dt)
    T = float(cur_param.period)
    Tx, Ty, Tz = cur_param.period_x, cur_param.period_y, cur_param.period_z
    p = params
    cur_time = cur_param.iterations if iterations is None else min(cur_param.iterations, iterations)
    start = [int(math.floor((-Tx / 4.0 - p.ax) / p.dx)), int(math.floor((-Ty / 4.0 - p.ay) / p.dy)),
             int(math.floor((-Tz / 4.0 - p.az) / p.dz))]
    stop = [int(math.floor((Tx / 4.0 - p.ax) / p.dx)), int(math.floor((Ty / 4.0 - p.ay) / p.dy)),
            int(math.floor((Tz / 4.0 - p.az) / p.dz))]
    two_pi = 2.0 * Const.PI

    def prof(lo, hi, d, period):
        return np.array([math.pow(math.cos(two_pi * (v * d) / period), 2.0) for v in range(lo, hi)])

    gx = prof(start[0], stop[0], p.dx, Tx)
    gy = prof(start[1], stop[1], p.dy, Ty)
    gz = prof(start[2], stop[2], p.dz, Tz)
    dt = cur_param.dt
    amp = np.array([math.sin(two_pi * ((t + 1) * dt) / T) for t in range(cur_time)])
    src = SeparableSource(7, start[0], start[1], start[2], gx, gy, gz, amp,
                          meta={"kind": "sample_box", "cur_time": cur_time})
    return src, cur_time


def _axis_profile(n, center, sigma, half_width):
    """Gaussian exp(-d^2/(2 sigma^2)) over a periodic window around `center`,
    d the minimum-image distance.  Returns (origin, table)."""
    if 2 * half_width + 1 >= n:
        origin, length = 0, n
    else:
        origin, length = (center - half_width) % n, 2 * half_width + 1
    idx = (origin + np.arange(length)) % n
    d = (idx - center + n / 2.0) % n - n / 2.0
    return origin, np.exp(-(d * d) / (2.0 * sigma * sigma))


def gaussian_pulse(params, center, sigma, A, T, t0, tau, n_steps, phase=0.0, comp="z",
                   cutoff_sigmas=9.0):
    """Gaussian-pulse current at cell `center` = (i, j, k)."""
    hw = int(math.ceil(cutoff_sigmas * sigma))
    i0, gx = _axis_profile(params.Ni, center[0], sigma, hw)
    j0, gy = _axis_profile(params.Nj, center[1], sigma, hw)
    k0, gz = _axis_profile(params.Nk, center[2], sigma, hw)
    n_amp = int(min(n_steps, math.floor(t0 + cutoff_sigmas * tau) + 1))
    s = np.arange(n_amp, dtype=np.float64) + 1.0
    amp = A * np.sin(2.0 * Const.PI * s / T + phase) * np.exp(-(((s - t0) / tau) ** 2))
    mask = {"x": 1, "y": 2, "z": 4}[comp]
    return SeparableSource(mask, i0, j0, k0, gx, gy, gz, amp,
                           meta={"kind": "gaussian_pulse", "center": tuple(center), "sigma": sigma,
                                 "A": A, "T": T, "t0": t0, "tau": tau, "phase": phase, "comp": comp})


def plane_wave_fields(params, axis=0, mode=1):
    """Initial E_y (x axis), E_z (y axis) or E_x (z axis) = sin(2 pi m u / L) on
    the E points and the matching B = sin(2 pi m (u + d/2) / L) on the
    staggered B points (the reference test's convention,
    src/FDTD_kokkos/test_FDTD_kokkos.cpp:7-66, with sign +1 pairs
    (Ey,Bz), (Ez,Bx), (Ex,By)).  Returns {component: flat array}."""
    from .fdtd import Component
    n = (params.Ni, params.Nj, params.Nk)[axis]
    u = np.arange(n, dtype=np.float64)
    e = np.sin(2.0 * Const.PI * mode * u / n)
    b = np.sin(2.0 * Const.PI * mode * (u + 0.5) / n)
    shape = (params.Nk, params.Nj, params.Ni)
    bshape = [1, 1, 1]
    bshape[2 - axis] = n
    E = np.broadcast_to(e.reshape(bshape), shape).reshape(-1).copy()
    B = np.broadcast_to(b.reshape(bshape), shape).reshape(-1).copy()
    pair = {0: (Component.EY, Component.BZ), 1: (Component.EZ, Component.BX), 2: (Component.EX, Component.BY)}[axis]
    return {pair[0]: E, pair[1]: B}


def baseline_pulse(params, seed=0, n_steps=1000, sigma=8.0):
    """One Jz Gaussian pulse at the grid centre with A ~ U[0.5, 2],
    T ~ U[20, 60] steps, tau = T, t0 = 3 tau (drawn from `seed`)."""
    rng = SplitMix64(seed)
    A = rng.uniform(0.5, 2.0)
    T = rng.uniform(20.0, 60.0)
    tau = T
    center = (params.Ni // 2, params.Nj // 2, params.Nk // 2)
    return gaussian_pulse(params, center, sigma, A, T, 3.0 * tau, tau, n_steps, comp="z")


def random_pulses(params, count, seed=0, n_steps=1000, sigma=8.0, comps=("z", "x")):
    """`count` pulses at uniform random cells with random phases; component
    drawn from `comps`."""
    rng = SplitMix64(seed)
    out = []
    for _ in range(count):
        A = rng.uniform(0.5, 2.0)
        T = rng.uniform(20.0, 60.0)
        phase = rng.uniform(0.0, 2.0 * math.pi)
        c = (rng.integer(0, params.Ni - 1), rng.integer(0, params.Nj - 1), rng.integer(0, params.Nk - 1))
        comp = comps[rng.integer(0, len(comps) - 1)]
        out.append(gaussian_pulse(params, c, sigma, A, T, 3.0 * T, T, n_steps, phase=phase, comp=comp))
    return out


def batch_workload(count=256, seed=0, n_steps=500, lo=32, hi=160, sigma=4.0):
    """The batched-form workload: `count` periodic domains with per-axis edge
    lengths uniform in [lo, hi]; each starts from a plane wave along a random
    axis with mode number 1..4 and carries one Gaussian-pulse source
    (A ~ U[0.5, 2], T ~ U[20, 60] steps, tau = T, t0 = 3 tau, random cell,
    random phase, Jz or Jx).  Returns a list of (params, {component: initial
    field}, source)."""
    rng = SplitMix64(seed)
    out = []
    for _ in range(count):
        p = normalised_parameters(rng.integer(lo, hi), rng.integer(lo, hi), rng.integer(lo, hi))
        axis = rng.integer(0, 2)
        mode = rng.integer(1, 4)
        init = plane_wave_fields(p, axis=axis, mode=mode)
        A = rng.uniform(0.5, 2.0)
        T = rng.uniform(20.0, 60.0)
        phase = rng.uniform(0.0, 2.0 * math.pi)
        c = (rng.integer(0, p.Ni - 1), rng.integer(0, p.Nj - 1), rng.integer(0, p.Nk - 1))
        comp = ("z", "x")[rng.integer(0, 1)]
        src = gaussian_pulse(p, c, sigma, A, T, 3.0 * T, T, n_steps, phase=phase, comp=comp)
        src.meta.update({"axis": axis, "mode": mode})
        out.append((p, init, src))
    return out
