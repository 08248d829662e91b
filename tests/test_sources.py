"""The seeded synthetic workloads, on the host.

The benchmark's inputs are built here, so their shapes and distributions are
what the measured numbers stand on: the generator (splitmix64, pinned to its
published first outputs for seed 0), the 512^3 Jz pulse (A ~ U[0.5, 2],
T ~ U[20, 60] steps, tau = T, t0 = 3 tau, sigma = 8 cells at the centre,
sampled at t = step + 1 like the reference sample,
perf-tests/kokkos_sample/kokkos_sample.cpp:89), the random pulses, the
batched workload (edges uniform in 32..160, plane wave along a random axis
with mode 1..4, one pulse) and the plane-wave initial fields.
"""
import math

import numpy as np
import pytest

from fdtd_method_gb300 import Const
from fdtd_method_gb300.sources import (SplitMix64, _axis_profile, baseline_pulse, batch_workload, gaussian_pulse,
                                       normalised_parameters, plane_wave_fields, random_pulses)


def test_splitmix64_published_outputs():
    r = SplitMix64(0)
    assert [r.next_u64() for _ in range(5)] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F,
                                                0xF88BB8A8724C81EC, 0x1B39896A51A8749B]
    u = SplitMix64(3)
    vals = [u.uniform(2.0, 5.0) for _ in range(1000)]
    assert min(vals) >= 2.0 and max(vals) < 5.0
    ints = [SplitMix64(s).integer(32, 160) for s in range(500)]
    assert min(ints) >= 32 and max(ints) <= 160


def test_axis_profile_is_periodic_gaussian():
    origin, g = _axis_profile(50, 1, 2.0, 6)
    assert origin == 45 and len(g) == 13
    idx = (origin + np.arange(13)) % 50
    d = np.array([((i - 1 + 25) % 50) - 25 for i in idx], dtype=float)
    np.testing.assert_allclose(g, np.exp(-d * d / 8.0), rtol=0, atol=0)
    assert g[6] == 1.0  # the centre cell
    origin, g = _axis_profile(10, 3, 2.0, 6)  # window wider than the axis: the whole axis
    assert origin == 0 and len(g) == 10 and g[3] == 1.0


@pytest.mark.parametrize("seed", [0, 1, 7])
def test_baseline_pulse(seed):
    p = normalised_parameters(512, 512, 512)
    src = baseline_pulse(p, seed=seed, n_steps=1000)
    m = src.meta
    A, T, t0, tau = m["A"], m["T"], m["t0"], m["tau"]
    assert 0.5 <= A <= 2.0 and 20.0 <= T <= 60.0 and tau == T and t0 == 3.0 * tau
    assert src.comp_mask == 4 and m["center"] == (256, 256, 256) and m["sigma"] == 8.0
    hw = int(math.ceil(9.0 * 8.0))
    for o, g in ((src.i0, src.gx), (src.j0, src.gy), (src.k0, src.gz)):
        assert o == 256 - hw and len(g) == 2 * hw + 1 and g[hw] == 1.0
        np.testing.assert_array_equal(g, g[::-1])
    s = np.arange(len(src.amp)) + 1.0  # sampled at t = step + 1
    want = A * np.sin(2.0 * Const.PI * s / T) * np.exp(-(((s - t0) / tau) ** 2))
    np.testing.assert_array_equal(src.amp, want)
    assert len(src.amp) == min(1000, math.floor(t0 + 9.0 * tau) + 1)
    again = baseline_pulse(p, seed=seed, n_steps=1000)
    np.testing.assert_array_equal(again.amp, src.amp)


def test_different_seeds_differ():
    p = normalised_parameters(64, 64, 64)
    a, b = baseline_pulse(p, seed=0), baseline_pulse(p, seed=1)
    assert (a.meta["A"], a.meta["T"]) != (b.meta["A"], b.meta["T"])


def test_random_pulses():
    p = normalised_parameters(100, 60, 40)
    srcs = random_pulses(p, 16, seed=5, n_steps=200, sigma=3.0)
    assert len(srcs) == 16
    for s in srcs:
        ci, cj, ck = s.meta["center"]
        assert 0 <= ci < 100 and 0 <= cj < 60 and 0 <= ck < 40
        assert s.comp_mask in (1, 4)
        assert 0.5 <= s.meta["A"] <= 2.0 and 20.0 <= s.meta["T"] <= 60.0
    again = random_pulses(p, 16, seed=5, n_steps=200, sigma=3.0)
    assert [s.meta["center"] for s in srcs] == [s.meta["center"] for s in again]


def test_batch_workload():
    wl = batch_workload(count=64, seed=0, n_steps=500)
    assert len(wl) == 64
    edges = [e for p, _, _ in wl for e in (p.Ni, p.Nj, p.Nk)]
    assert min(edges) >= 32 and max(edges) <= 160 and len(set(edges)) > 20
    for p, init, src in wl:
        axis, mode = src.meta["axis"], src.meta["mode"]
        assert axis in (0, 1, 2) and 1 <= mode <= 4
        assert src.comp_mask in (1, 4)
        assert len(init) == 2
        for v in init.values():
            assert v.shape == (p.cells,)


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_plane_wave_fields(axis):
    p = normalised_parameters(16, 12, 10)
    f = plane_wave_fields(p, axis=axis, mode=2)
    n = (p.Ni, p.Nj, p.Nk)[axis]
    u = np.arange(n)
    e_want = np.sin(2.0 * Const.PI * 2 * u / n)
    b_want = np.sin(2.0 * Const.PI * 2 * (u + 0.5) / n)
    (ec, ev), (bc, bv) = sorted(f.items(), key=lambda kv: int(kv[0]))
    assert int(ec) < 3 <= int(bc)
    e3 = ev.reshape(p.Nk, p.Nj, p.Ni)
    b3 = bv.reshape(p.Nk, p.Nj, p.Ni)
    line = [slice(0, 1)] * 3
    line[2 - axis] = slice(None)
    np.testing.assert_allclose(e3[tuple(line)].ravel(), e_want, rtol=0, atol=1e-15)
    np.testing.assert_allclose(b3[tuple(line)].ravel(), b_want, rtol=0, atol=1e-15)


def test_gaussian_pulse_cutoff_and_phase():
    p = normalised_parameters(40, 40, 40)
    s = gaussian_pulse(p, (0, 39, 20), 1.5, 1.0, 30.0, 6.0, 2.0, 500, phase=0.7, comp="x")
    assert s.comp_mask == 1
    assert len(s.amp) == math.floor(6.0 + 9.0 * 2.0) + 1  # silent after t0 + 9 tau
    st = np.arange(len(s.amp)) + 1.0
    np.testing.assert_array_equal(s.amp, np.sin(2.0 * Const.PI * st / 30.0 + 0.7) * np.exp(-(((st - 6.0) / 2.0) ** 2)))
