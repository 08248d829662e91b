"""The benchmark's own workloads against the oracle.

* 512^3 with the seeded Jz pulse (the workload bench.py times): the FP64
  drop-in against the oracle's restatement of the reference driver loop
  (sources written into the dense J arrays before every update_fields,
  perf-tests/kokkos_sample/kokkos_sample.cpp:88-113), bit for bit on all six
  components after 20 steps.
* The batched workload (domains with edges uniform in 32..160, plane wave and
  one pulse each): the first 8 domains of the seeded 256 through the batch,
  against FP64 handles of the same domains after 500 steps, rel-L2 <= 1e-5
  per domain (the precision forms' accuracy bar).
* The contracted FP64 arithmetic (fdtd_set_fp64_arith): within 1e-12 of the
  oracle, max-abs error normalised by the field amplitude, after 1000 steps
  on the 64^3 plane wave and on the pulse workload at 128^3.
"""
import numpy as np
import pytest

from oracle import Oracle

from fdtd_method_gb300 import FDTD, FDTDBatch, Precision, build, sources
from fdtd_method_gb300.sources import COURANT_DT, baseline_pulse, normalised_parameters

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def test_fp64_512_cubed_pulse_bitwise_vs_oracle_driver_loop():
    p = normalised_parameters(512, 512, 512)
    src = baseline_pulse(p, seed=0, n_steps=1000)
    steps = 20
    # the pulse must be on during these steps for the check to cover the current
    assert np.abs(src.amp[:steps]).max() > 0
    s = FDTD(p, COURANT_DT)
    s.add_source(src)
    s.step(steps)
    got = [s.copy_to_host(c) for c in range(6)]
    s.close()
    o = Oracle(p, COURANT_DT)
    o.add_source(src)
    o.step_driver(steps)
    for c in range(6):
        assert np.array_equal(got[c], o.f[c]), "component %d differs (max %g)" % (
            c, np.abs(got[c] - o.f[c]).max())
    assert np.abs(o.f[2]).max() > 0


def _rel_l2(a, b):
    num = sum(float(np.dot(x - y, x - y)) for x, y in zip(a, b))
    den = sum(float(np.dot(y, y)) for y in b)
    return (num / den) ** 0.5


def test_batched_workload_domains_follow_fp64():
    wl = sources.batch_workload(count=256, seed=0, n_steps=500)[:8]
    steps = 500
    b = FDTDBatch([w[0] for w in wl], COURANT_DT, Precision.FP32_COMP)
    for q, (p, init, src) in enumerate(wl):
        for c, v in init.items():
            b.copy_from_host(q, int(c), v)
        b.add_source(q, src)
    b.step(50)
    b.step(steps - 50)
    b.synchronize()
    for q, (p, init, src) in enumerate(wl):
        ref = FDTD(p, COURANT_DT)
        for c, v in init.items():
            ref.copy_from_host(int(c), v)
        ref.add_source(src)
        ref.step(steps)
        want = [ref.copy_to_host(c) for c in range(6)]
        ref.close()
        got = [b.copy_to_host(q, c) for c in range(6)]
        rel = _rel_l2(got, want)
        assert rel <= 1e-5, "domain %d (%dx%dx%d): rel-L2 %.3e" % (q, p.Ni, p.Nj, p.Nk, rel)
    b.close()


def _max_norm_error(sim, ref):
    amp = max(float(np.abs(ref.f[c]).max()) for c in range(6))
    return max(float(np.abs(sim.copy_to_host(c) - ref.f[c]).max()) for c in range(6)) / amp


def test_contracted_fp64_plane_wave_64_cubed():
    p = normalised_parameters(64, 64, 64)
    s = FDTD(p, COURANT_DT)
    s.set_fp64_arith(True)
    o = Oracle(p, COURANT_DT)
    for c, v in sources.plane_wave_fields(p, 0).items():
        s.copy_from_host(int(c), v)
        o.set(c, v)
    s.step(1000)
    o.step(1000)
    err = _max_norm_error(s, o)
    assert err <= 1e-12, err
    s.close()


def test_contracted_fp64_pulse_128_cubed():
    p = normalised_parameters(128, 128, 128)
    src = baseline_pulse(p, seed=0, n_steps=1000)
    s = FDTD(p, COURANT_DT)
    s.set_fp64_arith(True)
    s.add_source(src)
    o = Oracle(p, COURANT_DT)
    o.add_source(src)
    s.step(1000)
    o.step(1000)
    err = _max_norm_error(s, o)
    assert err <= 1e-12, err
    # and it is a different evaluation: not the bitwise form's bits
    assert any(not np.array_equal(s.copy_to_host(c), o.f[c]) for c in range(6))
    s.close()


def test_contracted_fp64_switches_back_to_bitwise():
    p = normalised_parameters(24, 20, 16)
    rng = np.random.default_rng(3)
    vals = [rng.standard_normal(p.cells) for _ in range(6)]
    s = FDTD(p, COURANT_DT)
    o = Oracle(p, COURANT_DT)
    for c, v in enumerate(vals):
        s.copy_from_host(c, v)
        o.set(c, v)
    s.set_fp64_arith(True)
    s.set_fp64_arith(False)
    s.step(5)
    o.step(5)
    for c in range(6):
        np.testing.assert_array_equal(s.copy_to_host(c), o.f[c])
    s.close()
