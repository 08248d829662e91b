"""Pins the oracle (CPU restatement, oracle/fdtd_oracle.c) to the reference:
against the golden numbers recorded from the reference's own build, and, where
that build is present (oracle/_ref), against the reference directly."""
import json
import os

import numpy as np
import pytest

from golden_inputs import CASES, PML_CASES, TWIN_CASES, case_inputs, case_params
from oracle import Oracle, OraclePML, RefKokkos, coefficients, field_sums, ref_available
from refcases import CONVERGENCE_CASES, run_convergence

from fdtd_method_gb300 import sources
from fdtd_method_gb300.fdtd import Component, CurrentParameters, Parameters

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


class OracleSolver:
    def __init__(self, p, dt):
        self.o = Oracle(p, dt)

    def set(self, comp, v):
        self.o.set(comp, v)

    def run(self, n):
        self.o.step(n)

    def get(self, comp):
        return self.o.get(comp)


def test_coefficients_follow_reference():
    # src/FDTD_kokkos/FDTD_kokkos.cpp:45-55
    p = Parameters(4, 5, 6, 0, 1, 0, 2, 0, 3, 0.25, 0.4, 0.5)
    dt = 1e-12
    c = coefficients(p, dt)
    cdt = 3e10 * dt
    assert list(c) == [cdt / 0.25, cdt / 0.4, cdt / 0.5, cdt / (2.0 * 0.25), cdt / (2.0 * 0.4),
                       cdt / (2.0 * 0.5), -4.0 * 3.14159265358 * dt]


@pytest.mark.parametrize("bad", [(0, 4, 4, 1.0), (4, -1, 4, 1.0), (4, 4, 0, 1.0), (4, 4, 4, 0.0),
                                 (4, 4, 4, -1e-12)])
def test_invalid_parameters_rejected(bad):
    Ni, Nj, Nk, dt = bad
    with pytest.raises(ValueError, match="invalid parameters"):
        coefficients(Parameters(Ni, Nj, Nk, 0, 1, 0, 1, 0, 1, 0.1, 0.1, 0.1), dt)


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference_golden_cases(name):
    """Bit-identical to FDTD_kokkos::FDTD on the recorded cases."""
    golden = np.load(os.path.join(GOLDEN, "reference_cases.npz"))
    spec = CASES[name]
    p, dt = case_params(spec)
    o = Oracle(p, dt)
    for c, v in case_inputs(spec).items():
        o.set(c, v)
    o.step(spec["steps"])
    for c in range(9):
        np.testing.assert_array_equal(o.get(c), golden["%s/%d" % (name, c)], err_msg="component %d" % c)


@pytest.mark.parametrize("name", sorted(TWIN_CASES))
def test_twin_restatement_matches_reference_twin_runs(name):
    """oracle_twin_run (the timed second CPU path) is the reference's OpenMP
    twin (src/FDTD/FDTD.cpp) bit for bit, its Jx line included."""
    golden = np.load(os.path.join(GOLDEN, "reference_twin_cases.npz"))
    spec = TWIN_CASES[name]
    p, dt = case_params(spec)
    o = Oracle(p, dt)
    for c, v in case_inputs(spec).items():
        o.set(c, v)
    o.step_twin(spec["steps"])
    for c in range(9):
        np.testing.assert_array_equal(o.get(c), golden["%s/%d" % (name, c)], err_msg="component %d" % c)


@pytest.mark.parametrize("shape", [(12, 10, 7), (1, 1, 1), (5, 1, 3), (16, 8, 4)])
def test_twin_equals_the_kokkos_path_without_current(shape):
    """At J = 0 the twin and the Kokkos path give the same bits (the twin's
    only arithmetic difference is its current line)."""
    Ni, Nj, Nk = shape
    p = Parameters(Ni, Nj, Nk, 0, 1, 0, 2, 0, 3, 1.0 / Ni, 2.0 / Nj, 3.0 / Nk)
    dt = 0.3 * min(p.dx, p.dy, p.dz) / 3e10
    rng = np.random.default_rng(Ni * 100 + Nj * 10 + Nk)
    a, b = Oracle(p, dt), Oracle(p, dt)
    for c in range(6):
        v = rng.standard_normal(p.cells)
        a.set(c, v)
        b.set(c, v)
    a.step(5)
    b.step_twin(5)
    for c in range(6):
        np.testing.assert_array_equal(a.get(c), b.get(c))


@pytest.mark.skipif(not ref_available(), reason="reference build (oracle/_ref) not present on this host")
def test_twin_restatement_bitwise_equal_to_reference_twin_build():
    p = Parameters(11, 6, 9, 0, 1, 0, 2, 0, 3, 1.0 / 11, 2.0 / 6, 3.0 / 9)
    dt = 0.3 * min(p.dx, p.dy, p.dz) / 3e10
    rng = np.random.default_rng(5)
    o, r = Oracle(p, dt), RefKokkos(p, dt, kind="openmp")
    for c in range(9):
        v = rng.standard_normal(p.cells)
        o.set(c, v)
        r.set(c, v)
    o.step_twin(6)
    r.update_fields(6)
    for c in range(9):
        np.testing.assert_array_equal(o.get(c), r.get(c))


@pytest.mark.parametrize("name,field,sel,grid", CONVERGENCE_CASES)
def test_oracle_convergence_matches_reference_unit_tests(name, field, sel, grid):
    """The reference's own convergence tests (unit-tests/test_FDTD_method_kokkos.cpp):
    the oracle reproduces the ratio the reference measured, and it is 4 +- 0.1."""
    golden = json.load(open(os.path.join(GOLDEN, "reference_unit_tests.json")))
    ref = golden["Convergence_kokkos." + name]
    ratio, errs = run_convergence(OracleSolver, field, sel, *grid)
    assert abs(ratio - 4.0) <= 0.1
    assert ratio == pytest.approx(ref["value"], rel=1e-12, abs=0)


def _sample_oracle(n, it):
    """The reference sample (perf-tests/kokkos_sample/kokkos_sample.cpp) run on
    the oracle: dx = C, dt = 0.2, box current for period/dt steps."""
    d = 3e10
    b = n / 2.0 * d
    p = Parameters(n, n, n, -b, b, -b, b, -b, b, d, d, d)
    cur = CurrentParameters(8, 4, 0.2)
    src, cur_time = sources.sample_box_source(p, cur, it)
    o = Oracle(p, cur.dt)
    o.add_source(src)
    o.step(it)
    return p, o


def _slice_rows(p, ex):
    # kokkos_sample.cpp:141-149: i = Nk/2, j and k over +-5 around the centre
    i = p.Nk // 2
    rows = []
    for j in range(p.Nj // 2 - 5, p.Nj // 2 + 5):
        rows.append("".join("%12.5f" % ex[i + j * p.Ni + k * p.Ni * p.Nj]
                            for k in range(p.Ni // 2 - 5, p.Ni // 2 + 5)))
    return rows


@pytest.mark.parametrize("key", ["16_60", "32_100", "20_30"])
def test_oracle_sample_matches_reference_program_output(key):
    """The Ex slice the reference's kokkos_sample prints (5 decimals)."""
    golden = json.load(open(os.path.join(GOLDEN, "reference_sample.json")))
    n, it = map(int, key.split("_"))
    p, o = _sample_oracle(n, it)
    rows = _slice_rows(p, o.get(Component.EX))
    assert [r.strip().split() for r in rows] == [r.strip().split() for r in golden[key]]


def test_field_sums_compensated():
    rng = np.random.default_rng(3)
    f = [rng.standard_normal(1000) for _ in range(6)]
    s = field_sums(f)
    for c in range(6):
        assert s[c] == pytest.approx(float(np.sum(f[c] * f[c])), rel=1e-13)
    assert s[6] == pytest.approx(float(np.sum(f[1] * f[5] - f[2] * f[4])), rel=1e-10, abs=1e-10)
    assert s[9] == 0
    f[2][5] = np.nan
    assert field_sums(f)[9] == 1


@pytest.mark.skipif(not ref_available(), reason="reference build (oracle/_ref) not present on this host")
@pytest.mark.parametrize("shape", [(12, 10, 7), (1, 1, 1), (5, 1, 3), (3, 8, 2)])
def test_oracle_bitwise_equal_to_reference_build(shape):
    Ni, Nj, Nk = shape
    p = Parameters(Ni, Nj, Nk, 0, 1, 0, 2, 0, 3, 1.0 / Ni, 2.0 / Nj, 3.0 / Nk)
    dt = 0.25 * min(p.dx, p.dy, p.dz) / 3e10
    rng = np.random.default_rng(sum(shape))
    o = Oracle(p, dt)
    r = RefKokkos(p, dt)
    for c in range(9):
        v = rng.standard_normal(Ni * Nj * Nk)
        o.set(c, v)
        r.set(c, v)
    o.step(6)
    r.update_fields(6)
    for c in range(9):
        np.testing.assert_array_equal(o.get(c), r.get(c))


@pytest.mark.skipif(not ref_available(), reason="reference build (oracle/_ref) not present on this host")
def test_reference_rejects_what_oracle_rejects():
    p = Parameters(0, 4, 4, 0, 1, 0, 1, 0, 1, 0.1, 0.1, 0.1)
    with pytest.raises(ValueError, match="ERROR: invalid parameters"):
        RefKokkos(p, 1e-12)
    r = RefKokkos(Parameters(2, 2, 2, 0, 1, 0, 1, 0, 1, 0.5, 0.5, 0.5), 1e-12)
    with pytest.raises(RuntimeError, match="Invalid field component"):
        r.get(9)


PML_GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_pml_cases.npz")


@pytest.mark.parametrize("name", sorted(PML_CASES))
def test_oracle_pml_matches_reference_golden_cases(name):
    """The PML restatement against the reference's own FDTD_PML
    (src/FDTD_kokkos/FDTD_PML_kokkos.cpp) on recorded runs, bit for bit."""
    spec = PML_CASES[name]
    params, dt = case_params(spec)
    o = OraclePML(params, dt, spec["pml"])
    for comp, values in case_inputs(spec).items():
        o.set(comp, values)
    o.step(spec["steps"])
    golden = np.load(PML_GOLDEN)
    for comp in range(6):
        np.testing.assert_array_equal(o.get(comp), golden["%s/%d" % (name, comp)], err_msg="component %d" % comp)


def test_oracle_pml_layer_profile():
    """Layer thickness (int)(N * pml_percent) per axis; conductivity zero in
    the main box, largest at the outer faces, symmetric (FDTD_PML_kokkos.cpp:71-136)."""
    p = Parameters(20, 16, 12, 0.0, 1.0, 0.0, 2.0, 0.0, 3.0, 0.05, 0.125, 0.25)
    o = OraclePML(p, 1e-13, 0.2)
    assert o.pml == [4, 3, 2]
    sx = o.sigma[0]
    assert np.all(sx[4:16] == 0.0) and np.all(sx[:4] > 0.0) and np.all(sx[16:] > 0.0)
    np.testing.assert_array_equal(sx[:4], sx[16:][::-1])
    assert np.all(np.diff(sx[:4]) < 0)
    o0 = OraclePML(p, 1e-13, 0.0)
    assert o0.pml == [0, 0, 0] and not any(s.any() for s in o0.sigma)


@pytest.mark.skipif(not ref_available(), reason="reference build (oracle/_ref) not present on this host")
@pytest.mark.parametrize("shape,pct", [((18, 14, 10), 0.2), ((9, 9, 9), 0.34), ((16, 1, 6), 0.25)])
def test_oracle_pml_bitwise_equal_to_reference_build(shape, pct):
    Ni, Nj, Nk = shape
    p = Parameters(Ni, Nj, Nk, 0.0, 1.0, 0.0, 2.0, 0.0, 3.0, 1.0 / Ni, 2.0 / Nj, 3.0 / Nk)
    dt = 0.3 * min(p.dx, p.dy, p.dz) / 3e10
    rng = np.random.default_rng(Ni + 31 * Nj)
    o = OraclePML(p, dt, pct)
    r = RefKokkos(p, dt, pml_percent=pct)
    for c in range(9):
        v = rng.standard_normal(p.Ni * p.Nj * p.Nk)
        o.set(c, v)
        r.set(c, v)
    o.step(5)
    r.update_fields(5)
    for c in range(6):
        np.testing.assert_array_equal(o.get(c), r.get(c))
    r.close()


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_oracle_follows_the_exact_discrete_plane_wave(axis):
    """The Yee scheme's exact solution for one periodic mode (its discrete
    dispersion relation and eigenvectors, tests/discrete_wave.py): the
    oracle follows it to FP64 rounding over 1000 steps along every axis."""
    import discrete_wave as dw
    from fdtd_method_gb300.sources import COURANT_DT, normalised_parameters
    shape = [4, 4, 4]
    shape[axis] = 64
    p = normalised_parameters(*shape)
    e0, b0 = dw.initial(p, axis)
    ce, cb = dw.PAIRS[axis]
    o = Oracle(p, COURANT_DT)
    o.set(ce, e0)
    o.set(cb, b0)
    o.step(1000)
    e, b = dw.exact(p, axis, COURANT_DT, 1000)
    assert np.abs(dw.line(o.get(ce), p, axis) - e).max() < 1e-13
    assert np.abs(dw.line(o.get(cb), p, axis) - b).max() < 1e-13
