"""One fused sweep per update_fields() call in the FP32-arithmetic forms.

The B-first sweep applies the B half steps that meet between two steps (the
previous step's trailing half, left pending, and this step's leading half)
and then E.  So the reference callers' pattern, update_fields() once per
step with reads in between (perf-tests/kokkos_sample/kokkos_sample.cpp:88-113,
unit-tests/test_FDTD_method_kokkos.cpp:36-38), must give the bits of
step(n), launch one kernel per call, and every reader must see B at the step
boundary.  Also here: the bounded device waits giving up (a test hook issues
no tile loads) and the handle staying usable afterwards.
"""
import numpy as np
import pytest

from oracle import Oracle

from fdtd_method_gb300 import FDTD, FDTDError, Precision, build, sources
from fdtd_method_gb300.sources import COURANT_DT, normalised_parameters

pytestmark = pytest.mark.gpu

FORMS = [Precision.FP32, Precision.FP32_COMP, Precision.FP16_SCALED]


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _make(p, prec, vals, srcs, pipeline="auto", cpt=0, dense_j=None):
    s = FDTD(p, COURANT_DT, prec)
    if prec == Precision.FP16_SCALED:
        s.set_fp16_exponents([4, 3, 5, 2, 4, 6])
    s.set_pipeline(pipeline, 0, 0, cpt)
    for c, v in enumerate(vals):
        s.copy_from_host(c, v)
    if dense_j is not None:
        for q, v in enumerate(dense_j):
            s.copy_from_host(6 + q, v)
    for q in srcs:
        s.add_source(q)
    return s


def _fields(s):
    return [s.copy_to_host(c) for c in range(6)]


def _setup(shape, seed):
    p = normalised_parameters(*shape)
    rng = np.random.default_rng(seed)
    vals = [rng.standard_normal(p.cells) * 0.5 for _ in range(6)]
    c = (shape[0] // 2, shape[1] // 3, shape[2] // 2)
    srcs = [sources.gaussian_pulse(p, c, 2.0, 1.0, 20.0, 3.0, 4.0, 40, comp="z"),
            sources.gaussian_pulse(p, (1, 2, 3), 1.5, 0.8, 25.0, 2.0, 3.0, 40, phase=0.5, comp="x")]
    return p, vals, srcs


@pytest.mark.parametrize("cpt", [1, 2])
@pytest.mark.parametrize("prec", FORMS)
def test_update_fields_with_reads_equals_step_n(prec, cpt):
    p, vals, srcs = _setup((45, 30, 26), 11)
    a = _make(p, prec, vals, srcs, cpt=cpt)
    a.step(9)
    want = _fields(a)
    e_want = a.field_sums()
    b = _make(p, prec, vals, srcs, cpt=cpt)
    for q in range(9):
        b.update_fields()
        if q % 3 == 1:  # reads between calls change nothing
            b.copy_to_host(q % 6)
            b.energy()
    got = _fields(b)
    for c in range(6):
        np.testing.assert_array_equal(got[c], want[c], err_msg="component %d" % c)
    np.testing.assert_array_equal(b.field_sums(), e_want)
    a.close()
    b.close()


@pytest.mark.parametrize("prec", FORMS)
def test_one_launch_per_update_fields_call(prec):
    p, vals, srcs = _setup((64, 40, 33), 3)
    s = _make(p, prec, vals, srcs)
    s.update_fields()
    s.synchronize()
    s.kernel_times()
    s.set_kernel_timing(True)
    for _ in range(12):
        s.update_fields()
    kt = s.kernel_times()
    assert kt["fused_step"][1] == 12
    assert kt["b_half"][1] == 0 and kt["b_double"][1] == 0 and kt["e_update"][1] == 0
    s.close()


@pytest.mark.parametrize("prec", FORMS)
def test_writes_and_pipeline_changes_apply_the_pending_half(prec):
    """Writing a field or switching to the split pipeline after B-first steps:
    the same bits as the split pipeline, which applies every half step in its
    own sweep."""
    p, vals, srcs = _setup((40, 22, 19), 7)
    rng = np.random.default_rng(8)
    new_ey = rng.standard_normal(p.cells) * 0.3
    runs = []
    for first in ("auto", "split"):
        s = _make(p, prec, vals, srcs, pipeline=first)
        s.step(4)
        s.copy_from_host(1, new_ey)  # E write: the pending half reads the old E
        s.step(3)
        s.set_pipeline("split")
        s.step(2)
        s.set_pipeline("auto")
        s.step(3)
        runs.append(_fields(s))
        s.close()
    for c in range(6):
        np.testing.assert_array_equal(runs[0][c], runs[1][c], err_msg="component %d" % c)


def test_fp16_exponent_change_applies_the_pending_half():
    p, vals, srcs = _setup((36, 20, 17), 9)
    runs = []
    for pipeline in ("auto", "split"):
        s = _make(p, Precision.FP16_SCALED, vals, srcs, pipeline=pipeline)
        s.step(5)
        s.set_fp16_exponents([5, 5, 5, 3, 3, 3])
        s.step(4)
        runs.append(_fields(s))
        s.close()
    for c in range(6):
        np.testing.assert_array_equal(runs[0][c], runs[1][c])


def test_dense_current_written_between_calls():
    """J is written between update_fields calls (the sample driver's pattern):
    the pending half does not read J, so the bits equal the split pipeline's."""
    p, vals, srcs = _setup((33, 18, 21), 5)
    runs = []
    for pipeline in ("auto", "split"):
        s = _make(p, Precision.FP32_COMP, vals, [], pipeline=pipeline)
        for q in range(5):
            s.copy_from_host(8, np.full(p.cells, 0.01 * (q + 1)))
            s.update_fields()
        runs.append(_fields(s))
        s.close()
    for c in range(6):
        np.testing.assert_array_equal(runs[0][c], runs[1][c])


@pytest.mark.parametrize("cpt", [1, 2])
def test_wait_that_gives_up_is_reported_and_the_context_stays_usable(cpt):
    """With the test hook no tile load is issued, so every bounded wait of the
    fused sweep runs out (after a few polls) with no copy in flight; the sweep
    stops, fdtd_synchronize reports FDTD_ERR_TIMEOUT, and both a new handle
    and the same handle (wait limit back to the default, fields set again)
    compute the oracle's results."""
    p = normalised_parameters(48, 30, 20)
    rng = np.random.default_rng(4)
    vals = [rng.standard_normal(p.cells) for _ in range(6)]
    s = FDTD(p, COURANT_DT, Precision.FP32_COMP)
    s.set_pipeline("fused", 0, 0, cpt)
    for c, v in enumerate(vals):
        s.copy_from_host(c, v)
    s.set_wait_limit(polls=8, withhold_loads=True)
    s.step(2)
    with pytest.raises(FDTDError, match="gave up"):
        s.synchronize()
    s.synchronize()  # the status was cleared
    o = Oracle(p, COURANT_DT)
    for c, v in enumerate(vals):
        o.set(c, v)
    o.step(3)
    want = [o.get(c) for c in range(6)]

    def rel(a):
        num = sum(float(((x - y) ** 2).sum()) for x, y in zip(a, want))
        return (num / sum(float((y * y).sum()) for y in want)) ** 0.5

    s.set_wait_limit(0, False)
    s.step_index = 0
    for c, v in enumerate(vals):
        s.copy_from_host(c, v)
    s.step(3)
    s.synchronize()
    assert rel(_fields(s)) <= 1e-6
    t = FDTD(p, COURANT_DT, Precision.FP32_COMP)
    for c, v in enumerate(vals):
        t.copy_from_host(c, v)
    t.step(3)
    t.synchronize()
    np.testing.assert_array_equal(np.concatenate(_fields(t)), np.concatenate(_fields(s)))
    s.close()
    t.close()


@pytest.mark.parametrize("tile_y", [6, 14, 30])
@pytest.mark.parametrize("prec", FORMS)
def test_tile_and_column_b_half_sweeps_agree(prec, tile_y):
    """The B half sweeps run on the fused sweep's tiles once a handle has its
    second copy (here: after a read with a half step pending), and as column
    sweeps before that; both give the bits of the other (split pipeline,
    several z chunks per column, sources and a pending half on every read)."""
    p, vals, srcs = _setup((70, 45, 53), 21)
    runs = []
    for read_early in (False, True):
        s = _make(p, prec, vals, srcs, pipeline="split", cpt=1)
        s.set_pipeline("split", tile_y, 16, 1)
        s.step(2)
        if read_early:
            s.copy_to_host(4)  # allocates the second copy: tile sweeps from here on
        s.step(5)
        s.update_fields()
        runs.append(_fields(s))
        s.close()
    for c in range(6):
        np.testing.assert_array_equal(runs[0][c], runs[1][c], err_msg="component %d" % c)
