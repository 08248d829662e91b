"""Temporal blocking: the depth-2 sweep (two steps per pass over the state)
against one-step sweeps.  Each of its four stages evaluates the split sweeps'
arithmetic on the stored values of the stage before, so a run at depth 2 must
give the bits of the same run at depth 1, whatever the grid shape (tiles
narrower or shorter than 32 x tile_y, grids thinner than the two-cell halo),
chunk length, sources, dense current or half step left pending."""
import numpy as np
import pytest

from fdtd_method_gb300 import FDTD, InvalidArgument, Precision, build, sources
from fdtd_method_gb300.sources import COURANT_DT, normalised_parameters

pytestmark = pytest.mark.gpu

FORMS = [Precision.FP32, Precision.FP32_COMP, Precision.FP16_SCALED]


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _run(p, prec, vals, srcs, calls, depth, tile_y=0, kchunk=0, dense_j=None):
    s = FDTD(p, COURANT_DT, prec)
    if prec == Precision.FP16_SCALED:
        s.set_fp16_exponents([4, 3, 5, 2, 4, 6])
    s.set_pipeline("fused", tile_y, kchunk, 1)
    s.set_temporal_depth(depth)
    for c, v in enumerate(vals):
        s.copy_from_host(c, v)
    if dense_j is not None:
        for q, v in enumerate(dense_j):
            s.copy_from_host(6 + q, v)
    for q in srcs:
        s.add_source(q)
    for n in calls:
        s.step(n)
    out = [s.copy_to_host(c) for c in range(6)]
    s.close()
    return out


def _case(shape, seed):
    p = normalised_parameters(*shape)
    rng = np.random.default_rng(seed)
    vals = [rng.standard_normal(p.cells) * 0.5 for _ in range(6)]
    c = (shape[0] // 2, shape[1] // 2, shape[2] // 2)
    srcs = [sources.gaussian_pulse(p, c, 2.0, 1.0, 20.0, 3.0, 4.0, 20, comp="z"),
            sources.gaussian_pulse(p, (0, 0, 0), 1.5, 0.8, 25.0, 2.0, 3.0, 20, phase=0.5, comp="x")]
    return p, vals, srcs


@pytest.mark.parametrize("prec", FORMS)
@pytest.mark.parametrize("shape,tile_y,kchunk", [((37, 19, 23), 14, 24), ((1, 1, 1), 14, 24), ((64, 28, 16), 14, 8),
                                                 ((31, 15, 129), 6, 48), ((2, 70, 3), 6, 2), ((33, 9, 40), 14, 7),
                                                 ((96, 42, 5), 6, 3), ((32, 20, 11), 14, 24), ((40, 17, 9), 6, 96),
                                                 ((128, 30, 12), 14, 96), ((3, 2, 2), 6, 1)])
def test_depth2_equals_depth1(prec, shape, tile_y, kchunk):
    p, vals, srcs = _case(shape, sum(shape))
    a = _run(p, prec, vals, srcs, [7], 1, tile_y, kchunk)
    b = _run(p, prec, vals, srcs, [7], 2, tile_y, kchunk)
    for c in range(6):
        np.testing.assert_array_equal(a[c], b[c], err_msg="component %d" % c)


@pytest.mark.parametrize("prec", [Precision.FP32, Precision.FP32_COMP])
def test_depth2_many_sources_dense_current_and_pending_halves(prec):
    """More sources than the kernel keeps in registers (the generic path),
    a dense current, and calls that start with a B half step pending."""
    p = normalised_parameters(40, 24, 20)
    rng = np.random.default_rng(2)
    vals = [rng.standard_normal(p.cells) * 0.1 for _ in range(6)]
    dj = [rng.standard_normal(p.cells) * 0.01 for _ in range(3)]
    srcs = sources.random_pulses(p, 6, seed=4, n_steps=30, sigma=2.0)
    a = _run(p, prec, vals, srcs, [1, 4, 3, 2], 1, dense_j=dj)
    b = _run(p, prec, vals, srcs, [1, 4, 3, 2], 2, dense_j=dj)
    for c in range(6):
        np.testing.assert_array_equal(a[c], b[c])


def test_depth2_launches_and_rejected_shapes():
    p, vals, srcs = _case((64, 40, 33), 5)
    s = FDTD(p, COURANT_DT, Precision.FP32)
    s.set_temporal_depth(2)
    s.add_source(srcs[0])
    s.step(1)
    s.synchronize()
    s.kernel_times()
    s.set_kernel_timing(True)
    s.step(9)
    kt = s.kernel_times()
    assert kt["fused_step2"][1] == 4 and kt["fused_step"][1] == 1
    with pytest.raises(InvalidArgument):
        s.set_pipeline("fused", 30, 0, 1)
    with pytest.raises(InvalidArgument):
        s.set_temporal_depth(3)
    s.close()
