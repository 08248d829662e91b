"""The autotuner times candidate launch shapes on the caller's own grid.  It
must leave the simulation state untouched and pick a shape whose results are
the same bits as any other shape's."""
import numpy as np
import pytest

from fdtd_method_gb300 import FDTD, FDTDBatch, FDTDError, Precision, build, sources
from fdtd_method_gb300.sources import COURANT_DT, normalised_parameters

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _setup(sim, p, seed):
    rng = np.random.default_rng(seed)
    for c in range(6):
        sim.get_field(c).assign(rng.standard_normal(p.cells) * 0.3)
    sim.add_source(sources.gaussian_pulse(p, (p.Ni // 2, p.Nj // 2, p.Nk // 2), 3.0, 1.5, 25.0, 3.0, 5.0, 40))


def _fields(sim):
    return [sim.get_field(c).numpy() for c in range(6)]


@pytest.mark.parametrize("prec", [Precision.FP32_COMP, Precision.FP16_SCALED])
def test_autotune_leaves_state_and_bits_unchanged(prec):
    p = normalised_parameters(70, 45, 40)
    a = FDTD(p, COURANT_DT, prec)
    b = FDTD(p, COURANT_DT, prec)
    for s in (a, b):
        if prec == Precision.FP16_SCALED:
            s.set_fp16_exponents([4] * 6)
        _setup(s, p, 3)
    before = _fields(a)
    r = a.autotune(sweeps=2, reuse=False)
    # (3 + 2 tile shapes) x 6 chunk lengths, and the depth-2 sweep's 2 x 3
    assert r["candidates"] == 36 and not r["cached"]
    assert (r["cells_per_thread"], r["tile_y"]) in {(1, 6), (1, 14), (1, 30), (2, 6), (2, 14)}
    assert r["kchunk"] in (16, 24, 32, 48, 64, 96) and r["ms_per_step"] > 0 and r["depth"] in (1, 2)
    for x, y in zip(before, _fields(a)):
        np.testing.assert_array_equal(x, y)
    a.step(7)
    b.step(7)
    for x, y in zip(_fields(a), _fields(b)):
        np.testing.assert_array_equal(x, y)
    c = FDTD(p, COURANT_DT, prec)
    r2 = c.autotune(reuse=True)
    assert r2["cached"] and (r2["tile_y"], r2["kchunk"], r2["cells_per_thread"], r2["depth"]) == (
        r["tile_y"], r["kchunk"], r["cells_per_thread"], r["depth"])


def test_autotune_rejects_fp64():
    p = normalised_parameters(8, 8, 8)
    s = FDTD(p, COURANT_DT)
    with pytest.raises(FDTDError):
        s.autotune()


def test_batch_autotune_leaves_state_and_bits_unchanged():
    shapes = [(40, 30, 20), (33, 17, 50), (64, 16, 9)]
    ps = [normalised_parameters(*sh) for sh in shapes]
    rng = np.random.default_rng(9)
    init = [[rng.standard_normal(p.cells) * 0.3 for _ in range(6)] for p in ps]
    srcs = [sources.gaussian_pulse(p, (p.Ni // 2, p.Nj // 2, p.Nk // 2), 2.0, 1.0, 25.0, 3.0, 5.0, 40) for p in ps]

    def make():
        b = FDTDBatch(ps, COURANT_DT, Precision.FP32_COMP)
        for q in range(len(ps)):
            for c in range(6):
                b.copy_from_host(q, c, init[q][c])
            b.add_source(q, srcs[q])
        return b

    a, b = make(), make()
    a.step(3)
    b.step(3)
    before = [[a.copy_to_host(q, c) for c in range(6)] for q in range(len(ps))]
    r = a.autotune(sweeps=2)
    assert r["candidates"] == 30 and r["tile_y"] in (6, 14, 30) and r["kchunk"] in (16, 24, 32, 48, 64)  # x 2 loops
    for q in range(len(ps)):
        for c in range(6):
            np.testing.assert_array_equal(before[q][c], a.copy_to_host(q, c))
    a.step(5)
    b.step(5)
    for q in range(len(ps)):
        for c in range(6):
            np.testing.assert_array_equal(a.copy_to_host(q, c), b.copy_to_host(q, c))
