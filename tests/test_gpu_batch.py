"""The batched form: many domains of uneven sizes in one persistent launch per
fused sweep.  Every domain must come out bit-identical to a single-domain
handle of the same storage form run alone (same arithmetic, same operation
order), whatever the tile shape, chunk length, graph use or step grouping."""
import numpy as np
import pytest

from fdtd_method_gb300 import FDTD, FDTDBatch, InvalidArgument, Precision, build, sources
from fdtd_method_gb300.sources import COURANT_DT, normalised_parameters

pytestmark = pytest.mark.gpu

SHAPES = [(37, 19, 23), (64, 28, 16), (33, 9, 40), (5, 70, 3), (96, 42, 5), (1, 1, 1), (32, 14, 24),
          (70, 61, 9)]


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _domains(shapes, seed):
    rng = np.random.default_rng(seed)
    out = []
    for q, sh in enumerate(shapes):
        p = normalised_parameters(*sh)
        vals = [rng.standard_normal(p.cells) * 0.5 for _ in range(6)]
        c = (sh[0] // 2, sh[1] // 3, sh[2] // 2)
        srcs = [] if q % 3 == 2 else [sources.gaussian_pulse(p, c, 2.0, 1.0 + 0.1 * q, 20.0, 3.0, 4.0, 30,
                                                              phase=0.3 * q, comp="zx"[q % 2])]
        out.append((p, vals, srcs))
    return out


def _single(p, prec, vals, srcs, groups, exps=None):
    s = FDTD(p, COURANT_DT, prec)
    if exps is not None:
        s.set_fp16_exponents(exps)
    for c, v in enumerate(vals):
        s.get_field(c).assign(v)
    for q in srcs:
        s.add_source(q)
    for n in groups:
        s.step(n)
    out = [s.get_field(c).numpy() for c in range(6)]
    sums = s.field_sums()
    s.close()
    return out, sums


def _batch(doms, prec, groups, tile_y=0, kchunk=0, graphs=True, exps=None, split=False):
    b = FDTDBatch([d[0] for d in doms], COURANT_DT, prec)
    b.set_config(tile_y, kchunk, graphs)
    b.set_split_sources(split)
    for q, (p, vals, srcs) in enumerate(doms):
        if exps is not None:
            b.set_fp16_exponents(q, exps)
        for c, v in enumerate(vals):
            b.copy_from_host(q, c, v)
        for s in srcs:
            b.add_source(q, s)
    for n in groups:
        b.step(n)
    b.synchronize()
    out = [[b.copy_to_host(q, c) for c in range(6)] for q in range(len(doms))]
    sums = [b.field_sums(q) for q in range(len(doms))]
    assert b.step_index == sum(groups)
    b.close()
    return out, sums


@pytest.mark.parametrize("split", [False, True])
@pytest.mark.parametrize("prec", [Precision.FP32, Precision.FP32_COMP, Precision.FP16_SCALED])
def test_batch_equals_single_domains(prec, split):
    """Every domain equals a single handle, with the sweep's plane loop
    compiled once or split into source and source-free copies."""
    doms = _domains(SHAPES, 3)
    exps = [4] * 6 if prec == Precision.FP16_SCALED else None
    got, sums = _batch(doms, prec, [5], exps=exps, split=split)
    for q, (p, vals, srcs) in enumerate(doms):
        want, wsums = _single(p, prec, vals, srcs, [5], exps=exps)
        for c in range(6):
            np.testing.assert_array_equal(got[q][c], want[c], err_msg="domain %d component %d" % (q, c))
        np.testing.assert_array_equal(sums[q], wsums)


@pytest.mark.parametrize("tile_y,kchunk,graphs", [(14, 24, True), (6, 7, True), (30, 64, False), (14, 1, False)])
def test_batch_shapes_graphs_and_step_groups(tile_y, kchunk, graphs):
    """Odd and even step groups (the copy parity flips with odd ones), graph
    replays of the same group, and several tile shapes."""
    doms = _domains(SHAPES[:5], 7)
    groups = [3, 3, 4, 1, 2]
    got, _ = _batch(doms, Precision.FP32_COMP, groups, tile_y, kchunk, graphs)
    for q, (p, vals, srcs) in enumerate(doms):
        want, _ = _single(p, Precision.FP32_COMP, vals, srcs, groups)
        for c in range(6):
            np.testing.assert_array_equal(got[q][c], want[c], err_msg="domain %d component %d" % (q, c))


def test_batch_workload_sample():
    """A slice of the batched workload generator (plane waves along random
    axes plus one pulse per domain) stepped 40 steps."""
    wl = sources.batch_workload(count=6, seed=5, n_steps=40, lo=20, hi=70)
    doms = []
    for p, init, src in wl:
        vals = [init.get(c, np.zeros(p.cells)) for c in range(6)]
        doms.append((p, vals, [src]))
    got, _ = _batch(doms, Precision.FP32_COMP, [40])
    for q, (p, vals, srcs) in enumerate(doms):
        want, _ = _single(p, Precision.FP32_COMP, vals, srcs, [40])
        for c in range(6):
            np.testing.assert_array_equal(got[q][c], want[c])


def test_batch_rejects_bad_arguments():
    p = normalised_parameters(8, 8, 8)
    with pytest.raises(InvalidArgument):
        FDTDBatch([], COURANT_DT)
    b = FDTDBatch([p, p], COURANT_DT, Precision.FP32)
    with pytest.raises(InvalidArgument):
        b.copy_to_host(2, 0)
    with pytest.raises(Exception):
        b.copy_from_host(0, 6, np.zeros(p.cells))
    with pytest.raises(InvalidArgument):
        b.step(-1)
    b.close()
