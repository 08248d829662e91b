"""Precision forms (FP32, compensated FP32, FP16 with per-component scale)
against the FP64 drop-in on the same GPU.  Each result is judged by its
relative L2 error over all six field components; the bars are stated per test."""
import math

import numpy as np
import pytest

from oracle import Oracle

from fdtd_method_gb300 import FDTD, Precision, build, sources
from fdtd_method_gb300.sources import COURANT_DT, normalised_parameters

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def rel_l2(a_list, b_list):
    num = sum(float(((a - b) ** 2).sum()) for a, b in zip(a_list, b_list))
    den = sum(float((b ** 2).sum()) for b in b_list)
    return math.sqrt(num / den)


def fields(sim):
    return [sim.get_field(c).numpy() for c in range(6)]


@pytest.mark.parametrize("prec,tol", [(Precision.FP32, 2.0 ** -23), (Precision.FP32_COMP, 2.0 ** -29),
                                      (Precision.FP16_SCALED, 2.0 ** -10)])
def test_host_round_trip(prec, tol):
    p = normalised_parameters(33, 17, 9)
    rng = np.random.default_rng(1)
    vals = [rng.standard_normal(p.cells) for _ in range(6)]
    s = FDTD(p, COURANT_DT, prec)
    if prec == Precision.FP16_SCALED:
        s.set_fp16_exponents([8] * 6)
        vals = [np.clip(v, -60, 60) for v in vals]
    for c, v in enumerate(vals):
        s.get_field(c).assign(v)
    for c, v in enumerate(vals):
        got = s.get_field(c).numpy()
        rel = np.abs(got - v) / np.maximum(np.abs(v), 1e-30)
        assert rel.max() <= tol * 1.01, (prec, c, rel.max())


def pulse_case(n=64, steps=400):
    p = normalised_parameters(n, n, n)
    src = sources.gaussian_pulse(p, (n // 2, n // 2, n // 2), 4.0, 1.3, 30.0, 90.0, 30.0, steps)
    return p, src


@pytest.fixture(scope="module")
def fp64_pulse():
    p, src = pulse_case()
    s = FDTD(p, COURANT_DT)
    s.add_source(src)
    s.step(400)
    return p, src, fields(s), s.energy()


@pytest.mark.parametrize("prec", [Precision.FP32, Precision.FP32_COMP, Precision.FP16_SCALED])
def test_pinned_host_buffers_match_pageable(prec):
    """Page-locked host buffers are converted in place by the device (no
    staging copy); the values must equal the staged path's, both ways."""
    torch = pytest.importorskip("torch")
    p = normalised_parameters(45, 21, 13)
    rng = np.random.default_rng(11)
    vals = [rng.standard_normal(p.cells) for _ in range(6)]
    a = FDTD(p, COURANT_DT, prec)
    b = FDTD(p, COURANT_DT, prec)
    for s_ in (a, b):
        if prec == Precision.FP16_SCALED:
            s_.set_fp16_exponents([6] * 6)
    pinned = [torch.from_numpy(v).pin_memory() for v in vals]
    for c in range(6):
        a.copy_from_host(c, vals[c])
        b.copy_from_host(c, pinned[c].numpy())
    a.step(3)
    b.step(3)
    for c in range(6):
        out = torch.zeros(p.cells, dtype=torch.float64).pin_memory()
        b.copy_to_host(c, out.numpy())
        np.testing.assert_array_equal(out.numpy(), a.get_field(c).numpy())


@pytest.mark.parametrize("prec,bar", [(Precision.FP32, 1e-5), (Precision.FP32_COMP, 1e-5),
                                      (Precision.FP16_SCALED, 5e-2)])
def test_pulse_rel_l2_vs_fp64(fp64_pulse, prec, bar):
    p, src, ref, e_ref = fp64_pulse
    s = FDTD(p, COURANT_DT, prec)
    if prec == Precision.FP16_SCALED:
        s.set_fp16_exponents([6] * 6)
    s.add_source(src)
    s.step(400)
    err = rel_l2(fields(s), ref)
    assert err <= bar, err
    assert abs(s.energy() - e_ref) / e_ref <= 10 * bar


def test_compensated_beats_plain_fp32(fp64_pulse):
    p, src, ref, _ = fp64_pulse
    errs = {}
    for prec in (Precision.FP32, Precision.FP32_COMP):
        s = FDTD(p, COURANT_DT, prec)
        s.add_source(src)
        s.step(400)
        errs[prec] = rel_l2(fields(s), ref)
    assert errs[Precision.FP32_COMP] < errs[Precision.FP32]


def _run(p, prec, vals, srcs, steps, pipeline, tile_y=0, kchunk=0, dense_j=None, cpt=0):
    s = FDTD(p, COURANT_DT, prec)
    if prec == Precision.FP16_SCALED:
        s.set_fp16_exponents([4] * 6)
    s.set_pipeline(pipeline, tile_y, kchunk, cpt)
    for c, v in enumerate(vals):
        s.get_field(c).assign(v)
    if dense_j is not None:
        for q, v in enumerate(dense_j):
            s.get_field(6 + q).assign(v)
    for q in srcs:
        s.add_source(q)
    s.step(steps)
    return fields(s)


@pytest.mark.parametrize("cpt", [1, 2])
@pytest.mark.parametrize("prec", [Precision.FP32, Precision.FP32_COMP, Precision.FP16_SCALED])
@pytest.mark.parametrize("shape,tile_y,kchunk", [((37, 19, 23), 14, 64), ((1, 1, 1), 14, 64),
                                                 ((64, 28, 16), 14, 8), ((31, 15, 129), 6, 64),
                                                 ((2, 70, 3), 6, 2), ((33, 9, 40), 14, 7),
                                                 ((96, 42, 5), 6, 3), ((70, 61, 9), 30, 4),
                                                 ((33, 31, 6), 30, 64), ((32, 20, 11), 14, 24),
                                                 ((40, 17, 9), 14, 24), ((128, 30, 12), 30, 24)])
def test_fused_step_equals_split_sweeps(prec, shape, tile_y, kchunk, cpt):
    if tile_y == 30 and cpt == 2:
        pytest.skip("30-row tiles exist for one cell per thread only")
    """The one-sweep-per-step kernel and the one-sweep-per-half-step kernels
    evaluate the same arithmetic: results are bit-identical, with sources."""
    p = normalised_parameters(*shape)
    rng = np.random.default_rng(sum(shape))
    vals = [rng.standard_normal(p.cells) * 0.5 for _ in range(6)]
    c = (shape[0] // 2, shape[1] // 2, shape[2] // 2)
    srcs = [sources.gaussian_pulse(p, c, 2.0, 1.0, 20.0, 3.0, 4.0, 20, comp="z"),
            sources.gaussian_pulse(p, (0, 0, 0), 1.5, 0.8, 25.0, 2.0, 3.0, 20, phase=0.5, comp="x")]
    a = _run(p, prec, vals, srcs, 5, "split")
    b = _run(p, prec, vals, srcs, 5, "fused", tile_y, kchunk, cpt=cpt)
    for q in range(6):
        np.testing.assert_array_equal(a[q], b[q], err_msg="component %d" % q)


@pytest.mark.parametrize("prec", [Precision.FP32, Precision.FP32_COMP, Precision.FP16_SCALED])
def test_fused_equals_split_with_signed_zeros(prec):
    """Mostly-zero fields with negative zeros, and values too small for FP16
    (stored as signed zeros): the fused and split pipelines give the same
    bits, the signs of zero results included (a difference formed as
    -(b - a) instead of a - b would flip them)."""
    p = normalised_parameters(45, 23, 17)
    rng = np.random.default_rng(12)
    vals = []
    for _ in range(6):
        v = rng.standard_normal(p.cells) * 0.5
        r = rng.random(p.cells)
        v[r < 0.45] = 0.0
        v[(r >= 0.45) & (r < 0.9)] = -0.0
        v[(r >= 0.9) & (r < 0.95)] *= 1e-12
        vals.append(v)
    srcs = [sources.gaussian_pulse(p, (20, 11, 8), 1.0, 1.0, 20.0, 3.0, 4.0, 20, comp="z")]
    for steps in (1, 3):
        a = _run(p, prec, vals, srcs, steps, "split")
        b = _run(p, prec, vals, srcs, steps, "fused", 14, 8, cpt=1)
        if steps == 1:
            assert any((x == 0).any() for x in a)  # zero results to compare
        for q in range(6):
            np.testing.assert_array_equal(np.ascontiguousarray(a[q]).view(np.uint64),
                                          np.ascontiguousarray(b[q]).view(np.uint64),
                                          err_msg="component %d after %d steps" % (q, steps))


@pytest.mark.parametrize("cpt", [1, 2])
@pytest.mark.parametrize("prec", [Precision.FP32, Precision.FP32_COMP])
def test_fused_many_sources_and_dense_current(prec, cpt):
    """More sources than the fused kernel keeps in registers (generic path),
    plus a dense current written by the host."""
    p = normalised_parameters(40, 24, 20)
    rng = np.random.default_rng(2)
    vals = [rng.standard_normal(p.cells) * 0.1 for _ in range(6)]
    dj = [rng.standard_normal(p.cells) * 0.01 for _ in range(3)]
    srcs = sources.random_pulses(p, 6, seed=4, n_steps=30, sigma=2.0)
    a = _run(p, prec, vals, srcs, 6, "split", dense_j=dj)
    b = _run(p, prec, vals, srcs, 6, "fused", dense_j=dj, cpt=cpt)
    for q in range(6):
        np.testing.assert_array_equal(a[q], b[q])


def test_fp32_forms_follow_oracle_on_random_fields():
    """Stencil and wrap of the FP32 kernels on odd sizes: one step from random
    fields agrees with the FP64 oracle to FP32 rounding."""
    p = normalised_parameters(37, 11, 6)
    rng = np.random.default_rng(5)
    vals = [rng.standard_normal(p.cells) for _ in range(6)]
    o = Oracle(p, COURANT_DT)
    for c, v in enumerate(vals):
        o.set(c, v)
    o.step(2)
    want = [o.get(c) for c in range(6)]
    for prec, bar in ((Precision.FP32, 1e-6), (Precision.FP32_COMP, 1e-7)):
        s = FDTD(p, COURANT_DT, prec)
        for c, v in enumerate(vals):
            s.get_field(c).assign(v)
        s.step(2)
        assert rel_l2(fields(s), want) <= bar, prec


@pytest.mark.parametrize("exps", [[2, 3, 1, 0, -1, 2], [-3, 4, 0, 5, 1, -2]])
def test_fp16_per_component_scales_follow_fp64(exps):
    """FP16 kernels compute on stored values with every coefficient carrying
    2^(e_dst - e_src): with a different exponent on every component (so a
    wrong pairing would scale a term by a power of two), analytic sources and
    a dense current, 12 steps stay within FP16 rounding of the FP64 run, in
    both pipelines."""
    p = normalised_parameters(40, 24, 20)
    rng = np.random.default_rng(8)
    vals = [rng.standard_normal(p.cells) * 0.5 for _ in range(6)]
    dj = [np.zeros(p.cells) for _ in range(3)]
    dj[2].reshape(p.Nk, p.Nj, p.Ni)[8:12, 6:14, 10:30] = 0.05
    srcs = sources.random_pulses(p, 2, seed=6, n_steps=20, sigma=2.0)
    ref = FDTD(p, COURANT_DT)
    for c, v in enumerate(vals):
        ref.get_field(c).assign(v)
    for c in range(3):
        ref.get_field(6 + c).assign(dj[c])
    for q in srcs:
        ref.add_source(q)
    ref.step(12)
    want = fields(ref)
    ref.close()
    for pipe in ("fused", "split"):
        s = FDTD(p, COURANT_DT, Precision.FP16_SCALED)
        s.set_pipeline(pipe)
        s.set_fp16_exponents(exps)
        for c, v in enumerate(vals):
            s.get_field(c).assign(v)
        for c in range(3):
            s.copy_from_host(6 + c, dj[c])
        for q in srcs:
            s.add_source(q)
        s.step(12)
        err = rel_l2(fields(s), want)
        s.close()
        assert err < 5e-3, (pipe, err)
