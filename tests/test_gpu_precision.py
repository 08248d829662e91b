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
