"""Per-component exponents of the FP16 storage form chosen by the engine.

Stored value = field * 2^e_c.  The kernels compute on stored values with
coefficients that carry the powers of two between components, so rescaling a
component is exact and changes results only where a value would otherwise
leave FP16's normal range (subnormal below 2^-14, overflow above 65504).
The autoscaler scans the stored peaks and re-encodes each component around
2^10, at most 2^5 above the strongest component's scale by default."""
import numpy as np
import pytest

from fdtd_method_gb300 import FDTD, Component, Precision, build, sources
from fdtd_method_gb300.sources import COURANT_DT, normalised_parameters

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _rel(a, b):
    d = float(np.sqrt(((a - b) ** 2).sum()))
    n = float(np.sqrt((b * b).sum()))
    return d / n


def _two_waves(p):
    """A weak wave along x (Ey, Bz; amplitude 1e-6) and a strong one along z
    (Ex, By; amplitude 1e3): orthogonal polarisations evolve independently."""
    f = {}
    for c, v in sources.plane_wave_fields(p, axis=0, mode=2).items():
        f[int(c)] = v * 1e-6
    for c, v in sources.plane_wave_fields(p, axis=2, mode=1).items():
        f[int(c)] = v * 1e3
    return f


def test_autoscale_picks_exponents_per_component_and_keeps_weak_fields():
    p = normalised_parameters(48, 16, 40)
    init = _two_waves(p)
    ref = FDTD(p, COURANT_DT, Precision.FP64)
    fixed = FDTD(p, COURANT_DT, Precision.FP16_SCALED)
    auto = FDTD(p, COURANT_DT, Precision.FP16_SCALED)
    for s in (ref, fixed, auto):
        for c, v in init.items():
            s.copy_from_host(c, v)
    # the two waves never exchange magnitude: a large headroom gives each
    # component its own scale
    exps = auto.fp16_autoscale(12, 40)
    # peaks: 1e-6 -> 2^12 needs e ~ 32; 1e3 -> e ~ 2; components without
    # field get the bound (2^40 above the strongest)
    assert exps[Component.EY] > 25 and exps[Component.BZ] > 25
    assert 0 < exps[Component.EX] < 5 and 0 < exps[Component.BY] < 5
    assert exps[Component.EZ] > 25 and exps[Component.BX] > 25
    for s in (ref, fixed, auto):
        s.step(60)
    for c in (Component.EY, Component.BZ):
        want = ref.copy_to_host(c)
        err_auto = _rel(auto.copy_to_host(c), want)
        err_fixed = _rel(fixed.copy_to_host(c), want)
        assert err_auto <= 5e-2, (c, err_auto)
        # 1e-6 lies below FP16's normal range (6.1e-5) at scale 1
        assert err_fixed > 0.05 and err_fixed > 5 * err_auto, (c, err_fixed)
    for c in (Component.EX, Component.BY):
        assert _rel(auto.copy_to_host(c), ref.copy_to_host(c)) <= 5e-2
    for s in (ref, fixed, auto):
        s.close()


def test_rescaling_is_exact_inside_the_normal_range():
    """The same run with fixed exponents and with rescans every 4 steps: the
    field values agree to the rounding of the rare values near zero that
    one of the two stores as FP16 subnormals."""
    p = normalised_parameters(40, 24, 18)
    rng = np.random.default_rng(12)
    vals = [rng.uniform(0.25, 1.0, p.cells) * rng.choice([-1.0, 1.0], p.cells) for _ in range(6)]
    src = sources.gaussian_pulse(p, (20, 12, 9), 2.5, 1.5, 20.0, 6.0, 6.0, 40, comp="z")
    a = FDTD(p, COURANT_DT, Precision.FP16_SCALED)
    b = FDTD(p, COURANT_DT, Precision.FP16_SCALED)
    a.set_fp16_exponents([6] * 6)
    b.set_fp16_exponents([6] * 6)
    b.set_fp16_autoscale(4, 13)  # stored peaks near 2^7: the wanted exponents are 5 or more above 6
    for s in (a, b):
        for c, v in enumerate(vals):
            s.copy_from_host(c, v)
        s.add_source(src)
        s.step(21)
    assert b.fp16_exponents() != [6] * 6
    for c in range(6):
        assert _rel(b.copy_to_host(c), a.copy_to_host(c)) <= 1e-6
    a.close()
    b.close()


def test_autoscale_follows_a_field_that_grows_from_zero():
    """A pulse source on zero fields: rescans every 10 steps keep every
    component in range while the field grows by orders of magnitude."""
    p = normalised_parameters(64, 64, 64)
    src = sources.baseline_pulse(p, seed=1, n_steps=300, sigma=4.0)
    ref = FDTD(p, COURANT_DT, Precision.FP64)
    h = FDTD(p, COURANT_DT, Precision.FP16_SCALED)
    h.set_fp16_autoscale(10)
    for s in (ref, h):
        s.add_source(src)
        s.step(220)
    num = den = 0.0
    for c in range(6):
        a, b = h.copy_to_host(c), ref.copy_to_host(c)
        assert np.isfinite(a).all()
        num += float(((a - b) ** 2).sum())
        den += float((b * b).sum())
    assert (num / den) ** 0.5 <= 5e-2
    e = h.fp16_exponents()
    assert len(set(e)) > 1  # Jz source: Ez, Bx, By carry the field, Ex, Ey and Bz less
    ref.close()
    h.close()
