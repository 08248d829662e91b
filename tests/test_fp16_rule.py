"""The FP16 form's exponent rule (fdtd_fp16_choose_exponents), on the host.

The rule a scan applies (the GPU side only supplies the six stored peaks):
k_c = ceil(log2 m_c) - e_c bounds component c's field peak by 2^k_c; with
k_all the largest, the wanted exponent is min(target - k_c, target +
headroom - k_all), clamped to [-60, 60] (a component with no field gets the
second term); a component is re-encoded when forced, when its exponent is
above the bound, or when the wanted one is 3 or more away.  Checked against
this restatement on seeded random cases and on the edge cases by hand.
"""
import math

import numpy as np
import pytest

from fdtd_method_gb300 import InvalidArgument, fp16_choose_exponents


def rule(peaks, cur, target, headroom, force):
    has = [m > 0 and math.isfinite(m) for m in peaks]
    k = [math.ceil(math.log2(m)) - e if h else 0 for m, e, h in zip(peaks, cur, has)]
    if not any(has):
        return list(cur)
    k_all = max(kc for kc, h in zip(k, has) if h)
    bound = target + headroom - k_all
    out = []
    for c in range(6):
        want = max(-60, min(60, min(target - k[c], bound) if has[c] else bound))
        keep = not force and cur[c] <= bound and abs(want - cur[c]) < 3
        out.append(cur[c] if keep else want)
    return out


def test_rule_on_seeded_cases():
    rng = np.random.default_rng(7)
    for _ in range(2000):
        peaks = [float(np.float32(10.0 ** rng.uniform(-8, 4.8))) if rng.random() > 0.1 else 0.0 for _ in range(6)]
        cur = [int(v) for v in rng.integers(-20, 21, 6)]
        target, headroom = int(rng.integers(0, 16)), int(rng.integers(0, 12))
        force = bool(rng.random() < 0.3)
        assert fp16_choose_exponents(peaks, cur, target, headroom, force) == rule(peaks, cur, target, headroom, force)


def test_weak_component_bounded_by_the_strongest():
    # Ez carries a 2^9 peak at exponent 0 (field 2^9); the others are at 2^-20.
    # Target 10, headroom 5: Ez -> 10 - 9 = 1; the weak ones -> min(10 + 20, 15 - 9) = 6.
    peaks = [2.0 ** -20] * 6
    peaks[2] = 2.0 ** 9
    assert fp16_choose_exponents(peaks, [0] * 6, 10, 5, False) == [6, 6, 0, 6, 6, 6]
    assert fp16_choose_exponents(peaks, [0] * 6, 10, 5, True) == [6, 6, 1, 6, 6, 6]


def test_hysteresis_and_bound():
    # every field peaks at 2^10 (stored peak 2^(10 + e)): wanted exponent 0
    cur = [2, -2, 0, 1, -1, 0]
    peaks = [2.0 ** (10 + e) for e in cur]
    # within 2 of the wanted exponent and not above the bound (15 - 10 = 5): kept
    assert fp16_choose_exponents(peaks, cur, 10, 5, False) == cur
    assert fp16_choose_exponents(peaks, cur, 10, 5, True) == [0] * 6
    # headroom 1 puts the bound at 1: the exponent 2 above it is re-encoded
    assert fp16_choose_exponents(peaks, cur, 10, 1, False) == [0, -2, 0, 1, -1, 0]
    # 3 or more from the wanted exponent: re-encoded
    cur3 = [-3, 0, 0, 0, 0, 0]
    assert fp16_choose_exponents([2.0 ** (10 + e) for e in cur3], cur3, 10, 5, False) == [0] * 6


def test_no_field_and_non_finite_peaks_leave_exponents():
    cur = [3, -4, 5, 0, 1, 2]
    assert fp16_choose_exponents([0.0] * 6, cur, 10, 5, True) == cur
    assert fp16_choose_exponents([math.inf, math.nan, 0.0, 0.0, 0.0, 0.0], cur, 10, 5, True) == cur
    # a NaN component with a finite one beside it takes the bound
    out = fp16_choose_exponents([math.nan, 2.0 ** 4, 0, 0, 0, 0], [0] * 6, 10, 5, True)
    assert out == [11, 6, 11, 11, 11, 11]


def test_clamped_to_sixty():
    assert fp16_choose_exponents([2.0 ** -100] + [0.0] * 5, [0] * 6, 15, 60, True)[0] == 60


@pytest.mark.parametrize("target,headroom,cur", [(-1, 5, [0] * 6), (16, 5, [0] * 6), (10, 61, [0] * 6),
                                                 (10, 5, [61, 0, 0, 0, 0, 0])])
def test_arguments_checked(target, headroom, cur):
    with pytest.raises(InvalidArgument):
        fp16_choose_exponents([1.0] * 6, cur, target, headroom)
