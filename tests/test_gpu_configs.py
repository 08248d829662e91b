"""Full-size runs of the precision workloads beside the 512^3 headline:

* 1024 x 1024 x 512 periodic grid, 8 seeded Gaussian-pulse Jz/Jx sources at
  random cells with random phases, 2000 steps: the compensated FP32 form
  against the FP64 drop-in on the same GPU (rel-L2 per component <= 1e-5,
  energy drift).
* 1536 x 1536 x 1024 periodic grid (2.4e9 cells, past the reference's int32
  indexing), 16 pulses, 1000 steps: FP16 storage with per-component
  power-of-two scales chosen by the engine (rescans every 25 steps) against
  plain FP32 on the same GPU, and the same 16 pulses rerun on 256^3 in FP16
  against the FP64 form.

Fields are compared on the device through fdtd_export_field; torch only
holds the FP64 comparison buffers."""
import math

import pytest

from fdtd_method_gb300 import FDTD, Precision, build, sources
from fdtd_method_gb300.sources import COURANT_DT, normalised_parameters

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

CHUNK = 1 << 27  # cells per comparison chunk (1 GiB of FP64 per buffer)
AUTOSCALE_EVERY = 25  # steps between the FP16 form's range checks


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def sq_sums(ref, other, cells):
    """Per component: sum (ref - other)^2 and sum ref^2 over the grid."""
    ba = torch.empty(min(CHUNK, cells), dtype=torch.float64, device="cuda")
    bb = torch.empty_like(ba)
    num, den = [0.0] * 6, [0.0] * 6
    for c in range(6):
        for off in range(0, cells, CHUNK):
            n = min(CHUNK, cells - off)
            ref.export_field(c, off, n, ba.data_ptr())
            other.export_field(c, off, n, bb.data_ptr())
            ref.synchronize()
            other.synchronize()
            a, b = ba[:n], bb[:n]
            num[c] += float(((a - b) ** 2).sum())
            den[c] += float((a * a).sum())
    return num, den


def rel_l2(num, den):
    total = sum(den)
    return math.sqrt(sum(num) / total), [math.sqrt(x / total) for x in num]


def test_compensated_1024x1024x512_8_pulses_2000_steps():
    p = normalised_parameters(1024, 1024, 512)
    steps = 2000
    srcs = sources.random_pulses(p, 8, seed=0, n_steps=steps, comps=("z", "x"))
    ref = FDTD(p, COURANT_DT, Precision.FP64)
    comp = FDTD(p, COURANT_DT, Precision.FP32_COMP)
    for s in (ref, comp):
        for q in srcs:
            s.add_source(q)
        s.step(steps)
    num, den = sq_sums(ref, comp, p.cells)
    total, per = rel_l2(num, den)
    drift = (comp.energy() - ref.energy()) / ref.energy()
    print("1024x1024x512 FP32_COMP: rel-L2 %.3e per component %s, energy drift %.3e"
          % (total, ["%.2e" % x for x in per], drift))
    assert total <= 1e-5 and max(per) <= 1e-5
    assert abs(drift) <= 1e-6
    ref.close()
    comp.close()


def _scaled_pulses(srcs, p_from, p_to):
    out = []
    for s in srcs:
        m = s.meta
        c = tuple(int(v * n_to // n_from) for v, n_from, n_to in
                  zip(m["center"], (p_from.Ni, p_from.Nj, p_from.Nk), (p_to.Ni, p_to.Nj, p_to.Nk)))
        out.append(sources.gaussian_pulse(p_to, c, m["sigma"], m["A"], m["T"], m["t0"], m["tau"], len(s.amp),
                                          phase=m["phase"], comp=m["comp"]))
    return out


def test_fp16_1536x1536x1024_16_pulses_1000_steps():
    p = normalised_parameters(1536, 1536, 1024)
    steps = 1000
    srcs = sources.random_pulses(p, 16, seed=0, n_steps=steps, comps=("z", "x"))
    half = FDTD(p, COURANT_DT, Precision.FP16_SCALED)
    half.set_fp16_autoscale(AUTOSCALE_EVERY)
    single = FDTD(p, COURANT_DT, Precision.FP32)
    for s in (half, single):
        for q in srcs:
            s.add_source(q)
        s.autotune(sweeps=3)
        s.step(steps)
    num, den = sq_sums(single, half, p.cells)
    total, per = rel_l2(num, den)
    exps = half.fp16_exponents()
    print("1536x1536x1024 FP16_SCALED vs FP32: rel-L2 %.3e per component %s, exponents %s"
          % (total, ["%.2e" % x for x in per], exps))
    assert total <= 5e-2
    assert len(set(exps)) > 1
    half.close()
    single.close()

    # the same 16 pulses, placed at the same relative cells of a 256^3 grid
    q = normalised_parameters(256, 256, 256)
    small = _scaled_pulses(srcs, p, q)
    ref = FDTD(q, COURANT_DT, Precision.FP64)
    h16 = FDTD(q, COURANT_DT, Precision.FP16_SCALED)
    h16.set_fp16_autoscale(AUTOSCALE_EVERY)
    for s in (ref, h16):
        for x in small:
            s.add_source(x)
        s.step(steps)
    num, den = sq_sums(ref, h16, q.cells)
    total, per = rel_l2(num, den)
    print("256^3 rerun FP16_SCALED vs FP64: rel-L2 %.3e" % total)
    assert total <= 5e-2
