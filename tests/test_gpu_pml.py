"""The PML form (the reference's FDTD_PML: split-field absorbing layer) on the
GPU against the oracle's restatement, which the CPU suite pins bit for bit to
the reference's own build and golden cases."""
import numpy as np
import pytest

from oracle import OraclePML

from fdtd_method_gb300 import FDTD, FDTD_PML, build, sources
from fdtd_method_gb300.fdtd import Parameters
from fdtd_method_gb300.sources import COURANT_DT, normalised_parameters

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _params(shape):
    Ni, Nj, Nk = shape
    p = Parameters(Ni, Nj, Nk, 0.0, 1.0, 0.0, 2.0, 0.0, 3.0, 1.0 / Ni, 2.0 / Nj, 3.0 / Nk)
    return p, 0.3 * min(p.dx, p.dy, p.dz) / 3e10


@pytest.mark.parametrize("shape,pct,steps", [((20, 16, 12), 0.2, 6), ((15, 12, 10), 0.25, 8), ((8, 8, 8), 0.0, 5),
                                             ((24, 6, 9), 0.15, 7), ((11, 13, 7), 0.3, 4), ((70, 33, 40), 0.1, 5),
                                             ((5, 1, 9), 0.4, 3)])
def test_pml_bitwise_equal_to_oracle(shape, pct, steps):
    p, dt = _params(shape)
    rng = np.random.default_rng(sum(shape))
    vals = [rng.standard_normal(p.cells) for _ in range(9)]
    o = OraclePML(p, dt, pct)
    s = FDTD_PML(p, dt, pct)
    assert s.pml_size == o.pml
    for c in range(9):
        o.set(c, vals[c])
        s.get_field(c).assign(vals[c])
    o.step(steps)
    s.step(steps)
    for c in range(6):
        np.testing.assert_array_equal(s.get_field(c).numpy(), o.get(c), err_msg="component %d" % c)


def test_pml_with_sources_and_step_groups():
    """Analytic sources (current only inside the layer's inner box), steps in
    several groups, update_fields one at a time."""
    p = normalised_parameters(40, 32, 28)
    pct = 0.2
    src = sources.gaussian_pulse(p, (20, 16, 14), 2.5, 1.2, 18.0, 8.0, 6.0, 40, comp="z")
    o = OraclePML(p, COURANT_DT, pct)
    s = FDTD_PML(p, COURANT_DT, pct)
    o.add_source(src)
    s.add_source(src)
    for n in (3, 1, 4):
        o.step(n)
        s.step(n)
    o.step(2)
    s.update_fields()
    s.update_fields()
    for c in range(6):
        np.testing.assert_array_equal(s.get_field(c).numpy(), o.get(c), err_msg="component %d" % c)


def test_pml_absorbs_an_outgoing_pulse():
    """A pulse radiated from the centre leaves through the layer: after the
    wave has crossed it, the PML grid holds a small fraction of the energy the
    periodic grid keeps."""
    p = normalised_parameters(48, 48, 48)
    # t0 = T: the current integrates to zero over the pulse, so no static field stays behind
    src = sources.gaussian_pulse(p, (24, 24, 24), 2.0, 1.0, 12.0, 12.0, 5.0, 60, comp="z")
    pml = FDTD_PML(p, COURANT_DT, 0.2)
    per = FDTD(p, COURANT_DT)
    for s in (pml, per):
        s.add_source(src)
        s.step(60)
    e60 = pml.energy()
    for s in (pml, per):
        s.step(140)
    assert pml.energy() < 0.05 * per.energy()
    assert pml.energy() < 0.2 * e60
