"""The compact C-ABI forms (fdtd_energy, fdtd_set_sources,
fdtd_field_device_ptr, fdtd_copy_field, fdtd_sync) agree with the entry points
they are built on."""
import ctypes

import numpy as np
import pytest

from fdtd_method_gb300 import FDTD, Precision, build, sources
from fdtd_method_gb300 import _lib
from fdtd_method_gb300.sources import COURANT_DT, normalised_parameters

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _sim(prec=Precision.FP64, seed=1):
    p = normalised_parameters(24, 18, 12)
    s = FDTD(p, COURANT_DT, prec)
    rng = np.random.default_rng(seed)
    for c in range(6):
        s.copy_from_host(c, rng.standard_normal(p.cells))
    return p, s


@pytest.mark.parametrize("prec", [Precision.FP64, Precision.FP32_COMP])
def test_energy_and_copy(prec):
    lib = _lib.load()
    p, s = _sim(prec)
    out = (ctypes.c_double * 3)()
    _lib.check(lib.fdtd_energy(s._handle(), out))
    sums = s.field_sums()
    dv = p.dx * p.dy * p.dz / (8.0 * 3.14159265358)
    assert out[0] == pytest.approx(sums[:3].sum() * dv, rel=1e-15)
    assert out[1] == pytest.approx(sums[3:6].sum() * dv, rel=1e-15)
    assert out[2] == pytest.approx(s.energy(), rel=1e-15)
    a = np.empty(p.cells)
    _lib.check(lib.fdtd_copy_field(s._handle(), 1, a.ctypes.data, 0))
    assert np.array_equal(a, s.copy_to_host(1))
    b = a[::-1].copy()
    _lib.check(lib.fdtd_copy_field(s._handle(), 1, b.ctypes.data, 1))
    assert np.array_equal(s.copy_to_host(1), _roundtrip(p, prec, b))
    with pytest.raises(_lib.InvalidArgument):
        _lib.check(lib.fdtd_copy_field(s._handle(), 1, b.ctypes.data, 2))
    _lib.check(lib.fdtd_sync(s._handle()))
    s.close()


def _roundtrip(p, prec, values):
    t = FDTD(p, COURANT_DT, prec)
    t.copy_from_host(1, values)
    out = t.copy_to_host(1)
    t.close()
    return out


def test_field_device_ptr_is_get_field():
    lib = _lib.load()
    p, s = _sim()
    ptr = ctypes.c_void_p()
    _lib.check(lib.fdtd_field_device_ptr(s._handle(), 3, ctypes.byref(ptr)))
    assert ptr.value == s.get_field(3).device_ptr
    s.close()


def test_set_sources_replaces_the_list_and_keeps_it_on_error():
    lib = _lib.load()
    p = normalised_parameters(24, 18, 12)
    srcs = [sources.gaussian_pulse(p, (12, 9, 6), 2.0, 1.0, 20.0, 8.0, 4.0, 30, comp="z"),
            sources.gaussian_pulse(p, (3, 4, 5), 1.5, 0.7, 15.0, 6.0, 3.0, 30, comp="x")]
    want = FDTD(p, COURANT_DT)
    for q in srcs:
        want.add_source(q)
    want.step(8)
    got = FDTD(p, COURANT_DT)
    got.add_source(srcs[1])  # replaced below
    cs = [q.to_c() for q in srcs]
    arr = (_lib.Source * 2)(cs[0][0], cs[1][0])
    _lib.check(lib.fdtd_set_sources(got._handle(), arr, 2))
    bad = (_lib.Source * 1)(cs[0][0])
    bad[0].comp_mask = 0  # invalid: the list stays as it was
    with pytest.raises(_lib.InvalidArgument):
        _lib.check(lib.fdtd_set_sources(got._handle(), bad, 1))
    got.step(8)
    for c in range(6):
        assert np.array_equal(got.copy_to_host(c), want.copy_to_host(c)), c
    want.close()
    got.close()
