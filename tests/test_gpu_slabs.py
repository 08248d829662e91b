"""z slabs on one GPU (the coarray program's decomposition, coarray/fdtd.F90,
with its halo exchange as device copies): a grid stepped as n slabs equals
the same grid stepped as one handle, bit for bit, in every precision form,
with sources that straddle slab faces and wrap around z, with dense
currents, and across several step calls; the FP64 slabs also equal the
oracle.  The FP32-arithmetic forms run both schedules: the split sweeps, and
one fused B-first sweep per step (FDTD_SWEEP_STEP) with its exchange."""
import numpy as np
import pytest

from oracle import Oracle

from fdtd_method_gb300 import FDTD, FDTDError, FDTDSlabs, InvalidArgument, Precision, Slab, build, sources
from fdtd_method_gb300 import _lib
from fdtd_method_gb300.sources import COURANT_DT, normalised_parameters

pytestmark = pytest.mark.gpu

FORMS = [Precision.FP64, Precision.FP32, Precision.FP32_COMP, Precision.FP16_SCALED]


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _case(seed=3):
    p = normalised_parameters(40, 24, 37)
    rng = np.random.default_rng(seed)
    f = [np.clip(rng.standard_normal(p.cells), -4, 4) for _ in range(6)]
    srcs = [
        # centred on a slab face of the 3-slab split (planes 13 | 25)
        sources.gaussian_pulse(p, (20, 12, 13), 1.5, 1.3, 20.0, 12.0, 6.0, 60, comp="z"),
        # a window that wraps around z (origin near Nk - 12)
        sources.gaussian_pulse(p, (7, 3, 1), 1.5, 0.8, 17.0, 9.0, 5.0, 60, phase=0.4, comp="x"),
        # a window as long as the grid
        sources.gaussian_pulse(p, (33, 20, 30), 3.0, 0.6, 25.0, 10.0, 6.0, 60, comp="y"),
    ]
    return p, f, srcs


def _load(sim, f, srcs, prec):
    if prec == Precision.FP16_SCALED:
        sim.set_fp16_exponents([1] * 6)
    for c in range(6):
        sim.copy_from_host(c, f[c])
    for s in srcs:
        sim.add_source(s)


def _fields(sim):
    return [sim.copy_to_host(c) for c in range(6)]


SCHEDULES = [(Precision.FP64, False)] + [(q, fz) for q in FORMS[1:] for fz in (False, True)]


@pytest.mark.parametrize("prec,fused", SCHEDULES)
@pytest.mark.parametrize("n", [1, 2, 3, 5])
def test_slabs_equal_the_whole_grid(prec, fused, n):
    p, f, srcs = _case()
    whole = FDTD(p, COURANT_DT, prec)
    if prec != Precision.FP64:
        whole.set_pipeline("split")
    _load(whole, f, srcs, prec)
    whole.step(4)
    whole.step(5)
    want = _fields(whole)
    with FDTDSlabs(p, COURANT_DT, n, prec, fused=fused) as sl:
        _load(sl, f, srcs, prec)
        sl.step(4)
        sl.step(5)
        got = _fields(sl)
        assert sl.step_index == whole.step_index == 9
    for c in range(6):
        assert np.array_equal(got[c], want[c]), (prec, n, c, np.abs(got[c] - want[c]).max())
    whole.close()


@pytest.mark.parametrize("prec,fused", [(Precision.FP64, False), (Precision.FP32_COMP, False),
                                        (Precision.FP32_COMP, True)])
def test_one_plane_slabs(prec, fused):
    # as many slabs as planes: every slab sends and receives its only plane
    p = normalised_parameters(24, 10, 7)
    rng = np.random.default_rng(11)
    f = [rng.standard_normal(p.cells) for _ in range(6)]
    src = [sources.gaussian_pulse(p, (12, 5, 3), 1.5, 1.0, 15.0, 6.0, 4.0, 30, comp="z")]
    whole = FDTD(p, COURANT_DT, prec)
    if prec != Precision.FP64:
        whole.set_pipeline("split")
    _load(whole, f, src, prec)
    whole.step(5)
    with FDTDSlabs(p, COURANT_DT, p.Nk, prec, fused=fused) as sl:
        _load(sl, f, src, prec)
        sl.step(5)
        for c in range(6):
            assert np.array_equal(sl.copy_to_host(c), whole.copy_to_host(c)), c
    whole.close()


@pytest.mark.parametrize("fused", [False, True])
def test_fp16_slabs_with_per_component_exponents(fused):
    p, f, srcs = _case(8)
    exps = [3, 1, -2, 0, 4, 2]
    whole = FDTD(p, COURANT_DT, Precision.FP16_SCALED)
    whole.set_pipeline("split")
    whole.set_fp16_exponents(exps)
    with FDTDSlabs(p, COURANT_DT, 3, Precision.FP16_SCALED, fused=fused) as sl:
        sl.set_fp16_exponents(exps)
        for sim in (whole, sl):
            for c in range(6):
                sim.copy_from_host(c, f[c] * 0.25)
            for q in srcs:
                sim.add_source(q)
            sim.step(6)
        for c in range(6):
            assert np.array_equal(sl.copy_to_host(c), whole.copy_to_host(c)), c
    whole.close()


@pytest.mark.parametrize("prec", [Precision.FP32, Precision.FP32_COMP])
def test_slabs_equal_the_fused_pipeline(prec):
    # the whole grid's default (fused) pipeline reproduces the split sweeps
    p, f, srcs = _case(4)
    whole = FDTD(p, COURANT_DT, prec)
    _load(whole, f, srcs, prec)
    whole.step(7)
    with FDTDSlabs(p, COURANT_DT, 3, prec) as sl:
        _load(sl, f, srcs, prec)
        sl.step(7)
        for c in range(6):
            assert np.array_equal(sl.copy_to_host(c), whole.copy_to_host(c)), (prec, c)
    whole.close()


@pytest.mark.parametrize("prec,fused", [(Precision.FP64, False), (Precision.FP32_COMP, False),
                                        (Precision.FP32_COMP, True), (Precision.FP32, True)])
def test_slabs_with_dense_current(prec, fused):
    p, f, _ = _case(5)
    rng = np.random.default_rng(9)
    j = np.zeros(p.cells)
    j.reshape(p.Nk, p.Nj, p.Ni)[10:16, 4:9, 3:30] = rng.standard_normal((6, 5, 27))
    whole = FDTD(p, COURANT_DT, prec)
    if prec != Precision.FP64:
        whole.set_pipeline("split")
    _load(whole, f, [], prec)
    whole.copy_from_host(8, j)
    whole.step(6)
    with FDTDSlabs(p, COURANT_DT, 2, prec, fused=fused) as sl:
        _load(sl, f, [], prec)
        sl.copy_from_host(8, j)
        sl.step(6)
        for c in range(6):
            assert np.array_equal(sl.copy_to_host(c), whole.copy_to_host(c)), (prec, c)
        assert np.array_equal(sl.copy_to_host(8), whole.copy_to_host(8))
    whole.close()


def test_fp64_slabs_equal_the_oracle():
    p, f, srcs = _case(6)
    o = Oracle(p, COURANT_DT)
    for c in range(6):
        o.set(c, f[c])
    for s in srcs:
        o.add_source(s)
    o.step(8)
    with FDTDSlabs(p, COURANT_DT, 4) as sl:
        _load(sl, f, srcs, Precision.FP64)
        sl.step(8)
        for c in range(6):
            assert np.array_equal(sl.copy_to_host(c), o.get(c)), c
        # the sums of the slabs are those of the grid, to rounding
        np.testing.assert_allclose(sl.field_sums()[:9], o.field_sums()[:9], rtol=1e-12, atol=1e-12)


def test_slab_errors():
    p = normalised_parameters(16, 8, 12)
    with pytest.raises(InvalidArgument):
        Slab(p, COURANT_DT, 5, 5)
    with pytest.raises(InvalidArgument):
        Slab(p, COURANT_DT, 0, 13)
    s = Slab(p, COURANT_DT, 0, 6)
    with pytest.raises(FDTDError):
        s.step(1)  # a slab steps through sweeps and exchanges
    with pytest.raises(FDTDError):
        s.set_pipeline("fused", 0, 0, 2)  # the slab's fused sweep has one cell per thread
    with pytest.raises(FDTDError):
        s.sweep(4)  # the FP64 form runs the split sweeps
    with pytest.raises(InvalidArgument):
        FDTDSlabs(p, COURANT_DT, 2, Precision.FP64, fused=True)
    t = Slab(p, COURANT_DT, 7, 12)  # leaves plane 6 uncovered
    import ctypes
    arr = (ctypes.c_void_p * 2)(s._handle().value, t._handle().value)
    with pytest.raises(InvalidArgument):
        _lib.check(_lib.load().fdtd_slab_exchange(arr, 2, 0))
    # the host-facing grid is the owned planes; halo planes are addressable
    assert s.parameters.Nk == 6 and s.copy_to_host(0).size == 16 * 8 * 6
    ptr, nb = s.plane(3, 0)
    assert ptr and nb == 16 * 8 * 8
    s.close()
    t.close()


@pytest.mark.parametrize("prec", [Precision.FP32, Precision.FP32_COMP, Precision.FP16_SCALED])
def test_fused_slabs_with_reads_writes_and_schedule_changes(prec):
    """Fused calls with reads between them (the pending half applied into the
    slabs' side arrays), a write (applied first), a split call and different
    launch shapes (several z chunks per slab): the whole grid's bits."""
    p, f, srcs = _case(12)
    rng = np.random.default_rng(13)
    new_ex = rng.standard_normal(p.cells) * 0.5
    whole = FDTD(p, COURANT_DT, prec)
    _load(whole, f, srcs, prec)
    with FDTDSlabs(p, COURANT_DT, 3, prec) as sl:
        _load(sl, f, srcs, prec)
        for s in sl.slabs:
            s.set_pipeline("auto", 6, 5, 1)
        for sim in (whole, sl):
            sim.step(3)
            sim.copy_to_host(4)
            sim.field_sums()
            sim.step(2)
            sim.copy_from_host(0, new_ex)
            sim.step(2)
        sl.fused = False
        sl.step(3)
        sl.fused = True
        whole.step(3)
        for s in sl.slabs:
            s.set_pipeline("auto", 30, 0, 1)
        sl.step(4)
        whole.step(4)
        for c in range(6):
            assert np.array_equal(sl.copy_to_host(c), whole.copy_to_host(c)), (prec, c)
        assert sl.step_index == whole.step_index == 14
    whole.close()


def test_fused_slab_step_is_one_launch_per_slab():
    p, f, srcs = _case(2)
    with FDTDSlabs(p, COURANT_DT, 3, Precision.FP32_COMP) as sl:
        _load(sl, f, srcs, Precision.FP32_COMP)
        sl.step(1)
        sl.synchronize()
        for s in sl.slabs:
            s.kernel_times()
            s.set_kernel_timing(True)
        sl.step(6)
        for s in sl.slabs:
            kt = s.kernel_times()
            assert kt["fused_step"][1] == 6
            assert kt["b_half"][1] == 0 and kt["b_double"][1] == 0 and kt["e_update"][1] == 0
