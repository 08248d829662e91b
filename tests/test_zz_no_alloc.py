"""fdtd_field_sums_noalloc against fdtd_field_sums.

The no-allocation entry point serves callers that cannot allocate device
memory themselves (an application whose pool allocator owns all device
memory, a monitor that must not call cudaMalloc next to a running
simulation).  It must give the same ten field sums as the handle-based entry
point, call after call, from the same device arrays.  This file is collected
last so that, if it fails, a run that stops at the first failure has already
run every other test.
"""
import ctypes

import numpy as np
import pytest

from fdtd_method_gb300 import FDTD, _lib, build
from fdtd_method_gb300.sources import COURANT_DT, normalised_parameters

pytestmark = pytest.mark.gpu


def _device_out(torch):
    return torch.zeros(_lib.DIAG_COUNT, dtype=torch.float64, device="cuda")


def test_noalloc_field_sums_match_handle_entry_point_twice():
    torch = pytest.importorskip("torch")
    build.build()
    lib = _lib.load()
    p = normalised_parameters(70, 33, 29)
    sim = FDTD(p, COURANT_DT)
    rng = np.random.default_rng(123)
    for c in range(6):
        sim.get_field(c).assign(rng.standard_normal(p.cells))
    sim.step(2)
    want = sim.field_sums()

    ptrs = (ctypes.c_void_p * 6)(*[sim.get_field(c).device_ptr for c in range(6)])
    for _ in range(2):
        out = _device_out(torch)
        rc = lib.fdtd_field_sums_noalloc(ptrs, p.cells, ctypes.c_void_p(out.data_ptr()), None)
        assert rc == 0, lib.fdtd_last_error()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        np.testing.assert_allclose(got[:6], want[:6], rtol=1e-12)
        scale = float(np.abs(want[:6]).sum())
        np.testing.assert_allclose(got[6:9], want[6:9], rtol=1e-9, atol=1e-12 * scale)
        assert got[9] == want[9] == 0


def test_noalloc_many_partials_non_finite_values_and_a_stream():
    """128^3 cells give 512 block partials, so the second pass folds more
    slots than it has threads; NaN and Inf values are counted; the call runs
    on a stream of the caller's."""
    torch = pytest.importorskip("torch")
    build.build()
    lib = _lib.load()
    p = normalised_parameters(128, 128, 128)
    sim = FDTD(p, COURANT_DT)
    rng = np.random.default_rng(7)
    vals = [rng.standard_normal(p.cells) for _ in range(6)]
    for c in range(6):
        sim.get_field(c).assign(vals[c])
    want = sim.field_sums()
    ptrs = (ctypes.c_void_p * 6)(*[sim.get_field(c).device_ptr for c in range(6)])
    stream = torch.cuda.Stream()
    out = _device_out(torch)
    rc = lib.fdtd_field_sums_noalloc(ptrs, p.cells, ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0, lib.fdtd_last_error()
    stream.synchronize()
    got = out.cpu().numpy()
    np.testing.assert_allclose(got[:6], want[:6], rtol=1e-12)
    scale = float(np.abs(want[:6]).sum())
    np.testing.assert_allclose(got[6:9], want[6:9], rtol=1e-9, atol=1e-12 * scale)
    assert got[9] == 0
    vals[2][12345] = np.nan
    vals[4][0] = np.inf
    vals[4][p.cells - 1] = -np.inf
    sim.get_field(2).assign(vals[2])
    sim.get_field(4).assign(vals[4])
    sim.synchronize()
    rc = lib.fdtd_field_sums_noalloc(ptrs, p.cells, ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0, lib.fdtd_last_error()
    stream.synchronize()
    assert out.cpu().numpy()[9] == 3 == sim.field_sums()[9]


def test_noalloc_rejects_grids_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    build.build()
    lib = _lib.load()
    p = normalised_parameters(8, 8, 8)
    sim = FDTD(p, COURANT_DT)
    ptrs = (ctypes.c_void_p * 6)(*[sim.get_field(c).device_ptr for c in range(6)])
    out = _device_out(torch)
    rc = lib.fdtd_field_sums_noalloc(ptrs, 268435456 + 1, ctypes.c_void_p(out.data_ptr()), None)
    assert rc == _lib.FDTD_ERR_INVALID_ARGUMENT
    assert b"too large" in lib.fdtd_last_error()
