"""The C-ABI library: it builds for sm_103a, loads, exports every symbol
include/fdtd_gb300.h declares, and validates arguments on the host before any
GPU work (so these run without a GPU)."""
import ctypes
import os
import re

import pytest

from fdtd_method_gb300 import FDTD, InvalidArgument, Parameters, Precision, _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fdtd_gb300.h")


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(fdtd_\w+)\s*\(", text, re.M)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("fdtd_create", "fdtd_destroy", "fdtd_update_fields", "fdtd_step",
                     "fdtd_zeroed_currents", "fdtd_get_field", "fdtd_copy_field_to_host",
                     "fdtd_copy_field_from_host", "fdtd_add_source", "fdtd_field_sums",
                     "fdtd_synchronize", "fdtd_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_abi_version(lib):
    assert lib.fdtd_abi_version() == 1


@pytest.mark.parametrize("dims,dt", [((0, 4, 4), 1e-12), ((4, 0, 4), 1e-12), ((4, 4, -2), 1e-12),
                                     ((4, 4, 4), 0.0), ((4, 4, 4), -1.0)])
def test_invalid_parameters_raise_like_the_reference(lib, dims, dt):
    # src/FDTD_kokkos/FDTD_kokkos.cpp:7-12 throws std::invalid_argument("ERROR: invalid parameters")
    p = Parameters(*dims, 0, 1, 0, 1, 0, 1, 0.25, 0.25, 0.25)
    with pytest.raises(InvalidArgument, match="ERROR: invalid parameters"):
        FDTD(p, dt)
    with pytest.raises(ValueError):
        FDTD(p, dt)


def test_invalid_precision_rejected(lib):
    p = Parameters(4, 4, 4, 0, 1, 0, 1, 0, 1, 0.25, 0.25, 0.25)
    h = ctypes.c_void_p()
    cp = p.to_c()
    assert lib.fdtd_create(ctypes.byref(cp), 1e-12, 7, ctypes.byref(h)) == _lib.FDTD_ERR_INVALID_ARGUMENT
    assert b"precision" in lib.fdtd_last_error()


def test_null_handle_calls_fail_cleanly(lib):
    assert lib.fdtd_step(None, 1) == _lib.FDTD_ERR_INVALID_ARGUMENT
    assert lib.fdtd_update_fields(None) == _lib.FDTD_ERR_INVALID_ARGUMENT
    assert lib.fdtd_destroy(None) == 0
    assert Precision.FP32_COMP == 2


def test_batch_arguments_checked_before_gpu_work(lib):
    p = Parameters(4, 4, 4, 0, 1, 0, 1, 0, 1, 0.25, 0.25, 0.25)
    arr = (_lib.Params * 1)(p.to_c())
    b = ctypes.c_void_p()
    assert lib.fdtd_batch_create(arr, 0, 1e-12, 2, ctypes.byref(b)) == _lib.FDTD_ERR_INVALID_ARGUMENT
    assert lib.fdtd_batch_create(arr, 1, 1e-12, 0, ctypes.byref(b)) == _lib.FDTD_ERR_UNSUPPORTED
    assert b"FP32" in lib.fdtd_last_error()
    assert lib.fdtd_batch_step(None, 1) == _lib.FDTD_ERR_INVALID_ARGUMENT
    assert lib.fdtd_batch_destroy(None) == 0


def test_pml_arguments_checked_before_gpu_work(lib):
    p = Parameters(8, 8, 8, 0, 1, 0, 1, 0, 1, 0.125, 0.125, 0.125).to_c()
    h = ctypes.c_void_p()
    for bad in (-0.1, 0.5, 0.7, float("nan")):
        assert lib.fdtd_create_pml(ctypes.byref(p), 1e-12, bad, 0, ctypes.byref(h)) == _lib.FDTD_ERR_INVALID_ARGUMENT
    assert lib.fdtd_create_pml(ctypes.byref(p), 1e-12, 0.2, 2, ctypes.byref(h)) == _lib.FDTD_ERR_UNSUPPORTED
    assert b"FP64" in lib.fdtd_last_error()


def test_slice_csv_matches_the_plotting_script_format(tmp_path):
    """OutFiles_<n>/<iteration>.csv as python_script_legend/visualization.py
    reads it: ';' separator, decimal comma, a header row."""
    import numpy as np

    from fdtd_method_gb300 import slices
    from fdtd_method_gb300.fdtd import Component

    p = Parameters(5, 4, 3, 0, 1, 0, 1, 0, 1, 0.2, 0.25, 0.33)
    values = np.arange(p.cells, dtype=np.float64) * -0.125

    class Stub:  # stands in for a solver: only get_field(c).numpy() is used
        parameters = p

        def get_field(self, c):
            return type("F", (), {"numpy": lambda self_: values})()

    path = slices.write_slice_csv(Stub(), Component.EY, 17, root=str(tmp_path))
    assert path.endswith(os.path.join("OutFiles_2", "17.csv"))
    lines = open(path).read().splitlines()
    assert lines[0].split(";") == ["0", "1", "2", "3", "4"]
    table = np.array([[float(x.replace(",", ".")) for x in ln.split(";")] for ln in lines[1:]])
    np.testing.assert_array_equal(table, values.reshape(3, 4, 5)[1])


def test_slab_and_compact_arguments_checked_before_gpu_work(lib):
    p = Parameters(8, 8, 12, 0, 1, 0, 1, 0, 1, 0.25, 0.25, 0.25).to_c()
    h = ctypes.c_void_p()
    # plane range outside the grid, or empty
    for k0, k1 in ((0, 13), (5, 5), (-1, 4)):
        assert lib.fdtd_slab_create(ctypes.byref(p), 1e-12, 0, k0, k1, ctypes.byref(h)) == _lib.FDTD_ERR_INVALID_ARGUMENT
    assert b"k_begin" in lib.fdtd_last_error()
    bad = _lib.Params(0, 8, 8, 0, 1, 0, 1, 0, 1, 0.25, 0.25, 0.25)
    assert lib.fdtd_slab_create(ctypes.byref(bad), 1e-12, 0, 0, 4, ctypes.byref(h)) == _lib.FDTD_ERR_INVALID_ARGUMENT
    assert lib.fdtd_last_error() == b"ERROR: invalid parameters"
    # exchange: no slabs, a null slab, a bad halo kind
    assert lib.fdtd_slab_exchange(None, 0, 0) == _lib.FDTD_ERR_INVALID_ARGUMENT
    arr = (ctypes.c_void_p * 1)(None)
    assert lib.fdtd_slab_exchange(arr, 1, 0) == _lib.FDTD_ERR_INVALID_ARGUMENT
    assert lib.fdtd_slab_exchange(arr, 1, 5) == _lib.FDTD_ERR_INVALID_ARGUMENT
    # compact forms and the batch loop switch on null handles
    out = (ctypes.c_double * 3)()
    assert lib.fdtd_energy(None, out) == _lib.FDTD_ERR_INVALID_ARGUMENT
    assert lib.fdtd_set_sources(None, None, 0) == _lib.FDTD_ERR_INVALID_ARGUMENT
    assert lib.fdtd_copy_field(None, 0, None, 0) == _lib.FDTD_ERR_INVALID_ARGUMENT
    assert lib.fdtd_sync(None) == _lib.FDTD_ERR_INVALID_ARGUMENT
    assert lib.fdtd_slab_sweep(None, 0) == _lib.FDTD_ERR_INVALID_ARGUMENT
    assert lib.fdtd_batch_set_split_sources(None, 1) == _lib.FDTD_ERR_INVALID_ARGUMENT
