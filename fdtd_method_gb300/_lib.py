"""ctypes binding of the engine's C ABI (include/fdtd_gb300.h).

The shared library is built in-tree by ``fdtd_method_gb300.build``; there is
no fallback: if the library is missing or fails to load, every entry point
raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfdtd_gb300.so")

FDTD_OK = 0
FDTD_ERR_INVALID_ARGUMENT = -1
FDTD_ERR_LOGIC = -2
FDTD_ERR_CUDA = -3
FDTD_ERR_OUT_OF_MEMORY = -4
FDTD_ERR_UNSUPPORTED = -5
FDTD_ERR_TIMEOUT = -6

DIAG_COUNT = 10


class FDTDError(RuntimeError):
    """A failed engine call (CUDA error, unsupported operation, ...)."""

    def __init__(self, code, message):
        super().__init__(message)
        self.code = code


class InvalidArgument(FDTDError, ValueError):
    """The reference's std::invalid_argument."""


class LogicError(FDTDError):
    """The reference's std::logic_error."""


class OutOfMemory(FDTDError, MemoryError):
    pass


class Params(ctypes.Structure):
    _fields_ = [("Ni", ctypes.c_int), ("Nj", ctypes.c_int), ("Nk", ctypes.c_int),
                ("ax", ctypes.c_double), ("bx", ctypes.c_double),
                ("ay", ctypes.c_double), ("by", ctypes.c_double),
                ("az", ctypes.c_double), ("bz", ctypes.c_double),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double)]


class Source(ctypes.Structure):
    _fields_ = [("comp_mask", ctypes.c_int),
                ("i0", ctypes.c_int), ("j0", ctypes.c_int), ("k0", ctypes.c_int),
                ("ni", ctypes.c_int), ("nj", ctypes.c_int), ("nk", ctypes.c_int),
                ("gx", ctypes.POINTER(ctypes.c_double)),
                ("gy", ctypes.POINTER(ctypes.c_double)),
                ("gz", ctypes.POINTER(ctypes.c_double)),
                ("amp", ctypes.POINTER(ctypes.c_double)),
                ("n_amp", ctypes.c_int64)]


class TuneResult(ctypes.Structure):
    _fields_ = [("tile_y", ctypes.c_int), ("kchunk", ctypes.c_int), ("cells_per_thread", ctypes.c_int),
                ("ms_per_sweep", ctypes.c_double), ("candidates", ctypes.c_int), ("cached", ctypes.c_int),
                ("split_sources", ctypes.c_int), ("depth", ctypes.c_int)]


_H = ctypes.c_void_p
_D = ctypes.POINTER(ctypes.c_double)

# name -> argument types (every function returns int unless listed in _RESTYPES)
SIGNATURES = {
    "fdtd_last_error": [],
    "fdtd_abi_version": [],
    "fdtd_create": [ctypes.POINTER(Params), ctypes.c_double, ctypes.c_int, ctypes.POINTER(_H)],
    "fdtd_destroy": [_H],
    "fdtd_create_pml": [ctypes.POINTER(Params), ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.POINTER(_H)],
    "fdtd_get_pml": [_H, ctypes.POINTER(ctypes.c_int)],
    "fdtd_update_fields": [_H],
    "fdtd_step": [_H, ctypes.c_int64],
    "fdtd_zeroed_currents": [_H],
    "fdtd_get_field": [_H, ctypes.c_int, ctypes.POINTER(_D)],
    "fdtd_copy_field_to_host": [_H, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t],
    "fdtd_copy_field_from_host": [_H, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t],
    "fdtd_add_source": [_H, ctypes.POINTER(Source), ctypes.POINTER(ctypes.c_int)],
    "fdtd_export_field": [_H, ctypes.c_int, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p],
    "fdtd_clear_sources": [_H],
    "fdtd_get_step": [_H, ctypes.POINTER(ctypes.c_int64)],
    "fdtd_set_step": [_H, ctypes.c_int64],
    "fdtd_field_sums": [_H, _D],
    "fdtd_get_params": [_H, ctypes.POINTER(Params), _D, ctypes.POINTER(ctypes.c_int)],
    "fdtd_set_stream": [_H, ctypes.c_void_p],
    "fdtd_synchronize": [_H],
    "fdtd_set_fp16_exponents": [_H, ctypes.POINTER(ctypes.c_int)],
    "fdtd_set_fp64_arith": [_H, ctypes.c_int],
    "fdtd_get_fp16_exponents": [_H, ctypes.POINTER(ctypes.c_int)],
    "fdtd_fp16_autoscale": [_H, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int)],
    "fdtd_fp16_choose_exponents": [ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                   ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int)],
    "fdtd_set_fp16_autoscale": [_H, ctypes.c_int, ctypes.c_int, ctypes.c_int],
    "fdtd_set_wait_limit": [_H, ctypes.c_int64, ctypes.c_int],
    "fdtd_set_temporal_depth": [_H, ctypes.c_int],
    "fdtd_measure_fp64_rate": [_D, _D],
    "fdtd_set_kernel_timing": [_H, ctypes.c_int],
    "fdtd_kernel_times": [_H, _D, ctypes.POINTER(ctypes.c_int64)],
    "fdtd_set_pipeline": [_H, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int],
    "fdtd_autotune": [_H, ctypes.c_int, ctypes.c_int, ctypes.POINTER(TuneResult)],
    "fdtd_batch_autotune": [_H, ctypes.c_int, ctypes.POINTER(TuneResult)],
    "fdtd_field_sums_noalloc": [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p],
    # batched form
    "fdtd_batch_create": [ctypes.POINTER(Params), ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.POINTER(_H)],
    "fdtd_batch_destroy": [_H],
    "fdtd_batch_size": [_H, ctypes.POINTER(ctypes.c_int)],
    "fdtd_batch_domain_params": [_H, ctypes.c_int, ctypes.POINTER(Params)],
    "fdtd_batch_add_source": [_H, ctypes.c_int, ctypes.POINTER(Source), ctypes.POINTER(ctypes.c_int)],
    "fdtd_batch_copy_field_to_host": [_H, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t],
    "fdtd_batch_copy_field_from_host": [_H, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t],
    "fdtd_batch_field_sums": [_H, ctypes.c_int, _D],
    "fdtd_batch_set_fp16_exponents": [_H, ctypes.c_int, ctypes.POINTER(ctypes.c_int)],
    "fdtd_batch_set_config": [_H, ctypes.c_int, ctypes.c_int, ctypes.c_int],
    "fdtd_batch_step": [_H, ctypes.c_int64],
    "fdtd_batch_get_step": [_H, ctypes.POINTER(ctypes.c_int64)],
    "fdtd_batch_tiles": [_H, ctypes.POINTER(ctypes.c_int64)],
    "fdtd_batch_set_stream": [_H, ctypes.c_void_p],
    "fdtd_batch_synchronize": [_H],
    "fdtd_batch_set_split_sources": [_H, ctypes.c_int],
    # compact forms
    "fdtd_energy": [_H, _D],
    "fdtd_set_sources": [_H, ctypes.POINTER(Source), ctypes.c_int],
    "fdtd_field_device_ptr": [_H, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)],
    "fdtd_copy_field": [_H, ctypes.c_int, ctypes.c_void_p, ctypes.c_int],
    "fdtd_sync": [_H],
    # z slabs
    "fdtd_slab_create": [ctypes.POINTER(Params), ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                         ctypes.POINTER(_H)],
    "fdtd_slab_info": [_H, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)],
    "fdtd_slab_sweep": [_H, ctypes.c_int],
    "fdtd_slab_plane": [_H, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                        ctypes.POINTER(ctypes.c_size_t)],
    "fdtd_slab_exchange": [ctypes.POINTER(_H), ctypes.c_int, ctypes.c_int],
}
_RESTYPES = {"fdtd_last_error": ctypes.c_char_p}

_lib = None


def load():
    """Loads the engine library (once).  Raises if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise FDTDError(FDTD_ERR_UNSUPPORTED,
                        "engine library %s is missing: build it with "
                        "`python -c 'import __graft_entry__ as g; g.build()'`" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RESTYPES.get(name, ctypes.c_int)
    _lib = lib
    return lib


def check(rc):
    if rc == FDTD_OK:
        return
    msg = load().fdtd_last_error().decode(errors="replace")
    cls = {FDTD_ERR_INVALID_ARGUMENT: InvalidArgument, FDTD_ERR_LOGIC: LogicError,
           FDTD_ERR_OUT_OF_MEMORY: OutOfMemory}.get(rc, FDTDError)
    raise cls(rc, msg)
