"""Host-side mirror of the reference's FDTD solver class over the CUDA engine.

Reference surface (Amazingkivas/FDTD_Method):
  struct Parameters          include/Structures.h:23-38
  struct CurrentParameters   include/Structures.h:13-21
  struct SelectedFields      include/Structures.h:8-11
  enum class Component/Axis  include/Enums.h:5-6
  FDTD_const::C, PI, ...     include/Constants.h:4-12
  class FDTD                 include/FDTD_kokkos/FDTD_kokkos.h:7-36
    FDTD(Parameters, FP dt)  src/FDTD_kokkos/FDTD_kokkos.cpp:5-67
    zeroed_currents()        src/FDTD_kokkos/FDTD_kokkos.cpp:69-73
    get_field(Component)     src/FDTD_kokkos/FDTD_kokkos.cpp:75-89
    update_fields()          src/FDTD_kokkos/FDTD_kokkos.cpp:91-104

Same names, argument meaning and error behaviour: invalid parameters raise
``InvalidArgument`` (a ValueError; the reference throws
std::invalid_argument("ERROR: invalid parameters")), an invalid component
raises ``LogicError`` (std::logic_error("ERROR: Invalid field component")).
All work runs through the C ABI of ``libfdtd_gb300.so``; nothing here
computes fields.
"""
import ctypes
import enum
from dataclasses import dataclass, field as dc_field

import numpy as np

from . import _lib
from ._lib import FDTDError, InvalidArgument, LogicError, OutOfMemory  # noqa: F401


class Const:
    """FDTD_const (include/Constants.h:4-12)."""
    C = 3e10
    R = 1e-12
    EPS0 = 1.0
    MU0 = 1.0
    N = 4.0
    PI = 3.14159265358


class Component(enum.IntEnum):
    EX = 0
    EY = 1
    EZ = 2
    BX = 3
    BY = 4
    BZ = 5
    JX = 6
    JY = 7
    JZ = 8


class Axis(enum.IntEnum):
    X = 0
    Y = 1
    Z = 2


class Precision(enum.IntEnum):
    FP64 = 0          # the drop-in: bit-identical to the reference
    FP32 = 1
    FP32_COMP = 2     # FP32 hi + BF16 lo compensated storage
    FP16_SCALED = 3   # FP16 storage, power-of-two scale per component


def fp16_choose_exponents(peaks, current, target_log2=10, headroom_log2=5, force=False):
    """The FP16 form's exponent rule on the host (fdtd_fp16_choose_exponents):
    from the six stored peaks (largest |stored value| per component; 0, Inf
    or NaN count as no field) and the current exponents, the exponents a scan
    re-encodes to."""
    lib = _lib.load()
    pk = (ctypes.c_float * 6)(*[float(v) for v in peaks])
    cur = (ctypes.c_int * 6)(*[int(e) for e in current])
    out = (ctypes.c_int * 6)()
    _lib.check(lib.fdtd_fp16_choose_exponents(pk, cur, int(target_log2), int(headroom_log2), 1 if force else 0, out))
    return list(out)


@dataclass
class Parameters:
    Ni: int
    Nj: int
    Nk: int
    ax: float
    bx: float
    ay: float
    by: float
    az: float
    bz: float
    dx: float
    dy: float
    dz: float

    def to_c(self):
        return _lib.Params(int(self.Ni), int(self.Nj), int(self.Nk),
                           float(self.ax), float(self.bx), float(self.ay), float(self.by),
                           float(self.az), float(self.bz),
                           float(self.dx), float(self.dy), float(self.dz))

    @property
    def cells(self):
        return int(self.Ni) * int(self.Nj) * int(self.Nk)


@dataclass
class SelectedFields:
    selected_E: Component
    selected_B: Component


@dataclass
class CurrentParameters:
    """include/Structures.h:13-21; period_* default to m * C as there."""
    period: int
    m: int
    dt: float
    iterations: int = 0
    period_x: float = None
    period_y: float = None
    period_z: float = None

    def __post_init__(self):
        for a in ("period_x", "period_y", "period_z"):
            if getattr(self, a) is None:
                setattr(self, a, float(self.m) * Const.C)


@dataclass
class SeparableSource:
    """A current source J_c(i,j,k,s) += amp[s] * gx[di] * gy[dj] * gz[dk] in a
    periodic box at (i0, j0, k0) of extent len(gx) x len(gy) x len(gz), for the
    components in comp_mask (bit 0 Jx, 1 Jy, 2 Jz).  See fdtd_source in
    include/fdtd_gb300.h."""
    comp_mask: int
    i0: int
    j0: int
    k0: int
    gx: np.ndarray
    gy: np.ndarray
    gz: np.ndarray
    amp: np.ndarray
    meta: dict = dc_field(default_factory=dict)

    def to_c(self):
        keep = [np.ascontiguousarray(a, dtype=np.float64) for a in (self.gx, self.gy, self.gz, self.amp)]
        ptr = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        s = _lib.Source(int(self.comp_mask), int(self.i0), int(self.j0), int(self.k0),
                        len(keep[0]), len(keep[1]), len(keep[2]),
                        ptr(keep[0]), ptr(keep[1]), ptr(keep[2]), ptr(keep[3]), len(keep[3]))
        return s, keep


class Field:
    """Handle to one component of a solver's state (the reference's
    Kokkos::View member).  It aliases the solver's storage: ``numpy()`` is the
    host mirror + deep_copy, ``assign()`` the copy back.  For the FP64 form
    ``device_ptr`` is the device address (and ``__cuda_array_interface__``
    lets array libraries wrap it without a copy)."""

    def __init__(self, solver, comp):
        self._solver = solver
        self.comp = Component(comp)

    def size(self):
        return self._solver.parameters.cells

    def __len__(self):
        return self.size()

    @property
    def device_ptr(self):
        return self._solver._device_ptr(self.comp)

    @property
    def __cuda_array_interface__(self):
        return {"shape": (self.size(),), "typestr": "<f8", "data": (self.device_ptr, False),
                "version": 3, "strides": None, "stream": None}

    def numpy(self, out=None):
        return self._solver.copy_to_host(self.comp, out)

    def assign(self, values):
        self._solver.copy_from_host(self.comp, values)


class FDTD:
    """Drop-in for FDTD_kokkos::FDTD on one GPU."""

    def __init__(self, parameters, dt, precision=Precision.FP64):
        self._h = None
        lib = _lib.load()
        self.parameters = parameters
        self.dt = float(dt)
        self.precision = Precision(precision)
        p = parameters.to_c()
        h = ctypes.c_void_p()
        _lib.check(lib.fdtd_create(ctypes.byref(p), self.dt, int(self.precision), ctypes.byref(h)))
        self._h = h
        self._lib = lib
        self._sources = []

    # -- lifetime -----------------------------------------------------------
    def close(self):
        if self._h is not None:
            self._lib.fdtd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _handle(self):
        if self._h is None:
            raise FDTDError(_lib.FDTD_ERR_INVALID_ARGUMENT, "solver is closed")
        return self._h

    # -- the reference's API ----------------------------------------------
    def get_field(self, comp):
        c = int(comp)
        if c < 0 or c > 8:
            raise LogicError(_lib.FDTD_ERR_LOGIC, "ERROR: Invalid field component")
        return Field(self, c)

    def update_fields(self):
        _lib.check(self._lib.fdtd_update_fields(self._handle()))

    def zeroed_currents(self):
        _lib.check(self._lib.fdtd_zeroed_currents(self._handle()))

    # -- extensions ---------------------------------------------------------
    def step(self, n):
        """n consecutive update_fields() calls."""
        _lib.check(self._lib.fdtd_step(self._handle(), int(n)))

    def synchronize(self):
        """Kokkos::fence() equivalent."""
        _lib.check(self._lib.fdtd_synchronize(self._handle()))

    def _device_ptr(self, comp):
        ptr = ctypes.POINTER(ctypes.c_double)()
        _lib.check(self._lib.fdtd_get_field(self._handle(), int(comp), ctypes.byref(ptr)))
        return ctypes.cast(ptr, ctypes.c_void_p).value

    def copy_to_host(self, comp, out=None):
        n = self.parameters.cells
        if out is None:
            out = np.empty(n, dtype=np.float64)
        if out.dtype != np.float64 or out.size != n or not out.flags.c_contiguous:
            raise InvalidArgument(_lib.FDTD_ERR_INVALID_ARGUMENT, "output must be a contiguous float64 array of Ni*Nj*Nk")
        _lib.check(self._lib.fdtd_copy_field_to_host(self._handle(), int(comp), out.ctypes.data, n))
        return out

    def copy_from_host(self, comp, values):
        n = self.parameters.cells
        a = np.ascontiguousarray(values, dtype=np.float64).reshape(-1)
        if a.size != n:
            raise InvalidArgument(_lib.FDTD_ERR_INVALID_ARGUMENT, "expected %d values, got %d" % (n, a.size))
        _lib.check(self._lib.fdtd_copy_field_from_host(self._handle(), int(comp), a.ctypes.data, n))

    def export_field(self, comp, offset, count, device_ptr):
        """FP64 values of E/B component `comp` at flat cells offset ..
        offset+count-1 into device memory at `device_ptr` (asynchronous on the
        solver's stream; synchronize() before reading them elsewhere)."""
        _lib.check(self._lib.fdtd_export_field(self._handle(), int(comp), int(offset), int(count),
                                               ctypes.c_void_p(int(device_ptr))))

    def add_source(self, src):
        c, keep = src.to_c()
        idx = ctypes.c_int()
        _lib.check(self._lib.fdtd_add_source(self._handle(), ctypes.byref(c), ctypes.byref(idx)))
        self._sources.append(src)
        return idx.value

    def clear_sources(self):
        _lib.check(self._lib.fdtd_clear_sources(self._handle()))
        self._sources = []

    @property
    def step_index(self):
        v = ctypes.c_int64()
        _lib.check(self._lib.fdtd_get_step(self._handle(), ctypes.byref(v)))
        return v.value

    @step_index.setter
    def step_index(self, value):
        _lib.check(self._lib.fdtd_set_step(self._handle(), int(value)))

    def field_sums(self):
        """FP64 sums over all cells: [Ex^2, Ey^2, Ez^2, Bx^2, By^2, Bz^2,
        (ExB)_x, (ExB)_y, (ExB)_z, non-finite count]."""
        out = (ctypes.c_double * _lib.DIAG_COUNT)()
        _lib.check(self._lib.fdtd_field_sums(self._handle(), out))
        return np.array(out[:], dtype=np.float64)

    def energy(self):
        """Total field energy (E^2 + B^2) dV / (8 pi), Gaussian units."""
        s = self.field_sums()
        p = self.parameters
        return float(s[:6].sum() * p.dx * p.dy * p.dz / (8.0 * Const.PI))

    def poynting(self):
        """Volume integral of the Poynting vector c/(4 pi) E x B (E and B taken
        at their own staggered points)."""
        s = self.field_sums()
        p = self.parameters
        return s[6:9] * Const.C * p.dx * p.dy * p.dz / (4.0 * Const.PI)

    def set_fp16_exponents(self, exps):
        arr = (ctypes.c_int * 6)(*[int(e) for e in exps])
        _lib.check(self._lib.fdtd_set_fp16_exponents(self._handle(), arr))

    def fp16_exponents(self):
        arr = (ctypes.c_int * 6)()
        _lib.check(self._lib.fdtd_get_fp16_exponents(self._handle(), arr))
        return list(arr)

    def fp16_autoscale(self, target_log2=10, headroom_log2=5):
        """FP16 form: choose every component's exponent now (peak at
        2^target, at most 2^headroom above the strongest component's scale;
        see fdtd_fp16_autoscale); returns the exponents."""
        arr = (ctypes.c_int * 6)()
        _lib.check(self._lib.fdtd_fp16_autoscale(self._handle(), int(target_log2), int(headroom_log2), arr))
        return list(arr)

    def set_fp16_autoscale(self, every_steps, target_log2=10, headroom_log2=5):
        """FP16 form: step() rescans the stored peaks every `every_steps`
        steps (0: never) and re-encodes components whose exponent drifted
        from the wanted one (fdtd_set_fp16_autoscale)."""
        _lib.check(self._lib.fdtd_set_fp16_autoscale(self._handle(), int(every_steps), int(target_log2),
                                                     int(headroom_log2)))

    def set_fp64_arith(self, contracted):
        """FP64 form: False keeps the reference's arithmetic bit for bit (the
        default); True accumulates each curl and current term with DFMA
        (fewer FP64 instructions; within a few ulps per step)."""
        _lib.check(self._lib.fdtd_set_fp64_arith(self._handle(), 1 if contracted else 0))

    def set_wait_limit(self, polls=0, withhold_loads=False):
        """Test hook of the bounded device waits (fdtd_set_wait_limit): waits
        give up after `polls` polls (0: the default); withhold_loads makes the
        fused sweeps issue no tile loads, so every wait gives up."""
        _lib.check(self._lib.fdtd_set_wait_limit(self._handle(), int(polls), 1 if withhold_loads else 0))

    KERNEL_KINDS = ("e_update", "b_half", "b_double", "fused_step", "fused_step2")
    PIPELINES = {"auto": 0, "split": 1, "fused": 2}

    def set_pipeline(self, pipeline="auto", tile_y=0, kchunk=0, cells_per_thread=0):
        """Step pipeline of the FP32-arithmetic forms: 'fused' (one sweep per
        step, the default) or 'split' (one sweep per half step); same results.
        tile_y (6, 14 or 30), kchunk and cells_per_thread (1 or 2) shape the fused
        launch; 0 keeps the default."""
        _lib.check(self._lib.fdtd_set_pipeline(self._handle(), self.PIPELINES[pipeline], int(tile_y), int(kchunk),
                                               int(cells_per_thread)))

    def autotune(self, sweeps=10, reuse=True):
        """Times every candidate launch shape of the fused sweep on this grid
        (the state is only read) and keeps the fastest.  Returns the choice
        as a dict; results are cached per (precision, grid) in the process."""
        r = _lib.TuneResult()
        _lib.check(self._lib.fdtd_autotune(self._handle(), int(sweeps), 1 if reuse else 0, ctypes.byref(r)))
        return {"tile_y": r.tile_y, "kchunk": r.kchunk, "cells_per_thread": r.cells_per_thread, "depth": r.depth,
                "ms_per_step": r.ms_per_sweep, "candidates": r.candidates, "cached": bool(r.cached)}

    def set_temporal_depth(self, depth):
        """Steps per pass over the state: 1, or 2 (temporal blocking; same
        bits).  See fdtd_set_temporal_depth."""
        _lib.check(self._lib.fdtd_set_temporal_depth(self._handle(), int(depth)))

    def set_kernel_timing(self, enabled):
        """Bracket every step-pipeline kernel launch with CUDA events."""
        _lib.check(self._lib.fdtd_set_kernel_timing(self._handle(), 1 if enabled else 0))

    def kernel_times(self):
        """{kind: (total ms, launches)} since the previous call."""
        ms = (ctypes.c_double * len(self.KERNEL_KINDS))()
        n = (ctypes.c_int64 * len(self.KERNEL_KINDS))()
        _lib.check(self._lib.fdtd_kernel_times(self._handle(), ms, n))
        return {k: (ms[q], n[q]) for q, k in enumerate(self.KERNEL_KINDS)}

    def set_stream(self, stream_handle):
        _lib.check(self._lib.fdtd_set_stream(self._handle(), ctypes.c_void_p(int(stream_handle or 0))))

    def coefficients(self):
        """The reference's coefficients (src/FDTD_kokkos/FDTD_kokkos.cpp:45-55)."""
        p, dt = self.parameters, self.dt
        cdt = Const.C * dt
        return {"coef_E": (cdt / p.dx, cdt / p.dy, cdt / p.dz),
                "coef_B": (cdt / (2.0 * p.dx), cdt / (2.0 * p.dy), cdt / (2.0 * p.dz)),
                "current_coef": -4.0 * Const.PI * dt}


def measure_fp64_rate():
    """Issue rate of the current GPU's FP64 pipe (DMUL/DADD instructions per
    second) and the probe's duration in ms (fdtd_measure_fp64_rate)."""
    lib = _lib.load()
    rate, ms = ctypes.c_double(), ctypes.c_double()
    _lib.check(lib.fdtd_measure_fp64_rate(ctypes.byref(rate), ctypes.byref(ms)))
    return rate.value, ms.value


class FDTD_PML(FDTD):
    """Drop-in for FDTD_kokkos::FDTD_PML (include/FDTD_kokkos/FDTD_PML_kokkos.h:10-33,
    src/FDTD_kokkos/FDTD_PML_kokkos.cpp): the solver with a split-field
    absorbing layer of (int)(N * pml_percent) cells on every face.
    update_fields follows FDTD_PML::update_fields (FP64, bit-identical to the
    reference)."""

    def __init__(self, parameters, dt, pml_percent):
        self._h = None
        lib = _lib.load()
        self.parameters = parameters
        self.dt = float(dt)
        self.precision = Precision.FP64
        self.pml_percent = float(pml_percent)
        p = parameters.to_c()
        h = ctypes.c_void_p()
        _lib.check(lib.fdtd_create_pml(ctypes.byref(p), self.dt, self.pml_percent, int(Precision.FP64),
                                       ctypes.byref(h)))
        self._h = h
        self._lib = lib
        self._sources = []

    @property
    def pml_size(self):
        """Layer thickness (cells) along x, y, z."""
        out = (ctypes.c_int * 3)()
        _lib.check(self._lib.fdtd_get_pml(self._handle(), out))
        return list(out)


class FDTDBatch:
    """Many independent periodic domains advanced together on one GPU (the
    batched form; the reference advances one grid per object).  Every domain
    has its own Parameters and sources and the same dt and precision (FP32,
    FP32_COMP or FP16_SCALED).  ``step(n)`` advances all domains by n steps:
    one persistent kernel launch per fused sweep works through the tile table
    of every domain, and the step group runs as one CUDA graph.  Each domain's
    results equal those of a single FDTD of the same form run alone."""

    def __init__(self, parameters, dt, precision=Precision.FP32_COMP):
        self._b = None
        lib = _lib.load()
        self.parameters = list(parameters)
        self.dt = float(dt)
        self.precision = Precision(precision)
        arr = (_lib.Params * len(self.parameters))(*[p.to_c() for p in self.parameters])
        b = ctypes.c_void_p()
        _lib.check(lib.fdtd_batch_create(arr, len(self.parameters), self.dt, int(self.precision), ctypes.byref(b)))
        self._b = b
        self._lib = lib

    def close(self):
        if self._b is not None:
            self._lib.fdtd_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __len__(self):
        return len(self.parameters)

    def _handle(self):
        if self._b is None:
            raise FDTDError(_lib.FDTD_ERR_INVALID_ARGUMENT, "batch is closed")
        return self._b

    def _params(self, domain):
        if not 0 <= int(domain) < len(self.parameters):
            raise InvalidArgument(_lib.FDTD_ERR_INVALID_ARGUMENT, "domain index out of range")
        return self.parameters[int(domain)]

    def add_source(self, domain, src):
        self._params(domain)
        c, keep = src.to_c()
        idx = ctypes.c_int()
        _lib.check(self._lib.fdtd_batch_add_source(self._handle(), int(domain), ctypes.byref(c), ctypes.byref(idx)))
        return idx.value

    def copy_to_host(self, domain, comp, out=None):
        n = self._params(domain).cells
        if out is None:
            out = np.empty(n, dtype=np.float64)
        if out.dtype != np.float64 or out.size != n or not out.flags.c_contiguous:
            raise InvalidArgument(_lib.FDTD_ERR_INVALID_ARGUMENT, "output must be a contiguous float64 array of Ni*Nj*Nk")
        _lib.check(self._lib.fdtd_batch_copy_field_to_host(self._handle(), int(domain), int(comp), out.ctypes.data, n))
        return out

    def copy_from_host(self, domain, comp, values):
        n = self._params(domain).cells
        a = np.ascontiguousarray(values, dtype=np.float64).reshape(-1)
        if a.size != n:
            raise InvalidArgument(_lib.FDTD_ERR_INVALID_ARGUMENT, "expected %d values, got %d" % (n, a.size))
        _lib.check(self._lib.fdtd_batch_copy_field_from_host(self._handle(), int(domain), int(comp), a.ctypes.data, n))

    def field_sums(self, domain):
        out = (ctypes.c_double * _lib.DIAG_COUNT)()
        _lib.check(self._lib.fdtd_batch_field_sums(self._handle(), int(domain), out))
        return np.array(out[:], dtype=np.float64)

    def energy(self, domain):
        s = self.field_sums(domain)
        p = self._params(domain)
        return float(s[:6].sum() * p.dx * p.dy * p.dz / (8.0 * Const.PI))

    def set_fp16_exponents(self, domain, exps):
        arr = (ctypes.c_int * 6)(*[int(e) for e in exps])
        _lib.check(self._lib.fdtd_batch_set_fp16_exponents(self._handle(), int(domain), arr))

    def set_config(self, tile_y=0, kchunk=0, graphs=True):
        _lib.check(self._lib.fdtd_batch_set_config(self._handle(), int(tile_y), int(kchunk), 1 if graphs else 0))

    def set_split_sources(self, on):
        """Compile the sweep's plane loop twice and run the source-free copy on
        tiles no source reaches (see fdtd_batch_set_split_sources)."""
        _lib.check(self._lib.fdtd_batch_set_split_sources(self._handle(), 1 if on else 0))

    def step(self, n):
        _lib.check(self._lib.fdtd_batch_step(self._handle(), int(n)))

    def autotune(self, sweeps=5):
        """Times the persistent fused sweep for every candidate tile shape,
        with the plane loop compiled once or split (the state is only read),
        and keeps the fastest."""
        r = _lib.TuneResult()
        _lib.check(self._lib.fdtd_batch_autotune(self._handle(), int(sweeps), ctypes.byref(r)))
        return {"tile_y": r.tile_y, "kchunk": r.kchunk, "ms_per_sweep": r.ms_per_sweep,
                "candidates": r.candidates, "split_sources": bool(r.split_sources)}

    def synchronize(self):
        _lib.check(self._lib.fdtd_batch_synchronize(self._handle()))

    def set_stream(self, stream_handle):
        _lib.check(self._lib.fdtd_batch_set_stream(self._handle(), ctypes.c_void_p(int(stream_handle or 0))))

    @property
    def step_index(self):
        v = ctypes.c_int64()
        _lib.check(self._lib.fdtd_batch_get_step(self._handle(), ctypes.byref(v)))
        return v.value

    def tiles(self):
        v = ctypes.c_int64()
        _lib.check(self._lib.fdtd_batch_tiles(self._handle(), ctypes.byref(v)))
        return v.value
