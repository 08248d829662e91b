"""ctypes access to the oracle (test infrastructure only).

``Oracle`` runs the C restatement in fdtd_oracle.c (each function there cites
the reference file:line it restates); ``OraclePML`` its PML subclass.  ``RefKokkos`` drives the reference's own
FDTD_kokkos::FDTD compiled from its sources in oracle/_ref (present only where
the reference checkout was available to build it).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_LIB = os.path.join(REF_DIR, "libfdtd_ref.so")

_D = ctypes.POINTER(ctypes.c_double)


class OracleParams(ctypes.Structure):
    _fields_ = [("Ni", ctypes.c_int), ("Nj", ctypes.c_int), ("Nk", ctypes.c_int),
                ("ax", ctypes.c_double), ("bx", ctypes.c_double),
                ("ay", ctypes.c_double), ("by", ctypes.c_double),
                ("az", ctypes.c_double), ("bz", ctypes.c_double),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double)]


class OracleSource(ctypes.Structure):
    _fields_ = [("comp_mask", ctypes.c_int),
                ("i0", ctypes.c_int), ("j0", ctypes.c_int), ("k0", ctypes.c_int),
                ("ni", ctypes.c_int), ("nj", ctypes.c_int), ("nk", ctypes.c_int),
                ("gx", _D), ("gy", _D), ("gz", _D), ("amp", _D), ("n_amp", ctypes.c_long)]


class OracleBox(ctypes.Structure):
    _fields_ = [(n, ctypes.c_long) for n in ("i0", "i1", "j0", "j1", "k0", "k1")]


def build_oracle(force=False):
    """Compiles liboracle.so (and nothing else) with the oracle's Makefile."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(os.path.join(HERE, "fdtd_oracle.c")):
        subprocess.run(["make", "-C", HERE, "liboracle.so"], check=True, capture_output=True)
    return LIB


_olib = None
_rlib = None


def oracle_lib():
    global _olib
    if _olib is None:
        build_oracle()
        lib = ctypes.CDLL(LIB)
        lib.oracle_coefficients.argtypes = [ctypes.POINTER(OracleParams), ctypes.c_double, _D]
        lib.oracle_coefficients.restype = ctypes.c_int
        lib.oracle_run.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_long, ctypes.POINTER(_D), _D,
                                   ctypes.POINTER(OracleSource), ctypes.c_int, ctypes.c_long, ctypes.c_int,
                                   ctypes.POINTER(_D)]
        lib.oracle_run.restype = None
        lib.oracle_run_driver.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_long, ctypes.POINTER(_D), _D,
                                          ctypes.POINTER(OracleSource), ctypes.c_int, ctypes.c_long, ctypes.c_int]
        lib.oracle_run_driver.restype = None
        lib.oracle_twin_run.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_long, ctypes.POINTER(_D), _D,
                                        ctypes.c_int]
        lib.oracle_twin_run.restype = None
        lib.oracle_pml_sizes.argtypes = [ctypes.POINTER(OracleParams), ctypes.c_double, ctypes.POINTER(ctypes.c_int)]
        lib.oracle_pml_sizes.restype = None
        lib.oracle_pml_sigma.argtypes = [ctypes.POINTER(OracleParams), ctypes.c_double, _D, _D, _D]
        lib.oracle_pml_sigma.restype = None
        lib.oracle_pml_run.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_long, ctypes.POINTER(_D), _D,
                                       ctypes.POINTER(ctypes.c_int), ctypes.POINTER(_D), ctypes.c_double,
                                       ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.POINTER(_D),
                                       ctypes.POINTER(OracleSource), ctypes.c_int, ctypes.c_long, ctypes.c_int,
                                       ctypes.POINTER(_D)]
        lib.oracle_pml_run.restype = None
        for name in ("oracle_update_B_box",):
            getattr(lib, name).argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_long, OracleBox] + [_D] * 6 + \
                [ctypes.c_double] * 3
            getattr(lib, name).restype = None
        lib.oracle_update_E_box.argtypes = [ctypes.c_long, ctypes.c_long, ctypes.c_long, OracleBox] + [_D] * 9 + \
            [ctypes.c_double] * 4
        lib.oracle_update_E_box.restype = None
        lib.oracle_field_sums.argtypes = [ctypes.c_long, ctypes.POINTER(_D), _D]
        lib.oracle_field_sums.restype = None
        lib.oracle_threads.restype = ctypes.c_int
        _olib = lib
    return _olib


def _ptr(a):
    return a.ctypes.data_as(_D)


def coefficients(params, dt):
    """[cEx, cEy, cEz, cBx, cBy, cBz, cJ] or raises ValueError like the
    reference's constructor."""
    p = OracleParams(params.Ni, params.Nj, params.Nk, params.ax, params.bx, params.ay, params.by,
                     params.az, params.bz, params.dx, params.dy, params.dz)
    out = np.zeros(7)
    if oracle_lib().oracle_coefficients(ctypes.byref(p), float(dt), _ptr(out)) != 0:
        raise ValueError("ERROR: invalid parameters")
    return out


def field_sums(fields):
    """Compensated FP64 sums: see oracle_field_sums in fdtd_oracle.c."""
    arrs = [np.ascontiguousarray(f, dtype=np.float64) for f in fields[:6]]
    ptrs = (_D * 6)(*[_ptr(a) for a in arrs])
    out = np.zeros(10)
    oracle_lib().oracle_field_sums(arrs[0].size, ptrs, _ptr(out))
    return out


class Oracle:
    """The reference's FDTD state and update, restated in C (fdtd_oracle.c).
    fields: dict component-index -> flat float64 array of Ni*Nj*Nk."""

    def __init__(self, params, dt, with_current=True):
        self.params = params
        self.dt = float(dt)
        self.coef = coefficients(params, dt)
        n = params.Ni * params.Nj * params.Nk
        self.f = [np.zeros(n) for _ in range(6)] + ([np.zeros(n) for _ in range(3)] if with_current else [None] * 3)
        self.sources = []
        self.step_index = 0
        self._jwork = None

    def set(self, comp, values):
        a = np.ascontiguousarray(values, dtype=np.float64).reshape(-1)
        if self.f[int(comp)] is None:
            self.f[int(comp)] = np.zeros_like(self.f[0])
        self.f[int(comp)][...] = a

    def get(self, comp):
        f = self.f[int(comp)]
        return np.zeros_like(self.f[0]) if f is None else f.copy()

    def add_source(self, src):
        self.sources.append(src)

    def _csources(self):
        keep = []
        csrc = (OracleSource * max(1, len(self.sources)))()
        for q, s in enumerate(self.sources):
            arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (s.gx, s.gy, s.gz, s.amp)]
            keep.append(arrs)
            csrc[q] = OracleSource(s.comp_mask, s.i0, s.j0, s.k0, len(arrs[0]), len(arrs[1]), len(arrs[2]),
                                   _ptr(arrs[0]), _ptr(arrs[1]), _ptr(arrs[2]), _ptr(arrs[3]), len(arrs[3]))
        return csrc, keep

    def step_driver(self, n=1):
        """The reference sample driver's loop: sources written into their
        boxes of the dense J arrays, then update_fields (oracle_run_driver)."""
        p = self.params
        for c in range(6, 9):
            if self.f[c] is None:
                self.f[c] = np.zeros_like(self.f[0])
        ptrs = (_D * 9)(*[_ptr(a) for a in self.f])
        csrc, keep = self._csources()
        oracle_lib().oracle_run_driver(p.Ni, p.Nj, p.Nk, ptrs, _ptr(self.coef), csrc, len(self.sources),
                                       self.step_index, int(n))
        self.step_index += int(n)

    def step_twin(self, n=1):
        """n update_fields of the reference's OpenMP twin (oracle_twin_run):
        the Kokkos path's results at J = 0; with current it keeps the twin's
        Jx line (src/FDTD/FDTD.cpp:82-90).  Sources are not evaluated."""
        p = self.params
        for c in range(6, 9):
            if self.f[c] is None:
                self.f[c] = np.zeros_like(self.f[0])
        ptrs = (_D * 9)(*[_ptr(a) for a in self.f])
        oracle_lib().oracle_twin_run(p.Ni, p.Nj, p.Nk, ptrs, _ptr(self.coef), int(n))
        self.step_index += int(n)

    def step(self, n=1):
        p = self.params
        ptrs = (_D * 9)(*[(_ptr(a) if a is not None else _D()) for a in self.f])
        csrc, keep = self._csources()
        if self.sources and self._jwork is None:
            self._jwork = [np.zeros_like(self.f[0]) for _ in range(3)]
        jw = (_D * 3)(*([_ptr(a) for a in self._jwork] if self._jwork else [_D(), _D(), _D()]))
        oracle_lib().oracle_run(p.Ni, p.Nj, p.Nk, ptrs, _ptr(self.coef), csrc, len(self.sources),
                                self.step_index, int(n), jw)
        self.step_index += int(n)

    def field_sums(self):
        return field_sums(self.f[:6])


def _cparams(params):
    return OracleParams(params.Ni, params.Nj, params.Nk, params.ax, params.bx, params.ay, params.by,
                        params.az, params.bz, params.dx, params.dy, params.dz)


class OraclePML(Oracle):
    """The reference's FDTD_PML (split-field absorbing layer of
    (int)(N * pml_percent) cells at both ends of every axis), restated in C
    (oracle_pml_run in fdtd_oracle.c)."""

    def __init__(self, params, dt, pml_percent, with_current=True):
        super().__init__(params, dt, with_current)
        self.pml_percent = float(pml_percent)
        cp = _cparams(params)
        sizes = (ctypes.c_int * 3)()
        oracle_lib().oracle_pml_sizes(ctypes.byref(cp), self.pml_percent, sizes)
        self.pml = list(sizes)
        self.sigma = [np.zeros(params.Ni), np.zeros(params.Nj), np.zeros(params.Nk)]
        oracle_lib().oracle_pml_sigma(ctypes.byref(cp), self.pml_percent, *[_ptr(a) for a in self.sigma])
        self.split = [np.zeros_like(self.f[0]) for _ in range(12)]

    def step(self, n=1):
        p = self.params
        ptrs = (_D * 9)(*[(_ptr(a) if a is not None else _D()) for a in self.f])
        csrc, keep = self._csources()
        if self.sources and self._jwork is None:
            self._jwork = [np.zeros_like(self.f[0]) for _ in range(3)]
        jw = (_D * 3)(*([_ptr(a) for a in self._jwork] if self._jwork else [_D(), _D(), _D()]))
        sig = (_D * 3)(*[_ptr(a) for a in self.sigma])
        spl = (_D * 12)(*[_ptr(a) for a in self.split])
        pml = (ctypes.c_int * 3)(*self.pml)
        oracle_lib().oracle_pml_run(p.Ni, p.Nj, p.Nk, ptrs, _ptr(self.coef), pml, sig, self.dt, p.dx, p.dy, p.dz,
                                    spl, csrc, len(self.sources), self.step_index, int(n), jw)
        self.step_index += int(n)

    def step_driver(self, n=1):
        raise NotImplementedError("the PML oracle steps through step()")


class OracleSlab:
    """A z slab of the oracle: planes [k_begin, k_end) of the grid `params`
    stored with one halo plane below and above (the layout of the coarray
    program's slabs with their next_E / pred_B halo arrays,
    coarray/fdtd.F90:90-98), updated by the box sweeps of fdtd_oracle.c over
    the owned planes.  J is dense (the owned planes of the whole grid's J)."""

    def __init__(self, params, dt, k_begin, k_end):
        self.coef = coefficients(params, dt)
        self.Ni, self.Nj = params.Ni, params.Nj
        self.nk = int(k_end) - int(k_begin)
        self.plane = params.Ni * params.Nj
        self.f = [np.zeros(self.plane * (self.nk + 2)) for _ in range(9)]
        self.step_index = 0
        self.pending = False  # a trailing B half step left pending (sweep kinds 3, 4)

    def owned(self, comp):
        """View of the owned planes of component comp (flat, i fastest)."""
        return self.f[int(comp)][self.plane:self.plane * (self.nk + 1)]

    def plane_view(self, comp, k):
        """View of stored plane k (0: halo below, nk + 1: halo above)."""
        return self.f[int(comp)][self.plane * k:self.plane * (k + 1)]

    def sweep(self, kind):
        """kind 0: B half step, 1: two B half steps, 2: E (kokkos_functors.h:128-151, :64-90),
        3: leave the step's trailing B half pending, 4: a whole step as the
        fused slab sweep does it: the pending half (if any) and the leading
        one on the owned planes and the halo plane below (which holds the
        neighbour's last plane of B and E), then E on the owned planes; the
        trailing half is left pending.  2 applies a pending half first; 0 and
        1 count it as their first half."""
        box = OracleBox(0, self.Ni, 0, self.Nj, 1, self.nk + 1)
        nk = self.nk + 2
        f, c = self.f, self.coef

        def b_half(b):
            oracle_lib().oracle_update_B_box(self.Ni, self.Nj, nk, b, *[_ptr(f[q]) for q in range(6)], c[3], c[4], c[5])

        def e_sweep():
            oracle_lib().oracle_update_E_box(self.Ni, self.Nj, nk, box, *[_ptr(f[q]) for q in (3, 4, 5, 6, 7, 8, 0, 1, 2)],
                                             c[6], c[0], c[1], c[2])
            self.step_index += 1

        if kind == 3:
            self.pending = True
            return
        if kind == 4:
            wide = OracleBox(0, self.Ni, 0, self.Nj, 0, self.nk + 1)
            for _ in range(2 if self.pending else 1):
                b_half(wide)
            e_sweep()
            self.pending = True
            return
        if kind == 2:
            if self.pending:
                b_half(box)
                self.pending = False
            e_sweep()
            return
        for _ in range(2 if kind == 1 else 1):
            b_half(box)
        self.pending = False


# ---------------------------------------------------------------------------
# The reference itself (oracle/_ref), where it was built.

def ref_available():
    return os.path.exists(REF_LIB)


def ref_lib():
    global _rlib
    if _rlib is None:
        if not ref_available():
            raise FileNotFoundError("reference build %s not present" % REF_LIB)
        lib = ctypes.CDLL(REF_LIB)
        lib.ref_kokkos_create.argtypes = [ctypes.POINTER(ctypes.c_int), _D, ctypes.c_double]
        lib.ref_kokkos_create.restype = ctypes.c_void_p
        lib.ref_kokkos_destroy.argtypes = [ctypes.c_void_p]
        lib.ref_kokkos_pml_create.argtypes = [ctypes.POINTER(ctypes.c_int), _D, ctypes.c_double, ctypes.c_double]
        lib.ref_kokkos_pml_create.restype = ctypes.c_void_p
        lib.ref_kokkos_pml_destroy.argtypes = [ctypes.c_void_p]
        lib.ref_kokkos_update_fields.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.ref_kokkos_zeroed_currents.argtypes = [ctypes.c_void_p]
        lib.ref_kokkos_field.argtypes = [ctypes.c_void_p, ctypes.c_int, _D, ctypes.c_long, ctypes.c_int]
        lib.ref_kokkos_field.restype = ctypes.c_int
        lib.ref_run_test_kokkos.argtypes = [ctypes.c_int] * 6
        lib.ref_run_test_kokkos.restype = ctypes.c_double
        lib.ref_last_error.restype = ctypes.c_char_p
        lib.ref_omp_create.argtypes = [ctypes.POINTER(ctypes.c_int), _D, ctypes.c_double]
        lib.ref_omp_create.restype = ctypes.c_void_p
        lib.ref_omp_destroy.argtypes = [ctypes.c_void_p]
        lib.ref_omp_update_fields.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.ref_omp_field.argtypes = [ctypes.c_void_p, ctypes.c_int, _D, ctypes.c_long, ctypes.c_int]
        lib.ref_omp_field.restype = ctypes.c_int
        _rlib = lib
    return _rlib


class RefKokkos:
    """FDTD_kokkos::FDTD from the reference's own sources (oracle/_ref).
    kind="kokkos" (the Kokkos solver class, the path the engine replaces) or "openmp" (its OpenMP twin)."""

    def __init__(self, params, dt, kind="kokkos", pml_percent=None):
        lib = ref_lib()
        self.kind = kind
        self.pml = pml_percent is not None
        n = (ctypes.c_int * 3)(params.Ni, params.Nj, params.Nk)
        b = (ctypes.c_double * 9)(params.ax, params.bx, params.ay, params.by, params.az, params.bz,
                                  params.dx, params.dy, params.dz)
        if self.pml:
            self.h = lib.ref_kokkos_pml_create(n, b, float(dt), float(pml_percent))
        else:
            create = lib.ref_kokkos_create if kind == "kokkos" else lib.ref_omp_create
            self.h = create(n, b, float(dt))
        if not self.h:
            raise ValueError(lib.ref_last_error().decode())
        self.n = params.Ni * params.Nj * params.Nk

    def close(self):
        if self.h:
            if self.pml:
                ref_lib().ref_kokkos_pml_destroy(self.h)
            else:
                (ref_lib().ref_kokkos_destroy if self.kind == "kokkos" else ref_lib().ref_omp_destroy)(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _field(self, comp, buf, direction):
        fn = ref_lib().ref_kokkos_field if self.kind == "kokkos" else ref_lib().ref_omp_field
        rc = fn(self.h, int(comp), _ptr(buf), self.n, direction)
        if rc == -2:
            raise RuntimeError(ref_lib().ref_last_error().decode())
        if rc != 0:
            raise ValueError(ref_lib().ref_last_error().decode())

    def set(self, comp, values):
        a = np.ascontiguousarray(values, dtype=np.float64).reshape(-1).copy()
        self._field(comp, a, 1)

    def get(self, comp):
        a = np.empty(self.n)
        self._field(comp, a, 0)
        return a

    def update_fields(self, steps=1):
        (ref_lib().ref_kokkos_update_fields if self.kind == "kokkos" else ref_lib().ref_omp_update_fields)(self.h, int(steps))

    def zeroed_currents(self):
        ref_lib().ref_kokkos_zeroed_currents(self.h)


def run_reference_unit_tests():
    """Runs the reference's own unit tests (oracle/_ref/ref_unit_tests) and
    returns {test name: (value, expected, tol, passed)}."""
    exe = os.path.join(REF_DIR, "ref_unit_tests")
    r = subprocess.run([exe], capture_output=True, text=True, check=True)
    out = {}
    for line in r.stdout.splitlines():
        parts = line.split()
        if parts and parts[0] == "NEAR":
            out[parts[1]] = (float(parts[2]), float(parts[3]), float(parts[4]), parts[5] == "PASS")
    return out
