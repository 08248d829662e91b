"""z-slab domain decomposition of the Yee step.

The reference's coarray program splits the grid into slabs of z planes, one
per image (coarray/fdtd.F90:149-164, init_decomposition: the first Nk mod n
images get one plane more), and between the sweeps of every step copies the
neighbours' boundary planes into halo arrays (:86-102):

    update_B;  pred_Bx, pred_By <- Bx, By of the image below, its last plane
    update_E;  next_Ex, next_Ey <- Ex, Ey of the image above, its first plane
    update_B

B at k+1 needs Ex, Ey there (include/FDTD_kokkos/kokkos_functors.h:141);
E at k-1 needs Bx, By there (:78); nothing else crosses a slab face.

Here a slab is an engine handle (``fdtd_slab_create``) that stores its owned
planes with one halo plane below and one above; its sweeps update the owned
planes only, and a halo exchange fills the halo planes.  ``step_schedule``
is the order of sweeps and exchanges that makes a set of slabs step exactly
like one handle of the whole grid (bit for bit: every cell sees the same
operands in the same order).  In the FP32-arithmetic forms a step can also be
one fused sweep (SWEEP_STEP: the single-grid engine's B-first kernel over the
owned planes), which reads E and B of the halo plane below and E of the one
above, so its exchange (HALO_STEP) carries Ex, Ey, Ez with Bx, By.  ``FDTDSlabs`` runs it on one GPU, the slabs
exchanging through device copies (``fdtd_slab_exchange``);
``ring_exchange`` is the same exchange between processes over
torch.distributed, one slab per rank.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import InvalidArgument
from .fdtd import FDTD, Parameters, Precision, Const

SWEEP_B_HALF, SWEEP_B_DOUBLE, SWEEP_E, SWEEP_B_DEFER, SWEEP_STEP = 0, 1, 2, 3, 4
HALO_E, HALO_B, HALO_STEP = 0, 1, 2
PLANE_HALO_BELOW, PLANE_FIRST, PLANE_LAST, PLANE_HALO_ABOVE = 0, 1, 2, 3


def slab_bounds(nk, n):
    """[k_begin, k_end) of each of n slabs of nk planes; the first nk mod n
    slabs have one plane more (coarray/fdtd.F90:149-164)."""
    nk, n = int(nk), int(n)
    if n <= 0 or n > nk:
        raise InvalidArgument(_lib.FDTD_ERR_INVALID_ARGUMENT, "need 1 <= slabs <= Nk")
    base, extra = divmod(nk, n)
    out, k = [], 0
    for s in range(n):
        size = base + (1 if s < extra else 0)
        out.append((k, k + size))
        k += size
    return out


def step_schedule(n, defer=False, pending=False, fused=False):
    """The operations of n update_fields steps on a set of slabs, in order:
    ("exchange", HALO_*) or ("sweep", SWEEP_*).

    One step is B/2, E, B/2 (src/FDTD_kokkos/FDTD_kokkos.cpp:91-104); the
    trailing B half step of one step and the leading one of the next share a
    sweep (SWEEP_B_DOUBLE), as in the single-grid engine.  With `defer` the
    last step's trailing half is left pending (SWEEP_B_DEFER, the
    FP32-arithmetic forms), and a call made with `pending` starts with the
    double sweep that applies it.  The E halo is exchanged first, so fields
    set from the host since the last step are seen across the slab faces.

    With `fused` (FP32-arithmetic forms: it needs `defer`), each step is one
    SWEEP_STEP, which applies the pending half itself; an exchange precedes
    the first sweep and follows every sweep, so the halo planes are current
    for any reader that applies the pending half between calls."""
    n = int(n)
    if n <= 0:
        return []
    if fused:
        if not defer:
            raise InvalidArgument(_lib.FDTD_ERR_INVALID_ARGUMENT,
                                  "the fused schedule leaves the trailing B half pending (defer)")
        ops = [("exchange", HALO_STEP)]
        for _ in range(n):
            ops += [("sweep", SWEEP_STEP), ("exchange", HALO_STEP)]
        return ops
    ops = [("exchange", HALO_E), ("sweep", SWEEP_B_DOUBLE if pending else SWEEP_B_HALF)]
    for s in range(n):
        last = SWEEP_B_DEFER if defer else SWEEP_B_HALF
        ops += [("exchange", HALO_B), ("sweep", SWEEP_E), ("exchange", HALO_E),
                ("sweep", SWEEP_B_DOUBLE if s + 1 < n else last)]
    return ops


def halo_groups(halo):
    """The parts of an exchange: a list of (components, sent plane, received
    plane, sent to the slab above).  E sends Ex, Ey of each slab's first
    plane to the slab below's halo above; B sends Bx, By of each slab's last
    plane to the slab above's halo below; STEP sends the E part and Bx, By,
    Ex, Ey, Ez of the last plane to the slab above's halo below."""
    e = ((0, 1), PLANE_FIRST, PLANE_HALO_ABOVE, False)
    if halo == HALO_E:
        return [e]
    if halo == HALO_B:
        return [((3, 4), PLANE_LAST, PLANE_HALO_BELOW, True)]
    if halo == HALO_STEP:
        return [e, ((3, 4, 0, 1, 2), PLANE_LAST, PLANE_HALO_BELOW, True)]
    raise InvalidArgument(_lib.FDTD_ERR_INVALID_ARGUMENT, "invalid halo")


def halo_planes(halo):
    """(components, sent plane, received plane) of HALO_E or HALO_B."""
    g = halo_groups(halo)
    if len(g) != 1:
        raise InvalidArgument(_lib.FDTD_ERR_INVALID_ARGUMENT, "the exchange has several parts: use halo_groups")
    return g[0][:3]


def ring_exchange(send, recv, halo, rank, world, group=None):
    """Halo exchange between processes, one slab per rank in plane order (the
    grid is periodic: rank world-1's neighbour above is rank 0).  send /
    recv: per component of ``halo_groups(halo)``, in order, the tensor of the
    plane this rank sends and the tensor its halo plane is received into.  E
    goes to the rank below, B to the rank above (coarray/fdtd.F90:90-91,
    97-98)."""
    import torch.distributed as dist
    reqs = []
    q = 0
    for g, (comps, _, _, up) in enumerate(halo_groups(halo)):
        to, frm = ((rank + 1) % world, (rank - 1) % world) if up else ((rank - 1) % world, (rank + 1) % world)
        for c in range(len(comps)):
            if world == 1:
                recv[q].copy_(send[q])
            else:
                tag = 100 * halo + 10 * g + c
                reqs.append(dist.isend(send[q], to, group=group, tag=tag))
                reqs.append(dist.irecv(recv[q], frm, group=group, tag=tag))
            q += 1
    for r in reqs:
        r.wait()


class Slab(FDTD):
    """One z slab on the current GPU: planes [k_begin, k_end) of the grid of
    ``parameters`` with a halo plane below and above.  ``parameters`` (the
    host-facing shape) describes the owned planes; ``global_parameters`` the
    whole grid.  Sources take whole-grid coordinates."""

    def __init__(self, parameters, dt, k_begin, k_end, precision=Precision.FP64):
        self._h = None
        lib = _lib.load()
        self.global_parameters = parameters
        self.k_begin, self.k_end = int(k_begin), int(k_end)
        self.dt = float(dt)
        self.precision = Precision(precision)
        p = parameters.to_c()
        h = ctypes.c_void_p()
        _lib.check(lib.fdtd_slab_create(ctypes.byref(p), self.dt, int(self.precision), self.k_begin, self.k_end,
                                        ctypes.byref(h)))
        self._h = h
        self._lib = lib
        self._sources = []
        nk = self.k_end - self.k_begin
        self.parameters = Parameters(parameters.Ni, parameters.Nj, nk, parameters.ax, parameters.bx,
                                     parameters.ay, parameters.by, parameters.az + self.k_begin * parameters.dz,
                                     parameters.az + (self.k_begin + nk) * parameters.dz,
                                     parameters.dx, parameters.dy, parameters.dz)

    def sweep(self, kind):
        """One sweep over the owned planes (SWEEP_B_HALF, SWEEP_B_DOUBLE,
        SWEEP_E, SWEEP_B_DEFER or SWEEP_STEP; SWEEP_E and SWEEP_STEP advance
        the step count)."""
        _lib.check(self._lib.fdtd_slab_sweep(self._handle(), int(kind)))

    def plane(self, comp, which, part=0):
        """(device address, bytes) of one stored plane of E/B component comp."""
        ptr, nb = ctypes.c_void_p(), ctypes.c_size_t()
        _lib.check(self._lib.fdtd_slab_plane(self._handle(), int(comp), int(which), int(part), ctypes.byref(ptr),
                                             ctypes.byref(nb)))
        return ptr.value, nb.value


class FDTDSlabs:
    """A periodic grid stepped as n z slabs on one GPU: the decomposition of
    the reference's coarray program (coarray/fdtd.F90), with its halo
    exchange done by device copies.  The API is FDTD's: the results (fields,
    sources, step count) are those of one FDTD of the whole grid in the same
    precision, bit for bit."""

    def __init__(self, parameters, dt, n_slabs, precision=Precision.FP64, fused=None):
        self.parameters = parameters
        self.dt = float(dt)
        self.precision = Precision(precision)
        self.bounds = slab_bounds(parameters.Nk, n_slabs)
        self.slabs = []
        try:
            for k0, k1 in self.bounds:
                self.slabs.append(Slab(parameters, dt, k0, k1, precision))
        except Exception:
            self.close()
            raise
        self._lib = _lib.load()
        self._arr = (ctypes.c_void_p * len(self.slabs))(*[s._handle().value for s in self.slabs])
        # FP32-arithmetic forms leave the last step's trailing B half pending,
        # as the whole-grid handle does (the FP64 form applies every half)
        self._defer = self.precision != Precision.FP64
        self._pending = False
        # one fused sweep per step (FP32-arithmetic forms; the default there)
        self.fused = self._defer if fused is None else bool(fused)
        if self.fused and not self._defer:
            self.close()
            raise InvalidArgument(_lib.FDTD_ERR_INVALID_ARGUMENT, "the FP64 form runs the split sweeps")

    def close(self):
        for s in self.slabs:
            s.close()
        self.slabs = []

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
        return len(self.slabs)

    def exchange(self, halo):
        if not self.slabs:
            raise InvalidArgument(_lib.FDTD_ERR_INVALID_ARGUMENT, "solver is closed")
        _lib.check(self._lib.fdtd_slab_exchange(self._arr, len(self.slabs), int(halo)))

    def step(self, n):
        """n consecutive update_fields() calls on every slab."""
        if int(n) < 0:
            raise InvalidArgument(_lib.FDTD_ERR_INVALID_ARGUMENT, "negative step count")
        if int(n) == 0:
            return
        for op, arg in step_schedule(n, self._defer, self._pending, self.fused):
            if op == "exchange":
                self.exchange(arg)
            else:
                for s in self.slabs:
                    s.sweep(arg)
        self._pending = self._defer

    def update_fields(self):
        self.step(1)

    def synchronize(self):
        for s in self.slabs:
            s.synchronize()

    def zeroed_currents(self):
        for s in self.slabs:
            s.zeroed_currents()

    def add_source(self, src):
        """A source in whole-grid coordinates; each slab keeps its part."""
        idx = None
        for s in self.slabs:
            idx = s.add_source(src)
        return idx

    def clear_sources(self):
        for s in self.slabs:
            s.clear_sources()

    def copy_to_host(self, comp, out=None):
        n = self.parameters.cells
        if out is None:
            out = np.empty(n, dtype=np.float64)
        if out.dtype != np.float64 or out.size != n or not out.flags.c_contiguous:
            raise InvalidArgument(_lib.FDTD_ERR_INVALID_ARGUMENT, "output must be a contiguous float64 array of Ni*Nj*Nk")
        plane = int(self.parameters.Ni) * int(self.parameters.Nj)
        for s, (k0, k1) in zip(self.slabs, self.bounds):
            s.copy_to_host(comp, out[k0 * plane:k1 * plane])
        return out

    def copy_from_host(self, comp, values):
        a = np.ascontiguousarray(values, dtype=np.float64).reshape(-1)
        if a.size != self.parameters.cells:
            raise InvalidArgument(_lib.FDTD_ERR_INVALID_ARGUMENT,
                                  "expected %d values, got %d" % (self.parameters.cells, a.size))
        plane = int(self.parameters.Ni) * int(self.parameters.Nj)
        for s, (k0, k1) in zip(self.slabs, self.bounds):
            s.copy_from_host(comp, a[k0 * plane:k1 * plane])
        if int(comp) < 6:
            self._pending = False  # every slab applied its pending half before the write

    def field_sums(self):
        """Sums over all cells (the slabs' FP64 sums added)."""
        return np.sum([s.field_sums() for s in self.slabs], axis=0)

    def energy(self):
        s = self.field_sums()
        p = self.parameters
        return float(s[:6].sum() * p.dx * p.dy * p.dz / (8.0 * Const.PI))

    def set_fp16_exponents(self, exps):
        for s in self.slabs:
            s.set_fp16_exponents(exps)
        self._pending = False

    @property
    def step_index(self):
        return self.slabs[0].step_index

    @step_index.setter
    def step_index(self, value):
        for s in self.slabs:
            s.step_index = value
