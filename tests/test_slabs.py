"""Host logic of the z-slab decomposition (fdtd_method_gb300/slabs.py), on
the CPU: the plane split of the reference's coarray program, the
sweep/exchange schedule, and the schedule run over the oracle's slabs, in
one process (any slab count) and as gloo ranks exchanging halo planes,
compared with the oracle on the whole grid bit for bit."""
import multiprocessing as mp
import os
import socket
import sys

import numpy as np
import pytest

from fdtd_method_gb300 import slabs
from fdtd_method_gb300.sources import COURANT_DT, normalised_parameters

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _coarray_decomposition(nk, images):
    """coarray/fdtd.F90:149-164 for images 1..n, as 0-based [k_begin, k_end)."""
    out = []
    for img in range(1, images + 1):
        remainder = nk % images
        k_local = nk // images
        if img <= remainder:
            k_local += 1
            offset = (img - 1) * k_local
        else:
            offset = remainder * (k_local + 1) + (img - remainder - 1) * k_local
        out.append((offset, offset + k_local))
    return out


@pytest.mark.parametrize("nk,n", [(64, 1), (64, 2), (37, 3), (37, 5), (10, 10), (513, 8)])
def test_slab_bounds_follow_the_coarray_decomposition(nk, n):
    assert slabs.slab_bounds(nk, n) == _coarray_decomposition(nk, n)


def test_slab_bounds_reject_more_slabs_than_planes():
    with pytest.raises(ValueError):
        slabs.slab_bounds(4, 5)
    with pytest.raises(ValueError):
        slabs.slab_bounds(4, 0)


def test_schedule_matches_the_reference_step_order():
    # B/2, E, B/2 per step (FDTD_kokkos.cpp:91-104); halos before the sweeps
    # that read them (coarray/fdtd.F90:86-102)
    ops = slabs.step_schedule(3)
    sweeps = [a for op, a in ops if op == "sweep"]
    assert sweeps == [slabs.SWEEP_B_HALF, slabs.SWEEP_E, slabs.SWEEP_B_DOUBLE, slabs.SWEEP_E,
                      slabs.SWEEP_B_DOUBLE, slabs.SWEEP_E, slabs.SWEEP_B_HALF]
    # every B sweep follows an E exchange, every E sweep a B exchange
    for q, (op, a) in enumerate(ops):
        if op == "sweep":
            want = slabs.HALO_B if a == slabs.SWEEP_E else slabs.HALO_E
            assert ops[q - 1] == ("exchange", want)
    assert slabs.step_schedule(0) == []


def test_schedule_with_a_pending_half_step():
    """FP32-arithmetic slabs leave the last trailing B half pending (as a
    whole-grid handle does): two calls of 2 steps make the sweeps of one call
    of 4, the pending half becoming the first half of the second call's
    double sweep."""
    first = [a for op, a in slabs.step_schedule(2, defer=True) if op == "sweep"]
    second = [a for op, a in slabs.step_schedule(2, defer=True, pending=True) if op == "sweep"]
    whole = [a for op, a in slabs.step_schedule(4, defer=True) if op == "sweep"]
    assert first[-1] == slabs.SWEEP_B_DEFER and second[0] == slabs.SWEEP_B_DOUBLE
    assert first[:-1] + second == whole


def test_fused_schedule():
    """One fused sweep per step, each followed by an exchange of what the next
    one reads (and what a reader applying the pending half reads)."""
    ops = slabs.step_schedule(3, defer=True, fused=True)
    assert ops == [("exchange", slabs.HALO_STEP)] + [("sweep", slabs.SWEEP_STEP), ("exchange", slabs.HALO_STEP)] * 3
    with pytest.raises(ValueError):
        slabs.step_schedule(2, fused=True)
    # the halo the fused sweep reads: E above; B and E below
    groups = slabs.halo_groups(slabs.HALO_STEP)
    assert groups == [((0, 1), slabs.PLANE_FIRST, slabs.PLANE_HALO_ABOVE, False),
                      ((3, 4, 0, 1, 2), slabs.PLANE_LAST, slabs.PLANE_HALO_BELOW, True)]
    with pytest.raises(ValueError):
        slabs.halo_planes(slabs.HALO_STEP)


def _initial_fields(p, seed):
    rng = np.random.default_rng(seed)
    n = p.Ni * p.Nj * p.Nk
    f = [rng.standard_normal(n) for _ in range(6)]
    j = [np.zeros(n) for _ in range(3)]
    # a current box that crosses slab faces and the periodic z wrap
    shape = (p.Nk, p.Nj, p.Ni)
    for c in range(3):
        jj = j[c].reshape(shape)
        for k in list(range(p.Nk - 3, p.Nk)) + list(range(0, 4)):
            jj[k, 2:6, 1:5] = rng.standard_normal((4, 4))
    return f + j


def _whole_grid(p, dt, fields, steps):
    from oracle import Oracle
    o = Oracle(p, dt)
    for c in range(9):
        o.set(c, fields[c])
    o.step(steps)
    return [o.get(c) for c in range(6)]


def _run_slab(slab, rank, world, fields, plane, k0, k1, steps, exchange, fused=False):
    for c in range(9):
        slab.owned(c)[...] = fields[c][k0 * plane:k1 * plane]
    for op, arg in slabs.step_schedule(steps, defer=fused, fused=fused):
        if op == "sweep":
            slab.sweep(arg)
        else:
            exchange(arg)
    if fused:
        slab.sweep(slabs.SWEEP_B_HALF)


def _exchange_in_process(ss, halo):
    n = len(ss)
    for comps, frm, to, up in slabs.halo_groups(halo):
        for r, s in enumerate(ss):
            dst = ss[(r + 1) % n] if up else ss[(r - 1) % n]
            kf = 1 if frm == slabs.PLANE_FIRST else s.nk
            kt = dst.nk + 1 if to == slabs.PLANE_HALO_ABOVE else 0
            for c in comps:
                dst.plane_view(c, kt)[...] = s.plane_view(c, kf)


@pytest.mark.parametrize("fused", [False, True])
def test_oracle_slabs_in_one_process_equal_the_whole_grid(fused):
    """The split schedule, and the fused one in FP64 arithmetic (two calls of
    3 steps; the pending half applied at the end by a B half sweep, which
    reads the E halo the last exchange left current)."""
    from oracle import OracleSlab
    p = normalised_parameters(12, 10, 23)
    fields = _initial_fields(p, 5)
    want = _whole_grid(p, COURANT_DT, fields, 6)
    plane = p.Ni * p.Nj
    for n in (1, 2, 3, 7):
        bounds = slabs.slab_bounds(p.Nk, n)
        ss = [OracleSlab(p, COURANT_DT, k0, k1) for k0, k1 in bounds]
        for s, (k0, k1) in zip(ss, bounds):
            for c in range(9):
                s.owned(c)[...] = fields[c][k0 * plane:k1 * plane]
        calls = [(3, False), (3, True)] if fused else [(6, False)]
        for steps, pending in calls:
            for op, arg in slabs.step_schedule(steps, defer=fused, pending=pending, fused=fused):
                if op == "sweep":
                    for s in ss:
                        s.sweep(arg)
                else:
                    _exchange_in_process(ss, arg)
        if fused:
            for s in ss:
                s.sweep(slabs.SWEEP_B_HALF)
        for c in range(6):
            got = np.concatenate([s.owned(c) for s in ss])
            assert np.array_equal(got, want[c]), (n, c)
        assert all(s.step_index == 6 for s in ss)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, steps, out, fused=False):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      OMP_NUM_THREADS="1")
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist

    from fdtd_method_gb300 import slabs as sl
    from fdtd_method_gb300.sources import COURANT_DT as dt, normalised_parameters as npar
    from oracle import OracleSlab
    dist.init_process_group("gloo", rank=rank, world_size=world)
    p = npar(12, 10, 23)
    fields = _initial_fields(p, 5)
    k0, k1 = sl.slab_bounds(p.Nk, world)[rank]
    slab = OracleSlab(p, dt, k0, k1)

    def exchange(halo):
        send, recv, dst = [], [], []
        for comps, frm, to, _ in sl.halo_groups(halo):
            kf = 1 if frm == sl.PLANE_FIRST else slab.nk
            kt = slab.nk + 1 if to == sl.PLANE_HALO_ABOVE else 0
            for c in comps:
                send.append(torch.from_numpy(slab.plane_view(c, kf).copy()))
                recv.append(torch.empty_like(send[-1]))
                dst.append((c, kt))
        sl.ring_exchange(send, recv, halo, rank, world)
        for (c, kt), t in zip(dst, recv):
            slab.plane_view(c, kt)[...] = t.numpy()

    _run_slab(slab, rank, world, fields, p.Ni * p.Nj, k0, k1, steps, exchange, fused)
    out.put((rank, [slab.owned(c).copy() for c in range(6)]))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world,fused", [(2, False), (3, False), (2, True), (3, True)])
def test_gloo_ranks_exchanging_halo_planes_equal_the_whole_grid(world, fused):
    pytest.importorskip("torch")
    p = normalised_parameters(12, 10, 23)
    steps = 5
    want = _whole_grid(p, COURANT_DT, _initial_fields(p, 5), steps)
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, steps, out, fused)) for r in range(world)]
    for pr in procs:
        pr.start()
    res = dict(out.get(timeout=180) for _ in procs)
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    for c in range(6):
        got = np.concatenate([res[r][c] for r in range(world)])
        assert np.array_equal(got, want[c]), c
