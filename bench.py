#!/usr/bin/env python3
"""Benchmark of the Yee step on one GB300 (one JSON line on stdout).

Workload (the headline configuration): 512^3 periodic grid in normalised
units (dx = dy = dz = C, dt = 0.5/sqrt(3)), zero initial fields, one Jz
Gaussian-pulse source at the centre (A, T drawn from seed 0, tau = T,
t0 = 3 tau, sigma = 8 cells), run length 1000 steps.  A "step" is one
update_fields (B/2, E, B/2) over the whole grid.

  value      Gcell-steps/s of the chosen form (compensated FP32 storage, FP32
             arithmetic), device-timed with CUDA events over K steps on the
             launching stream, state resident in HBM.
  fp64       the same for the FP64 drop-in (bit-identical to the reference),
             with its own e2e leg, its roofline against the FP64 pipe rate
             measured in this run, and the contracted FP64 arithmetic beside it.
  e2e        the chosen form through the C ABI with host buffers: upload the
             six FP64 fields from pinned host memory, K steps, download them.
  accuracy   rel-L2 (whole state and per component) and energy difference of
             the chosen form against the FP64 run after the run length; every
             entry of `forms` and `batched` carries the same.
  roofline   the dominant kernel's algorithmic bytes / its mean CUDA-event
             duration against the measured HBM copy bandwidth.
  cpu_baseline  the reference's CPU path (restated in oracle/, OpenMP on all
             host cores, the reference driver's loop) on a bounded sample;
             cpu_baseline_openmp_twin the reference's OpenMP twin (J = 0).
  batched    the batched form on its own workload (256 domains with edges
             uniform in 32..160 cells, plane wave + one pulse each), CUDA-graph
             step groups, one persistent launch per fused sweep.
  forms      the other storage forms (FP32, FP16 with per-component scale, or
             the compensated form) on the same workload and timing: value and
             their fused kernel's roofline.

--impl reference runs only that CPU path on the same workload (exactly
--steps timed steps after --warmup, unless a stated time budget caps them)
and prints its own line.  Under torchrun every rank runs its own replica (no
data exchange; weak scaling) and rank 0 prints the line.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gcell-steps/s chosen vs plain FP64, 1 GB300, rel-L2≤1e-5; % of HBM roofline"
UNIT = "Gcell-steps/s"
FALLBACK_HBM_GBS = 6800.0
# FP64 instructions per cell-step of the split FP64 sweeps (a merged double B
# half step: 21, E: 18; contracted: 12 + 12); the pipe's issue rate is
# measured in the run (fdtd_measure_fp64_rate).
FP64_INSTR_PER_CELL_STEP = 39
FP64_FMA_INSTR_PER_CELL_STEP = 24
# time budget of the reference arm's timed steps (the CPU path runs ~0.2 s per
# 512^3 step on 16 cores)
REFERENCE_BUDGET_S = 600.0


def parse_args():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=512, help="grid edge (cells)")
    ap.add_argument("--grid", type=int, nargs=3, metavar=("NI", "NJ", "NK"), default=None,
                    help="grid extents (overrides --n; profiling captures of part of the benchmark grid)")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--precision", default="fp32_comp", choices=["fp32_comp", "fp32", "fp16_scaled"])
    ap.add_argument("--pipeline", default="auto", choices=["auto", "fused", "split"])
    ap.add_argument("--tile-y", type=int, default=0)
    ap.add_argument("--kchunk", type=int, default=0)
    ap.add_argument("--cells-per-thread", type=int, default=0)
    ap.add_argument("--depth", type=int, default=0, help="steps per sweep of the chosen form (0: the autotuner's)")
    ap.add_argument("--run-length", type=int, default=1000, help="steps of the accuracy run")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--fp64-steps", type=int, default=0, help="timed FP64 steps (default max(20, K/5))")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--no-forms", action="store_true", help="skip the other storage forms' lines")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-form leg")
    ap.add_argument("--batch-only", action="store_true", help="run only the batched-form leg and print it")
    ap.add_argument("--batch-domains", type=int, default=256)
    ap.add_argument("--batch-group", type=int, default=50, help="steps per CUDA-graph step group of the batch")
    ap.add_argument("--no-batch-accuracy", action="store_true", help="skip the batched form's FP64 comparison")
    ap.add_argument("--cpu-worker", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--cpu-kind", default="kokkos", choices=["kokkos", "twin"], help=argparse.SUPPRESS)
    ap.add_argument("--cpu-steps", type=int, default=0, help=argparse.SUPPRESS)
    ap.add_argument("--cpu-warmup", type=int, default=1, help=argparse.SUPPRESS)
    ap.add_argument("--cpu-budget-s", type=float, default=15.0, help=argparse.SUPPRESS)
    return ap.parse_args()


def workload(args):
    from fdtd_method_gb300.sources import baseline_pulse, normalised_parameters
    p = normalised_parameters(*(args.grid or (args.n, args.n, args.n)))
    src = baseline_pulse(p, seed=args.seed, n_steps=args.run_length)
    return p, src


def config_dict(args, p, src):
    m = src.meta
    shape = "%d^3" % args.n if not args.grid else "%dx%dx%d" % tuple(args.grid)
    return {"workload": "%s periodic Yee step, 1 Jz Gaussian pulse (sigma 8 cells, A=%.3f, T=%.2f steps, seed %d), "
                        "FP32-compensated vs FP64" % (shape, m["A"], m["T"], args.seed),
            "grid": [p.Ni, p.Nj, p.Nk], "cells": p.cells, "dt": "0.5/sqrt(3) (c=1, dx=1)",
            "chosen_precision": args.precision, "run_length": args.run_length,
            "l2": "inputs larger than L2 (state >= 4 GB per form vs 129 MB L2); no flush",
            "parallelism": "replicas" if args.gpus > 1 else "single GPU"}


# ---------------------------------------------------------------------------
# CPU baseline: the reference's path restated in oracle/ (OpenMP), run in a
# child process so its OpenMP runtime owns every host core.

def cpu_worker(args):
    """Times the reference's CPU path restated in oracle/: the Kokkos path's
    driver loop (kind kokkos: sources written into the dense J arrays, three
    sweeps per step) or its OpenMP twin (kind twin: src/FDTD/FDTD.cpp's loops,
    valid at J = 0, so run without the source).  `--cpu-steps` 0 picks the
    step count from --cpu-budget-s after the warm-up; a positive count is
    capped only by that budget."""
    import numpy as np  # noqa: F401
    from oracle import Oracle
    from oracle.oracle import oracle_lib
    from fdtd_method_gb300.sources import COURANT_DT
    p, src = workload(args)
    o = Oracle(p, COURANT_DT)
    twin = args.cpu_kind == "twin"
    if not twin:
        o.add_source(src)
    for c in range(9):  # first touch
        if o.f[c] is None:
            o.f[c] = np.zeros_like(o.f[0])
        o.f[c][...] = 0.0
    run = o.step_twin if twin else o.step_driver
    warm = max(1, args.cpu_warmup)
    t0 = time.perf_counter()
    run(warm)
    t_first = (time.perf_counter() - t0) / warm
    fit = int(max(1, args.cpu_budget_s / max(t_first, 1e-3)))
    steps = min(args.cpu_steps, fit) if args.cpu_steps else int(max(2, min(50, fit)))
    t0 = time.perf_counter()
    run(steps)
    dt_s = time.perf_counter() - t0
    print(json.dumps({"steps": steps, "warmup": warm, "seconds": dt_s, "threads": int(oracle_lib().oracle_threads()),
                      "value": p.cells * steps / dt_s / 1e9, "kind": args.cpu_kind,
                      "capped": bool(args.cpu_steps and steps < args.cpu_steps)}))


def run_cpu_baseline(args, steps=0, warmup=1, budget=15.0, kind="kokkos"):
    cmd = [sys.executable, os.path.abspath(__file__), "--cpu-worker", "--n", str(args.n), "--seed", str(args.seed),
           "--run-length", str(args.run_length), "--cpu-steps", str(steps), "--cpu-warmup", str(warmup),
           "--cpu-budget-s", str(budget), "--cpu-kind", kind] + (["--grid"] + [str(v) for v in args.grid] if args.grid else [])
    env = dict(os.environ)
    env.setdefault("OMP_PROC_BIND", "close")
    r = subprocess.run(cmd, capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError("CPU baseline failed: %s" % r.stderr[-2000:])
    return json.loads(r.stdout.strip().splitlines()[-1])


def cpu_baseline_obj(res, n):
    if res.get("kind") == "twin":
        return {"value": res["value"], "unit": UNIT, "cores": res["threads"], "kind": "port",
                "sample": "%d steps of the %d^3 grid at J = 0 (the twin ignores Jy, Jz), oracle/fdtd_oracle.c "
                          "restatement of the reference's OpenMP twin src/FDTD/FDTD.cpp (pinned bit for bit to "
                          "its build), OpenMP" % (res["steps"], n)}
    return {"value": res["value"], "unit": UNIT, "cores": res["threads"], "kind": "port",
            "sample": "%d steps of the %d^3 workload (reference driver loop: box current + B/2,E,B/2 sweeps), "
                      "oracle/fdtd_oracle.c restatement of the reference's Kokkos path, OpenMP" % (res["steps"], n)}


# ---------------------------------------------------------------------------
# Clocks sampled during the timed region.

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.path = None
        self.gpu = gpu_index

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(prefix="clocks_", suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.3)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for q, nm in enumerate(names):
                if parts[5 + q].lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------

def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "of measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "of fallback"


def ncu_traffic(kernel_kind, precision):
    """DRAM bytes per cell of one launch, from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.json")
    try:
        d = json.load(open(path))
        return float(d[precision][kernel_kind]["dram_bytes_per_cell"])
    except (OSError, KeyError, ValueError, TypeError):
        return None


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group(backend="nccl")
    else:
        torch.cuda.set_device(0)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, x):
    """The largest x over all ranks (the slowest replica's time)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(world, cells, steps, ms):
    """Whole-job Gcell-steps/s of `world` replicas that each advanced `cells`
    cells by `steps` steps, the slowest taking `ms` milliseconds (weak
    scaling: the work per GPU is fixed)."""
    return world * cells * steps / (ms / 1e3) / 1e9


def timed_steps(sim, stream, steps, world):
    import torch
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    sim.step(steps)
    t1.record(stream)
    t1.synchronize()
    torch.cuda.synchronize()
    barrier(world)
    return t0.elapsed_time(t1)


PREC = {"fp32_comp": 2, "fp32": 1, "fp16_scaled": 3}
# FP16 form: per-component power-of-two scales chosen by the engine, which
# scans the stored peaks every FP16_AUTOSCALE_EVERY steps (the scan is inside
# the timed steps).  The batched form keeps one fixed scale per component
# (FP16_EXPONENTS; its fields peak near 1e1).
FP16_AUTOSCALE_EVERY = 25
FP16_EXPONENTS = [6] * 6


def make_sim(p, precision_name):
    from fdtd_method_gb300 import FDTD
    from fdtd_method_gb300.sources import COURANT_DT
    s = FDTD(p, COURANT_DT, PREC[precision_name])
    if precision_name == "fp16_scaled":
        s.set_fp16_autoscale(FP16_AUTOSCALE_EVERY)
    return s
BYTES_PER_VALUE = {"fp32_comp": 6, "fp32": 4, "fp16_scaled": 2, "fp64": 8}
# update_fields steps one launch of each fused kernel kind advances
STEPS_PER_LAUNCH = {"fused_step": 1, "fused_step2": 2}


def launch_roofline(kind, alg_bytes, launch_ms, hbm, note):
    """A kernel's algorithmic bytes per launch over its mean launch time,
    against the HBM peak.  A depth-2 sweep reads and writes the state once for
    two steps: `effective_frac` counts the bytes two one-step sweeps would
    move (it can exceed 1)."""
    gbs = alg_bytes / (launch_ms / 1e3) / 1e9
    steps = STEPS_PER_LAUNCH.get(kind, 1)
    return {"bound": "hbm", "kernel": kind, "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
            "peak_note": note, "mean_launch_ms": launch_ms, "steps_per_launch": steps,
            "effective_frac": steps * gbs / hbm}


# ---------------------------------------------------------------------------
# Accuracy against FP64, computed on the GPU from exported FP64 fields.

def device_fields(sim, cells):
    """The six E/B components of `sim` as FP64 device tensors (fdtd_export_field)."""
    import torch
    out = []
    for c in range(6):
        t = torch.empty(cells, dtype=torch.float64, device="cuda")
        sim.export_field(c, 0, cells, t.data_ptr())
        out.append(t)
    sim.synchronize()
    return out


NAMES = ["Ex", "Ey", "Ez", "Bx", "By", "Bz"]


def accuracy_obj(got, ref, e_got, e_ref, steps):
    """rel-L2 of `got` against the FP64 fields `ref` over all six components
    (and each component's error against the norm of all six), the max-abs
    error against the largest FP64 amplitude, and the energy difference."""
    num = den = 0.0
    per = {}
    amp = max(float(r.abs().max()) for r in ref)
    worst = 0.0
    for c in range(6):
        d = got[c] - ref[c]
        per[NAMES[c]] = float((d * d).sum())
        num += per[NAMES[c]]
        den += float((ref[c] * ref[c]).sum())
        worst = max(worst, float(d.abs().max()))
    return {"steps": steps, "rel_l2": math.sqrt(num / den) if den else None,
            "rel_l2_per_component": {k: math.sqrt(v / den) if den else None for k, v in per.items()},
            "max_abs_over_amplitude": worst / amp if amp else None,
            "energy_fp64": e_ref, "energy": e_got, "energy_rel_diff": (e_got - e_ref) / e_ref if e_ref else None,
            "bar": 1e-5}


class Fp64Reference:
    """The FP64 drop-in run of the workload for the run length, kept as FP64
    device tensors for the forms' comparisons."""

    def __init__(self, args, p, src):
        from fdtd_method_gb300 import FDTD, Precision
        from fdtd_method_gb300.sources import COURANT_DT
        a = FDTD(p, COURANT_DT, Precision.FP64)
        a.add_source(src)
        a.step(args.run_length)
        self.fields = device_fields(a, p.cells)
        self.energy = a.energy()
        self.steps = args.run_length
        a.close()

    def compare(self, sim, cells):
        sim.synchronize()
        got = device_fields(sim, cells)
        out = accuracy_obj(got, self.fields, sim.energy(), self.energy, self.steps)
        del got
        return out


def form_accuracy(args, p, src, precision, ref):
    sim = make_sim(p, precision)
    sim.add_source(src)
    sim.step(args.run_length)
    out = ref.compare(sim, p.cells)
    if precision == "fp16_scaled":
        out["fp16_exponents"] = sim.fp16_exponents()
    sim.close()
    return out


def batch_accuracy(wl, b, steps):
    """Every domain of the batch `b` (stepped `steps` steps from the workload's
    initial state) against an FP64 handle of the same domain: rel-L2 over all
    domains and components, the worst domain's rel-L2, and the total energy."""
    import torch
    from fdtd_method_gb300 import FDTD, Precision
    from fdtd_method_gb300.sources import COURANT_DT
    num = den = 0.0
    worst = 0.0
    e_b = e_ref = 0.0
    for q, (p, init, src) in enumerate(wl):
        ref = FDTD(p, COURANT_DT, Precision.FP64)
        for c, v in init.items():
            ref.copy_from_host(int(c), v)
        ref.add_source(src)
        ref.step(steps)
        want = device_fields(ref, p.cells)
        e_ref += ref.energy()
        ref.close()
        got = []
        for c in range(6):
            h = b.copy_to_host(q, c)
            got.append(torch.from_numpy(h).cuda())
        e_b += b.energy(q)
        dn = sum(float(((g - w) ** 2).sum()) for g, w in zip(got, want))
        dd = sum(float((w * w).sum()) for w in want)
        num += dn
        den += dd
        worst = max(worst, math.sqrt(dn / dd) if dd else 0.0)
    return {"steps": steps, "domains": len(wl), "rel_l2": math.sqrt(num / den) if den else None,
            "worst_domain_rel_l2": worst, "energy_fp64": e_ref, "energy": e_b,
            "energy_rel_diff": (e_b - e_ref) / e_ref if e_ref else None, "bar": 1e-5}


def run_batched(args, stream, world, with_accuracy=False):
    """The batched form on its own workload: `--batch-domains` periodic domains
    with edges uniform in 32..160 cells, a plane wave along a random axis and
    one Gaussian pulse each (seeded), stepped in CUDA-graph step groups of
    `--batch-group` steps (one persistent launch per fused sweep).  With
    `with_accuracy` a second batch runs the workload's 500 steps and every
    domain is compared with an FP64 handle."""
    import torch
    from fdtd_method_gb300 import FDTDBatch
    from fdtd_method_gb300.sources import COURANT_DT, batch_workload
    G = max(2, args.batch_group // 2 * 2)  # even: replays start from the same copy
    groups = max(1, args.steps // G)
    wl = batch_workload(count=args.batch_domains, seed=args.seed, n_steps=500)

    def make_batch():
        b = FDTDBatch([w[0] for w in wl], COURANT_DT, PREC[args.precision])
        b.set_stream(stream.cuda_stream)
        for q, (p, init, src) in enumerate(wl):
            if args.precision == "fp16_scaled":
                b.set_fp16_exponents(q, FP16_EXPONENTS)
            for c, v in init.items():
                b.copy_from_host(q, int(c), v)
            b.add_source(q, src)
        return b

    b = make_batch()
    cells = sum(w[0].cells for w in wl)
    tuned = None if args.no_autotune else b.autotune(sweeps=5)
    b.step(G)  # captures the group's graph and warms up
    b.synchronize()
    torch.cuda.synchronize()
    barrier(world)
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for _ in range(groups):
        b.step(G)
    t1.record(stream)
    t1.synchronize()
    b.synchronize()
    barrier(world)
    ms = max_over_ranks(world, t0.elapsed_time(t1))
    steps = groups * G
    tiles = b.tiles()
    cfg = tuned
    b.close()
    acc = None
    if with_accuracy:
        b = make_batch()
        if tuned:
            b.set_config(tuned["tile_y"], tuned["kchunk"], True)
            b.set_split_sources(tuned["split_sources"])
        b.step(G)
        b.step(500 - G)
        b.synchronize()
        acc = batch_accuracy(wl, b, 500)
        b.close()
    bpv = BYTES_PER_VALUE[args.precision]
    gbs = 12 * bpv * cells * steps / (ms / 1e3) / 1e9
    hbm, note = measured_peaks()
    edges = [w[0].Ni for w in wl] + [w[0].Nj for w in wl] + [w[0].Nk for w in wl]
    return {"value": world * cells * steps / (ms / 1e3) / 1e9, "unit": UNIT, "domains": len(wl), "cells": cells,
            "edge_min": min(edges), "edge_max": max(edges), "tiles_per_sweep": tiles, "steps": steps,
            "group_steps": G, "ms_per_step": ms / steps, "launches_per_group": G + 1, "autotune": cfg,
            "step_roofline": {"algorithmic_bytes_per_cell_step": 12 * bpv, "achieved": gbs, "peak": hbm,
                              "frac": gbs / hbm, "peak_note": note},
            "accuracy": acc,
            "workload": "%d periodic domains, edges uniform in 32..160 cells, plane wave (random axis, mode 1-4) "
                        "+ 1 Gaussian pulse each (A in [0.5,2], T in [20,60] steps), seed %d, %s"
                        % (len(wl), args.seed, args.precision)}


def time_form(args, p, src, precision, stream, world):
    """K autotuned steps of one storage form on the workload: Gcell-steps/s
    and its fused kernel's mean launch time against the HBM roofline."""
    cells, K, W = p.cells, args.steps, args.warmup
    sim = make_sim(p, precision)
    sim.set_stream(stream.cuda_stream)
    sim.add_source(src)
    tuned = None if args.no_autotune else sim.autotune(sweeps=10, reuse=False)
    sim.step(W)
    sim.synchronize()
    sim.kernel_times()
    sim.set_kernel_timing(True)
    ms = max_over_ranks(world, timed_steps(sim, stream, K, world))
    kt = sim.kernel_times()
    sim.set_kernel_timing(False)
    exps = sim.fp16_exponents() if precision == "fp16_scaled" else None
    sim.close()
    hbm, note = measured_peaks()
    out = {"value": replica_value(world, cells, K, ms), "unit": UNIT, "ms_per_step": ms / K, "autotune": tuned}
    if exps is not None:
        out["fp16_exponents"] = exps
        out["fp16_autoscale_every"] = FP16_AUTOSCALE_EVERY
    kinds = {k: v for k, v in kt.items() if v[1] > 0 and k in STEPS_PER_LAUNCH}
    if kinds:
        kind = max(kinds, key=lambda k: kinds[k][0])
        launch_ms = kinds[kind][0] / kinds[kind][1]
        out["roofline"] = dict(launch_roofline(kind, 12 * BYTES_PER_VALUE[precision] * cells, launch_ms, hbm, note),
                               traffic=(lambda t: t * cells if t else None)(ncu_traffic(kind, precision)))
    return out


def e2e_leg(args, p, src, make, K, W, world, tuned=None):
    """The job through the C ABI with host buffers: upload the six FP64 fields
    from pinned host memory, K steps, download the six fields; all inside the
    timed region (wall clock, the step's result read back to the host)."""
    import torch
    cells = p.cells
    host = [torch.zeros(cells, dtype=torch.float64).pin_memory().numpy() for _ in range(6)]
    s = make()
    if tuned:
        s.autotune(reuse=True)  # the shape chosen before (cached)
    s.add_source(src)
    for c in range(6):  # warm-up job (not timed)
        s.copy_from_host(c, host[c])
    s.step(W)
    for c in range(6):
        s.copy_to_host(c, host[c])
    s.step_index = 0
    for c in range(6):
        host[c][...] = 0.0
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for c in range(6):
        s.copy_from_host(c, host[c])
    s.step(K)
    for c in range(6):
        s.copy_to_host(c, host[c])
    e2e_s = max_over_ranks(world, time.perf_counter() - t0)
    s.close()
    moved = 6 * cells * 8
    return {"value": world * cells * K / e2e_s / 1e9, "unit": UNIT,
            "h2d_bytes_per_step": moved / K, "d2h_bytes_per_step": moved / K,
            "job": "upload 6 FP64 fields (pinned) -> %d steps -> download 6 FP64 fields, via "
                   "fdtd_copy_field_*/fdtd_step" % K}


def fp64_leg(args, p, src, stream, world, K, W):
    """The FP64 drop-in: device-timed steps in the bitwise arithmetic and in
    the contracted one, each against the FP64 pipe's issue rate measured here."""
    from fdtd_method_gb300 import FDTD, Precision
    from fdtd_method_gb300.fdtd import measure_fp64_rate
    from fdtd_method_gb300.sources import COURANT_DT
    cells = p.cells
    peak, probe_ms = measure_fp64_rate()
    out = {"pipe_peak_instr_per_s": peak, "pipe_peak_note": "measured in this run: DMUL/DADD chains on every SM "
                                                             "(fdtd_measure_fp64_rate, %.1f ms)" % probe_ms}
    for name, contracted, instr in (("bitwise", False, FP64_INSTR_PER_CELL_STEP),
                                    ("contracted", True, FP64_FMA_INSTR_PER_CELL_STEP)):
        s = FDTD(p, COURANT_DT, Precision.FP64)
        s.set_fp64_arith(contracted)
        s.set_stream(stream.cuda_stream)
        s.add_source(src)
        s.step(min(W, 3))
        s.synchronize()
        ms = max_over_ranks(world, timed_steps(s, stream, K, world))
        s.close()
        v = replica_value(world, cells, K, ms)
        rate = v * 1e9 * instr / world
        out[name] = {"value": v, "unit": UNIT, "steps": K, "ms_per_step": ms / K,
                     "roofline": {"bound": "fp64-pipe", "instr_per_cell_step": instr, "achieved_instr_per_s": rate,
                                  "peak_instr_per_s": peak, "frac": rate / peak}}
    return out


def run_ours(args):
    import torch
    from fdtd_method_gb300 import FDTD, Precision
    from fdtd_method_gb300.sources import COURANT_DT

    world, rank, local = dist_init(args)
    if args.batch_only:
        stream = torch.cuda.Stream()
        out = run_batched(args, stream, world, with_accuracy=not args.no_batch_accuracy and rank == 0)
        if rank == 0:
            print(json.dumps(out))
        return
    p, src = workload(args)
    cells = p.cells
    K, W = args.steps, args.warmup
    hbm, hbm_note = measured_peaks()
    stream = torch.cuda.Stream()

    # --- chosen form, device-timed ---------------------------------------
    sim = make_sim(p, args.precision)
    sim.set_pipeline(args.pipeline, args.tile_y, args.kchunk, args.cells_per_thread)
    sim.set_stream(stream.cuda_stream)
    sim.add_source(src)
    tuned = None
    if not args.no_autotune and args.pipeline != "split" and not (args.tile_y or args.kchunk or args.cells_per_thread
                                                                   or args.depth):
        tuned = sim.autotune(sweeps=10, reuse=False)  # before the timed region; the state is only read
    if args.depth:
        sim.set_temporal_depth(args.depth)
    sim.step(W)
    sim.synchronize()
    sim.kernel_times()
    sim.set_kernel_timing(True)
    clocks = ClockSampler(local)
    clocks.start()
    ms = timed_steps(sim, stream, K, world)
    clk = clocks.stop()
    kt = sim.kernel_times()
    sim.set_kernel_timing(False)
    ms = max_over_ranks(world, ms)
    value = replica_value(world, cells, K, ms)
    launches = int(sum(n for _, n in kt.values()))

    bpv = BYTES_PER_VALUE[args.precision]
    kinds = {k: v for k, v in kt.items() if v[1] > 0}
    dom = max(kinds, key=lambda k: kinds[k][0])
    dom_ms = kinds[dom][0] / kinds[dom][1]
    dom_values = {"e_update": 9, "b_double": 9, "b_half": 9, "fused_step": 12, "fused_step2": 12}[dom]
    dom_bytes = dom_values * bpv * cells
    traffic_pc = ncu_traffic(dom, args.precision)
    roofline = dict(launch_roofline(dom, dom_bytes, dom_ms, hbm, hbm_note),
                    traffic=traffic_pc * cells if traffic_pc else None,
                    algorithmic_bytes_per_launch=dom_bytes,
                    per_kernel_ms={k: v[0] / v[1] for k, v in kinds.items()},
                    launches={k: v[1] for k, v in kinds.items()})
    step_alg = 12 * bpv  # per cell-step, zero stored J (sources evaluated in-kernel)
    step_roof = {"algorithmic_bytes_per_cell_step": step_alg,
                 "achieved": step_alg * cells * K / (ms / 1e3) / 1e9, "frac": step_alg * cells * K / (ms / 1e3) / 1e9 / hbm}
    # the reference callers' pattern: update_fields() once per step
    # (kokkos_sample.cpp:88-113), against step(K) just measured
    sim.synchronize()
    sim.kernel_times()
    sim.set_kernel_timing(True)
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t0.record(stream)
    for _ in range(K):
        sim.update_fields()
    t1.record(stream)
    t1.synchronize()
    kt_loop = sim.kernel_times()
    sim.set_kernel_timing(False)
    ms_loop = t0.elapsed_time(t1)
    update_loop = {"value": replica_value(world, cells, K, max_over_ranks(world, ms_loop)), "unit": UNIT,
                   "ms_per_step": ms_loop / K, "vs_step_n": (ms / K) / (ms_loop / K),
                   "launches": {k: v[1] for k, v in kt_loop.items() if v[1] > 0},
                   "job": "%d update_fields() calls, one step each (the reference driver's pattern)" % K}
    sim.close()
    del sim
    torch.cuda.empty_cache()

    # --- the other FP32-arithmetic forms (same workload and timing) -------
    forms = None
    if not args.no_forms:
        forms = {}
        for name in ("fp32_comp", "fp32", "fp16_scaled"):
            if name != args.precision:
                forms[name] = time_form(args, p, src, name, stream, world)
                torch.cuda.empty_cache()

    # --- batched form ------------------------------------------------------
    batched = None
    if not args.no_batch:
        batched = run_batched(args, stream, world, with_accuracy=not args.no_batch_accuracy and rank == 0)
        torch.cuda.empty_cache()

    # --- FP64 drop-in (bitwise and contracted) -----------------------------
    K64 = args.fp64_steps or max(20, K // 5)
    fp64 = fp64_leg(args, p, src, stream, world, K64, W)
    v64 = fp64["bitwise"]["value"]
    torch.cuda.empty_cache()

    # --- e2e through the C ABI with host buffers -------------------------
    e2e = None
    if not args.no_e2e:
        def make_chosen():
            s = make_sim(p, args.precision)
            s.set_pipeline(args.pipeline, args.tile_y, args.kchunk, args.cells_per_thread)
            return s
        e2e = e2e_leg(args, p, src, make_chosen, K, W, world, tuned)
        fp64["e2e"] = e2e_leg(args, p, src, lambda: FDTD(p, COURANT_DT, Precision.FP64), K, W, world)
        torch.cuda.empty_cache()

    # --- accuracy after the run length (every form against one FP64 run) --
    acc = None
    if not args.no_accuracy and rank == 0:
        ref = Fp64Reference(args, p, src)
        acc = form_accuracy(args, p, src, args.precision, ref)
        for name in (forms or {}):
            forms[name]["accuracy"] = form_accuracy(args, p, src, name, ref)
        s64 = FDTD(p, COURANT_DT, Precision.FP64)
        s64.set_fp64_arith(True)
        s64.add_source(src)
        s64.step(args.run_length)
        fp64["contracted"]["accuracy"] = ref.compare(s64, cells)
        s64.close()
        del ref
        torch.cuda.empty_cache()

    cpu = twin = None
    if not args.no_cpu and rank == 0 and world == 1:
        for kind in ("kokkos", "twin"):
            try:
                res = cpu_baseline_obj(run_cpu_baseline(args, kind=kind), args.n)
            except Exception as exc:  # reported, not fatal
                res = {"value": None, "unit": UNIT, "error": str(exc)[:300]}
            if kind == "kokkos":
                cpu = res
            else:
                twin = res

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
                "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "synthetic (seeded Gaussian-pulse source, zero initial fields)",
                "config": dict(config_dict(args, p, src), autotune=tuned), "clocks": clk, "e2e": e2e,
                "gpu_launches": launches, "update_fields_loop": update_loop,
                "roofline": roofline, "step_roofline": step_roof, "cpu_baseline": cpu,
                "cpu_baseline_openmp_twin": twin,
                "fp64": dict(fp64, value=v64, unit=UNIT, steps=K64, chosen_vs_fp64=value / v64),
                "accuracy": acc, "batched": batched, "forms": forms}
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_reference(args):
    """The reference's CPU path on the machine's host cores: the Kokkos path's
    driver loop restated in oracle/ (bit-identical to the reference's build),
    exactly --steps timed steps after --warmup (at least one), unless the
    steps would outrun REFERENCE_BUDGET_S; then as many as fit, and the line
    says so.  Under torchrun only rank 0 runs and prints."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    p, src = workload(args)
    warm = max(1, args.warmup)
    res = run_cpu_baseline(args, steps=max(1, args.steps), warmup=warm, budget=REFERENCE_BUDGET_S)
    cb = cpu_baseline_obj(res, args.n)
    note = ("reference Kokkos path restated in oracle/fdtd_oracle.c (bit-identical to the reference's own build), "
            "OpenMP on all host cores")
    if res.get("capped"):
        note += "; timed steps capped at %d by the %.0f s budget" % (res["steps"], REFERENCE_BUDGET_S)
    line = {"impl": "reference", "metric": METRIC, "value": res["value"], "unit": UNIT, "n_gpus": world,
            "steps": res["steps"], "warmup": res["warmup"], "ms_per_step": res["seconds"] / res["steps"] * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Gaussian-pulse source, zero initial fields)",
            "config": config_dict(args, p, src), "cpu_baseline": cb,
            "e2e": {"value": res["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": note}
    print(json.dumps(line))


def main():
    args = parse_args()
    if args.cpu_worker:
        cpu_worker(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
