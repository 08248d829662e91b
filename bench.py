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
  fp64       the same for the FP64 drop-in (bit-identical to the reference).
  e2e        the chosen form through the C ABI with host buffers: upload the
             six FP64 fields from pinned host memory, K steps, download them.
  accuracy   rel-L2 of the chosen form against the FP64 run after 1000 steps.
  roofline   the dominant kernel's algorithmic bytes / its mean CUDA-event
             duration against the measured HBM copy bandwidth.
  cpu_baseline  the reference's CPU path (restated in oracle/, OpenMP on all
             host cores, the reference driver's loop) on a bounded sample.
  batched    the batched form on its own workload (256 domains with edges
             uniform in 32..160 cells, plane wave + one pulse each), CUDA-graph
             step groups, one persistent launch per fused sweep.
  forms      the other storage forms (FP32, FP16 with per-component scale, or
             the compensated form) on the same workload and timing: value and
             their fused kernel's roofline.

--impl reference runs only that CPU path on the same workload and prints its
own line.  Under torchrun every rank runs its own replica (no data exchange;
weak scaling) and rank 0 prints the line.
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
# FP64 instructions per cell-step of the split FP64 pipeline (a merged
# double B half step: 21; E: 18); the GB300 FP64 pipe issues ~5.0e11/s.
FP64_INSTR_PER_CELL_STEP = 39
FP64_PIPE_PEAK = 5.0e11


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
    ap.add_argument("--cpu-worker", action="store_true", help=argparse.SUPPRESS)
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
    import numpy as np  # noqa: F401
    from oracle import Oracle
    from oracle.oracle import oracle_lib
    from fdtd_method_gb300.sources import COURANT_DT
    p, src = workload(args)
    o = Oracle(p, COURANT_DT)
    o.add_source(src)
    for c in range(9):  # first touch
        o.f[c][...] = 0.0
    t0 = time.perf_counter()
    o.step_driver(max(1, args.cpu_warmup))
    t_first = (time.perf_counter() - t0) / max(1, args.cpu_warmup)
    steps = args.cpu_steps or int(max(2, min(50, args.cpu_budget_s / max(t_first, 1e-3))))
    t0 = time.perf_counter()
    o.step_driver(steps)
    dt_s = time.perf_counter() - t0
    print(json.dumps({"steps": steps, "seconds": dt_s, "threads": int(oracle_lib().oracle_threads()),
                      "value": p.cells * steps / dt_s / 1e9}))


def run_cpu_baseline(args, steps=0, warmup=1, budget=15.0):
    cmd = [sys.executable, os.path.abspath(__file__), "--cpu-worker", "--n", str(args.n), "--seed", str(args.seed),
           "--run-length", str(args.run_length), "--cpu-steps", str(steps), "--cpu-warmup", str(warmup),
           "--cpu-budget-s", str(budget)] + (["--grid"] + [str(v) for v in args.grid] if args.grid else [])
    env = dict(os.environ)
    env.setdefault("OMP_PROC_BIND", "close")
    r = subprocess.run(cmd, capture_output=True, text=True, env=env)
    if r.returncode != 0:
        raise RuntimeError("CPU baseline failed: %s" % r.stderr[-2000:])
    return json.loads(r.stdout.strip().splitlines()[-1])


def cpu_baseline_obj(res, n):
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
# power-of-two storage scale of every component in the FP16 form (fields of
# this workload peak near 1e1; 2^6 keeps them clear of the subnormal range)
FP16_EXPONENTS = [6] * 6


def make_sim(p, precision_name):
    from fdtd_method_gb300 import FDTD
    from fdtd_method_gb300.sources import COURANT_DT
    s = FDTD(p, COURANT_DT, PREC[precision_name])
    if precision_name == "fp16_scaled":
        s.set_fp16_exponents(FP16_EXPONENTS)
    return s
BYTES_PER_VALUE = {"fp32_comp": 6, "fp32": 4, "fp16_scaled": 2, "fp64": 8}


def run_batched(args, stream, world):
    """The batched form on its own workload: `--batch-domains` periodic domains
    with edges uniform in 32..160 cells, a plane wave along a random axis and
    one Gaussian pulse each (seeded), stepped in CUDA-graph step groups of
    `--batch-group` steps (one persistent launch per fused sweep)."""
    import torch
    from fdtd_method_gb300 import FDTDBatch
    from fdtd_method_gb300.sources import COURANT_DT, batch_workload
    G = max(2, args.batch_group // 2 * 2)  # even: replays start from the same copy
    groups = max(1, args.steps // G)
    wl = batch_workload(count=args.batch_domains, seed=args.seed, n_steps=500)
    b = FDTDBatch([w[0] for w in wl], COURANT_DT, PREC[args.precision])
    b.set_stream(stream.cuda_stream)
    for q, (p, init, src) in enumerate(wl):
        if args.precision == "fp16_scaled":
            b.set_fp16_exponents(q, FP16_EXPONENTS)
        for c, v in init.items():
            b.copy_from_host(q, int(c), v)
        b.add_source(q, src)
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
    b.close()
    bpv = BYTES_PER_VALUE[args.precision]
    gbs = 12 * bpv * cells * steps / (ms / 1e3) / 1e9
    hbm, note = measured_peaks()
    edges = [w[0].Ni for w in wl] + [w[0].Nj for w in wl] + [w[0].Nk for w in wl]
    return {"value": world * cells * steps / (ms / 1e3) / 1e9, "unit": UNIT, "domains": len(wl), "cells": cells,
            "edge_min": min(edges), "edge_max": max(edges), "tiles_per_sweep": tiles, "steps": steps,
            "group_steps": G, "ms_per_step": ms / steps, "launches_per_group": G + 2, "autotune": tuned,
            "step_roofline": {"algorithmic_bytes_per_cell_step": 12 * bpv, "achieved": gbs, "peak": hbm,
                              "frac": gbs / hbm, "peak_note": note},
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
    del sim
    hbm, note = measured_peaks()
    fused = kt.get("fused_step")
    out = {"value": replica_value(world, cells, K, ms), "unit": UNIT, "ms_per_step": ms / K, "autotune": tuned}
    if fused and fused[1] > 0:
        launch_ms = fused[0] / fused[1]
        alg = 12 * BYTES_PER_VALUE[precision] * cells
        gbs = alg / (launch_ms / 1e3) / 1e9
        traffic_pc = ncu_traffic("fused_step", precision)
        out["roofline"] = {"bound": "hbm", "kernel": "fused_step", "achieved": gbs, "peak": hbm, "unit": "GB/s",
                           "frac": gbs / hbm, "peak_note": note, "mean_launch_ms": launch_ms,
                           "traffic": traffic_pc * cells if traffic_pc else None}
    return out


def run_ours(args):
    import numpy as np
    import torch
    from fdtd_method_gb300 import FDTD, Precision
    from fdtd_method_gb300.sources import COURANT_DT

    world, rank, local = dist_init(args)
    if args.batch_only:
        stream = torch.cuda.Stream()
        out = run_batched(args, stream, world)
        if rank == 0:
            print(json.dumps(out))
        return
    p, src = workload(args)
    cells = p.cells
    K, W = args.steps, args.warmup
    hbm, hbm_note = measured_peaks()
    stream = torch.cuda.Stream()
    out = {}

    # --- chosen form, device-timed ---------------------------------------
    sim = make_sim(p, args.precision)
    sim.set_pipeline(args.pipeline, args.tile_y, args.kchunk, args.cells_per_thread)
    sim.set_stream(stream.cuda_stream)
    sim.add_source(src)
    tuned = None
    if not args.no_autotune and args.pipeline != "split" and not (args.tile_y or args.kchunk or args.cells_per_thread):
        tuned = sim.autotune(sweeps=10, reuse=False)  # before the timed region; the state is only read
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
    dom_values = {"e_update": 9, "b_double": 9, "b_half": 9, "fused_step": 12}[dom]
    dom_bytes = dom_values * bpv * cells
    achieved = dom_bytes / (dom_ms / 1e3) / 1e9
    traffic_pc = ncu_traffic(dom, args.precision)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "peak_note": hbm_note,
                "traffic": traffic_pc * cells if traffic_pc else None,
                "algorithmic_bytes_per_launch": dom_bytes,
                "mean_launch_ms": dom_ms,
                "per_kernel_ms": {k: v[0] / v[1] for k, v in kinds.items()}}
    step_alg = 12 * bpv  # per cell-step, zero stored J (sources evaluated in-kernel)
    step_roof = {"algorithmic_bytes_per_cell_step": step_alg,
                 "achieved": step_alg * cells * K / (ms / 1e3) / 1e9, "frac": step_alg * cells * K / (ms / 1e3) / 1e9 / hbm}
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
        batched = run_batched(args, stream, world)
        torch.cuda.empty_cache()

    # --- FP64 drop-in ------------------------------------------------------
    K64 = args.fp64_steps or max(20, K // 5)
    s64 = FDTD(p, COURANT_DT, Precision.FP64)
    s64.set_stream(stream.cuda_stream)
    s64.add_source(src)
    s64.step(min(W, 3))
    s64.synchronize()
    ms64 = max_over_ranks(world, timed_steps(s64, stream, K64, world))
    v64 = world * cells * K64 / (ms64 / 1e3) / 1e9
    del s64

    # --- e2e through the C ABI with host buffers -------------------------
    e2e = None
    if not args.no_e2e:
        host = [torch.zeros(cells, dtype=torch.float64).pin_memory().numpy() for _ in range(6)]
        s = make_sim(p, args.precision)
        s.set_pipeline(args.pipeline, args.tile_y, args.kchunk, args.cells_per_thread)
        if tuned:
            s.autotune(reuse=True)  # the shape chosen above (cached)
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
        moved = 6 * cells * 8
        e2e = {"value": world * cells * K / e2e_s / 1e9, "unit": UNIT,
               "h2d_bytes_per_step": moved / K, "d2h_bytes_per_step": moved / K,
               "job": "upload 6 FP64 fields (pinned) -> %d steps -> download 6 FP64 fields, via fdtd_copy_field_*/fdtd_step" % K}
        del s, host

    # --- accuracy after the run length -----------------------------------
    acc = None
    if not args.no_accuracy and rank == 0:
        a = FDTD(p, COURANT_DT, Precision.FP64)
        b = make_sim(p, args.precision)
        b.set_pipeline(args.pipeline, args.tile_y, args.kchunk, args.cells_per_thread)
        for x in (a, b):
            x.add_source(src)
            x.step(args.run_length)
        num = den = 0.0
        per = {}
        bufa = np.empty(cells)
        bufb = np.empty(cells)
        names = ["Ex", "Ey", "Ez", "Bx", "By", "Bz"]
        for c in range(6):
            a.copy_to_host(c, bufa)
            b.copy_to_host(c, bufb)
            d = float(np.dot(bufa - bufb, bufa - bufb))
            n2 = float(np.dot(bufa, bufa))
            per[names[c]] = d
            num += d
            den += n2
        # each component's error normalised by the norm of all six FP64 fields
        per = {k: math.sqrt(v / den) for k, v in per.items()}
        ea, eb = a.energy(), b.energy()
        acc = {"steps": args.run_length, "rel_l2": math.sqrt(num / den), "rel_l2_per_component": per,
               "energy_fp64": ea, "energy_chosen": eb, "energy_rel_diff": (eb - ea) / ea if ea else None,
               "bar": 1e-5}
        del a, b

    cpu = None
    if not args.no_cpu and rank == 0 and world == 1:
        try:
            cpu = cpu_baseline_obj(run_cpu_baseline(args), args.n)
        except Exception as exc:  # reported, not fatal
            cpu = {"value": None, "unit": UNIT, "error": str(exc)[:300]}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
                "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "synthetic (seeded Gaussian-pulse source, zero initial fields)",
                "config": dict(config_dict(args, p, src), autotune=tuned), "clocks": clk, "e2e": e2e,
                "gpu_launches": launches,
                "roofline": roofline, "step_roofline": step_roof, "cpu_baseline": cpu,
                "fp64": {"value": v64, "unit": UNIT, "steps": K64, "ms_per_step": ms64 / K64,
                         "chosen_vs_fp64": value / v64,
                         "roofline": {"bound": "fp64-pipe", "achieved_instr_per_s": v64 * 1e9 * FP64_INSTR_PER_CELL_STEP / world,
                                      "peak_instr_per_s": FP64_PIPE_PEAK,
                                      "frac": v64 * 1e9 * FP64_INSTR_PER_CELL_STEP / world / FP64_PIPE_PEAK}},
                "accuracy": acc, "batched": batched, "forms": forms}
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_reference(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    p, src = workload(args)
    steps = max(1, min(args.steps, 30))
    res = run_cpu_baseline(args, steps=steps, warmup=max(1, min(args.warmup, 3)))
    cb = cpu_baseline_obj(res, args.n)
    line = {"impl": "reference", "metric": METRIC, "value": res["value"], "unit": UNIT, "n_gpus": world,
            "steps": res["steps"], "warmup": max(1, min(args.warmup, 3)), "ms_per_step": res["seconds"] / res["steps"] * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Gaussian-pulse source, zero initial fields)",
            "config": config_dict(args, p, src), "cpu_baseline": cb,
            "e2e": {"value": res["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference Kokkos path restated in oracle/fdtd_oracle.c (bit-identical to the reference's "
                    "own build), OpenMP on all host cores; timed steps capped at 30"}
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
