"""The benchmark's JSON contract, checked on the host.

* The reference arm (`bench.py --impl reference`, the reference's CPU path
  restated in oracle/) prints one line with the metric, exactly --steps timed
  steps after --warmup, a cpu_baseline describing its own run and an e2e
  object with no host transfers; under torchrun only rank 0 prints.
* The roofline helper's arithmetic, and the committed DRAM-traffic table the
  bench line's `traffic` comes from (one entry per FP32-arithmetic form).
"""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _reference_line(extra_env=None, steps=3, warmup=3):
    env = dict(os.environ)
    env.update(extra_env or {})
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--grid", "24", "20",
                        "16", "--steps", str(steps), "--warmup", str(warmup)],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    return lines


def test_reference_arm_prints_one_contract_line():
    lines = _reference_line(steps=4, warmup=3)
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["steps"] == 4 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["value"] > 0 and d["higher_is_better"] is True and d["vs_baseline"] is None
    assert d["dtype"] == "f64" and "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_print_nothing():
    lines = _reference_line({"WORLD_SIZE": "2", "RANK": "1", "LOCAL_RANK": "1"})
    assert lines == []


def test_launch_roofline_arithmetic():
    r = bench.launch_roofline("fused_step", 72 * 512 ** 3, 1.8, 6674.8, "of measured")
    assert r["achieved"] == pytest.approx(72 * 512 ** 3 / 1.8e-3 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / 6674.8)
    assert r["effective_frac"] == pytest.approx(r["frac"]) and r["unit"] == "GB/s" and r["bound"] == "hbm"
    r2 = bench.launch_roofline("fused_step2", 72 * 512 ** 3, 3.6, 6674.8, "of measured")
    assert r2["steps_per_launch"] == 2 and r2["effective_frac"] == pytest.approx(2 * r2["frac"])


@pytest.mark.parametrize("prec,alg", [("fp32_comp", 72), ("fp32", 48), ("fp16_scaled", 24)])
def test_traffic_table_has_every_form(prec, alg):
    t = bench.ncu_traffic("fused_step", prec)
    assert t is not None
    # actual DRAM bytes sit at or above the algorithmic bytes, and not far above
    assert alg <= t <= 1.3 * alg
