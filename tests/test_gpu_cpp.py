"""The C++ drop-in class (include/fdtd_gb300.hpp) as a user of the reference's
API would drive it: the reference's convergence tests restated in C++ and the
GPU twin of the reference's sample program, checked against the reference's
own recorded results."""
import json
import os
import subprocess

import pytest

from fdtd_method_gb300 import build

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
BIN = os.path.dirname(os.path.abspath(build.__file__))


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def test_cpp_convergence_tests_reproduce_reference_ratios():
    r = subprocess.run([os.path.join(BIN, "convergence_tests")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    golden = json.load(open(os.path.join(GOLDEN, "reference_unit_tests.json")))
    lines = [ln.split() for ln in r.stdout.splitlines() if ln.startswith("NEAR")]
    assert len(lines) == 12
    for _, name, value, _, _, status in lines:
        assert status == "PASS"
        assert float(value) == pytest.approx(golden[name]["value"], rel=1e-12, abs=0)


@pytest.mark.parametrize("key", ["16_60", "32_100", "20_30"])
def test_cpp_sample_twin_prints_reference_slice(key):
    golden = json.load(open(os.path.join(GOLDEN, "reference_sample.json")))
    n, it = key.split("_")
    r = subprocess.run([os.path.join(BIN, "fdtd_sample"), n, it], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    rows = [ln for ln in r.stdout.splitlines() if ln.strip() and "Execution" not in ln]
    assert [x.split() for x in rows] == [x.split() for x in golden[key]]


def test_cpp_sample_rejects_wrong_argument_count():
    r = subprocess.run([os.path.join(BIN, "fdtd_sample"), "16"], capture_output=True, text=True)
    assert r.returncode == 1
    assert "Incorrect number of parameters" in r.stdout
