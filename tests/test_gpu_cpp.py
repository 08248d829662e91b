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


def test_cpp_sample_pml_run_uses_the_pml_class():
    """The sample's PML option (the reference sample's __PML_TEST__ block)
    drives FDTD_gb300::FDTD_PML; the periodic slice is unchanged and the
    layer's field sum matches the Python PML class on the same job."""
    golden = json.load(open(os.path.join(GOLDEN, "reference_sample.json")))
    r = subprocess.run([os.path.join(BIN, "fdtd_sample"), "16", "60", "pml"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "Execution time (PML)" in r.stdout
    rows = [ln for ln in r.stdout.splitlines() if ln.strip() and "Execution" not in ln and "PML" not in ln]
    assert [x.split() for x in rows] == [x.split() for x in golden["16_60"]]
    value = float([ln for ln in r.stdout.splitlines() if ln.startswith("PML field square sum")][0].split()[-1])

    from fdtd_method_gb300 import FDTD_PML, sources
    from fdtd_method_gb300.fdtd import CurrentParameters, Parameters
    d = 3e10
    p = Parameters(16, 16, 16, -8 * d, 8 * d, -8 * d, 8 * d, -8 * d, 8 * d, d, d, d)
    cp = CurrentParameters(8, 4, 0.2)
    src, _ = sources.sample_box_source(p, cp, iterations=60)
    s = FDTD_PML(p, cp.dt, 0.2)
    s.add_source(src)
    s.step(60)
    assert value == pytest.approx(float(s.field_sums()[:6].sum()), rel=1e-6)


def _coarray_job(n, iterations):
    """The coarray program's grid and box current (coarray/fdtd.F90:36-52 and
    init_currents, :184-204), as a whole-grid source."""
    import math

    import numpy as np

    from fdtd_method_gb300 import Const, Parameters, SeparableSource
    C, PI = Const.C, Const.PI
    dx, dt, TT = C, 0.2, 8.0
    Tx = 4 * C
    current_time = min(int(TT / dt), iterations)
    bnd = n / 2.0 * dx
    start = int(math.floor((-Tx / 4.0 + bnd) / dx))
    stop = int(math.floor((Tx / 4.0 + bnd) / dx))
    g = np.array([math.pow(math.cos(2.0 * PI * v * dx / Tx), 2.0) for v in range(start, stop + 1)])
    amp = np.array([math.sin(2.0 * PI * (t + 1) * dt / TT) for t in range(current_time)])
    p = Parameters(n, n, n, -bnd, bnd, -bnd, bnd, -bnd, bnd, dx, dx, dx)
    return p, dt, SeparableSource(7, start % n, start % n, start % n, g, g, g, amp)


@pytest.mark.parametrize("slabs", [1, 3, 5])
def test_cpp_coarray_twin_slabs_print_the_whole_grid_slice(slabs):
    """The coarray program's twin on z slabs prints the slice that one
    whole-grid handle computes for the same job, digit for digit."""
    from fdtd_method_gb300 import FDTD
    n, it = 32, 20
    r = subprocess.run([os.path.join(BIN, "fdtd_coarray_sample"), str(n), str(it), str(slabs)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    assert lines[0] == "Running on %d images" % slabs
    assert lines[1].startswith("Total execution time: ") and lines[1].endswith(" seconds")
    got = [ln.split() for ln in lines[2:] if ln.strip()]
    p, dt, src = _coarray_job(n, it)
    sim = FDTD(p, dt)
    sim.add_source(src)
    sim.step(it)
    ex = sim.get_field(0).numpy().reshape(n, n, n)  # (k, j, i)
    want = [["%.5f" % ex[n // 2, j, i] for i in range(n // 2 - 5, n // 2 + 5)] for j in range(n // 2 - 5, n // 2 + 5)]
    assert got == want
    assert any(float(v) != 0.0 for row in got for v in row)
    sim.close()
