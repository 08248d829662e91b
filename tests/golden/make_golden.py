"""Generates the golden fixtures in this directory from the reference itself.

Runs only where the reference checkout has been compiled into oracle/_ref
(`make -C oracle ref`): the reference's own FDTD_kokkos sources, built
unmodified against the host Kokkos stand-in.  Outputs:

  reference_unit_tests.json  the values the reference's 24 convergence tests
                             measure (unit-tests/test_FDTD_method*.cpp)
  reference_cases.npz        final fields of small runs of FDTD_kokkos::FDTD
                             on seeded inputs (inputs are regenerated from the
                             seeds by `case_inputs`, exactly, on any host)
  reference_sample.json      stdout slices of the reference's kokkos_sample
                             program (perf-tests/kokkos_sample/kokkos_sample.cpp)
  reference_pml_cases.npz    final E and B of small runs of FDTD_kokkos::FDTD_PML
                             (src/FDTD_kokkos/FDTD_PML_kokkos.cpp) on seeded inputs
  reference_twin_cases.npz   final fields of small runs of the reference's
                             OpenMP twin FDTD_openmp::FDTD (src/FDTD/FDTD.cpp)

    python tests/golden/make_golden.py            # every fixture
    python tests/golden/make_golden.py twin pml   # the named ones only
"""
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from golden_inputs import CASES, PML_CASES, TWIN_CASES, case_inputs, case_params  # noqa: E402
from oracle import RefKokkos, run_reference_unit_tests  # noqa: E402
from oracle.oracle import REF_DIR  # noqa: E402


def unit_tests():
    tests = run_reference_unit_tests()
    with open(os.path.join(HERE, "reference_unit_tests.json"), "w") as f:
        json.dump({k: {"value": v[0], "expected": v[1], "tol": v[2], "passed": v[3]}
                   for k, v in sorted(tests.items())}, f, indent=1)


def runs(cases, kind, path):
    out = {}
    for name, spec in cases.items():
        params, dt = case_params(spec)
        ref = RefKokkos(params, dt, kind=kind)
        for comp, values in case_inputs(spec).items():
            ref.set(comp, values)
        ref.update_fields(spec["steps"])
        for comp in range(9):
            out["%s/%d" % (name, comp)] = ref.get(comp)
        ref.close()
    np.savez_compressed(os.path.join(HERE, path), **out)


def pml():
    out = {}
    for name, spec in PML_CASES.items():
        params, dt = case_params(spec)
        ref = RefKokkos(params, dt, pml_percent=spec["pml"])
        for comp, values in case_inputs(spec).items():
            ref.set(comp, values)
        ref.update_fields(spec["steps"])
        for comp in range(6):
            out["%s/%d" % (name, comp)] = ref.get(comp)
        ref.close()
    np.savez_compressed(os.path.join(HERE, "reference_pml_cases.npz"), **out)


def sample():
    sample = {}
    for n, it in ((16, 60), (32, 100), (20, 30)):
        r = subprocess.run([os.path.join(REF_DIR, "kokkos_sample"), str(n), str(it)],
                           capture_output=True, text=True, check=True, env=dict(os.environ, OMP_NUM_THREADS="2"))
        rows = [ln for ln in r.stdout.splitlines() if ln.strip() and ln.strip()[0] in "-0123456789"
                and "." in ln and "Execution" not in ln]
        sample["%d_%d" % (n, it)] = rows
    with open(os.path.join(HERE, "reference_sample.json"), "w") as f:
        json.dump(sample, f, indent=1)


FIXTURES = {
    "unit": unit_tests,
    "cases": lambda: runs(CASES, "kokkos", "reference_cases.npz"),
    "pml": pml,
    "sample": sample,
    "twin": lambda: runs(TWIN_CASES, "openmp", "reference_twin_cases.npz"),
}


def main(names):
    for name in names or sorted(FIXTURES):
        FIXTURES[name]()
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main(sys.argv[1:])
