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

    python tests/golden/make_golden.py
"""
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from golden_inputs import CASES, PML_CASES, case_inputs, case_params  # noqa: E402
from oracle import RefKokkos, run_reference_unit_tests  # noqa: E402
from oracle.oracle import REF_DIR  # noqa: E402


def main():
    tests = run_reference_unit_tests()
    with open(os.path.join(HERE, "reference_unit_tests.json"), "w") as f:
        json.dump({k: {"value": v[0], "expected": v[1], "tol": v[2], "passed": v[3]}
                   for k, v in sorted(tests.items())}, f, indent=1)

    out = {}
    for name, spec in CASES.items():
        params, dt = case_params(spec)
        ref = RefKokkos(params, dt)
        for comp, values in case_inputs(spec).items():
            ref.set(comp, values)
        ref.update_fields(spec["steps"])
        for comp in range(9):
            out["%s/%d" % (name, comp)] = ref.get(comp)
        ref.close()
    np.savez_compressed(os.path.join(HERE, "reference_cases.npz"), **out)

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

    sample = {}
    for n, it in ((16, 60), (32, 100), (20, 30)):
        r = subprocess.run([os.path.join(REF_DIR, "kokkos_sample"), str(n), str(it)],
                           capture_output=True, text=True, check=True, env=dict(os.environ, OMP_NUM_THREADS="2"))
        rows = [ln for ln in r.stdout.splitlines() if ln.strip() and ln.strip()[0] in "-0123456789"
                and "." in ln and "Execution" not in ln]
        sample["%d_%d" % (n, it)] = rows
    with open(os.path.join(HERE, "reference_sample.json"), "w") as f:
        json.dump(sample, f, indent=1)
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
