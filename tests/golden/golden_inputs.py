"""Seeded inputs of the golden reference cases (shared by the generator and
the tests).  Values are k / 2^20 for integers k drawn by numpy's PCG64, so
every host regenerates them bit for bit."""
import numpy as np

# name -> grid, domain, steps, seed, which components get random data
CASES = {
    "random_12x10x7": {"n": (12, 10, 7), "steps": 5, "seed": 11, "comps": range(9)},
    "random_noJ_9x6x5": {"n": (9, 6, 5), "steps": 7, "seed": 12, "comps": range(6)},
    "tiny_1x1x1": {"n": (1, 1, 1), "steps": 4, "seed": 13, "comps": range(9)},
    "line_5x1x3": {"n": (5, 1, 3), "steps": 4, "seed": 14, "comps": range(9)},
    "line_1x7x1": {"n": (1, 7, 1), "steps": 3, "seed": 15, "comps": range(9)},
    "odd_7x3x5": {"n": (7, 3, 5), "steps": 6, "seed": 16, "comps": range(9)},
    "wide_33x2x2": {"n": (33, 2, 2), "steps": 5, "seed": 17, "comps": range(9)},
}


# Runs of the reference's OpenMP twin (FDTD_openmp::FDTD, src/FDTD/FDTD.cpp);
# with J != 0 they record its Jx line (:82-90), with J = 0 the Kokkos path
TWIN_CASES = {
    "twin_random_12x10x7": {"n": (12, 10, 7), "steps": 5, "seed": 31, "comps": range(9)},
    "twin_noJ_9x6x5": {"n": (9, 6, 5), "steps": 7, "seed": 32, "comps": range(6)},
    "twin_odd_7x3x5": {"n": (7, 3, 5), "steps": 6, "seed": 33, "comps": range(9)},
    "twin_tiny_1x1x1": {"n": (1, 1, 1), "steps": 4, "seed": 34, "comps": range(9)},
}


# PML cases (FDTD_PML(Parameters, dt, pml_percent)); same domain and inputs
PML_CASES = {
    "pml_random_20x16x12_p20": {"n": (20, 16, 12), "steps": 6, "seed": 21, "comps": range(9), "pml": 0.2},
    "pml_noJ_15x12x10_p25": {"n": (15, 12, 10), "steps": 8, "seed": 22, "comps": range(6), "pml": 0.25},
    "pml_zero_8x8x8_p0": {"n": (8, 8, 8), "steps": 5, "seed": 23, "comps": range(9), "pml": 0.0},
    "pml_flat_24x6x9_p15": {"n": (24, 6, 9), "steps": 7, "seed": 24, "comps": range(9), "pml": 0.15},
    "pml_odd_11x13x7_p30": {"n": (11, 13, 7), "steps": 4, "seed": 25, "comps": range(9), "pml": 0.3},
}


def case_params(spec):
    from fdtd_method_gb300.fdtd import Parameters
    Ni, Nj, Nk = spec["n"]
    # the reference unit tests' domain [0,1]x[0,2]x[0,3] (unit-tests/test_FDTD_method_kokkos.cpp:21-31)
    p = Parameters(Ni, Nj, Nk, 0.0, 1.0, 0.0, 2.0, 0.0, 3.0, 1.0 / Ni, 2.0 / Nj, 3.0 / Nk)
    # Courant number 0.3 on the finest axis
    dt = 0.3 * min(p.dx, p.dy, p.dz) / 3e10
    return p, dt


def case_inputs(spec):
    rng = np.random.default_rng(spec["seed"])
    n = spec["n"][0] * spec["n"][1] * spec["n"][2]
    return {c: rng.integers(-(1 << 20), 1 << 20, size=n).astype(np.float64) / float(1 << 20)
            for c in spec["comps"]}
