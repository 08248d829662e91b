"""ORACLE — test infrastructure only.

CPU restatement of the reference's Yee step (fdtd_oracle.c, liboracle.so) and,
where the reference checkout is present, the reference's own sources compiled
against host stand-ins of Kokkos and googletest (_ref/).  Only the tests, the
engine's smoke check and the benchmark's CPU-baseline leg use this package, and
only as the checker; the engine never imports it.
"""
from .oracle import (Oracle, OraclePML, OracleSlab, RefKokkos, build_oracle, coefficients, field_sums, oracle_lib,  # noqa: F401
                     ref_available, ref_lib, run_reference_unit_tests)
