"""The cdu driver restated (compiler/cdu.py): its report format on CPU, its run through the runtime on GPU."""

import numpy as np
import pytest

from compiler import cdu
from compiler import workloads as wl


def test_fortran_es24_16_format():
    assert cdu.fortran_es(123456.78901234567) == "  1.2345678901234567E+05"
    assert cdu.fortran_es(-0.001) == " -1.0000000000000000E-03"
    assert cdu.fortran_es(0.0) == "  0.0000000000000000E+00"
    assert len(cdu.fortran_es(1e-150)) == 24 and cdu.fortran_es(1e-150).endswith("-150")


def test_sequential_sum_is_left_to_right():
    values = np.array([1e16, 1.0, -1e16, 1.0])
    # pairwise summation would give 2.0 or 0.0 in another order; left to right: (1e16 + 1) - 1e16 + 1 = 1.0
    assert cdu.sequential_sum(values) == ((1e16 + 1.0) - 1e16) + 1.0


def test_report_lines():
    text = cdu.report({"nx": 8, "ny": 4, "nz": 2, "iterations": 3, "warmup": 1, "total_ms": 1.5,
                       "ms_per_iter": 0.5, "checksum": 2.0})
    assert text.splitlines() == [
        "--- CDU benchmark ---", "grid:         8 x 4 x 2", "iterations:   3", "warmup_iters: 1",
        "total_ms:              1.500 ms", "ms_per_iter:           0.500 ms",
        "checksum:       2.0000000000000000E+00"]


@pytest.mark.gpu
def test_driver_checksum_equals_the_oracle(cuda):
    from oracle import api

    nx, ny, nz = 40, 24, 16
    r = cdu.run(nx, ny, nz, iterations=3, warmup=1, seed=7)
    f = wl.reference_driver_fields(nx, ny, nz, 7)
    ref = api.momentum("cdu", np.zeros_like(f.U), f.U, f.V, f.W, f.geometry.dx, f.geometry.dy, f.geometry.dz, 1)
    interior = (slice(1, nz + 1), slice(1, ny + 1), slice(1, nx + 1))
    assert np.array_equal(r["u2"][interior].view(np.int64), ref[interior].view(np.int64))
    assert r["checksum"] == cdu.sequential_sum(ref[interior])


@pytest.mark.gpu
def test_driver_fast_fp_is_within_the_tolerance(cuda):
    from oracle import api
    from tolerance import check

    nx, ny, nz = 40, 24, 16
    r = cdu.run(nx, ny, nz, iterations=2, warmup=1, seed=7, fast_fp=True)
    f = wl.reference_driver_fields(nx, ny, nz, 7)
    ref = api.momentum("cdu", np.zeros_like(f.U), f.U, f.V, f.W, f.geometry.dx, f.geometry.dy, f.geometry.dz, 1)
    interior = (slice(1, nz + 1), slice(1, ny + 1), slice(1, nx + 1))
    check(r["u2"][interior], ref[interior], "U2")
    assert not np.array_equal(r["u2"][interior].view(np.int64), ref[interior].view(np.int64))  # the fast kernel ran
