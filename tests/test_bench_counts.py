"""The bench's per-point operation counts: FP64-pipe and integer-pipe operations add up to each kernel's DAG.

The fast-fp DAG is 65 + 5 + 7·NS operations for U, V, W and NS scalars (51 without scalars), the strict one
90 + 3 + 11·NS (93 without scalars, the halving of U, V, W included); the bench reports them split by the pipe
that runs them.
"""
import sys
from pathlib import Path

import pytest

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
import bench  # noqa: E402


@pytest.mark.parametrize("nscalar", [0, 1, 2, 3, 4])
def test_counts_add_up_to_the_dag(nscalar):
    fast = 51 + (8 + 7 * nscalar if nscalar else 0)
    strict = 93 + (3 + 11 * nscalar if nscalar else 0)
    assert bench.fp64_ops_per_point(nscalar, "fast") + bench.int_pipe_ops_per_point(nscalar, "fast") == fast
    assert bench.fp64_ops_per_point(nscalar, "strict") + bench.int_pipe_ops_per_point(nscalar, "strict") == strict


def test_headline_counts():
    # the three-scalar step the bench line reports: 62 + 18 fast-fp, 99 + 30 strict
    assert (bench.fp64_ops_per_point(3, "fast"), bench.int_pipe_ops_per_point(3, "fast")) == (62, 18)
    assert (bench.fp64_ops_per_point(3, "strict"), bench.int_pipe_ops_per_point(3, "strict")) == (99, 30)
    # an advance keeps the leading FMA of each sum on the FP64 pipe
    assert bench.fp64_ops_per_point(3, "fast", mode="advance") == 68
