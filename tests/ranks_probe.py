"""Run by tests/test_bench_ranks.py under torchrun: the bench's rank plumbing on gloo, without a GPU."""

import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import torch  # noqa: E402

import bench  # noqa: E402

dist, rank, world, local = bench.dist_setup()
bench.barrier(dist, torch)
slowest = bench.max_over_ranks(dist, torch, 10.0 + rank)  # rank r "took" 10 + r ms
value = bench.whole_job_value(1_000_000, world, 5, slowest)
bench.barrier(dist, torch)
if rank == 0:
    print(json.dumps({"world": world, "backend": dist.get_backend(), "slowest_ms": slowest, "value": value}))
dist.destroy_process_group()
