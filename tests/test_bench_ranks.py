"""The bench's multi-process path on CPU: torchrun with two gloo ranks (no GPU).

`bench.py --gpus N` runs N independent replicas (the advection step has no data-path exchange): each rank times its
own steps, the slowest rank's time is taken by an all-reduce, and rank 0 prints the whole-job value. The reference
arm runs on rank 0 only; the other ranks exit 0 without work.
"""

import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _torchrun(args, timeout=300):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_port()), *args]
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", OMP_NUM_THREADS="2")
    return subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=timeout)


def _json_lines(text):
    return [json.loads(line) for line in text.splitlines() if line.startswith("{")]


def test_two_gloo_ranks_take_the_slowest_time():
    run = _torchrun(["tests/ranks_probe.py"])
    assert run.returncode == 0, run.stderr[-2000:]
    lines = _json_lines(run.stdout)
    assert len(lines) == 1  # rank 0 alone prints
    line = lines[0]
    assert (line["world"], line["backend"], line["slowest_ms"]) == (2, "gloo", 11.0)
    assert abs(line["value"] - 2 * 1_000_000 * 5 / 11e-3 / 1e9) < 1e-12


def test_reference_arm_runs_on_rank_zero_only():
    run = _torchrun(["bench.py", "--impl", "reference", "--size", "48", "40", "16", "--steps", "2", "--warmup", "3"])
    assert run.returncode == 0, run.stderr[-2000:]
    lines = _json_lines(run.stdout)
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["unit"] == "Gpts/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
