"""The integer-pipe binary64 additions and multiply (csrc/kernels/soft_fp64.cuh) against IEEE arithmetic.

The advection kernels compute their products with ``mul_rn_int`` instead of DMUL, so every bit-exact parity test
of the strict kernel already exercises it on the GPU; these tests check the two functions directly, over operand
distributions chosen to reach every rounding case (ties, cancellation, exponent ends, special values): on the host
against the host's IEEE doubles, and on the GPU against DADD/DMUL.
"""
import ctypes
import json
import shutil
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent / "soft_fp64"
KERNELS = Path(__file__).resolve().parents[1] / "fortran-to-cuda_gb300" / "csrc" / "kernels"


def test_host_matches_ieee(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    fake = tmp_path / "inc"
    fake.mkdir()
    (fake / "cuda_runtime.h").write_text("// empty: the check compiles the header as host C++\n")
    exe = tmp_path / "soft_fp64_host"
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", f"-I{fake}", f"-I{KERNELS}", f"-I{HERE}",
                    str(HERE / "soft_fp64_host.cpp"), "-o", str(exe)], check=True)
    run = subprocess.run([str(exe), "1000000"], capture_output=True, text=True, timeout=300)
    lines = [json.loads(line) for line in run.stdout.splitlines()]
    assert len(lines) == 21
    assert all(line["mismatches"] == 0 for line in lines), lines
    assert run.returncode == 0


@pytest.mark.gpu
def test_device_matches_dadd_dmul(cuda, tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    lib = tmp_path / "soft_fp64_device.so"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-shared",
                    "-Xcompiler", "-fPIC", f"-I{KERNELS}", f"-I{HERE}", str(HERE / "soft_fp64_device.cu"),
                    "-o", str(lib)], check=True)
    check = ctypes.CDLL(str(lib)).soft_fp64_device_check
    check.restype = ctypes.c_longlong
    check.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong, ctypes.c_ulonglong]
    for op in (0, 1, 2):
        for dist in range(7):
            for seed in (1, 2):
                assert check(op, dist, 0x5eed0000 + 977 * seed + 31 * dist + op, 1 << 24) == 0, (op, dist, seed)
