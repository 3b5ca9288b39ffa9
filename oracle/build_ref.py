"""Recipe: build the reference's own residency runtime with its CPU test backend (test infrastructure only).

Compiles compiler/runtime/scoped_runtime.cu of the reference, where it lies,
with g++ and the reference's own CPU-test and fault-injection switches
(-DFORT_SCOPE_CPU_TEST -DFORT_SCOPE_TEST_FAULTS, as its tests do in
compiler/tests/test_scoped_runtime.py:140-165 and test_scoped_access_batch.py:64-70)
into oracle/_ref/libscoped_ref.so. Tests use it to check that this repository's
runtime answers the same ABI calls with the same statuses and host values.
Nothing is copied: the source is read from the reference checkout, which
exists only on the development machine; elsewhere the recipe does nothing.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

# The reference checkout: F2C_REFERENCE_ROOT, else where the development machine keeps it.
REFERENCE = Path(os.environ.get("F2C_REFERENCE_ROOT", "/root/reference"))
SOURCE = REFERENCE / "compiler" / "runtime" / "scoped_runtime.cu"
OUT_DIR = Path(__file__).resolve().parent / "_ref"
LIBRARY = OUT_DIR / "libscoped_ref.so"
FLAGS = ["-DFORT_SCOPE_CPU_TEST", "-DFORT_SCOPE_TEST_FAULTS"]
STAMP = OUT_DIR / "libscoped_ref.flags"


def build_if_available() -> Path | None:
    if not SOURCE.exists():
        return LIBRARY if LIBRARY.exists() else None
    stamped = STAMP.exists() and STAMP.read_text() == " ".join(FLAGS)
    if LIBRARY.exists() and stamped and LIBRARY.stat().st_mtime >= SOURCE.stat().st_mtime:
        return LIBRARY
    cxx = shutil.which(os.environ.get("CXX", "g++"))
    if not cxx:
        return None
    OUT_DIR.mkdir(exist_ok=True)
    tmp = LIBRARY.with_suffix(f".{os.getpid()}.tmp")
    cmd = [cxx, "-std=c++17", "-O1", "-fPIC", "-shared", "-pthread", *FLAGS, "-x", "c++", str(SOURCE), "-o",
           str(tmp)]
    result = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    if result.returncode != 0:
        return None
    os.replace(tmp, LIBRARY)
    STAMP.write_text(" ".join(FLAGS))
    return LIBRARY


if __name__ == "__main__":
    print(build_if_available())
