"""Build recipe for the C oracle (test infrastructure only).

Compiles advection_oracle.c and stencil_oracle.c into oracle/_build/liboracle.so
with the reference's strict host numerical contract (-ffp-contract=off,
compiler/emission/numerical_contract.py:13-15) and OpenMP. Plain gcc, no
machine-specific flags, so the same recipe builds on x86_64 and aarch64.
"""

from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SOURCES = ("advection_oracle.c", "stencil_oracle.c")
OUT_DIR = HERE / "_build"
LIBRARY = OUT_DIR / "liboracle.so"
FLAGS = ("-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-std=c11", "-Wall")


def build(force: bool = False) -> Path:
    sources = [HERE / s for s in SOURCES]
    if (not force and LIBRARY.exists()
            and all(LIBRARY.stat().st_mtime >= s.stat().st_mtime for s in sources)):
        return LIBRARY
    OUT_DIR.mkdir(exist_ok=True)
    tmp = LIBRARY.with_suffix(f".{os.getpid()}.tmp")
    cc = os.environ.get("CC", "gcc")
    subprocess.run([cc, *FLAGS, *map(str, sources), "-o", str(tmp), "-lm"], check=True)
    os.replace(tmp, LIBRARY)
    return LIBRARY


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
