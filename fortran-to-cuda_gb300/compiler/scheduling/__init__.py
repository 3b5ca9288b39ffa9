"""Schedule choices of the advection templates and the autotuner that makes them.

The reference schedules every nest the same way: axis order by unit-stride
locality, no tiling, 256-thread blocks (compiler/scheduling/planner.py:82-123,
compiler/ir/plan.py:31). Here the column-tile shape is fixed by the kernel
(32 x 8 points, one warp per row plus an edge warp), and what varies is the
depth of the z-chunk an item of work covers: deep chunks amortise the per-chunk
prologue (the bottom faces of the first level), shallow chunks give the
persistent batched kernel more items to balance across SMs. The best depth
depends on the instance's height, so the autotuner picks one per nz bucket by
timing the real batched step on the GPU (coordinate descent over the buckets),
and caches the choice per GPU name, scalar count and bucket set in
``tuned.json`` next to this file.
"""

from __future__ import annotations

import json
import time
from pathlib import Path

CACHE = Path(__file__).with_name("tuned.json")
CANDIDATES = (8, 16, 24, 32, 48, 64, 96)
DEFAULT_KZ = 32


def bucket(nz: int) -> str:
    """Height bucket of an instance: the reference ensemble draws nz from {32, 64, 96}."""
    for bound in (16, 32, 48, 64, 96, 128, 192, 256):
        if nz <= bound:
            return f"nz<={bound}"
    return "nz>256"


def _key(gpu: str, nscalar: int, mask: int) -> str:
    return f"{gpu}|scalars={nscalar}|mask={mask}"


def load_cache() -> dict:
    if CACHE.exists():
        return json.loads(CACHE.read_text())
    return {}


def kz_for(shapes, gpu: str, nscalar: int, mask: int = 7) -> list[int]:
    """Per-instance z-chunk depths from the cache (DEFAULT_KZ where nothing was tuned)."""
    table = load_cache().get(_key(gpu, nscalar, mask), {})
    return [int(table.get(bucket(nz), DEFAULT_KZ)) for (_, _, nz) in shapes]


def tune(shapes, gpu: str, nscalar: int, time_step, mask: int = 7, passes: int = 2, write: bool = True) -> dict:
    """Pick a depth per bucket. ``time_step(kz_list) -> seconds per step`` runs the batch on the GPU."""
    buckets = sorted({bucket(nz) for (_, _, nz) in shapes})
    choice = {b: DEFAULT_KZ for b in buckets}

    def kz_list(table):
        return [table[bucket(nz)] for (_, _, nz) in shapes]

    best = time_step(kz_list(choice))
    history = [{"kz": dict(choice), "seconds": best}]
    for _ in range(passes):
        improved = False
        for b in buckets:
            heights = [nz for (_, _, nz) in shapes if bucket(nz) == b]
            for cand in CANDIDATES:
                if cand == choice[b] or cand > max(heights):
                    continue
                trial = dict(choice)
                trial[b] = cand
                t = time_step(kz_list(trial))
                history.append({"kz": dict(trial), "seconds": t})
                if t < best * 0.995:
                    best, choice, improved = t, trial, True
        if not improved:
            break
    result = {"choice": choice, "seconds_per_step": best, "trials": len(history),
              "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())}
    if write:
        cache = load_cache()
        cache[_key(gpu, nscalar, mask)] = dict(choice)
        cache.setdefault("_history", {})[_key(gpu, nscalar, mask)] = result
        CACHE.write_text(json.dumps(cache, indent=1, sort_keys=True) + "\n")
    return result
