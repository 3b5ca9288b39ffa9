"""Schedule choices of the advection templates and the autotuner that makes them.

The reference schedules every nest the same way: axis order by unit-stride
locality, no tiling, 256-thread blocks (compiler/scheduling/planner.py:82-123,
compiler/ir/plan.py:31). Here a batched step has two shape choices: the tile
height (4, 8 or 16 rows of 32 points; one warp per row plus an edge warp, the
fast-fp kernel for 4 and 16) for the whole persistent launch, and per instance
the depth of the z-chunk an item of work covers: deep chunks amortise the
per-chunk prologue (the bottom faces of the first level), shallow chunks and
short tiles give the persistent kernel more items to balance across SMs. The
best choice depends on the instances' sizes, so the autotuner times the real
batched step on the GPU (coordinate descent: the tile height, then a depth
per nz bucket, repeated while it improves) and caches the choice per GPU name,
scalar count, output mask and numerical contract in ``tuned.json`` next to
this file.
"""

from __future__ import annotations

import json
import time
from pathlib import Path

CACHE = Path(__file__).with_name("tuned.json")
CANDIDATES = (8, 16, 24, 32, 48, 64, 96)
ROWS = (4, 8, 16)
DEFAULT_KZ = 32
DEFAULT_ROWS = 8


def bucket(nz: int) -> str:
    """Height bucket of an instance: the reference ensemble draws nz from {32, 64, 96}."""
    for bound in (16, 32, 48, 64, 96, 128, 192, 256):
        if nz <= bound:
            return f"nz<={bound}"
    return "nz>256"


def _key(gpu: str, nscalar: int, mask: int, numerics: str = "strict") -> str:
    base = f"{gpu}|scalars={nscalar}|mask={mask}"
    return base if numerics == "strict" else f"{base}|{numerics}"


def load_cache() -> dict:
    if CACHE.exists():
        return json.loads(CACHE.read_text())
    return {}


def _table(gpu: str, nscalar: int, mask: int, numerics: str) -> dict:
    cache = load_cache()
    return cache.get(_key(gpu, nscalar, mask, numerics)) or cache.get(_key(gpu, nscalar, mask), {})


def kz_for(shapes, gpu: str, nscalar: int, mask: int = 7, numerics: str = "strict") -> list[int]:
    """Per-instance z-chunk depths from the cache (DEFAULT_KZ where nothing was tuned)."""
    table = _table(gpu, nscalar, mask, numerics)
    return [int(table.get(bucket(nz), DEFAULT_KZ)) for (_, _, nz) in shapes]


def rows_for(gpu: str, nscalar: int, mask: int = 7, numerics: str = "strict") -> int:
    """The tile height from the cache (8 where nothing was tuned; always 8 for the strict kernel)."""
    if numerics == "strict":
        return DEFAULT_ROWS
    return int(_table(gpu, nscalar, mask, numerics).get("tile_rows", DEFAULT_ROWS))


def tune(shapes, gpu: str, nscalar: int, time_step, mask: int = 7, passes: int = 2, write: bool = True,
         numerics: str = "strict") -> dict:
    """Pick a tile height and a depth per bucket. ``time_step(kz_list, rows) -> seconds per step`` runs the batch.

    The strict kernel has 8-row tiles only; the fast-fp kernel tries 4, 8 and 16."""
    buckets = sorted({bucket(nz) for (_, _, nz) in shapes})
    choice = {b: DEFAULT_KZ for b in buckets}
    rows = DEFAULT_ROWS
    row_candidates = ROWS if numerics == "fast" else (DEFAULT_ROWS,)

    def kz_list(table):
        return [table[bucket(nz)] for (_, _, nz) in shapes]

    best = time_step(kz_list(choice), rows)
    history = [{"kz": dict(choice), "tile_rows": rows, "seconds": best}]
    for _ in range(passes):
        improved = False
        for cand in row_candidates:
            if cand == rows:
                continue
            t = time_step(kz_list(choice), cand)
            history.append({"kz": dict(choice), "tile_rows": cand, "seconds": t})
            if t < best * 0.995:
                best, rows, improved = t, cand, True
        for b in buckets:
            heights = [nz for (_, _, nz) in shapes if bucket(nz) == b]
            for cand in CANDIDATES:
                if cand == choice[b] or cand > max(heights):
                    continue
                trial = dict(choice)
                trial[b] = cand
                t = time_step(kz_list(trial), rows)
                history.append({"kz": dict(trial), "tile_rows": rows, "seconds": t})
                if t < best * 0.995:
                    best, choice, improved = t, trial, True
        if not improved:
            break
    result = {"choice": {**choice, "tile_rows": rows}, "seconds_per_step": best, "trials": len(history),
              "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())}
    if write:
        cache = load_cache()
        key = _key(gpu, nscalar, mask, numerics)
        cache[key] = {**choice, "tile_rows": rows}
        cache.setdefault("_history", {})[key] = result
        CACHE.write_text(json.dumps(cache, indent=1, sort_keys=True) + "\n")
    return result
