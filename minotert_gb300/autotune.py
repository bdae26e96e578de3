"""Autotuner for the traversal launch schedule (mrt_tuning).

Sweeps persistent blocks per SM (warps per SM = 4 x blocks), the work-fetch
mode of the persistent kernels, the primary-ray kernel form, the ray-sort
threshold, the path tail, the spreading of triangle tests over the warp and
the refill threshold on a caller-supplied frame function, timing each
candidate with CUDA events on the frame's stream, and keeps the fastest.
Results are cached as JSON keyed by GPU and workload, so a renderer pays
for the sweep once.

    best = autotune(ctx, run_frame, stream, key="icospheres_1080p")
    ctx.set_tuning(**best["tuning"])
"""
from __future__ import annotations

import itertools
import json
import statistics
from pathlib import Path

from ._lib import Context, MrtError

DEFAULT_CACHE = Path(__file__).resolve().parent / "_build" / "autotune.json"


SORT_NEVER = 0xFFFFFFFF


def candidates(max_blocks_per_sm: int, sort: bool = False):
    blocks = sorted({b for b in (1, 2, 3, 4, 5, 6, 8) if b <= max_blocks_per_sm} | {max_blocks_per_sm})
    sort_thr = [SORT_NEVER, 1 << 18, 1 << 14] if sort else [SORT_NEVER]
    # dynamic_fetch bit 0: extension rays, bit 1: shadow rays
    # tail_bounce: 0 = wavefront passes for every bounce, 3 = one persistent
    # launch finishes the paths alive at bounce 3
    # tri_spread bit 0: the extension rays' triangle tests spread over the warp
    # refill_min: idle lanes a warp waits for before fetching new rays
    for b, dyn, prim, thr, tail, spread, rmin in itertools.product(blocks, (1, 3, 0, 2), (0, 1), sort_thr, (3, 0),
                                                                   (1, 0), (8, 1)):
        yield {"trace_blocks_per_sm": b, "dynamic_fetch": dyn, "primary_persistent": prim, "sort_min_rays": thr,
               "tail_bounce": tail, "tri_spread": spread, "refill_min": rmin}


def time_frames(ctx: Context, run_frame, stream, frames: int, warmup: int) -> float:
    """Median milliseconds of `frames` calls of run_frame(stream)."""
    for _ in range(warmup):
        run_frame(stream)
    evs = [(ctx.event(), ctx.event()) for _ in range(frames)]
    for a, b in evs:
        ctx.record(a, stream)
        run_frame(stream)
        ctx.record(b, stream)
    ctx.sync(stream)
    return statistics.median(ctx.elapsed_ms(a, b) for a, b in evs)


def autotune(ctx: Context, run_frame, stream=None, key: str = "default", frames: int = 5, warmup: int = 2,
             cache: Path | None = DEFAULT_CACHE, sort: bool = False, space=None) -> dict:
    gpu_key = None
    if cache is not None and cache.exists():
        try:
            db = json.loads(cache.read_text())
        except ValueError:
            db = {}
    else:
        db = {}
    info = ctx.device_info()
    gpu_key = f"{info.name.decode(errors='replace')}:sm{info.cc_major}{info.cc_minor}"
    full_key = f"{gpu_key}:{key}"
    if full_key in db and space is None:
        ctx.set_tuning(**db[full_key]["tuning"])
        return db[full_key]
    saved = ctx.tuning()
    max_b = max(1, int(info.trace_blocks_per_sm_max))
    results = []
    for cand in (space or candidates(max_b, sort)):
        try:
            ctx.set_tuning(**cand)
            ms = time_frames(ctx, run_frame, stream, frames, warmup)
        except MrtError as e:  # a schedule this workload cannot run (e.g. a stack below its BVH depth)
            results.append({"tuning": cand, "ms": None, "refused": str(e)})
            continue
        results.append({"tuning": cand, "ms": ms})
    best = min((r for r in results if r["ms"] is not None), key=lambda r: r["ms"])
    ctx.set_tuning(**best["tuning"])
    out = {"tuning": best["tuning"], "ms": best["ms"], "results": results,
           "default_ms": next((r["ms"] for r in results
                               if all(_as_dict(saved).get(k) == v for k, v in r["tuning"].items())), None)}
    if cache is not None:
        cache.parent.mkdir(parents=True, exist_ok=True)
        db[full_key] = out
        cache.write_text(json.dumps(db, indent=1))
    return out


def _as_dict(t) -> dict:
    return {f: int(getattr(t, f)) for f, _ in t._fields_}
