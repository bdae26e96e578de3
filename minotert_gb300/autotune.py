"""Autotuner for the traversal launch schedule (mrt_tuning).

Tunes persistent blocks per SM (warps per SM = 4 x blocks), the work-fetch
mode of the persistent kernels, the primary-ray kernel form, the ray-sort
threshold, the path tail (and whether it starts from the wavefront's hits),
the spreading of triangle tests over the warp, the refill threshold and the
overlapped shadow rays on a caller-supplied
frame function, timing each candidate with CUDA events on the frame's
stream, and keeps the fastest.  The default search is coordinate-wise: from
the current schedule, each knob in turn takes each of its values with the
others held, a change is kept when it is at least 0.5 % faster, and the
pass repeats until nothing changes (at most `rounds` passes) -- tens of
candidates instead of the thousands of the full product.  An explicit
`space` (a list of tuning dicts) is swept exhaustively instead.  Results are
cached as JSON keyed by GPU and workload, so a renderer pays for the search
once.

    best = autotune(ctx, run_frame, stream, key="icospheres_1080p")
    ctx.set_tuning(**best["tuning"])
"""
from __future__ import annotations

import json
import statistics
from pathlib import Path

from ._lib import Context, MrtError

DEFAULT_CACHE = Path(__file__).resolve().parent / "_build" / "autotune.json"


SORT_NEVER = 0xFFFFFFFF


def knobs(max_blocks_per_sm: int, sort: bool = False) -> dict:
    """The values each schedule knob may take in the coordinate search."""
    blocks = sorted({b for b in (2, 4, 6, 8) if b <= max_blocks_per_sm} | {max_blocks_per_sm, 0})
    return {
        "trace_blocks_per_sm": blocks,            # 0 = occupancy maximum
        "dynamic_fetch": [3, 1, 0, 2],            # bit 0 extension, bit 1 shadow rays
        "tri_spread": [11, 3, 1, 0, 15],          # bit 0 extension, 1 shadow, 2 primary rays, 3 the tail
        "refill_min": [8, 4, 12, 1],              # idle lanes before a refill
        "overlap_shadow": [1, 0],                 # shadow rays beside the next extension trace
        "tail_bounce": [3, 0, 2, 4],              # paths alive at this bounce finish in one launch
        "tail_from_hits": [1, 0],                 # ... starting from that bounce's wavefront hits
        "primary_persistent": [0, 1],
        "sort_min_rays": [SORT_NEVER, 1 << 18, 1 << 14] if sort else [SORT_NEVER],
    }


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


def coordinate_search(measure, start: dict, space: dict, rounds: int = 2, min_gain: float = 0.005):
    """Coordinate descent over `space` (knob -> values) from `start`.
    `measure(tuning) -> ms or None` (None: a schedule the workload cannot
    run).  Returns (best tuning, its ms, [every measurement])."""
    results = []
    seen = {}

    def timed(t):
        key = tuple(sorted(t.items()))
        if key not in seen:
            seen[key] = measure(t)
            results.append({"tuning": dict(t), "ms": seen[key]})
        return seen[key]

    best = dict(start)
    best_ms = timed(best)
    if best_ms is None:
        raise MrtError(-1, "autotune: the starting schedule does not run")
    for _ in range(rounds):
        changed = False
        for k, values in space.items():
            for v in values:
                if v == best.get(k):
                    continue
                cand = dict(best, **{k: v})
                ms = timed(cand)
                if ms is not None and ms < best_ms * (1.0 - min_gain):
                    best, best_ms, changed = cand, ms, True
        if not changed:
            break
    return best, best_ms, results


def autotune(ctx: Context, run_frame, stream=None, key: str = "default", frames: int = 5, warmup: int = 2,
             cache: Path | None = DEFAULT_CACHE, sort: bool = False, space=None, rounds: int = 2) -> dict:
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
    saved = _as_dict(ctx.tuning())

    def measure(cand):
        try:
            ctx.set_tuning(**cand)
            return time_frames(ctx, run_frame, stream, frames, warmup)
        except MrtError:  # a schedule this workload cannot run (e.g. a stack below its BVH depth)
            return None

    try:
        if space is None:
            space_k = knobs(max(1, int(info.trace_blocks_per_sm_max)), sort)
            best, best_ms, results = coordinate_search(measure, saved, space_k, rounds=rounds)
        else:
            results = [{"tuning": cand, "ms": measure(cand)} for cand in space]
            ok = [r for r in results if r["ms"] is not None]
            if not ok:
                raise MrtError(-1, "autotune: no candidate schedule runs")
            best_r = min(ok, key=lambda r: r["ms"])
            best, best_ms = best_r["tuning"], best_r["ms"]
    except MrtError:
        ctx.set_tuning(**saved)
        raise
    ctx.set_tuning(**best)
    out = {"tuning": best, "ms": best_ms, "results": results,
           "default_ms": next((r["ms"] for r in results
                               if all(saved.get(k) == v for k, v in r["tuning"].items())), None)}
    if cache is not None:
        cache.parent.mkdir(parents=True, exist_ok=True)
        db[full_key] = out
        cache.write_text(json.dumps(db, indent=1))
    return out


def _as_dict(t) -> dict:
    return {f: int(getattr(t, f)) for f, _ in t._fields_}
