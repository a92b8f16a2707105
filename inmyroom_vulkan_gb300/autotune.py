"""Autotuner of the batched collide launch.

Picks, for one batch of queries on one context, the launch settings of the
persistent traversal and the narrow phase that give the shortest device time:

  queue depth      queue_capacity (node pairs the global work queue holds)
                   and donate_min (the stack depth above which a warp hands
                   node pairs to idle warps)
  warps            warps_per_block and blocks_per_sm of the persistent
                   traversal (lanes per node pair are picked per step by the
                   kernel itself from the width of its work: 8, 16 or 32)
  stack / tile     stack_entries (per-warp shared-memory node-pair stack) and
                   leaf_flush (candidate leaf pairs a warp gathers before it
                   appends them to the narrow phase's list)

Search: coordinate descent from the context's current settings, one setting
at a time over its candidate values, keeping a change only when it is faster
by more than `tol`, until a pass changes nothing (at most `passes`). Each
candidate is timed with CUDA events over `reps` launches after `warmup`
launches; a candidate that fails (queue overflow, a launch that does not fit)
or whose triangle-test, leaf-pair and colliding-pair counts differ from the
starting settings' is dropped, so a tuned launch computes the same sets.

Cache: with `cache` (a JSON file path), results are kept per shape signature
(the device's name and SM count, the batch's query count and flags, and a
workload tag the caller gives, e.g. the scene's name). A later tuning of the
same signature takes the stored settings after one check launch (its counts
must equal the starting settings' and it must not fail) instead of
searching; a missing, unreadable or mismatching entry is searched and written
again.
"""
from __future__ import annotations

import json
import os
import tempfile
from dataclasses import dataclass, field

import numpy as np

SPACE: dict[str, tuple] = {
    "warps_per_block": (2, 4, 8),
    "blocks_per_sm": (1, 2, 3),
    "stack_entries": (256, 512, 1024),
    "donate_min": (8, 16, 32, 64),
    "leaf_flush": (8, 16, 32),
    "queue_capacity": (1 << 18, 1 << 20, 1 << 22),
}


@dataclass
class Trial:
    config: dict
    ms: float | None          # None: the candidate was dropped
    error: str = ""


@dataclass
class Result:
    best: dict
    best_ms: float
    start_ms: float
    trials: list = field(default_factory=list)

    cached: bool = False

    def as_dict(self) -> dict:
        return {"best": self.best, "best_ms": self.best_ms, "start_ms": self.start_ms,
                "trials": len(self.trials), "dropped": sum(t.ms is None for t in self.trials), "cached": self.cached}


def load_cache(path: str) -> dict:
    """The cache's entries, or {} when the file is missing or unreadable."""
    try:
        with open(path) as f:
            d = json.load(f)
        return d if isinstance(d, dict) else {}
    except (OSError, ValueError):
        return {}


def store_cache(path: str, signature: str, res: Result, space: dict) -> None:
    """Writes (atomically: a temporary file renamed over the old one) the
    entry of `signature`, keeping the others."""
    entries = load_cache(path)
    entries[signature] = {"best": res.best, "best_ms": res.best_ms, "start_ms": res.start_ms,
                          "space": sorted(space)}
    folder = os.path.dirname(os.path.abspath(path))
    os.makedirs(folder, exist_ok=True)
    fd, tmp = tempfile.mkstemp(dir=folder, suffix=".tmp")
    with os.fdopen(fd, "w") as f:
        json.dump(entries, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def cached_descent(measure, start: dict, space: dict, signature: str, cache: str | None, **kw) -> Result:
    """coordinate_descent, or the cache's settings for `signature` when they
    cover the same settings and one measurement of them succeeds."""
    if cache:
        e = load_cache(cache).get(signature)
        if isinstance(e, dict) and e.get("space") == sorted(space) and isinstance(e.get("best"), dict) and \
                set(e["best"]) == set(space):
            try:
                ms = float(measure(dict(e["best"])))
                return Result(dict(e["best"]), ms, float(e.get("start_ms", ms)), [], cached=True)
            except Exception:  # noqa: BLE001 - a stale entry is searched again
                pass
    res = coordinate_descent(measure, start, space, **kw)
    if cache:
        store_cache(cache, signature, res, space)
    return res


def shape_signature(n: int, flags: int, workload: str = "") -> str:
    """Device name, SM count, query count, flags and the caller's workload tag."""
    import torch

    p = torch.cuda.get_device_properties(torch.cuda.current_device())
    return f"{p.name}|sm{p.multi_processor_count}|queries{n}|flags{flags}|{workload}"


def coordinate_descent(measure, start: dict, space: dict, passes: int = 2, tol: float = 0.01) -> Result:
    """measure(config) -> milliseconds, or raises to drop the candidate."""
    cache: dict = {}

    def run(cfg: dict) -> Trial:
        key = tuple(sorted(cfg.items()))
        if key not in cache:
            try:
                cache[key] = Trial(dict(cfg), float(measure(dict(cfg))))
            except Exception as e:  # noqa: BLE001 - a failing candidate is dropped, not fatal
                cache[key] = Trial(dict(cfg), None, str(e))
        return cache[key]

    first = run(start)
    if first.ms is None:
        raise RuntimeError(f"the starting configuration fails: {first.error}")
    best, best_ms = dict(start), first.ms
    for _ in range(passes):
        changed = False
        for name, values in space.items():
            for v in values:
                if v == best.get(name):
                    continue
                t = run({**best, name: v})
                if t.ms is not None and t.ms < best_ms * (1.0 - tol):
                    best, best_ms, changed = dict(t.config), t.ms, True
        if not changed:
            break
    return Result(best, best_ms, first.ms, list(cache.values()))


def tune_collide(ctx, d_queries: int, n: int, flags: int = 0, space: dict | None = None, reps: int = 5,
                 warmup: int = 2, passes: int = 2, flush=None, cache: str | None = None,
                 workload: str = "") -> Result:
    """Tunes ctx (a capi.Context) for the batch at device pointer d_queries
    (n queries) and leaves it configured with the best settings. `flush`, a
    CUDA tensor larger than L2, is rewritten before every timed launch.
    `cache`: a JSON file of earlier results by shape signature (`workload`
    names the batch's scene in it)."""
    import torch

    space = dict(SPACE if space is None else space)
    cur = ctx.config()
    start = {k: int(getattr(cur, k)) for k in space}
    stream = torch.cuda.Stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    want: list = []

    def measure(cfg: dict) -> float:
        ctx.reconfigure(**cfg)
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                ctx.collide_async(d_queries, n, flags, stream.cuda_stream)
            st = ctx.sync_stats()  # raises on an error status
            counts = (st["tri_tests"], st["leaf_pairs"], st["tri_pairs"])
            if not want:
                want.append(counts)
            elif counts != want[0]:
                raise RuntimeError(f"counts {counts} differ from {want[0]}")
            times = []
            for k in range(reps):
                if flush is not None:
                    flush.fill_(k & 0xff)
                ev0.record(stream)
                ctx.collide_async(d_queries, n, flags, stream.cuda_stream)
                ev1.record(stream)
                ev1.synchronize()
                times.append(ev0.elapsed_time(ev1))
            ctx.sync_stats()
        return float(np.median(times))

    if cache:
        # the starting settings' counts, which a cached setting must reproduce
        ctx.reconfigure(**start)
        with torch.cuda.stream(stream):
            ctx.collide_async(d_queries, n, flags, stream.cuda_stream)
            st = ctx.sync_stats()
        want.append((st["tri_tests"], st["leaf_pairs"], st["tri_pairs"]))
    res = cached_descent(measure, start, space, shape_signature(n, flags, workload), cache, passes=passes)
    ctx.reconfigure(**res.best)
    return res
