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
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

SPACE: dict[str, tuple] = {
    "warps_per_block": (2, 4, 8),
    "blocks_per_sm": (1, 2),
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

    def as_dict(self) -> dict:
        return {"best": self.best, "best_ms": self.best_ms, "start_ms": self.start_ms,
                "trials": len(self.trials), "dropped": sum(t.ms is None for t in self.trials)}


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
                 warmup: int = 2, passes: int = 2, flush=None) -> Result:
    """Tunes ctx (a capi.Context) for the batch at device pointer d_queries
    (n queries) and leaves it configured with the best settings. `flush`, a
    CUDA tensor larger than L2, is rewritten before every timed launch."""
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

    res = coordinate_descent(measure, start, space, passes=passes)
    ctx.reconfigure(**res.best)
    return res
