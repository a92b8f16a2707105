"""The autotuner's search (inmyroom_vulkan_gb300/autotune.py) on synthetic
cost functions: it finds the separable optimum, drops failing candidates,
keeps the start when nothing is faster, and refuses a failing start; its
cache of results by shape signature."""
import json

import pytest

from inmyroom_vulkan_gb300.autotune import SPACE, cached_descent, coordinate_descent


def test_finds_the_separable_optimum():
    target = {"warps_per_block": 8, "blocks_per_sm": 1, "stack_entries": 1024, "donate_min": 16, "leaf_flush": 8,
              "queue_capacity": 1 << 22}
    cost = lambda c: 1.0 + sum(abs(SPACE[k].index(c[k]) - SPACE[k].index(v)) for k, v in target.items())  # noqa: E731
    start = {k: v[0] for k, v in SPACE.items()}
    res = coordinate_descent(cost, start, SPACE)
    assert res.best == target and res.best_ms == 1.0 and res.start_ms > 1.0
    assert len(res.trials) < 40


def test_drops_failing_candidates():
    def cost(c):
        if c["stack_entries"] == 1024:
            raise RuntimeError("does not fit")
        return 10.0 - c["stack_entries"] / 512 - c["warps_per_block"]

    start = {"warps_per_block": 2, "stack_entries": 256}
    res = coordinate_descent(cost, start, {"warps_per_block": (2, 4, 8), "stack_entries": (256, 512, 1024)})
    assert res.best == {"warps_per_block": 8, "stack_entries": 512}
    dropped = [t for t in res.trials if t.ms is None]
    assert dropped and all("does not fit" in t.error for t in dropped)


def test_keeps_the_start_within_tolerance():
    res = coordinate_descent(lambda c: 5.0 - 0.001 * c["leaf_flush"], {"leaf_flush": 16}, {"leaf_flush": (8, 16, 32)},
                             tol=0.05)
    assert res.best == {"leaf_flush": 16}


def test_failing_start_raises():
    with pytest.raises(RuntimeError):
        coordinate_descent(lambda c: 1 / 0, {"leaf_flush": 16}, {"leaf_flush": (8, 16)})


def test_cache_round_trip(tmp_path):
    """The first tuning searches and writes the cache; the same signature then
    takes the stored settings with one measurement; another signature, a
    changed search space or a damaged file searches again."""
    path = str(tmp_path / "sub" / "autotune.json")
    space = {"warps_per_block": (2, 4, 8), "leaf_flush": (8, 16, 32)}
    calls = []

    def cost(c):
        calls.append(dict(c))
        return 1.0 + abs(c["warps_per_block"] - 8) + abs(c["leaf_flush"] - 16) / 8

    start = {"warps_per_block": 2, "leaf_flush": 8}
    sig = "gpu|sm152|queries516|flags48|scene"
    r1 = cached_descent(cost, start, space, sig, path)
    assert not r1.cached and r1.best == {"warps_per_block": 8, "leaf_flush": 16} and len(calls) > 3
    assert json.load(open(path))[sig]["best"] == r1.best
    calls.clear()
    r2 = cached_descent(cost, start, space, sig, path)
    assert r2.cached and r2.best == r1.best and len(calls) == 1
    calls.clear()
    r3 = cached_descent(cost, start, space, "gpu|sm152|queries1000|flags48|scene", path)
    assert not r3.cached and len(calls) > 3 and len(json.load(open(path))) == 2
    r4 = cached_descent(cost, start, {**space, "blocks_per_sm": (1, 2)}, sig, path)
    assert not r4.cached
    open(path, "w").write("{not json")
    r5 = cached_descent(cost, start, space, sig, path)
    assert not r5.cached and r5.best == r1.best and json.load(open(path))


def test_cache_entry_that_fails_is_searched_again(tmp_path):
    path = str(tmp_path / "autotune.json")
    space = {"stack_entries": (256, 512, 1024)}
    cached_descent(lambda c: 3.0 - c["stack_entries"] / 1024, {"stack_entries": 256}, space, "sig", path)

    def cost(c):
        if c["stack_entries"] == 1024:
            raise RuntimeError("does not fit any more")
        return 3.0 - c["stack_entries"] / 1024

    r = cached_descent(cost, {"stack_entries": 256}, space, "sig", path)
    assert not r.cached and r.best == {"stack_entries": 512}
