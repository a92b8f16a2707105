"""The autotuner's search (inmyroom_vulkan_gb300/autotune.py) on synthetic
cost functions: it finds the separable optimum, drops failing candidates,
keeps the start when nothing is faster, and refuses a failing start."""
import pytest

from inmyroom_vulkan_gb300.autotune import SPACE, coordinate_descent


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
