"""The host-side fan-out of a frame's results to the entities' ancestors
(cg_frame_callbacks) against the oracle's restatement of
CollisionDetection.cpp:104-124 and EntitiesHandler::GetEntityAncestors, on
random entity hierarchies; no device involved."""
import numpy as np
import pytest

from inmyroom_vulkan_gb300 import capi
from oracle import frame


def random_hierarchy(rng, n_ids):
    parent = np.zeros(n_ids, np.uint32)
    for e in range(1, n_ids):
        parent[e] = rng.integers(0, e)  # parents come first: no cycles
    return parent


def as_calls(cb) -> dict:
    out: dict = {}
    for r in cb:
        out.setdefault(int(r["receiver"]), []).append(
            (int(r["family_entity"]), int(r["collide_with"]), tuple(np.asarray(r["delta"], np.float32).tolist())))
    return out


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_fan_out_matches_oracle(seed):
    rng = np.random.default_rng(seed)
    n_ids = 200
    parent = random_hierarchy(rng, n_ids)
    n = 60
    entity_ids = rng.choice(np.arange(1, n_ids), n, replace=False).astype(np.uint32)
    res = np.zeros(150, capi.FRAME_RESULT_DTYPE)
    res["first"] = rng.integers(0, n, len(res))
    res["second"] = (res["first"] + rng.integers(1, n, len(res))) % n
    res["first_delta"] = rng.normal(size=(len(res), 3))
    res["second_delta"] = rng.normal(size=(len(res), 3))
    cb = capi.frame_callbacks(res, entity_ids, parent)
    want = frame.fan_out([(r["first"], r["second"], r["first_delta"], r["second_delta"]) for r in res],
                         entity_ids, parent)
    assert as_calls(cb) == want
    assert np.all(np.diff(cb["receiver"].astype(np.int64)) >= 0)  # grouped by receiver


def test_fan_out_edge_cases():
    # 0 <- 1 <- 2 <- 3, 0 <- 4: an entity and its own ancestor, siblings under the root
    parent = np.array([0, 0, 1, 2, 0], np.uint32)
    ids = np.array([3, 1, 4], np.uint32)
    res = np.zeros(2, capi.FRAME_RESULT_DTYPE)
    res[0]["first"], res[0]["second"] = 0, 1   # 3 under 1: 3's chain gets 2 and 3, 1's nothing
    res[1]["first"], res[1]["second"] = 1, 2   # 1 and 4 share only the root
    res["first_delta"] = [[1, 2, 3], [4, 5, 6]]
    res["second_delta"] = [[-1, -2, -3], [-4, -5, -6]]
    cb = capi.frame_callbacks(res, ids, parent)
    got = [(int(r["receiver"]), int(r["family_entity"]), int(r["collide_with"])) for r in cb]
    assert got == [(1, 1, 4), (2, 3, 1), (3, 3, 1), (4, 4, 1)]
    assert len(capi.frame_callbacks(res[:0], ids, parent)) == 0
    with pytest.raises(capi.CgError):
        capi.frame_callbacks(res, ids, np.array([0, 2, 1, 2, 0], np.uint32))  # 1 and 2 form a cycle
    with pytest.raises(capi.CgError):
        capi.frame_callbacks(res, np.array([3, 1, 9], np.uint32), parent)  # no entity 9
