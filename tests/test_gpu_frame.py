"""GPU collision frame (cg_collision_frame) against one frame of
CollisionDetection::ExecuteCollisionDetection
(src/CollisionDetection/CollisionDetection.cpp:38-103): the reference's golden
pairs and deltas on the 256-entity scene, the oracle's frame with other
motions, the composition of the frame from its own collide step's rays, and
the edge cases.

The pairs with rays are exact. The deltas are the reference's arithmetic on
the frame's own rays, which match the reference's up to the last bits of the
rays that start at a contact's weighted average point (summed in another
order). Hence two bars:
* composition: every delta within 1e-4 relative of the oracle's shooting and
  split run on the frame's own rays and ray averages (only the order in which
  a pair's force responses are summed differs);
* reference: at least 95% of the pairs within 2e-4 relative of the
  reference's deltas, every pair within 2% of its delta's length (a ray that
  grazes a triangle's edge, or that sets the shooting's maximum, can move a
  delta by up to a percent).
Pairs where neither entity moved have exactly zero deltas on both sides."""
import os

import numpy as np
import pytest

from inmyroom_vulkan_gb300 import capi, scenes
from oracle import frame

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
RTOL, ATOL = 2e-4, 1e-5     # against the reference: most pairs
ROW_TOL = 2e-2              # against the reference: every pair, relative to the delta's length
COMPOSE_RTOL = 1e-4         # against the oracle on the frame's own rays


def as_arrays(res):
    p = np.stack([res["first"], res["second"]], 1).astype(np.uint32)
    d = np.concatenate([res["first_delta"], res["second_delta"]], 1).astype(np.float32)
    o = np.lexsort((p[:, 1], p[:, 0]))
    return p[o], d[o]


def check_against_reference(p, d, wp, wd):
    assert np.array_equal(p, wp)
    tight = np.isclose(d, wd, rtol=RTOL, atol=ATOL).all(1)
    assert tight.mean() >= 0.95, (tight.sum(), len(tight))
    for half in (slice(0, 3), slice(3, 6)):
        err = np.linalg.norm(d[:, half] - wd[:, half], axis=1)
        assert (err <= ROW_TOL * np.linalg.norm(wd[:, half], axis=1) + ATOL).all()


@pytest.fixture(scope="module")
def scene_trees(gpu_ctx, port):
    sc = scenes.scene()
    trees = [port.tree_build(m.points, m.indices, m.normals) for m in sc.meshes]
    ids = np.array([gpu_ctx.upload_flat(t.export()) for t in trees], np.uint32)
    yield sc, trees, ids
    for i in ids:
        gpu_ctx.free_tree(int(i))


def test_golden_frame(gpu_ctx, scene_trees):
    sc, _, ids = scene_trees
    want = np.load(os.path.join(GOLD, "frame_scene.npz"))
    for _ in range(2):  # the second frame reuses the buffers
        p, d = as_arrays(gpu_ctx.collision_frame(ids, sc.mats, want["previous"], want["callback"]))
        check_against_reference(p, d, want["pairs"], want["deltas"])
        still = ~np.abs(want["deltas"]).any(1)
        assert still.any() and not np.abs(d[still]).any()


def test_frame_composition(gpu_ctx, port, scene_trees):
    """Each record from the oracle's shooting and split, run on the frame's own
    rays (cg_read_rays, by the record's query) and ray averages."""
    sc, trees, ids = scene_trees
    want = np.load(os.path.join(GOLD, "frame_scene.npz"))
    prev = want["previous"]
    res = gpu_ctx.collision_frame(ids, sc.mats, prev, want["callback"])
    rays, avgs = gpu_ctx.rays(), gpu_ctx.ray_averages()
    assert len(res) == len(np.unique(rays["query"]))
    moved_rows = 0
    for r in res:
        a, b, k = int(r["first"]), int(r["second"]), int(r["query"])
        mine = rays[rays["query"] == k]
        ra = np.concatenate([mine["origin"], mine["direction"]], 1)[mine["side"] == 0]
        rb = np.concatenate([mine["origin"], mine["direction"]], 1)[mine["side"] == 1]
        assert avgs[k]["rays_first"] == len(ra) and avgs[k]["rays_second"] == len(rb)
        if np.array_equal(sc.mats[a], prev[a]) and np.array_equal(sc.mats[b], prev[b]):
            assert not np.abs(r["first_delta"]).any() and not np.abs(r["second_delta"]).any()
            continue
        moved_rows += 1
        delta = port.shoot_rays(trees[a], trees[b], sc.mats[a], sc.mats[b], ra, rb)
        with np.errstate(invalid="ignore", divide="ignore"):
            m1 = frame.point_movement(avgs[k]["first"], sc.mats[a], prev[a])
            m2 = frame.point_movement(avgs[k]["second"], sc.mats[b], prev[b])
            total = np.float32(m1 + m2)
            d1 = -delta * np.float32(m1 / total)
            d2 = delta * np.float32(m2 / total)
        scale = float(np.linalg.norm(delta)) + 1e-6
        np.testing.assert_allclose(r["first_delta"], d1, rtol=COMPOSE_RTOL, atol=COMPOSE_RTOL * scale)
        np.testing.assert_allclose(r["second_delta"], d2, rtol=COMPOSE_RTOL, atol=COMPOSE_RTOL * scale)
    assert moved_rows > 150


def test_frames_against_oracle(gpu_ctx, port, scene_trees):
    sc, trees, ids = scene_trees
    for seed, still_every, step, share, params in ((5, 2, 0.2, 0.3, None), (6, 4, 0.01, 1.0, (0.3, 1.2, 1.5))):
        prev, cb = scenes.frame_motion(sc, seed=seed, still_every=still_every, step=step, callback_share=share)
        p, d = as_arrays(gpu_ctx.collision_frame(ids, sc.mats, prev, cb, params))
        wp, wd = frame.as_arrays(frame.collision_frame(port, trees, sc.mats, prev, cb, params))
        assert len(wp) > 50
        check_against_reference(p, d, wp, wd)


def test_frame_edge_cases(gpu_ctx, scene_trees):
    sc, _, ids = scene_trees
    n = len(ids)
    # nothing moved: every pair with rays, all deltas zero
    p, d = as_arrays(gpu_ctx.collision_frame(ids, sc.mats, sc.mats))
    assert len(p) > 100 and not np.abs(d).any()
    # no entity calls back: no broad pairs, and no collide step to read
    assert len(gpu_ctx.collision_frame(ids, sc.mats, sc.mats, np.zeros(n, np.uint8))) == 0
    with pytest.raises(capi.CgError):
        gpu_ctx.rays()
    # fewer than two entities
    assert len(gpu_ctx.collision_frame(ids[:1], sc.mats[:1], sc.mats[:1])) == 0
    assert len(gpu_ctx.collision_frame(ids[:0], sc.mats[:0], sc.mats[:0])) == 0
    # the result capacity: an overflow error
    with pytest.raises(capi.CgError) as e:
        gpu_ctx.collision_frame(ids, sc.mats, sc.mats, cap=10)
    assert e.value.code == capi.CG_ERR_OUTPUT_OVERFLOW
    # more broad pairs than the context's max_queries: refused with the count
    with capi.Context(max_queries=32) as small:  # the first 40 entities make 47 broad pairs
        sids = small.build_trees(sc.meshes[:40])
        with pytest.raises(capi.CgError) as e:
            small.collision_frame(sids, sc.mats[:40], sc.mats[:40])
        assert e.value.code == capi.CG_ERR_OUTPUT_OVERFLOW
    # an unknown tree id
    bad = ids.copy()
    bad[3] = 0xFFFFFF
    with pytest.raises(capi.CgError) as e:
        gpu_ctx.collision_frame(bad, sc.mats, sc.mats)
    assert e.value.code == capi.CG_ERR_NOT_FOUND
