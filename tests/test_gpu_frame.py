"""GPU collision frame (cg_collision_frame) against one frame of
CollisionDetection::ExecuteCollisionDetection
(src/CollisionDetection/CollisionDetection.cpp:38-103): the reference's golden
pairs and deltas on the 256-entity scene, the oracle's frame with other
motions, and the edge cases.

The pairs with rays are exact. The deltas are within 2e-4 relative (1e-5
absolute): the GPU sums each pair's force responses over its rays in the
order the contact kernels emitted them, the reference in its unordered_map's
order, so the mean force direction can differ in its last bits; pairs where
neither entity moved have exactly zero deltas on both."""
import os

import numpy as np
import pytest

from inmyroom_vulkan_gb300 import capi, scenes
from oracle import frame

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
RTOL, ATOL = 2e-4, 1e-5


def as_arrays(res):
    p = np.stack([res["first"], res["second"]], 1).astype(np.uint32)
    d = np.concatenate([res["first_delta"], res["second_delta"]], 1).astype(np.float32)
    o = np.lexsort((p[:, 1], p[:, 0]))
    return p[o], d[o]


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
        assert np.array_equal(p, want["pairs"])
        assert np.allclose(d, want["deltas"], rtol=RTOL, atol=ATOL)
        still = ~np.abs(want["deltas"]).any(1)
        assert still.any() and not np.abs(d[still]).any()


def test_frames_against_oracle(gpu_ctx, port, scene_trees):
    sc, trees, ids = scene_trees
    for seed, still_every, step, share, params in ((5, 2, 0.2, 0.3, None), (6, 4, 0.01, 1.0, (0.3, 1.2, 1.5))):
        prev, cb = scenes.frame_motion(sc, seed=seed, still_every=still_every, step=step, callback_share=share)
        p, d = as_arrays(gpu_ctx.collision_frame(ids, sc.mats, prev, cb, params))
        wp, wd = frame.as_arrays(frame.collision_frame(port, trees, sc.mats, prev, cb, params))
        assert len(wp) > 50
        assert np.array_equal(p, wp)
        assert np.allclose(d, wd, rtol=RTOL, atol=ATOL)


def test_frame_edge_cases(gpu_ctx, scene_trees):
    sc, _, ids = scene_trees
    n = len(ids)
    # nothing moved: every pair with rays, all deltas zero
    p, d = as_arrays(gpu_ctx.collision_frame(ids, sc.mats, sc.mats))
    assert len(p) > 100 and not np.abs(d).any()
    # no entity calls back: no broad pairs
    assert len(gpu_ctx.collision_frame(ids, sc.mats, sc.mats, np.zeros(n, np.uint8))) == 0
    # fewer than two entities
    assert len(gpu_ctx.collision_frame(ids[:1], sc.mats[:1], sc.mats[:1])) == 0
    assert len(gpu_ctx.collision_frame(ids[:0], sc.mats[:0], sc.mats[:0])) == 0
    # the result capacity: an overflow error, the count still exact
    with pytest.raises(capi.CgError) as e:
        gpu_ctx.collision_frame(ids, sc.mats, sc.mats, cap=10)
    assert e.value.code == capi.CG_ERR_OUTPUT_OVERFLOW
    # a freed tree id
    bad = ids.copy()
    bad[3] = 0xFFFFFF
    with pytest.raises(capi.CgError) as e:
        gpu_ctx.collision_frame(bad, sc.mats, sc.mats)
    assert e.value.code == capi.CG_ERR_NOT_FOUND
