"""GPU collision frame (cg_collision_frame) against one frame of
CollisionDetection::ExecuteCollisionDetection
(src/CollisionDetection/CollisionDetection.cpp:38-103): the reference's golden
pairs and deltas on the 256-entity scene, the oracle's frame with other
motions, the composition of the frame from its own collide step's rays, and
the edge cases.

Bit for bit: the pairs with rays, and every delta, against the oracle's
frame (the frame's rays are the reference's rays in the reference's order, so
the shooting's sums and the split are the reference's arithmetic on the same
operands), and against the reference's golden frame on every pair whose
triangle tests the reference defines: a pair with a fragile test (the
second interval degenerates, Triangle.cpp:960-966, where the reference reads
uninitialised values; the oracle and the GPU define it as no intersection)
has no defined reference delta (two runs of the same reference build gave
different deltas for the golden frame's one such pair), so the golden
comparison leaves it out. Pairs where neither entity moved have exactly zero
deltas on both sides."""
import os

import numpy as np
import pytest

from inmyroom_vulkan_gb300 import capi, scenes
from oracle import frame

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def bits(x):
    return np.ascontiguousarray(x, np.float32).view(np.uint32)


def same_bits(got, want, what=""):
    got = np.ascontiguousarray(got, np.float32)
    want = np.ascontiguousarray(want, np.float32)
    assert got.shape == want.shape, what
    nan = np.isnan(want)
    assert np.array_equal(np.isnan(got), nan), what
    bad = np.argwhere(bits(got) != bits(want))
    bad = bad[~nan[tuple(bad.T)]] if len(bad) else bad
    assert not len(bad), (what, bad[:5], got[tuple(bad[:5].T)], want[tuple(bad[:5].T)])


def as_arrays(res):
    p = np.stack([res["first"], res["second"]], 1).astype(np.uint32)
    d = np.concatenate([res["first_delta"], res["second_delta"]], 1).astype(np.float32)
    o = np.lexsort((p[:, 1], p[:, 0]))
    return p[o], d[o]


def check_against_reference(p, d, wp, wd, defined=None):
    assert np.array_equal(p, wp)
    if defined is None:
        defined = np.ones(len(p), bool)
    same_bits(d[defined], wd[defined], "deltas")


def reference_defined(port, trees, mats, pairs):
    """Rows whose pair has no fragile triangle test (the reference's result
    is defined there)."""
    ok = []
    for a, b in pairs:
        _, _, _, fragile = port.mid_phase(trees[a], trees[b], mats[a], mats[b]).narrow()
        ok.append(fragile == 0)
    return np.array(ok, bool)


@pytest.fixture(scope="module")
def scene_trees(gpu_ctx, port):
    sc = scenes.scene()
    trees = [port.tree_build(m.points, m.indices, m.normals) for m in sc.meshes]
    ids = np.array([gpu_ctx.upload_flat(t.export()) for t in trees], np.uint32)
    yield sc, trees, ids
    for i in ids:
        gpu_ctx.free_tree(int(i))


def test_golden_frame(gpu_ctx, port, scene_trees):
    sc, trees, ids = scene_trees
    want = np.load(os.path.join(GOLD, "frame_scene.npz"))
    defined = reference_defined(port, trees, sc.mats, want["pairs"])
    assert defined.sum() >= len(defined) - 2
    for _ in range(2):  # the second frame reuses the buffers
        p, d = as_arrays(gpu_ctx.collision_frame(ids, sc.mats, want["previous"], want["callback"]))
        check_against_reference(p, d, want["pairs"], want["deltas"], defined)
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
        same_bits(r["first_delta"], d1, (a, b, "first delta"))
        same_bits(r["second_delta"], d2, (a, b, "second delta"))
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
