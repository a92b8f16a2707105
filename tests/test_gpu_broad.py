"""GPU broad phase (cg_broad_phase) against SweepAndPrune::ExecuteSweepAndPrune
(src/CollisionDetection/SweepAndPrune.cpp:15-88): the reference's golden pairs
on the 256-entity scene and the oracle's with other axes and callback
patterns, oriented the same way; edge cases."""
import os

import numpy as np
import pytest

from inmyroom_vulkan_gb300 import capi, scenes

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def sorted_pairs(p):
    p = np.asarray(p, np.uint32).reshape(-1, 2)
    return p[np.lexsort((p[:, 1], p[:, 0]))]


def test_scene_pairs(gpu_ctx, port):
    want = np.load(os.path.join(GOLD, "sap_scene.npz"))
    sc = scenes.scene()
    trees = [port.tree_build(m.points, m.indices, m.normals) for m in sc.meshes]
    ids = np.array([gpu_ctx.upload_flat(t.export()) for t in trees], np.uint32)
    got = gpu_ctx.broad_phase(ids, sc.mats, want["callback"])
    assert np.array_equal(sorted_pairs(got), want["pairs"])
    rng = np.random.default_rng(11)
    axes = np.linalg.qr(rng.normal(size=(3, 3)))[0].T.astype(np.float32)
    for cb in (None, (rng.random(len(ids)) < 0.2).astype(np.uint8)):
        for ax in (None, axes):
            g = gpu_ctx.broad_phase(ids, sc.mats, cb, ax)
            w = port.sweep_and_prune(trees, sc.mats, cb, ax)
            assert np.array_equal(sorted_pairs(g), sorted_pairs(w))
    # capacity: exact count, first records written
    with pytest.raises(capi.CgError) as e:
        gpu_ctx.broad_phase(ids, sc.mats, None, None, cap=10)
    assert e.value.code == capi.CG_ERR_OUTPUT_OVERFLOW
    assert len(gpu_ctx.broad_phase(ids[:1], sc.mats[:1])) == 0
    assert len(gpu_ctx.broad_phase(ids[:0], sc.mats[:0])) == 0
    for i in ids:
        gpu_ctx.free_tree(int(i))
