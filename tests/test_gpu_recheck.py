"""The FP64 recheck of the plane distances on the GPU (CG_RECHECK, CG_ROBUST)
against the oracle's restatement (test_oracle_recheck.py pins that one to
exact arithmetic and to the reference's golden verdicts).

* CG_RECHECK keeps the reference's colliding pairs and segments bit for bit
  and counts what the oracle counts (distances recomputed, tests with a
  changed class);
* CG_ROBUST gives the oracle's robust pairs and segments bit for bit;
on the 256-entity scene and on the near-epsilon golden pairs (single-triangle
trees, coordinates up to 1e3, corners within a few 1e-6 of the other plane).
"""
import os

import numpy as np
import pytest

from inmyroom_vulkan_gb300 import capi, scenes

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def table(q, ia, ib, src, tgt):
    t = np.concatenate([np.stack([q, ia, ib], 1).astype(np.uint32),
                        np.ascontiguousarray(np.concatenate([src, tgt], 1), np.float32).view(np.uint32)], 1)
    return t[np.lexsort(t.T[::-1])] if len(t) else t


def gpu_table(p):
    return table(p["query"], p["tri_a"], p["tri_b"], p["source"], p["target"])


def port_table(pairs, segs):
    return table(pairs[:, 0], pairs[:, 1], pairs[:, 2], segs[:, :3], segs[:, 3:])


def run_modes(ctx, port, trees_a, trees_b, ids_a, ids_b, mats_a, mats_b):
    rel = np.stack([capi.relative_matrix(a, b) for a, b in zip(mats_a, mats_b)])
    q = capi.make_queries(ids_a, ids_b, rel)
    out = {}
    for name, flags, mode in (("plain", 0, None), ("recheck", capi.CG_RECHECK, 1), ("robust", capi.CG_ROBUST, 2)):
        st = ctx.collide(q, flags=flags)
        assert st["status"] == 0
        got = gpu_table(ctx.tri_pairs())
        if mode is None:
            pairs, segs, tests, _ = port.collide_pairs(trees_a, trees_b, mats_a, mats_b)
            counts = (0, 0)
        else:
            pairs, segs, tests, _, counts = port.collide_pairs(trees_a, trees_b, mats_a, mats_b, recheck_mode=mode)
        assert st["tri_tests"] == tests, name
        assert np.array_equal(got, port_table(pairs, segs)), name
        assert (st["rechecked"], st["disagreements"]) == counts, (name, st["rechecked"], st["disagreements"], counts)
        out[name] = (got, counts)
    assert np.array_equal(out["plain"][0], out["recheck"][0])
    return out


def test_scene_recheck_and_robust(gpu_ctx, port):
    sc = scenes.scene()
    tp = [port.tree_build(m.points, m.indices, m.normals) for m in sc.meshes]
    ids = np.array([gpu_ctx.upload_flat(t.export()) for t in tp], np.uint32)
    qa, qb = sc.pairs[:, 0], sc.pairs[:, 1]
    out = run_modes(gpu_ctx, port, [tp[i] for i in qa], [tp[j] for j in qb], ids[qa], ids[qb], sc.mats[qa],
                    sc.mats[qb])
    assert out["recheck"][1][0] > 0
    for i in ids:
        gpu_ctx.free_tree(int(i))


def test_near_epsilon_pairs(gpu_ctx, port):
    g = np.load(os.path.join(GOLD, "tritri_near.npz"))
    n = len(g["a"])
    idx = np.arange(3, dtype=np.uint32)
    ta = [port.tree_build(g["a"][i].reshape(3, 3), idx) for i in range(n)]
    tb = [port.tree_build(g["b"][i].reshape(3, 3), idx) for i in range(n)]
    ida = np.array([gpu_ctx.upload_flat(t.export()) for t in ta], np.uint32)
    idb = np.array([gpu_ctx.upload_flat(t.export()) for t in tb], np.uint32)
    eye = np.tile(np.eye(4, dtype=np.float32).reshape(1, 16), (n, 1))
    out = run_modes(gpu_ctx, port, ta, tb, ida, idb, eye, eye)
    assert out["recheck"][1][1] > 10  # tests whose FP32 classes the FP64 recheck corrects
    assert not np.array_equal(out["plain"][0], out["robust"][0])
    for i in np.concatenate([ida, idb]):
        gpu_ctx.free_tree(int(i))
