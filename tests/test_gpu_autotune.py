"""Autotuned batch (a small batch-sweep workload: uneven rigid mesh pairs,
256..4,096 triangles): the colliding triangle pairs and their segments equal
the oracle's bit for bit before tuning, and the tuned settings give the same
pairs again."""
import numpy as np
import pytest
import torch

from inmyroom_vulkan_gb300 import autotune, capi, scenes

pytestmark = pytest.mark.gpu


def pair_table(q, ia, ib, segs):
    """(n, 9) uint32 rows [query, ia, ib, segment bits] sorted lexicographically."""
    t = np.concatenate([np.stack([q, ia, ib], 1).astype(np.uint32),
                        np.ascontiguousarray(segs, np.float32).view(np.uint32).reshape(-1, 6)], 1)
    return t[np.lexsort(t.T[::-1])]


def gpu_table(p):
    return pair_table(p["query"], p["tri_a"], p["tri_b"], np.concatenate([p["source"], p["target"]], 1))


def test_tuned_batch_matches_oracle(port):
    bs = scenes.batch_sweep(n_queries=600, pool=10, tri_hi=4096)
    trees = [port.tree_build(m.points, m.indices, m.normals) for m in bs.meshes]
    with capi.Context(max_queries=1024) as ctx:
        ids = np.array([ctx.upload_flat(t.export()) for t in trees], np.uint32)
        rel = np.stack([capi.relative_matrix(a, b) for a, b in zip(bs.mats_a, bs.mats_b)])
        q = capi.make_queries(ids[bs.qa], ids[bs.qb], rel)
        st = ctx.collide(q)
        assert st["status"] == 0 and st["tri_pairs"] > 1000
        got = gpu_table(ctx.tri_pairs())
        pairs, segs, tests, _ = port.collide_pairs([trees[i] for i in bs.qa], [trees[i] for i in bs.qb], bs.mats_a,
                                                  bs.mats_b)
        assert st["tri_tests"] == tests
        assert np.array_equal(got, pair_table(pairs[:, 0], pairs[:, 1], pairs[:, 2], segs))
        d_q = torch.from_numpy(q.view(np.uint8).copy()).cuda()
        space = {"warps_per_block": (4, 8), "donate_min": (16, 32), "leaf_flush": (16, 32)}
        res = autotune.tune_collide(ctx, d_q.data_ptr(), len(q), space=space, reps=3, warmup=1)
        cfg = ctx.config()
        assert all(getattr(cfg, k) == v for k, v in res.best.items())
        assert res.best_ms <= res.start_ms and all(t.ms is not None for t in res.trials)
        st2 = ctx.collide(q)
        assert st2["status"] == 0 and st2["tri_tests"] == st["tri_tests"]
        assert np.array_equal(gpu_table(ctx.tri_pairs()), got)
