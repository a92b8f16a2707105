"""GPU parity: the CUDA path (through the C ABI) against the reference's golden
outputs and against the oracle restatement, bit for bit.

Colliding triangle pairs, their segments and the candidate leaf pairs must be
identical; the comparison is over sets because the GPU emits them in a
different order than the reference's depth-first recursion.
"""
import os

import numpy as np
import pytest

import oracle
from inmyroom_vulkan_gb300 import capi, scenes

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def bits(x):
    return np.ascontiguousarray(x, np.float32).view(np.uint32)


def pair_table(q, ia, ib, segs):
    """(n, 9) uint32 rows [query, ia, ib, seg bits...] sorted lexicographically."""
    t = np.concatenate([np.stack([q, ia, ib], 1).astype(np.uint32), bits(segs).reshape(-1, 6)], 1)
    return t[np.lexsort(t.T[::-1])] if len(t) else t


def gpu_pair_table(pairs):
    segs = np.concatenate([pairs["source"], pairs["target"]], 1)
    return pair_table(pairs["query"], pairs["tri_a"], pairs["tri_b"], segs)


def leaf_table(rows):
    rows = np.asarray(rows, np.uint32).reshape(-1, 5)
    return rows[np.lexsort(rows.T[::-1])] if len(rows) else rows


def gpu_leaf_table(lp):
    return leaf_table(np.stack([lp["query"], lp["offset_a"], lp["count_a"], lp["offset_b"], lp["count_b"]], 1))


def test_golden_rigid_pair_matches_reference_outputs(gpu_ctx):
    g = np.load(os.path.join(GOLD, "rigid_small.npz"))

    def flat(tag):
        k = f"tree_{tag}_"
        return oracle.FlatTree(g[k + "root"], g[k + "node_obbs"], g[k + "node_ref"], g[k + "node_cnt"],
                               g[k + "tri_pos"], g[k + "tri_nrm"], g[k + "tri_idx"])

    ida, idb = gpu_ctx.upload_flat(flat("a")), gpu_ctx.upload_flat(flat("b"))
    rel = np.stack([capi.relative_matrix(a, b) for a, b in zip(g["mats_a"], g["mats_b"])])
    q = capi.make_queries(np.full(len(rel), ida), np.full(len(rel), idb), rel)
    st = gpu_ctx.collide(q, flags=capi.CG_KEEP_LEAF_PAIRS)
    assert st["status"] == 0 and st["fragile"] == 0
    assert st["tri_tests"] == int(g["tests"].sum())
    got = gpu_pair_table(gpu_ctx.tri_pairs())
    want = pair_table(g["pairs"][:, 0], g["pairs"][:, 1], g["pairs"][:, 2], g["segs"])
    assert np.array_equal(got, want)
    lp = g["leaf_pairs"]
    assert np.array_equal(gpu_leaf_table(gpu_ctx.leaf_pairs()), leaf_table(lp[:, [0, 1, 2, 3, 4]]))
    gpu_ctx.free_tree(ida)
    gpu_ctx.free_tree(idb)


def run_both(ctx, port, trees_port, ids, qa, qb, mats_a, mats_b, flags=capi.CG_KEEP_LEAF_PAIRS):
    rel = np.stack([port.relative_matrix(a, b) for a, b in zip(mats_a, mats_b)])
    q = capi.make_queries(np.asarray(ids)[qa], np.asarray(ids)[qb], rel)
    st = ctx.collide(q, flags=flags)
    pairs, segs, tests, nleaf = port.collide_pairs([trees_port[i] for i in qa], [trees_port[j] for j in qb],
                                                    mats_a, mats_b)
    return st, pairs, segs, tests, nleaf


def test_rigid_pair_1000_poses_bit_exact(gpu_ctx, port):
    rp = scenes.rigid_pair(n_poses=1000)
    tp = [port.tree_build(m.points, m.indices, m.normals) for m in (rp.mesh_a, rp.mesh_b)]
    ids = [gpu_ctx.upload_flat(t.export()) for t in tp]
    n = len(rp.mats_a)
    st, pairs, segs, tests, nleaf = run_both(gpu_ctx, port, tp, ids, np.zeros(n, int), np.ones(n, int),
                                             rp.mats_a, rp.mats_b)
    assert st["status"] == 0
    assert st["tri_tests"] == tests and st["leaf_pairs"] == nleaf
    assert st["tri_pairs"] == len(pairs) > 100000
    assert np.array_equal(gpu_pair_table(gpu_ctx.tri_pairs()), pair_table(pairs[:, 0], pairs[:, 1], pairs[:, 2], segs))
    # candidate leaf pairs of a few poses
    lps = gpu_ctx.leaf_pairs()
    for k in (0, 17, 999):
        m = port.mid_phase(tp[0], tp[1], rp.mats_a[k], rp.mats_b[k])
        want = m.leaf_pairs()
        got = lps[lps["query"] == k]
        assert np.array_equal(gpu_leaf_table(got)[:, 1:], leaf_table(np.c_[np.full(len(want), k), want])[:, 1:])
    for i in ids:
        gpu_ctx.free_tree(i)


@pytest.fixture(scope="module")
def scene_setup(port):
    sc = scenes.scene()
    tp = [port.tree_build(m.points, m.indices, m.normals) for m in sc.meshes]
    return sc, tp


def test_scene_256_entities_bit_exact(gpu_ctx, port, scene_setup):
    sc, tp = scene_setup
    ids = [gpu_ctx.upload_flat(t.export()) for t in tp]
    qa, qb = sc.pairs[:, 0], sc.pairs[:, 1]
    st, pairs, segs, tests, nleaf = run_both(gpu_ctx, port, tp, ids, qa, qb, sc.mats[qa], sc.mats[qb])
    assert st["status"] == 0
    assert st["tri_tests"] == tests and st["leaf_pairs"] == nleaf and st["tri_pairs"] == len(pairs)
    assert np.array_equal(gpu_pair_table(gpu_ctx.tri_pairs()), pair_table(pairs[:, 0], pairs[:, 1], pairs[:, 2], segs))
    # repeated launches give the same set (the work distribution varies)
    st2 = gpu_ctx.collide(capi.make_queries(np.asarray(ids)[qa], np.asarray(ids)[qb],
                                            np.stack([capi.relative_matrix(sc.mats[i], sc.mats[j])
                                                      for i, j in zip(qa, qb)])))
    assert st2["tri_pairs"] == st["tri_pairs"] and st2["tri_tests"] == st["tri_tests"]
    for i in ids:
        gpu_ctx.free_tree(i)


def test_edge_cases(gpu_ctx, port):
    rng = np.random.Generator(np.random.PCG64(99))
    meshes = {
        "empty": (np.zeros((0, 3), np.float32), np.zeros(0, np.uint32)),
        "one": (rng.normal(size=(3, 3)).astype(np.float32) * 0.5, np.arange(3, dtype=np.uint32)),
        "four": (rng.normal(size=(12, 3)).astype(np.float32) * 0.5, np.arange(12, dtype=np.uint32)),
        "five": (rng.normal(size=(15, 3)).astype(np.float32) * 0.5, np.arange(15, dtype=np.uint32)),
    }
    sph = scenes.octa_sphere(3, 0.5, 0.0, rng)
    meshes["sphere"] = (sph.points, sph.indices)
    names = list(meshes)
    tp = [port.tree_build(*meshes[k]) for k in names]
    ids = [gpu_ctx.upload_flat(t.export()) for t in tp]
    qa, qb, ma, mb = [], [], [], []
    for i in range(len(names)):
        for j in range(len(names)):
            for k in range(3):
                qa.append(i)
                qb.append(j)
                ma.append(scenes.pose(scenes.random_rotation(rng), rng.normal(size=3) * 0.1))
                mb.append(scenes.pose(scenes.random_rotation(rng), rng.normal(size=3) * 0.1))
    # identical placement: every triangle of the sphere against itself is coplanar
    qa.append(4)
    qb.append(4)
    ma.append(scenes.pose(np.eye(3), [0, 0, 0]))
    mb.append(scenes.pose(np.eye(3), [0, 0, 0]))
    # far apart
    qa.append(4)
    qb.append(4)
    ma.append(scenes.pose(np.eye(3), [0, 0, 0]))
    mb.append(scenes.pose(np.eye(3), [50, 0, 0]))
    st, pairs, segs, tests, nleaf = run_both(gpu_ctx, port, tp, ids, np.array(qa), np.array(qb), np.array(ma),
                                             np.array(mb))
    assert st["status"] == 0 and st["tri_tests"] == tests and st["leaf_pairs"] == nleaf
    assert np.array_equal(gpu_pair_table(gpu_ctx.tri_pairs()), pair_table(pairs[:, 0], pairs[:, 1], pairs[:, 2], segs))
    # zero queries
    st = gpu_ctx.collide(capi.make_queries([], [], np.zeros((0, 16), np.float32)))
    assert st["status"] == 0 and st["tri_tests"] == 0
    for i in ids:
        gpu_ctx.free_tree(i)


def test_output_overflow_reports_exact_count_then_retry(port):
    rp = scenes.rigid_pair(n_poses=50)
    tp = [port.tree_build(m.points, m.indices, m.normals) for m in (rp.mesh_a, rp.mesh_b)]
    with capi.Context(max_tri_pairs=1000) as ctx:
        ids = [ctx.upload_flat(t.export()) for t in tp]
        rel = np.stack([capi.relative_matrix(a, b) for a, b in zip(rp.mats_a, rp.mats_b)])
        q = capi.make_queries(np.full(50, ids[0]), np.full(50, ids[1]), rel)
        st = ctx.collide(q, check=False)
        assert st["rc"] == -5 and st["tri_pairs"] > 1000
        need = st["tri_pairs"]
        ctx.reconfigure(max_tri_pairs=need)
        st = ctx.collide(q)
        assert st["tri_pairs"] == need and len(ctx.tri_pairs()) == need


def test_unknown_tree_is_rejected(gpu_ctx):
    q = capi.make_queries([12345], [0], np.eye(4, dtype=np.float32).reshape(1, 16))
    with pytest.raises(capi.CgError) as e:
        gpu_ctx.collide(q)
    assert e.value.code == -8


def test_malformed_tree_is_rejected(gpu_ctx):
    root = np.zeros(12, np.float32)
    obbs = np.zeros((1, 2, 12), np.float32)
    with pytest.raises(capi.CgError) as e:
        gpu_ctx.upload_tree(root, obbs, [[0, 0]], [[0, 0]], np.zeros((4, 9), np.float32))  # child points to itself
    assert e.value.code == -7
    with pytest.raises(capi.CgError) as e:
        gpu_ctx.upload_tree(root, obbs, [[0, 3]], [[2, 2]], np.zeros((4, 9), np.float32))  # range past the end
    assert e.value.code == -7


@pytest.mark.parametrize("shape", [dict(warps_per_block=4, stack_entries=256, donate_min=64, leaf_flush=1),
                                   dict(warps_per_block=6, stack_entries=1024, donate_min=900, leaf_flush=33),
                                   dict(warps_per_block=8, stack_entries=512, blocks_per_sm=1, leaf_flush=16)])
def test_launch_shapes_give_identical_sets(port, scene_setup, shape):
    sc, tp = scene_setup
    sel = sc.pairs[:120]
    with capi.Context(**shape) as ctx:
        ids = [ctx.upload_flat(t.export()) for t in tp]
        qa, qb = sel[:, 0], sel[:, 1]
        st, pairs, segs, tests, nleaf = run_both(ctx, port, tp, ids, qa, qb, sc.mats[qa], sc.mats[qb])
        assert st["status"] == 0 and st["tri_tests"] == tests
        assert np.array_equal(gpu_pair_table(ctx.tri_pairs()), pair_table(pairs[:, 0], pairs[:, 1], pairs[:, 2], segs))


def test_large_leaves_bit_exact(gpu_ctx, port):
    """Leaves far above the builder's four triangles (a tree that is one leaf
    of 40 or 18 triangles, and one of 3): the narrow phase's long and
    multi-round leaf pairs, with the full integer division, against the
    oracle on the same flat trees."""
    rng = np.random.Generator(np.random.PCG64(7))
    big = 10.0
    root = np.array([0, 0, 0, big, 0, 0, 0, big, 0, 0, 0, big], np.float32)

    def leaf_tree(n_tris):
        pos = (rng.normal(size=(n_tris, 9)) * 0.4).astype(np.float32)
        nrm = np.tile(np.array([0, 0, 1], np.float32), (n_tris, 3))
        idx = np.arange(3 * n_tris, dtype=np.uint32).reshape(-1, 3)
        return oracle.FlatTree(root, np.zeros((0, 2, 12), np.float32), np.zeros((0, 2), np.uint32),
                               np.zeros((0, 2), np.uint32), pos, nrm, idx)

    flats = [leaf_tree(40), leaf_tree(18), leaf_tree(3)]
    tp = [port.tree_import(f) for f in flats]
    ids = [gpu_ctx.upload_flat(f) for f in flats]
    qa, qb, ma, mb = [], [], [], []
    for i in range(3):
        for j in range(3):
            for _ in range(4):
                qa.append(i)
                qb.append(j)
                ma.append(scenes.pose(scenes.random_rotation(rng), rng.normal(size=3) * 0.1))
                mb.append(scenes.pose(scenes.random_rotation(rng), rng.normal(size=3) * 0.1))
    st, pairs, segs, tests, nleaf = run_both(gpu_ctx, port, tp, ids, np.array(qa), np.array(qb), np.array(ma),
                                             np.array(mb))
    assert st["status"] == 0 and st["tri_tests"] == tests and tests > 10000 and st["leaf_pairs"] == nleaf
    assert len(pairs) > 100
    assert np.array_equal(gpu_pair_table(gpu_ctx.tri_pairs()), pair_table(pairs[:, 0], pairs[:, 1], pairs[:, 2], segs))
    for i in ids:
        gpu_ctx.free_tree(i)


def test_leaf_pairs_in_the_reference_order(gpu_ctx, port):
    """CG_DFS_ORDER: every query's candidate leaf pairs in the order the
    reference's recursion emits them (OBBtree.cpp:414-476), on the scene."""
    sc = scenes.scene()
    tp = [port.tree_build(m.points, m.indices, m.normals) for m in sc.meshes]
    ids = np.array([gpu_ctx.upload_flat(t.export()) for t in tp], np.uint32)
    qa, qb = sc.pairs[:, 0], sc.pairs[:, 1]
    rel = np.stack([capi.relative_matrix(sc.mats[i], sc.mats[j]) for i, j in zip(qa, qb)])
    q = capi.make_queries(ids[qa], ids[qb], rel)
    with pytest.raises(capi.CgError):  # the order applies to kept leaf pairs
        gpu_ctx.collide(q, flags=capi.CG_DFS_ORDER)
    st = gpu_ctx.collide(q, flags=capi.CG_KEEP_LEAF_PAIRS | capi.CG_DFS_ORDER | capi.CG_MID_ONLY)
    assert st["status"] == 0
    lp = gpu_ctx.leaf_pairs()
    assert len(lp) == st["leaf_pairs"] and np.all(np.diff(lp["query"].astype(np.int64)) >= 0)
    starts = np.searchsorted(lp["query"], np.arange(len(q) + 1))
    for k in range(len(q)):
        want = port.mid_phase(tp[qa[k]], tp[qb[k]], sc.mats[qa[k]], sc.mats[qb[k]]).leaf_pairs()
        g = lp[starts[k]:starts[k + 1]]
        got = np.stack([g["offset_a"], g["count_a"], g["offset_b"], g["count_b"]], 1).astype(np.uint32)
        assert np.array_equal(got, want.astype(np.uint32)), k
    for i in ids:
        gpu_ctx.free_tree(int(i))
