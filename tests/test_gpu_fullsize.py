"""Parity at the benchmark's full sizes, bit for bit against the oracle:

* the batch sweep: 10,000 uneven rigid mesh-pair queries over 48 meshes of
  256..65,536 triangles in one launch (trees built on the GPU, bit-identical
  to the oracle's builder); colliding pairs, segments, triangle tests and
  candidate leaf pairs;
* the deforming frame: 64 skinned and morphed 12,000-triangle tubes (deformed
  and refitted on the GPU) against the 198k-triangle heightfield; the
  colliding pairs and segments equal the oracle's on its own refit of the
  same deformed vertices (the pairs do not depend on the boxes)."""
import numpy as np
import pytest

from inmyroom_vulkan_gb300 import capi, scenes

pytestmark = pytest.mark.gpu


def table(q, a, b, segs):
    t = np.concatenate([np.stack([q, a, b], 1).astype(np.uint32), np.ascontiguousarray(segs, np.float32).view(np.uint32)],
                       1)
    return t[np.lexsort(t.T[::-1])] if len(t) else t


def gpu_table(p):
    return table(p["query"], p["tri_a"], p["tri_b"], np.concatenate([p["source"], p["target"]], 1))


def test_batch_sweep_full(port):
    from test_gpu_build import same

    bs = scenes.batch_sweep()
    assert len(bs.qa) == 10000
    with capi.Context(max_queries=16384, max_tri_pairs=1 << 23, max_leaf_pairs=1 << 24) as ctx:
        ids = ctx.build_trees(bs.meshes)
        tp = [port.tree_build(m.points, m.indices, m.normals) for m in bs.meshes]
        for i, t, m in zip(ids, tp, bs.meshes):
            same(ctx.export_tree(int(i)), t.export(), normals=m.normals is not None)
        rel = np.stack([capi.relative_matrix(a, b) for a, b in zip(bs.mats_a, bs.mats_b)])
        st = ctx.collide(capi.make_queries(ids[bs.qa], ids[bs.qb], rel))
        assert st["status"] == 0 and st["tri_pairs"] > 1000000
        pairs, segs, tests, leafs = port.collide_pairs([tp[i] for i in bs.qa], [tp[j] for j in bs.qb], bs.mats_a,
                                                       bs.mats_b)
        assert st["tri_tests"] == tests and st["leaf_pairs"] == leafs
        assert np.array_equal(gpu_table(ctx.tri_pairs()), table(pairs[:, 0], pairs[:, 1], pairs[:, 2], segs))


def test_deforming_frame_full(port):
    torch = pytest.importorskip("torch")
    from test_gpu_deform import deform_on_gpu

    sc = scenes.deforming()
    n = sc.vertices.shape[0]
    assert n == 64 and sc.mesh.n_tris == 12000 and sc.field.n_tris > 190000
    rest = port.tree_build(sc.mesh.points, sc.mesh.indices, sc.mesh.normals).export()
    field = port.tree_build(sc.field.points, sc.field.indices, sc.field.normals)
    with capi.Context(max_tri_pairs=1 << 22) as ctx:
        outs, _ = deform_on_gpu(torch, ctx, sc)
        ids = [ctx.upload_flat(rest) for _ in range(n)]
        fid = ctx.upload_flat(field.export())
        ctx.tree_refit_batch(ids, [o.data_ptr() for o in outs], [o.shape[0] for o in outs])
        eye = np.eye(4, dtype=np.float32).reshape(16)
        rel = np.stack([capi.relative_matrix(sc.models[m], eye) for m in range(n)])
        st = ctx.collide(capi.make_queries(ids, [fid] * n, rel), flags=capi.CG_CONTACTS)
        assert st["status"] == 0 and st["tri_pairs"] > 10000
        got = gpu_table(ctx.tri_pairs())
        refit = []
        for m in range(n):
            pos = outs[m].cpu().numpy()
            want = port.deform(sc.vertices[m], sc.morph_weights[m], sc.joints, sc.weights, sc.joint_matrices[m],
                               sc.inverse_bind)
            assert np.array_equal(pos.view(np.uint32), want.view(np.uint32)), m
            refit.append(port.tree_import(port.tree_refit(rest, pos)))
        pairs, segs, _, _ = port.collide_pairs(refit, [field] * n, sc.models, [eye] * n)
        assert np.array_equal(got, table(pairs[:, 0], pairs[:, 1], pairs[:, 2], segs))
