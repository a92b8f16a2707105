"""Skinned, morphed meshes and rigid meshes in one launch: the tubes are
deformed (morph targets + linear-blend skinning) and their trees refitted on
the GPU, then ONE cg_collide batch holds the tube-against-heightfield queries
interleaved with rigid entity pairs of the 256-entity scene, with contacts
and rays. Everything equals the oracle bit for bit: colliding pairs and
segments, triangle tests and candidate leaf pairs over the whole batch, and
per query the contact records, rays and mean origins in the reference's
order (for the tubes, the oracle collides the GPU's refitted trees)."""
import numpy as np
import pytest

import oracle
from inmyroom_vulkan_gb300 import capi, scenes

pytestmark = pytest.mark.gpu


def table(q, a, b, segs):
    t = np.concatenate([np.stack([q, a, b], 1).astype(np.uint32), np.ascontiguousarray(segs, np.float32).view(np.uint32)],
                       1)
    return t[np.lexsort(t.T[::-1])] if len(t) else t


def test_skinned_and_rigid_in_one_launch(port):
    torch = pytest.importorskip("torch")
    from test_gpu_contacts import check_grouped, check_query
    from test_gpu_deform import deform_on_gpu

    ds = scenes.deforming(n_meshes=6, rings=40, around=24, grid=96)
    n_tubes = ds.vertices.shape[0]
    sc = scenes.scene()
    keep = (sc.pairs[:, 0] < 48) & (sc.pairs[:, 1] < 48)
    rqa, rqb = sc.pairs[keep, 0], sc.pairs[keep, 1]
    rest = port.tree_build(ds.mesh.points, ds.mesh.indices, ds.mesh.normals).export()
    field = port.tree_build(ds.field.points, ds.field.indices, ds.field.normals)
    rigid = [port.tree_build(m.points, m.indices, m.normals) for m in sc.meshes[:48]]
    eye = np.eye(4, dtype=np.float32).reshape(16)
    with capi.Context() as ctx:
        outs, _ = deform_on_gpu(torch, ctx, ds)
        tube_ids = [ctx.upload_flat(rest) for _ in range(n_tubes)]
        fid = ctx.upload_flat(field.export())
        rigid_ids = [ctx.upload_flat(t.export()) for t in rigid]
        ctx.tree_refit_batch(tube_ids, [o.data_ptr() for o in outs], [o.shape[0] for o in outs])
        # the oracle collides the GPU's refitted boxes (leaf pairs and the
        # descent order depend on them; the refit itself is tested for
        # containment elsewhere), with the rest tree's topology and normals
        refit = []
        for m in range(n_tubes):
            root, obbs, tri = ctx.tree_download(tube_ids[m], rest.n_nodes, rest.n_tris)
            refit.append(port.tree_import(oracle.FlatTree(root, obbs, rest.node_ref, rest.node_cnt, tri, rest.tri_nrm,
                                                          rest.tri_idx)))
        # the batch: rigid pairs with a tube query after every few of them
        ida, idb, ta, tb, ma, mb, is_tube = [], [], [], [], [], [], []
        every = max(1, len(rqa) // n_tubes)
        t_next = 0
        for k in range(len(rqa)):
            i, j = int(rqa[k]), int(rqb[k])
            ida.append(rigid_ids[i]), idb.append(rigid_ids[j]), ta.append(rigid[i]), tb.append(rigid[j])
            ma.append(sc.mats[i]), mb.append(sc.mats[j]), is_tube.append(False)
            if k % every == 0 and t_next < n_tubes:
                ida.append(tube_ids[t_next]), idb.append(fid), ta.append(refit[t_next]), tb.append(field)
                ma.append(ds.models[t_next]), mb.append(eye), is_tube.append(True)
                t_next += 1
        assert t_next == n_tubes
        is_tube = np.array(is_tube)
        rel = np.stack([capi.relative_matrix(a, b) for a, b in zip(ma, mb)])
        st = ctx.collide(capi.make_queries(ida, idb, rel), flags=capi.CG_CONTACTS)
        assert st["status"] == 0
        pairs, segs, tests, leafs = port.collide_pairs(ta, tb, ma, mb)
        assert st["tri_tests"] == tests and st["leaf_pairs"] == leafs
        p = ctx.tri_pairs()
        got = table(p["query"], p["tri_a"], p["tri_b"], np.concatenate([p["source"], p["target"]], 1))
        assert np.array_equal(got, table(pairs[:, 0], pairs[:, 1], pairs[:, 2], segs))
        hit_q = np.unique(pairs[:, 0])
        assert is_tube[hit_q].any() and (~is_tube[hit_q]).any()  # both kinds collide
        contacts, rays, averages = ctx.contacts(), ctx.rays(), ctx.ray_averages()
        check_grouped(contacts, rays)
        for k in range(len(ida)):
            m = port.mid_phase(ta[k], tb[k], ma[k], mb[k])
            check_query(port, m, k, contacts, rays, averages)
