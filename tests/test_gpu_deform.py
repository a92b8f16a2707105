"""Deforming meshes on the GPU against the oracle: morph + linear-blend
skinning (the engine's skinning shader, restated) bit for bit; the tree refit
to the deformed vertices (boxes that contain their subtrees, with axes from the same eigen procedure; where the covariance is nearly
degenerate, as across a tube, any axes fit, so boxes are not compared
directly); the colliding triangle pairs of refitted trees against a
heightfield, which do not depend on the boxes, bit for bit."""
import numpy as np
import pytest

import oracle
from inmyroom_vulkan_gb300 import capi, scenes

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def deform_on_gpu(torch, ctx, sc):
    n = sc.vertices.shape[0]
    V = sc.vertices.shape[1]
    keep = []
    views, outs = [], []
    j = _dev(torch, sc.joints.view(np.int16))
    w = _dev(torch, sc.weights)
    ib = _dev(torch, sc.inverse_bind)
    keep += [j, w, ib]
    for m in range(n):
        v = _dev(torch, sc.vertices[m])
        mw = _dev(torch, sc.morph_weights[m])
        jm = _dev(torch, sc.joint_matrices[m])
        out = torch.zeros((V, 4), dtype=torch.float32, device="cuda")
        keep += [v, mw, jm, out]
        views.append(capi.cg_deform_view(V, sc.vertices.shape[2] - 1, 1, sc.joint_matrices.shape[1], v.data_ptr(),
                                         mw.data_ptr(), j.data_ptr(), w.data_ptr(), jm.data_ptr(), ib.data_ptr()))
        outs.append(out)
    ctx.deform_batch(views, [o.data_ptr() for o in outs])
    torch.cuda.synchronize()
    return outs, keep


def test_deform_bit_exact(port):
    torch = pytest.importorskip("torch")
    sc = scenes.deforming(n_meshes=3, rings=24, around=16, grid=32)
    with capi.Context() as ctx:
        outs, _ = deform_on_gpu(torch, ctx, sc)
        for m in range(3):
            want = port.deform(sc.vertices[m], sc.morph_weights[m], sc.joints, sc.weights, sc.joint_matrices[m],
                               sc.inverse_bind)
            got = outs[m].cpu().numpy()
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), m
            assert np.abs(got[:, :3] - sc.vertices[m][:, 0, :3]).max() > 0.05  # it did deform


def record_ranges(ft):
    """(first, count) of the subtree triangles of the root and every child box."""
    n = ft.n_nodes
    node_rg = [None] * n
    boxes = []
    for k in range(n - 1, -1, -1):
        rs = []
        for s2 in range(2):
            ref, cnt = int(ft.node_ref[k, s2]), int(ft.node_cnt[k, s2])
            rs.append((ref, cnt) if cnt else node_rg[ref])
        lo = min(r[0] for r in rs if r[1])
        hi = max(r[0] + r[1] for r in rs if r[1])
        node_rg[k] = (lo, hi - lo)
        boxes.append((k, rs))
    root = node_rg[0] if n else (0, ft.n_tris)
    return root, dict(boxes)


def contains(box, pts):
    """max |t| over points p = c + t_u u + t_v v + t_w w (FP64)."""
    c = box[0:3].astype(np.float64)
    H = np.stack([box[3:6], box[6:9], box[9:12]], 1).astype(np.float64)
    t = np.linalg.solve(H, (pts.astype(np.float64) - c).T)
    return np.abs(t).max()


def test_refit_contains_and_collides_like_oracle(port):
    """The refit boxes contain every corner of their subtree; the colliding
    triangle pairs (and segments) against a heightfield equal the oracle's on
    its own FP64 refit of the same deformed vertices."""
    torch = pytest.importorskip("torch")
    sc = scenes.deforming(n_meshes=4, rings=40, around=24, grid=96)
    rest = port.tree_build(sc.mesh.points, sc.mesh.indices, sc.mesh.normals).export()
    field = port.tree_build(sc.field.points, sc.field.indices, sc.field.normals)
    root_rg, node_rgs = record_ranges(rest)
    with capi.Context() as ctx:
        outs, _ = deform_on_gpu(torch, ctx, sc)
        ids = [ctx.upload_flat(rest) for _ in range(4)]
        fid = ctx.upload_flat(field.export())
        ctx.tree_refit_batch(ids, [o.data_ptr() for o in outs], [o.shape[0] for o in outs])
        torch.cuda.synchronize()
        refit_port = []
        for m in range(4):
            pos = outs[m].cpu().numpy()
            want = port.tree_refit(rest, pos)
            root, obbs, tri = ctx.tree_download(ids[m], rest.n_nodes, rest.n_tris)
            assert np.array_equal(tri.view(np.uint32), want.tri_pos.view(np.uint32)), m
            corners = tri.reshape(-1, 3, 3)
            pts = lambda rg: corners[rg[0]:rg[0] + rg[1]].reshape(-1, 3)  # noqa: E731
            worst = contains(root, pts(root_rg))
            for k, rs in node_rgs.items():
                for s2 in range(2):
                    worst = max(worst, contains(obbs[k, s2], pts(rs[s2])))
            assert worst <= 1.0, (m, worst)
            refit_port.append(port.tree_import(want))
        eye = np.eye(4, dtype=np.float32).reshape(16)
        rel = np.stack([capi.relative_matrix(sc.models[m], eye) for m in range(4)])
        st = ctx.collide(capi.make_queries(ids, [fid] * 4, rel))
        pairs, segs, tests, nleaf = port.collide_pairs(refit_port, [field] * 4, sc.models, [eye] * 4)
        assert st["status"] == 0 and st["tri_pairs"] == len(pairs) > 0
        got = ctx.tri_pairs()
        key = lambda q, a, b, s: np.lexsort(np.c_[q, a, b, np.ascontiguousarray(s, np.float32).view(np.uint32)].T[::-1])
        gs = np.concatenate([got["source"], got["target"]], 1)
        gk = key(got["query"], got["tri_a"], got["tri_b"], gs)
        wk = key(pairs[:, 0], pairs[:, 1], pairs[:, 2], segs)
        assert np.array_equal(got["query"][gk], pairs[wk, 0]) and np.array_equal(got["tri_a"][gk], pairs[wk, 1])
        assert np.array_equal(got["tri_b"][gk], pairs[wk, 2])
        assert np.array_equal(gs[gk].view(np.uint32), segs[wk].view(np.uint32))
