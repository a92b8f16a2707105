"""GPU uncollide-ray shooting (cg_shoot_rays) against the oracle: the deltas
of ShootUncollideRays::ExecuteShootUncollideRays
(src/CollisionDetection/ShootUncollideRays.cpp:14-98) bit for bit, for the
reference's golden vectors, a 200-pose rigid pair and the scene's pairs with
the rays the GPU's own contact step made."""
import os

import numpy as np
import pytest

import oracle
from inmyroom_vulkan_gb300 import capi, scenes

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def bits(x):
    return np.ascontiguousarray(x, np.float32).view(np.uint32)


def test_golden_deltas(gpu_ctx):
    g = np.load(os.path.join(GOLD, "rigid_small.npz"))
    want = np.load(os.path.join(GOLD, "shoot_small.npz"))["deltas"]

    def flat(tag):
        k = f"tree_{tag}_"
        return oracle.FlatTree(g[k + "root"], g[k + "node_obbs"], g[k + "node_ref"], g[k + "node_cnt"],
                               g[k + "tri_pos"], g[k + "tri_nrm"], g[k + "tri_idx"])

    ida, idb = gpu_ctx.upload_flat(flat("a")), gpu_ctx.upload_flat(flat("b"))
    n = len(g["mats_a"])
    ra = [g["rays_a"][g["rays_a"][:, 0] == k, 1:] for k in range(n)]
    rb = [g["rays_b"][g["rays_b"][:, 0] == k, 1:] for k in range(n)]
    got = gpu_ctx.shoot_rays([ida] * n, [idb] * n, g["mats_a"], g["mats_b"], ra, rb)
    assert np.array_equal(bits(got), bits(want))
    gpu_ctx.free_tree(ida)
    gpu_ctx.free_tree(idb)


def test_rigid_pair_200_poses(gpu_ctx, port):
    rp = scenes.rigid_pair(n_poses=200)
    tp = [port.tree_build(m.points, m.indices, m.normals) for m in (rp.mesh_a, rp.mesh_b)]
    ids = [gpu_ctx.upload_flat(t.export()) for t in tp]
    n = len(rp.mats_a)
    ra, rb = [], []
    for k in range(n):
        a, b, _ = port.mid_phase(tp[0], tp[1], rp.mats_a[k], rp.mats_b[k]).rays()
        ra.append(a)
        rb.append(b)
    for params in (None, (0.3, 1.2, 1.5)):
        got = gpu_ctx.shoot_rays([ids[0]] * n, [ids[1]] * n, rp.mats_a, rp.mats_b, ra, rb, params)
        want = np.stack([port.shoot_rays(tp[0], tp[1], rp.mats_a[k], rp.mats_b[k], ra[k], rb[k],
                                         None if params is None else np.array(params, np.float32))
                         for k in range(n)])
        assert np.array_equal(bits(got), bits(want))
        assert (np.abs(got).sum(1) > 0).sum() > 150
    for i in ids:
        gpu_ctx.free_tree(i)


def test_scene_with_its_own_rays(gpu_ctx, port):
    sc = scenes.scene()
    keep = (sc.pairs[:, 0] < 96) & (sc.pairs[:, 1] < 96)
    qa, qb = sc.pairs[keep, 0], sc.pairs[keep, 1]
    tp = {i: port.tree_build(sc.meshes[i].points, sc.meshes[i].indices, sc.meshes[i].normals)
          for i in np.unique(np.concatenate([qa, qb]))}
    ids = {i: gpu_ctx.upload_flat(t.export()) for i, t in tp.items()}
    rel = np.stack([capi.relative_matrix(sc.mats[i], sc.mats[j]) for i, j in zip(qa, qb)])
    q = capi.make_queries([ids[i] for i in qa], [ids[j] for j in qb], rel)
    assert gpu_ctx.collide(q, flags=capi.CG_CONTACTS)["status"] == 0
    rays = gpu_ctx.rays()
    rays = rays[np.lexsort((rays["side"], rays["query"]))]  # per query, side 0 then 1 (order within: as emitted)
    n = len(qa)
    ra, rb = [], []
    for k in range(n):
        mine = rays[rays["query"] == k]
        ra.append(np.concatenate([mine["origin"][mine["side"] == 0], mine["direction"][mine["side"] == 0]], 1))
        rb.append(np.concatenate([mine["origin"][mine["side"] == 1], mine["direction"][mine["side"] == 1]], 1))
    got = gpu_ctx.shoot_rays([ids[i] for i in qa], [ids[j] for j in qb], sc.mats[qa], sc.mats[qb], ra, rb)
    want = np.stack([port.shoot_rays(tp[qa[k]], tp[qb[k]], sc.mats[qa[k]], sc.mats[qb[k]], ra[k], rb[k])
                     for k in range(n)])
    assert np.array_equal(bits(got), bits(want))
    assert (np.abs(got).sum(1) > 0).sum() > 20
    for i in ids.values():
        gpu_ctx.free_tree(i)
