"""GPU OBB-tree construction (cg_tree_build) against OBBtree::OBBtree
(src/Geometry/OBBtree.cpp:321-358): the whole flat tree (root box, node
boxes, child links and counts, triangles with normals and indices in leaf
order) bit for bit, for the reference's golden trees, the 256-entity scene,
the deforming workload's tube and heightfield, the batch sweep's meshes and
degenerate meshes."""
import os

import numpy as np
import pytest

import oracle
from inmyroom_vulkan_gb300 import capi, scenes

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


class M:
    def __init__(self, points, indices, normals=None):
        self.points = np.asarray(points, np.float32).reshape(-1, 3)
        self.indices = np.asarray(indices, np.uint32).reshape(-1, 3)
        self.normals = None if normals is None else np.asarray(normals, np.float32).reshape(-1, 3)


def same(got: capi.TreeArrays, want, normals=True):
    a, b = got.arrays(), want.arrays()
    keys = ["root", "node_obbs", "node_ref", "node_cnt", "tri_pos", "tri_idx"] + (["tri_nrm"] if normals else [])
    for k in keys:
        x, y = a[k], b[k]
        assert x.shape == y.shape, (k, x.shape, y.shape)
        if x.dtype == np.float32:
            x, y = x.view(np.uint32), y.view(np.uint32)
        assert np.array_equal(x, y), k


def build_and_check(ctx, port, meshes):
    ids = ctx.build_trees(meshes)
    for m, tid in zip(meshes, ids):
        want = port.tree_build(m.points, m.indices, m.normals).export()
        same(ctx.export_tree(int(tid)), want, normals=m.normals is not None)
    for tid in ids:
        ctx.free_tree(int(tid))


def test_golden_trees(gpu_ctx):
    g = np.load(os.path.join(GOLD, "rigid_small.npz"))
    meshes = [M(g["points_" + s], g["indices_" + s], g["normals_" + s]) for s in "ab"]
    ids = gpu_ctx.build_trees(meshes)
    for s, tid in zip("ab", ids):
        k = f"tree_{s}_"
        want = oracle.FlatTree(g[k + "root"], g[k + "node_obbs"], g[k + "node_ref"], g[k + "node_cnt"],
                               g[k + "tri_pos"], g[k + "tri_nrm"], g[k + "tri_idx"])
        same(gpu_ctx.export_tree(int(tid)), want)
        gpu_ctx.free_tree(int(tid))


def test_scene_trees(gpu_ctx, port):
    sc = scenes.scene()
    build_and_check(gpu_ctx, port, sc.meshes)


def test_deforming_and_sweep_meshes(gpu_ctx, port):
    ds = scenes.deforming(n_meshes=2)
    bs = scenes.batch_sweep(n_queries=10)
    build_and_check(gpu_ctx, port, [ds.mesh, ds.field] + list(bs.meshes[:12]))


def test_degenerate_meshes(gpu_ctx, port):
    rng = np.random.default_rng(3)
    pts = rng.normal(size=(40, 3)).astype(np.float32)
    cases = [
        M(pts[:3], [[0, 1, 2]]),                                   # one triangle: leaf root
        M(pts[:12], np.arange(12).reshape(4, 3)),                  # four: leaf root
        M(pts[:15], np.arange(15).reshape(5, 3), pts[:15]),        # five: one split
        M(np.zeros((3, 3)), np.zeros((7, 3))),                     # one distinct point
        M(pts[:3], np.tile([[0, 1, 2]], (9, 1))),                  # the same triangle 9 times
        M(np.outer(np.arange(30), [1.0, 2.0, -0.5]), rng.integers(0, 30, (25, 3))),  # collinear points
        M(np.round(pts * 4) / 4, rng.integers(0, 40, (200, 3))),   # equal projections, signed zeros
    ]
    build_and_check(gpu_ctx, port, cases)
    # an empty mesh between two others in one batch
    mixed = gpu_ctx.build_trees([cases[2], M(np.zeros((0, 3)), np.zeros((0, 3))), cases[6]])
    for tid, m in zip((mixed[0], mixed[2]), (cases[2], cases[6])):
        same(gpu_ctx.export_tree(int(tid)), port.tree_build(m.points, m.indices, m.normals).export(),
             normals=m.normals is not None)
    assert gpu_ctx.tree_info(int(mixed[1]))[:2] == (0, 0)
    for tid in mixed:
        gpu_ctx.free_tree(int(tid))
    # an empty mesh: the empty box and no triangles
    tid = int(gpu_ctx.build_trees([M(np.zeros((0, 3)), np.zeros((0, 3)))])[0])
    t = gpu_ctx.export_tree(tid)
    assert t.node_obbs.shape[0] == 0 and t.tri_pos.shape[0] == 0
    eps = np.finfo(np.float32).eps
    assert np.array_equal(t.root, np.array([0, 0, 0, eps, 0, 0, 0, eps, 0, 0, 0, eps], np.float32))
    gpu_ctx.free_tree(tid)


def test_large_node_sums(gpu_ctx, port):
    """Nodes of more than 256 triangles take their coordinate sums without the
    chain, replaying its roundings: meshes whose sums cannot be replayed (one
    coordinate or all), round a few times or too often, or hold only zeros,
    against the oracle's sequential sums."""
    rng = np.random.default_rng(11)
    n_pts = 1500
    base = rng.normal(size=(n_pts, 3)).astype(np.float32)
    wide = base * (10.0 ** rng.uniform(-30, 3, (n_pts, 1))).astype(np.float32)  # exponents too far apart
    grow = base.copy()                                                               # x's running sum too long
    grow[:, 0] = 1.0 + rng.random(n_pts, dtype=np.float32)
    grow[::97, 0] = 2.0 ** -20
    flat = base.copy()                                                               # z all zeros, signed
    flat[:, 2] = np.where(rng.random(n_pts) < 0.5, 0.0, -0.0)
    idx = rng.integers(0, n_pts, (2400, 3))
    meshes = [M(base, idx), M(wide, idx), M(grow, idx), M(flat, idx)]
    # y near 20 with a few values near 2^-20: the sequential y sum rounds 33
    # times (replayed), or 65 and more (more than the replay takes: the chain)
    for frac in (0.005, 0.05):
        t = base.copy()
        r2 = np.random.default_rng(12)
        sel = r2.random(n_pts) < frac
        t[:, 1] += np.float32(20.0)
        t[sel, 1] = ((1.0 + r2.random(sel.sum())) * 2.0 ** -20).astype(np.float32)
        meshes.append(M(t, idx))
    build_and_check(gpu_ctx, port, meshes)


def test_bad_index(gpu_ctx):
    with pytest.raises(capi.CgError) as e:
        gpu_ctx.build_trees([M(np.zeros((3, 3)), [[0, 1, 3]])])
    assert e.value.code == capi.CG_ERR_BAD_TREE


@pytest.mark.parametrize("pageable", ["1", "0"])
def test_mesh_input_paths(port, monkeypatch, pageable):
    """The meshes read by the device from the caller's arrays (where it reads
    pageable host memory) or copied (CG_PAGEABLE_ACCESS=0): the same trees;
    the first bad vertex index by mesh, then position, is the one reported,
    and the context builds again afterwards."""
    monkeypatch.setenv("CG_PAGEABLE_ACCESS", pageable)
    rng = np.random.default_rng(5)
    pts = rng.normal(size=(300, 3)).astype(np.float32)
    good = [M(pts, rng.integers(0, 300, (700, 3)), pts), M(pts[:40], rng.integers(0, 40, (60, 3)))]
    with capi.Context() as ctx:
        build_and_check(ctx, port, good)
        bad_a = np.array(good[1].indices)
        bad_a[17, 2] = 40
        bad_a[30, 0] = 99
        bad_b = np.array(good[0].indices)
        bad_b[3, 1] = 300
        with pytest.raises(capi.CgError) as e:
            ctx.build_trees([good[0], M(pts[:40], bad_a), M(pts, bad_b)])
        assert e.value.code == capi.CG_ERR_BAD_TREE
        assert "mesh 1 index 53 is vertex 40 of 40" in str(e.value)
        build_and_check(ctx, port, good)


def test_misaligned_mesh_arrays(gpu_ctx, port):
    """Mesh arrays 2 bytes off a 4-byte boundary are copied rather than read
    by the device's 4-byte loads: the same trees."""
    rng = np.random.default_rng(9)
    pts = rng.normal(size=(300, 3)).astype(np.float32)
    idx = rng.integers(0, 300, (500, 3)).astype(np.uint32)

    def shifted(a):
        buf = np.zeros(a.nbytes + 2, np.uint8)
        v = buf[2:2 + a.nbytes].view(a.dtype).reshape(a.shape)
        v[...] = a
        assert not v.flags.aligned
        return v

    build_and_check(gpu_ctx, port, [M(shifted(pts), shifted(idx), shifted(pts)), M(pts, shifted(idx))])


def test_built_trees_collide_like_uploaded(gpu_ctx, port):
    """The scene step on GPU-built trees: the same colliding pairs as on the
    oracle's uploaded trees."""
    sc = scenes.scene()
    ids = gpu_ctx.build_trees(sc.meshes[:64])
    keep = (sc.pairs[:, 0] < 64) & (sc.pairs[:, 1] < 64)
    qa, qb = sc.pairs[keep, 0], sc.pairs[keep, 1]
    rel = np.stack([capi.relative_matrix(sc.mats[i], sc.mats[j]) for i, j in zip(qa, qb)])
    st = gpu_ctx.collide(capi.make_queries(ids[qa], ids[qb], rel))
    got = gpu_ctx.tri_pairs()
    trees = [port.tree_build(m.points, m.indices, m.normals) for m in sc.meshes[:64]]
    pairs, _, tests, _ = port.collide_pairs([trees[i] for i in qa], [trees[j] for j in qb], sc.mats[qa], sc.mats[qb])
    assert st["tri_tests"] == tests and len(got) == len(pairs) > 1000
    for tid in ids:
        gpu_ctx.free_tree(int(tid))


def test_built_tree_refits_like_uploaded(gpu_ctx, port):
    """A GPU-built tree's refit side arrays (subtree ranges, parents, leaf
    list) are the upload's: refitting both to the same moved vertices gives
    the same boxes, bit for bit."""
    import torch

    ds = scenes.deforming(n_meshes=2)
    m = ds.mesh
    built = int(gpu_ctx.build_trees([m])[0])
    uploaded = gpu_ctx.upload_flat(port.tree_build(m.points, m.indices, m.normals).export())
    rng = np.random.default_rng(5)
    moved = np.concatenate([m.points + rng.normal(scale=0.05, size=m.points.shape), np.ones((len(m.points), 1))], 1)
    pos = torch.from_numpy(moved.astype(np.float32)).cuda()
    gpu_ctx.tree_refit_batch([built, uploaded], [pos.data_ptr()] * 2, [len(moved)] * 2)
    a, b = gpu_ctx.export_tree(built), gpu_ctx.export_tree(uploaded)
    for k in ("root", "node_obbs", "tri_pos"):
        assert np.array_equal(a.arrays()[k].view(np.uint32), b.arrays()[k].view(np.uint32)), k
    assert not np.array_equal(a.root, port.tree_build(m.points, m.indices, m.normals).export().root)
    gpu_ctx.free_tree(built)
    gpu_ctx.free_tree(uploaded)


def test_tree_cache_round_trip(gpu_ctx, tmp_path):
    """cg_tree_save / cg_tree_load: the same flat tree back; a damaged or
    truncated file is refused."""
    sc = scenes.scene()
    meshes = [sc.meshes[3], M(sc.meshes[4].points, sc.meshes[4].indices)]  # with and without normals
    ids = gpu_ctx.build_trees(meshes)
    for k, tid in enumerate(ids):
        path = str(tmp_path / f"tree{k}.cgtree")
        gpu_ctx.save_tree(int(tid), path)
        back = gpu_ctx.load_tree(path)
        a, b = gpu_ctx.export_tree(int(tid)).arrays(), gpu_ctx.export_tree(back).arrays()
        assert a.keys() == b.keys()
        for key in a:
            assert np.array_equal(a[key].view(np.uint32), b[key].view(np.uint32)), key
        gpu_ctx.free_tree(back)
        raw = bytearray(open(path, "rb").read())
        raw[100] ^= 1
        open(path, "wb").write(bytes(raw))
        with pytest.raises(capi.CgError) as e:
            gpu_ctx.load_tree(path)
        assert e.value.code == capi.CG_ERR_BAD_TREE
        open(path, "wb").write(bytes(raw[:-9]))
        with pytest.raises(capi.CgError) as e:
            gpu_ctx.load_tree(path)
        assert e.value.code == capi.CG_ERR_BAD_TREE
    with pytest.raises(capi.CgError) as e:
        gpu_ctx.load_tree(str(tmp_path / "missing.cgtree"))
    assert e.value.code == capi.CG_ERR_NOT_FOUND
    for tid in ids:
        gpu_ctx.free_tree(int(tid))


def test_trees_from_gltf(gpu_ctx, port, tmp_path):
    """Meshes through a glTF file (inmyroom_vulkan_gb300.gltf) built on the
    device: the oracle's trees of the same triangles, bit for bit; the
    instances' matrices come back exactly."""
    from inmyroom_vulkan_gb300 import gltf

    sc = scenes.scene(n_entities=12)
    meshes = [gltf.Mesh(f"m{k}", m.points, m.normals if k % 3 else None, np.asarray(m.indices).reshape(-1, 3))
              for k, m in enumerate(sc.meshes)]
    path = str(tmp_path / "scene.gltf")
    gltf.save(path, gltf.Scene(meshes, [gltf.Instance(k, sc.mats[k]) for k in range(12)]))
    back = gltf.load(path)
    assert all(np.array_equal(a.matrix, sc.mats[a.mesh]) for a in back.instances)
    build_and_check(gpu_ctx, port, [M(m.points, m.indices, m.normals) for m in back.meshes])
