"""The oracle restatement against the live reference build on larger seeded
workloads (skipped where the reference sources are absent)."""
import numpy as np

from inmyroom_vulkan_gb300 import scenes


def bits(x):
    return np.ascontiguousarray(x, np.float32).view(np.uint32)


def test_rigid_pair_full_size(port, ref):
    rp = scenes.rigid_pair(n_poses=40)
    tp = [port.tree_build(m.points, m.indices, m.normals) for m in (rp.mesh_a, rp.mesh_b)]
    tr = [ref.tree_build(m.points, m.indices, m.normals) for m in (rp.mesh_a, rp.mesh_b)]
    for a, b in zip(tp, tr):
        assert a.export().equal(b.export())
    hits = 0
    for k in range(len(rp.mats_a)):
        mp = port.mid_phase(tp[0], tp[1], rp.mats_a[k], rp.mats_b[k])
        mr = ref.mid_phase(tr[0], tr[1], rp.mats_a[k], rp.mats_b[k])
        assert np.array_equal(mp.leaf_pairs(), mr.leaf_pairs())
        p1, s1, t1, _ = mp.narrow()
        p2, s2, t2, _ = mr.narrow()
        assert np.array_equal(p1, p2) and np.array_equal(bits(s1), bits(s2)) and t1 == t2
        hits += len(p1)
    assert hits > 1000


def test_scene_trees_and_pairs(port, ref):
    sc = scenes.scene(n_entities=24, seed=2024)
    tp = [port.tree_build(m.points, m.indices, m.normals) for m in sc.meshes]
    tr = [ref.tree_build(m.points, m.indices, m.normals) for m in sc.meshes]
    for a, b in zip(tp, tr):
        assert a.export().equal(b.export())
    # all entity pairs, overlapping or not
    for i in range(0, 24, 3):
        for j in range(i + 1, 24, 5):
            mp = port.mid_phase(tp[i], tp[j], sc.mats[i], sc.mats[j])
            mr = ref.mid_phase(tr[i], tr[j], sc.mats[i], sc.mats[j])
            assert np.array_equal(mp.leaf_pairs(), mr.leaf_pairs())
            p1, s1, _, _ = mp.narrow()
            p2, s2, _, _ = mr.narrow()
            assert np.array_equal(p1, p2) and np.array_equal(bits(s1), bits(s2))


def test_face_normal_fallback_and_small_trees(port, ref):
    # (An empty index list crashes the reference's CreateTriangleIndicesList,
    # Triangle.cpp:244, which dereferences max_element of it; the oracle's
    # empty tree is tested on its own in test_oracle_edge_cases.py.)
    rng = np.random.Generator(np.random.PCG64(7))
    for n_tris in (1, 3, 4, 5, 9, 17):
        pts = rng.normal(size=(n_tris * 3, 3)).astype(np.float32)
        idx = np.arange(n_tris * 3, dtype=np.uint32)
        a = port.tree_build(pts, idx, None)
        b = ref.tree_build(pts, idx, None)
        assert a.export().equal(b.export()), n_tris


def test_batch_counts_match(port, ref):
    sc = scenes.scene(n_entities=32, seed=77, cube=8.0)
    tp = [port.tree_build(m.points, m.indices, m.normals) for m in sc.meshes]
    tr = [ref.tree_build(m.points, m.indices, m.normals) for m in sc.meshes]
    ma, mb = sc.mats[sc.pairs[:, 0]], sc.mats[sc.pairs[:, 1]]
    r1 = port.collide_batch([tp[i] for i in sc.pairs[:, 0]], [tp[j] for j in sc.pairs[:, 1]], ma, mb, threads=4)
    r2 = ref.collide_batch([tr[i] for i in sc.pairs[:, 0]], [tr[j] for j in sc.pairs[:, 1]], ma, mb, threads=4)
    assert r1["tests"] == r2["tests"] and r1["rays"] == r2["rays"]


def test_shoot_rays_full_size(port, ref):
    """ShootUncollideRays with the engine's settings and with others, on the
    full rigid pair: port and reference give the same deltas, bit for bit."""
    rp = scenes.rigid_pair(n_poses=30)
    tp = [port.tree_build(m.points, m.indices, m.normals) for m in (rp.mesh_a, rp.mesh_b)]
    tr = [ref.tree_build(m.points, m.indices, m.normals) for m in (rp.mesh_a, rp.mesh_b)]
    moved = 0
    for k in range(len(rp.mats_a)):
        ra, rb, _ = port.mid_phase(tp[0], tp[1], rp.mats_a[k], rp.mats_b[k]).rays()
        for params in (None, np.array([0.3, 1.2, 1.5], np.float32)):
            a = port.shoot_rays(tp[0], tp[1], rp.mats_a[k], rp.mats_b[k], ra, rb, params)
            b = ref.shoot_rays(tr[0], tr[1], rp.mats_a[k], rp.mats_b[k], ra, rb, params)
            assert np.array_equal(bits(a), bits(b)), (k, a, b)
            moved += int(np.any(a != 0))
    assert moved > 30


def test_sweep_and_prune_axes_and_callbacks(port, ref):
    """SweepAndPrune with the engine's axes and with others, all and some
    entities calling back: port and reference give the same oriented pairs."""
    sc = scenes.scene(n_entities=128, seed=1077)
    tp = [port.tree_build(m.points, m.indices, m.normals) for m in sc.meshes]
    tr = [ref.tree_build(m.points, m.indices, m.normals) for m in sc.meshes]
    rng = np.random.default_rng(3)
    axes = np.linalg.qr(rng.normal(size=(3, 3)))[0].T.astype(np.float32)
    for cb in (np.ones(len(tp), np.uint8), (rng.random(len(tp)) < 0.3).astype(np.uint8)):
        for ax in (None, axes):
            a = port.sweep_and_prune(tp, sc.mats, cb, ax)
            b = ref.sweep_and_prune(tr, sc.mats, cb, ax)
            assert set(map(tuple, a)) == set(map(tuple, b)) and len(a) == len(b)


def _same_bits(a, b):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    nan = np.isnan(b)
    return a.shape == b.shape and np.array_equal(np.isnan(a), nan) and np.array_equal(bits(a)[~nan], bits(b)[~nan])


def test_scene256_full_size(port, ref):
    """The full 256-entity scene: every tree of the port's builder equals the
    reference builder's, and for every AABB-overlap query the leaf pairs (in
    the descent's order), the colliding pairs and segments, the uncollide rays
    (in the order of the reference's unordered_map) and the mean origins are
    the reference's, bit for bit."""
    sc = scenes.scene()
    tp = [port.tree_build(m.points, m.indices, m.normals) for m in sc.meshes]
    tr = [ref.tree_build(m.points, m.indices, m.normals) for m in sc.meshes]
    for k, (a, b) in enumerate(zip(tp, tr)):
        assert a.export().equal(b.export()), k
    n_rays = 0
    for i, j in sc.pairs:
        mp = port.mid_phase(tp[i], tp[j], sc.mats[i], sc.mats[j])
        mr = ref.mid_phase(tr[i], tr[j], sc.mats[i], sc.mats[j])
        assert np.array_equal(mp.leaf_pairs(), mr.leaf_pairs()), (i, j)
        p1, s1, t1, _ = mp.narrow()
        p2, s2, t2, _ = mr.narrow()
        assert np.array_equal(p1, p2) and np.array_equal(bits(s1), bits(s2)) and t1 == t2, (i, j)
        ra1, rb1, avg1 = mp.rays()
        ra2, rb2, avg2 = mr.rays()
        assert _same_bits(ra1, ra2) and _same_bits(rb1, rb2), (i, j)
        assert _same_bits(avg1, avg2), (i, j, avg1, avg2)
        n_rays += len(ra1) + len(rb1)
    assert n_rays > 20000
