"""The oracle restatement reproduces the reference's own outputs (golden fixtures
made by tests/golden/make_golden.py from the reference sources) bit for bit."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLD, name))


def bits(x):
    return np.ascontiguousarray(x, np.float32).view(np.uint32)


def tri_tri_ex(port, a, b):
    cop, fr = C.c_int(), C.c_int()
    s, t = np.zeros(3, np.float32), np.zeros(3, np.float32)
    hit = port.fn("tri_tri_ex")(np.ascontiguousarray(a, np.float32), np.ascontiguousarray(b, np.float32),
                                C.byref(cop), C.byref(fr), s, t)
    return hit, cop.value, fr.value, s, t


def test_tri_tri_matches_reference(port):
    """Every case where the reference's behaviour is defined matches bit for bit.
    The "fragile" cases (U's plane distances all below the absolute epsilon while
    V's are not) make the reference read uninitialised interval values
    (Triangle.cpp:960-966); the oracle defines them as no intersection and flags
    them, and they are the only cases allowed to differ."""
    g = load("tritri.npz")
    fragile = 0
    for i in range(len(g["a"])):
        hit, cop, fr, s, t = tri_tri_ex(port, g["a"][i], g["b"][i])
        if fr:
            fragile += 1
            assert hit == 0 and cop == 0
            continue
        assert hit == g["hit"][i] and cop == g["coplanar"][i], i
        if hit and not cop:
            assert np.array_equal(bits(s), bits(g["src"][i])) and np.array_equal(bits(t), bits(g["tgt"][i])), i
    # the near-epsilon and small-scale cases exercise the degenerate branch
    assert 0 < fragile < 40
    # every hand-built case is well defined
    for i in range(25):
        assert tri_tri_ex(port, g["a"][i], g["b"][i])[2] == 0, i


def test_tri_transform_matches_reference(port):
    g = load("tritri.npz")
    for i in range(0, len(g["a"]), 7):
        assert np.array_equal(bits(port.transform_tri(g["mats"][i % 64], g["a"][i])), bits(g["xformed"][i]))


def test_sat_surface_transform_match_reference(port):
    g = load("boxes.npz")
    for i in range(len(g["a"])):
        assert port.sat(g["a"][i], g["b"][i]) == g["sat"][i], i
        assert np.float32(port.surface(g["a"][i])).view(np.uint32) == bits(g["surface"][i]), i
        assert np.array_equal(bits(port.transform_box(g["mats"][i % 64], g["a"][i])), bits(g["xformed"][i])), i
    # the cases separate on different axes, and both outcomes occur
    assert 0 < g["sat"].sum() < len(g["sat"])


def test_relative_matrix_matches_reference(port):
    g = load("boxes.npz")
    m = g["mats"]
    for i in range(64):
        assert np.array_equal(bits(port.relative_matrix(m[i], m[(i * 7 + 3) % 64])), bits(g["relative"][i]))


def test_eig3_matches_reference(port):
    g = load("fits.npz")
    for i in range(len(g["A"])):
        v, d = port.eig3(g["A"][i])
        assert np.array_equal(v.reshape(9).view(np.uint64), g["V"][i].view(np.uint64)), i
        assert np.array_equal(d.view(np.uint64), g["d"][i].view(np.uint64)), i


def test_obb_fit_matches_reference(port):
    g = load("fits.npz")
    off = 0
    for i, n in enumerate(g["lens"]):
        pts = g["pts"][off:off + n]
        off += n
        assert np.array_equal(bits(port.obb_from_points(pts)), bits(g["boxes"][i])), i


@pytest.fixture(scope="module")
def rigid():
    return load("rigid_small.npz")


def _flat(g, tag):
    k = f"tree_{tag}_"
    return oracle.FlatTree(g[k + "root"], g[k + "node_obbs"], g[k + "node_ref"], g[k + "node_cnt"],
                           g[k + "tri_pos"], g[k + "tri_nrm"], g[k + "tri_idx"])


def test_tree_build_matches_reference(port, rigid):
    for tag in ("a", "b"):
        t = port.tree_build(rigid[f"points_{tag}"], rigid[f"indices_{tag}"], rigid[f"normals_{tag}"])
        assert t.export().equal(_flat(rigid, tag))


def test_mid_and_narrow_phase_match_reference(port, rigid):
    ta = port.tree_import(_flat(rigid, "a"))
    tb = port.tree_import(_flat(rigid, "b"))
    for k in range(len(rigid["mats_a"])):
        m = port.mid_phase(ta, tb, rigid["mats_a"][k], rigid["mats_b"][k])
        lp = rigid["leaf_pairs"][rigid["leaf_pairs"][:, 0] == k][:, 1:]
        assert np.array_equal(m.leaf_pairs(), lp), k
        pairs, segs, tests, fragile = m.narrow()
        sel = rigid["pairs"][:, 0] == k
        assert np.array_equal(pairs, rigid["pairs"][sel][:, 1:]), k
        assert np.array_equal(bits(segs), bits(rigid["segs"][sel])), k
        assert tests == rigid["tests"][k]
        ra, rb, avg = m.rays()
        for got, want in ((ra, rigid["rays_a"]), (rb, rigid["rays_b"])):
            want = want[want[:, 0] == k][:, 1:]
            key = lambda r: r[np.lexsort(bits(r).T[::-1])]  # noqa: E731
            assert np.array_equal(bits(key(got)), bits(key(want))), k
        np.testing.assert_allclose(avg, rigid["avgs"][k], rtol=1e-5, atol=1e-6)


def test_shoot_rays_matches_reference(port):
    """ShootUncollideRays::ExecuteShootUncollideRays on the rigid_small poses
    with the reference's rays: the deltas bit for bit."""
    g = load("rigid_small.npz")
    want = load("shoot_small.npz")["deltas"]
    ta = port.tree_build(g["points_a"], g["indices_a"], g["normals_a"])
    tb = port.tree_build(g["points_b"], g["indices_b"], g["normals_b"])
    for k in range(len(g["mats_a"])):
        ra = g["rays_a"][g["rays_a"][:, 0] == k, 1:]
        rb = g["rays_b"][g["rays_b"][:, 0] == k, 1:]
        got = port.shoot_rays(ta, tb, g["mats_a"][k], g["mats_b"][k], ra, rb)
        assert np.array_equal(bits(got), bits(want[k])), k


def test_sweep_and_prune_matches_reference(port):
    """SweepAndPrune::ExecuteSweepAndPrune on the 256-entity scene: the same
    pairs, oriented the same way."""
    from inmyroom_vulkan_gb300 import scenes

    want = load("sap_scene.npz")
    sc = scenes.scene()
    trees = [port.tree_build(m.points, m.indices, m.normals) for m in sc.meshes]
    got = port.sweep_and_prune(trees, sc.mats, want["callback"])
    got = got[np.lexsort((got[:, 1], got[:, 0]))]
    assert np.array_equal(got, want["pairs"])


def test_collision_frame_matches_reference(port):
    """One frame of CollisionDetection::ExecuteCollisionDetection on the
    256-entity scene with a previous frame (a third of the entities still):
    the same pairs with rays and the same deltas, bit for bit, including the
    zero deltas of pairs where neither entity moved."""
    from inmyroom_vulkan_gb300 import scenes
    from oracle import frame

    want = load("frame_scene.npz")
    sc = scenes.scene()
    prev, cb = scenes.frame_motion(sc)
    assert np.array_equal(prev, want["previous"]) and np.array_equal(cb, want["callback"])
    trees = [port.tree_build(m.points, m.indices, m.normals) for m in sc.meshes]
    pairs, deltas = frame.as_arrays(frame.collision_frame(port, trees, sc.mats, prev, cb))
    assert np.array_equal(pairs, want["pairs"])
    assert np.array_equal(bits(deltas), bits(want["deltas"]))
    still = (pairs[:, 0] % 3 == 0) & (pairs[:, 1] % 3 == 0)
    assert still.any() and not np.abs(deltas[still]).any()
    assert np.abs(deltas[~still]).sum(1).min() > 0
    # fewer than two entities: nothing (CollisionDetection.cpp:40)
    assert frame.collision_frame(port, trees[:1], sc.mats[:1], prev[:1], cb[:1]) == []
