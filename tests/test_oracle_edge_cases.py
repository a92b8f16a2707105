"""Edge cases of the oracle that the reference cannot run or that need no reference."""
import numpy as np

EPS = np.float32(np.finfo(np.float32).eps)


def test_empty_tree_is_empty_obb_leaf(port):
    t = port.tree_build(np.zeros((0, 3), np.float32), np.zeros(0, np.uint32))
    f = t.export()
    assert f.n_nodes == 0 and f.n_tris == 0
    # OBB::EmptyOBB (OBB.cpp:168-178)
    assert np.array_equal(f.root, np.float32([0, 0, 0, EPS, 0, 0, 0, EPS, 0, 0, 0, EPS]))


def test_point_and_two_point_fits(port):
    b = port.obb_from_points(np.ones((4, 3), np.float32))
    assert np.array_equal(b, np.float32([1, 1, 1, EPS, 0, 0, 0, EPS, 0, 0, 0, EPS]))
    b = port.obb_from_points(np.float32([[0, 0, 0], [2, 0, 0]]))
    assert np.isclose(np.linalg.norm(b[3:12].reshape(3, 3), axis=1).max(), 1.0 + EPS)


def test_leaf_root_tree_keeps_input_order(port):
    pts = np.arange(36, dtype=np.float32).reshape(12, 3) * np.float32(0.1)
    idx = np.arange(12, dtype=np.uint32)
    f = port.tree_build(pts, idx).export()
    assert f.n_nodes == 0 and f.n_tris == 4
    assert np.array_equal(f.tri_idx.reshape(-1), idx)


def test_far_apart_has_no_leaf_pairs(port):
    from inmyroom_vulkan_gb300 import scenes

    rp = scenes.rigid_pair(n_poses=1, subdiv=2)
    ta = port.tree_build(rp.mesh_a.points, rp.mesh_a.indices, rp.mesh_a.normals)
    tb = port.tree_build(rp.mesh_b.points, rp.mesh_b.indices, rp.mesh_b.normals)
    far = scenes.pose(np.eye(3), [10.0, 0, 0])
    m = port.mid_phase(ta, tb, rp.mats_a[0], far)
    assert len(m.leaf_pairs()) == 0
    p, s, t, fr = m.narrow()
    assert len(p) == 0 and t == 0
