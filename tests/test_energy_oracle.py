"""The FP64 reference of the penetration energy (oracle/energy.py), pinned on
the CPU: its posing equals the deforming scene's bone chain, its morph + skin
equals the C++ restatement of the skinning shader
(shaders/dynamicMeshShader_glsl.comp:78-145), and its autograd gradient equals
FP64 central differences (h = 1e-4) on every parameter of a small scene."""
import numpy as np
import torch

from inmyroom_vulkan_gb300 import scenes
from oracle import energy as oe


def chain_skeleton(sc):
    B = sc.axis_angles.shape[1]
    parent = [-1] + list(range(B - 1))
    offsets = np.array([[0.0, 0.0, 0.0]] + [[0.0, sc.bone_len, 0.0]] * (B - 1))
    return parent, offsets


def small_problem(port):
    sc = scenes.deforming(n_meshes=3, rings=24, around=12, n_bones=8, grid=48)
    n = sc.vertices.shape[0]
    parent, offsets = chain_skeleton(sc)
    rest = port.tree_build(sc.mesh.points, sc.mesh.indices, sc.mesh.normals)
    field = port.tree_build(sc.field.points, sc.field.indices, sc.field.normals)
    rf, ff = rest.export(), field.export()
    eye = np.eye(4, dtype=np.float32).reshape(16)
    trees = [port.tree_import(port.tree_refit(rf, port.deform(sc.vertices[m], sc.morph_weights[m], sc.joints,
                                                                 sc.weights, sc.joint_matrices[m], sc.inverse_bind)))
             for m in range(n)]
    pairs, _, _, _ = port.collide_pairs(trees, [field] * n, sc.models, [eye] * n)
    rel = np.stack([port.relative_matrix(sc.models[m], eye) for m in range(n)])
    pr = oe.Problem(parent, offsets, sc.inverse_bind, sc.vertices, sc.joints, sc.weights, rf.tri_idx, ff.tri_pos, rel,
                    pairs)
    return sc, pr, pairs


def test_pose_is_the_scene_chain():
    sc = scenes.deforming(n_meshes=4, rings=8, around=6, n_bones=50, grid=8)
    parent, offsets = chain_skeleton(sc)
    G = oe.pose(torch.as_tensor(sc.axis_angles), parent, offsets).numpy()
    for m in range(len(G)):
        np.testing.assert_allclose(G[m], scenes.chain_matrices(sc.axis_angles[m], sc.bone_len), rtol=0, atol=1e-12)


def test_skin_matches_the_restatement(port):
    sc = scenes.deforming(n_meshes=3, rings=24, around=12, n_bones=8, grid=8)
    ibm = oe.from_col_major(sc.inverse_bind)
    G = oe.from_col_major(sc.joint_matrices.astype(np.float64))
    pos = oe.deform(G, ibm, sc.vertices, torch.as_tensor(sc.morph_weights, dtype=torch.float64), sc.joints,
                    sc.weights).numpy()
    for m in range(len(pos)):
        want = np.asarray(port.deform(sc.vertices[m], sc.morph_weights[m], sc.joints, sc.weights, sc.joint_matrices[m],
                                      sc.inverse_bind))[:, :3]
        np.testing.assert_allclose(pos[m], want, rtol=0, atol=2e-6 * np.abs(want).max())


def test_gradient_equals_central_differences(port):
    sc, pr, pairs = small_problem(port)
    assert len(pairs) > 50
    e, ga, gw = pr.value_and_grad(sc.axis_angles, sc.morph_weights)
    assert e > 0
    fd_a = np.array([pr.central_difference(sc.axis_angles, sc.morph_weights, "axis_angles", i)
                     for i in np.ndindex(ga.shape)]).reshape(ga.shape)
    fd_w = np.array([pr.central_difference(sc.axis_angles, sc.morph_weights, "morph_weights", i)
                     for i in np.ndindex(gw.shape)]).reshape(gw.shape)
    for fd, g in ((fd_a, ga), (fd_w, gw)):
        assert np.linalg.norm(fd - g) <= 1e-5 * np.linalg.norm(g)
        np.testing.assert_allclose(fd, g, rtol=1e-4, atol=1e-6 * np.abs(g).max())


def test_energy_terms_by_hand():
    """One pair: a triangle in z = 0 (normal +z) and one with a vertex 0.5
    below it and the others above; the reverse direction adds the first
    triangle's vertices below the second's plane."""
    pa = np.array([[[0, 0, 0], [1, 0, 0], [0, 1, 0]]], np.float64)
    pb = np.array([[[0.2, 0.2, -0.5], [0.2, 0.2, 1.0], [0.6, 0.2, 1.0]]], np.float64)
    t = oe.plane_terms(torch.as_tensor(pa), torch.as_tensor(pb)).item()
    assert abs(t - 0.25) < 1e-15
    # the reverse direction against the second triangle's plane, worked out here
    n = np.cross(pb[0, 1] - pb[0, 0], pb[0, 2] - pb[0, 0])
    n /= np.linalg.norm(n)
    s = (pa[0] - pb[0, 0]) @ n
    want = float((np.minimum(s, 0) ** 2).sum())
    assert abs(oe.plane_terms(torch.as_tensor(pb), torch.as_tensor(pa)).item() - want) < 1e-15
