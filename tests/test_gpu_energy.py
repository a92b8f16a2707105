"""GPU penetration energy and its hand-written adjoint (cg_pose, cg_energy,
cg_energy_backward, cg_pose_backward behind PenetrationEnergy) on the
deforming workload (64 skinned + morphed 12,000-triangle tubes against a
198,450-triangle heightfield), against the FP64 reference of oracle/energy.py
evaluated on the GPU's own colliding pair set:

* energy within E_RTOL relative;
* gradients with respect to the 64 x 50 x 3 axis angles and 64 x 8 morph
  weights within GRAD_RTOL (2-norm relative error, the whole gradient and each
  mesh's), and against FP64 central differences (h = 1e-4) on the largest
  entries.
"""
import numpy as np
import pytest
import torch

from inmyroom_vulkan_gb300 import capi, scenes
from inmyroom_vulkan_gb300.energy import DeformingCollider, current_stream, penetration_energy
from oracle import energy as oe

pytestmark = pytest.mark.gpu

E_RTOL = 1e-4
GRAD_RTOL = 1e-3
FD_RTOL = 2e-3


def make(ctx, port, **kw):
    sc = scenes.deforming(**kw)
    parent, offsets = scenes.chain_skeleton(sc)
    rest = port.tree_build(sc.mesh.points, sc.mesh.indices, sc.mesh.normals)
    field = port.tree_build(sc.field.points, sc.field.indices, sc.field.normals)
    rf, ff = rest.export(), field.export()
    fid = ctx.upload_flat(ff)
    eye = np.eye(4, dtype=np.float32).reshape(16)
    rel = np.stack([capi.relative_matrix(m, eye) for m in sc.models])
    col = DeformingCollider(ctx, rf, capi.Skeleton(parent, offsets), sc.vertices, sc.joints, sc.weights,
                            sc.inverse_bind, fid, rel)
    pr = lambda pairs: oe.Problem(parent, offsets.astype(np.float64), sc.inverse_bind, sc.vertices,  # noqa: E731
                                  sc.joints, sc.weights, rf.tri_idx, ff.tri_pos, rel, pairs)
    return sc, col, pr, fid


def leaf(t):
    return torch.tensor(np.asarray(t, np.float32), device="cuda", requires_grad=True)


def pair_array(col):
    p = col.tri_pairs()
    return np.stack([p["query"], p["tri_a"], p["tri_b"]], 1).astype(np.int64)


def test_pose_matches_fp64(gpu_ctx):
    sc = scenes.deforming(n_meshes=8, rings=4, around=4, grid=8)
    parent, offsets = scenes.chain_skeleton(sc)
    skel = capi.Skeleton(parent, offsets)
    aa = torch.tensor(sc.axis_angles, dtype=torch.float32, device="cuda")
    aa[0, :5] = 0.0  # the series branch
    aa[1, :5] *= 1e-3
    jm = torch.zeros(8, aa.shape[1], 16, device="cuda")
    gpu_ctx.pose(skel, aa.data_ptr(), 8, jm.data_ptr(), current_stream())
    want = oe.col_major(oe.pose(aa.cpu().double(), parent, offsets.astype(np.float64))).numpy()
    np.testing.assert_allclose(jm.cpu().numpy(), want, rtol=0, atol=5e-6)


def test_energy_and_gradient_match_fp64(gpu_ctx, port):
    sc, col, problem, fid = make(gpu_ctx, port)
    aa, mw = leaf(sc.axis_angles), leaf(sc.morph_weights)
    E = penetration_energy(aa, mw, col)
    E.backward()
    pairs = pair_array(col)
    assert len(pairs) > 1000
    pr = problem(pairs)
    e64, ga64, gw64 = pr.value_and_grad(aa.detach().cpu().double().numpy(), mw.detach().cpu().double().numpy())
    assert abs(E.item() - e64) <= E_RTOL * e64, (E.item(), e64)
    ga, gw = aa.grad.cpu().numpy().astype(np.float64), mw.grad.cpu().numpy().astype(np.float64)
    for got, want in ((ga, ga64), (gw, gw64)):
        assert np.linalg.norm(got - want) <= GRAD_RTOL * np.linalg.norm(want)
        for m in range(len(want)):
            if np.linalg.norm(want[m]) > 0:
                assert np.linalg.norm(got[m] - want[m]) <= GRAD_RTOL * np.linalg.norm(want[m]), m
            else:
                assert not got[m].any(), m
    a64, w64 = aa.detach().cpu().double().numpy(), mw.detach().cpu().double().numpy()
    for which, g, g64 in (("axis_angles", ga, ga64), ("morph_weights", gw, gw64)):
        for flat in np.argsort(-np.abs(g64).ravel())[:3]:
            idx = np.unravel_index(flat, g64.shape)
            fd = pr.central_difference(a64, w64, which, idx)
            assert abs(g[idx] - fd) <= FD_RTOL * abs(fd), (which, idx, g[idx], fd)
    col.close()
    gpu_ctx.free_tree(fid)


def test_backward_after_another_forward_raises(gpu_ctx, port):
    sc, col, _, fid = make(gpu_ctx, port, n_meshes=4, rings=20, around=12, grid=64)
    aa, mw = leaf(sc.axis_angles), leaf(sc.morph_weights)
    E1 = penetration_energy(aa, mw, col)
    E2 = penetration_energy(aa, mw, col)
    E2.backward()
    with pytest.raises(RuntimeError):
        E1.backward()
    # the same inputs again: the same pair set and energy
    assert torch.equal(E1, E2)
    col.close()
    gpu_ctx.free_tree(fid)


def test_energy_needs_the_pairs(gpu_ctx, port):
    sc, col, _, fid = make(gpu_ctx, port, n_meshes=2, rings=8, around=8, grid=16)
    col.flags = capi.CG_MID_ONLY
    with pytest.raises(capi.CgError):
        penetration_energy(leaf(sc.axis_angles), leaf(sc.morph_weights), col)
    col.close()
    gpu_ctx.free_tree(fid)
