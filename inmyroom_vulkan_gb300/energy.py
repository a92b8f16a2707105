"""Differentiable penetration energy of skinned, morphed meshes against static
trees, behind a torch.autograd.Function.

The engine itself only resolves collisions; this is the differentiable form of
the same path. Per forward, on the current CUDA stream: skeletons posed from
axis angles (cg_pose), morph + skin (cg_deform_batch), tree refit
(cg_tree_refit_batch), the collide step (cg_collide_async) and the energy of
its colliding pairs (cg_energy). The backward runs the hand-written adjoints
(cg_energy_backward, which recomputes the deformed vertices it needs, then
cg_pose_backward). Every step is a CUDA kernel of libcollide_gpu.so; there is
no CPU path.
"""
from __future__ import annotations

import numpy as np
import torch

from . import capi

# cudaStreamLegacy: torch reports its legacy default stream as handle 0, which
# the C ABI reads as "the context's own stream"; this handle names the legacy
# default stream itself, so the kernels stay ordered with torch's work on it.
CUDA_STREAM_LEGACY = 1


def current_stream() -> int:
    return torch.cuda.current_stream().cuda_stream or CUDA_STREAM_LEGACY


class DeformingCollider:
    """n meshes of one rest topology (one OBB tree each, refitted every
    forward), each collided with one static tree.

    vertices (n, V, 1 + targets, 4) float32: base (w = 1) then target offsets;
    joints (V, groups, 4) uint16 and weights (V, groups, 4) float32 shared;
    inverse_bind (bones, 16) column-major; relative (n, 16) the queries'
    matrices inverse(mesh placement) * static placement.
    """

    def __init__(self, ctx: capi.Context, rest_tree, skeleton: capi.Skeleton, vertices, joints, weights, inverse_bind,
                 static_tree_id: int, relative, flags: int = 0):
        dev = torch.device("cuda")
        vertices = np.ascontiguousarray(vertices, np.float32)
        self.ctx, self.skeleton, self.flags = ctx, skeleton, flags
        self.n, self.V, tp1, _ = vertices.shape
        self.T = tp1 - 1
        self.B = skeleton.n_bones
        self.groups = joints.shape[1]
        self.ids = [ctx.upload_flat(rest_tree) for _ in range(self.n)]
        t = lambda a, dt=None: torch.from_numpy(np.ascontiguousarray(a, dt)).to(dev)  # noqa: E731
        self.vertices = t(vertices)
        self.joints = t(np.asarray(joints, np.uint16).view(np.int16))
        self.weights = t(weights, np.float32)
        self.inverse_bind = t(inverse_bind, np.float32)
        # stable buffers: the batch tables hold their addresses
        self.axis_angles = torch.zeros(self.n, self.B, 3, device=dev)
        self.morph_weights = torch.zeros(self.n, max(self.T, 1), device=dev)
        self.joint_matrices = torch.zeros(self.n, self.B, 16, device=dev)
        self.positions = torch.zeros(self.n, self.V, 4, device=dev)
        self.energy_out = torch.zeros((), dtype=torch.float64, device=dev)
        self.grad_joint = torch.zeros(self.n, self.B, 16, device=dev)
        self.grad_morph = torch.zeros(self.n, max(self.T, 1), device=dev)
        self.grad_axis_angles = torch.zeros(self.n, self.B, 3, device=dev)
        self.views = [capi.cg_deform_view(self.V, self.T, self.groups, self.B, self.vertices[m].data_ptr(),
                                          self.morph_weights[m].data_ptr(), self.joints.data_ptr(),
                                          self.weights.data_ptr(), self.joint_matrices[m].data_ptr(),
                                          self.inverse_bind.data_ptr()) for m in range(self.n)]
        self.out_ptrs = [self.positions[m].data_ptr() for m in range(self.n)]
        self.side = capi.EnergySide(self.views, self.B, self.T, self.grad_joint.data_ptr(),
                                    self.grad_morph.data_ptr() if self.T else None)
        q = capi.make_queries(self.ids, [static_tree_id] * self.n, np.asarray(relative, np.float32))
        self.queries = torch.from_numpy(q.view(np.uint8).copy()).to(dev)
        self.generation = 0

    def close(self):
        for i in self.ids:
            self.ctx.free_tree(i)
        self.ids = []

    # -- the two passes, on device buffers --

    def forward_pass(self, axis_angles: torch.Tensor, morph_weights: torch.Tensor) -> torch.Tensor:
        s = current_stream()
        self.axis_angles.copy_(axis_angles.detach().reshape(self.n, self.B, 3))
        if self.T:
            self.morph_weights.copy_(morph_weights.detach().reshape(self.n, self.T))
        c = self.ctx
        c.pose(self.skeleton, self.axis_angles.data_ptr(), self.n, self.joint_matrices.data_ptr(), s)
        c.deform_batch(self.views, self.out_ptrs, s)
        c.tree_refit_batch(self.ids, self.out_ptrs, [self.V] * self.n, s)
        c.collide_async(self.queries.data_ptr(), self.n, self.flags, s)
        c.energy(self.energy_out.data_ptr(), s)
        self.generation += 1
        return self.energy_out

    def backward_pass(self, grad_energy: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
        s = current_stream()
        g = grad_energy.detach().to(device=self.energy_out.device, dtype=torch.float64).reshape(()).contiguous()
        c = self.ctx
        c.energy_backward(g.data_ptr(), self.side, None, s)
        c.pose_backward(self.skeleton, self.axis_angles.data_ptr(), self.joint_matrices.data_ptr(),
                        self.grad_joint.data_ptr(), self.n, self.grad_axis_angles.data_ptr(), s)
        return self.grad_axis_angles, self.grad_morph[:, :self.T]

    def tri_pairs(self) -> np.ndarray:
        """The colliding pairs of the last forward (host copy)."""
        return self.ctx.tri_pairs()


class PenetrationEnergy(torch.autograd.Function):
    """E(axis_angles (n, bones, 3), morph_weights (n, targets)) as a float64
    scalar; its backward gives dE/d axis_angles and dE/d morph_weights (float32).
    The colliding pair set is the forward's (piecewise constant in the inputs).
    A later forward on the same collider replaces that set: backward then
    raises."""

    @staticmethod
    def forward(ctx, axis_angles, morph_weights, collider: DeformingCollider):
        e = collider.forward_pass(axis_angles, morph_weights).clone()
        ctx.collider = collider
        ctx.generation = collider.generation
        return e

    @staticmethod
    def backward(ctx, grad_energy):
        col: DeformingCollider = ctx.collider
        if col.generation != ctx.generation:
            raise RuntimeError("the collider ran another forward since this one: its colliding pairs and "
                               "deformation were replaced; run forward again before backward")
        ga, gw = col.backward_pass(grad_energy)
        return ga.clone(), gw.clone(), None


def penetration_energy(axis_angles: torch.Tensor, morph_weights: torch.Tensor,
                       collider: DeformingCollider) -> torch.Tensor:
    return PenetrationEnergy.apply(axis_angles, morph_weights, collider)
