"""FP64 reference of the differentiable penetration energy. Test
infrastructure (the checker of the GPU energy and its adjoint), NOT part of the
product.

Every step in float64 torch on the CPU, differentiated by torch autograd:

* posing: bone j's world matrix G_j = G_parent(j) @ T(offset_j) @ R(a_j), R(a)
  = matrix_exp([a]x) (an independent route to the rotation the GPU forms by
  Rodrigues' formula);
* morph + skin, the engine's skinning shader restated
  (shaders/dynamicMeshShader_glsl.comp:78-145, position path): u = base +
  sum_i w_i target_i, p = sum over influences weight * (G_j @ IBM_j) @ u;
* energy over a FIXED list of colliding pairs (query, triangle of the
  deforming tree, triangle of the static tree), both directions of the
  vertex-vs-plane test of src/CollisionDetection/CreateUncollideRays.cpp:102-112:
  sum of min(0, s)^2 with s = n . (p - p0), n the unit normal of
  cross(p1 - p0, p2 - p0) of the other triangle (Plane.cpp:5-20), in the
  deforming tree's space (the static triangle moved by the query's matrix).

With the pair list fixed the energy is a smooth (C1) function of the
parameters, so central finite differences check its autograd gradient.
"""
from __future__ import annotations

import numpy as np
import torch

F64 = torch.float64


def skew(a: torch.Tensor) -> torch.Tensor:
    z = torch.zeros_like(a[..., 0])
    return torch.stack([torch.stack([z, -a[..., 2], a[..., 1]], -1),
                        torch.stack([a[..., 2], z, -a[..., 0]], -1),
                        torch.stack([-a[..., 1], a[..., 0], z], -1)], -2)


def pose(axis_angles: torch.Tensor, parent, offsets) -> torch.Tensor:
    """(P, B, 3) -> world matrices (P, B, 4, 4)."""
    P, B, _ = axis_angles.shape
    R = torch.linalg.matrix_exp(skew(axis_angles))
    off = torch.as_tensor(np.asarray(offsets, np.float64).reshape(B, 3), dtype=F64)
    G = []
    for j in range(B):
        L = torch.zeros(P, 4, 4, dtype=F64)
        L[:, :3, :3] = R[:, j]
        L[:, :3, 3] = off[j]
        L[:, 3, 3] = 1.0
        G.append(L if parent[j] < 0 else G[parent[j]] @ L)
    return torch.stack(G, 1)


def col_major(M: torch.Tensor) -> torch.Tensor:
    """(..., 4, 4) -> (..., 16) column-major."""
    return M.transpose(-1, -2).reshape(M.shape[:-2] + (16,))


def from_col_major(a) -> torch.Tensor:
    t = torch.as_tensor(np.asarray(a, np.float64), dtype=F64)
    return t.reshape(t.shape[:-1] + (4, 4)).transpose(-1, -2)


def deform(G: torch.Tensor, inverse_bind: torch.Tensor, vertices, morph_weights: torch.Tensor, joints,
           weights) -> torch.Tensor:
    """G (P, B, 4, 4), inverse_bind (B, 4, 4), vertices (P, V, 1 + T, 4),
    morph_weights (P, T), joints / weights (V, groups, 4) -> (P, V, 3)."""
    vx = torch.as_tensor(np.asarray(vertices, np.float64), dtype=F64)
    u = vx[:, :, 0] + torch.einsum("pt,pvtc->pvc", morph_weights, vx[:, :, 1:])
    S = G @ inverse_bind  # (P, B, 4, 4)
    j = torch.as_tensor(np.asarray(joints, np.int64).reshape(joints.shape[0], -1))
    w = torch.as_tensor(np.asarray(weights, np.float64).reshape(weights.shape[0], -1), dtype=F64)
    Sv = S[:, j]  # (P, V, 4 * groups, 4, 4)
    out = torch.einsum("vk,pvkrc,pvc->pvr", w, Sv, u)
    return out[..., :3]


def plane_terms(q: torch.Tensor, p: torch.Tensor) -> torch.Tensor:
    """q, p (N, 3, 3): sum over p's vertices of min(0, s)^2 against q's plane."""
    c = torch.cross(q[:, 1] - q[:, 0], q[:, 2] - q[:, 0], dim=-1)
    n = c / torch.linalg.norm(c, dim=-1, keepdim=True)
    s = torch.einsum("nc,nkc->nk", n, p - q[:, :1])
    return torch.clamp(s, max=0.0).square().sum(-1)


def energy(positions: torch.Tensor, tri_idx, static_tri_pos, relative, pairs) -> torch.Tensor:
    """positions (P, V, 3) of the deforming meshes; tri_idx (Ta, 3) vertex
    indices of the deforming tree's triangles (tree order); static_tri_pos
    (Tb, 9) the static tree's triangles (tree order); relative (P, 16) the
    queries' matrices (column-major); pairs (N, 3) [query, tri_a, tri_b]."""
    pairs = np.asarray(pairs, np.int64).reshape(-1, 3)
    if not len(pairs):
        return positions.sum() * 0.0
    qi, ta, tb = (torch.as_tensor(pairs[:, k]) for k in range(3))
    idx = torch.as_tensor(np.asarray(tri_idx, np.int64))[ta]  # (N, 3)
    pa = positions[qi.unsqueeze(1), idx]  # (N, 3, 3)
    M = from_col_major(np.asarray(relative, np.float32).astype(np.float64))[qi]  # (N, 4, 4)
    sb = torch.as_tensor(np.asarray(static_tri_pos, np.float64).reshape(-1, 3, 3), dtype=F64)[tb]
    pb = torch.einsum("nrc,nkc->nkr", M[:, :3, :3], sb) + M[:, None, :3, 3]
    return plane_terms(pb, pa).sum() + plane_terms(pa, pb).sum()


class Problem:
    """The energy as a function of (axis angles, morph weights) for one fixed
    pair list, with its gradient by autograd and by central differences."""

    def __init__(self, parent, offsets, inverse_bind_cm, vertices, joints, weights, tri_idx, static_tri_pos,
                 relative, pairs):
        self.parent, self.offsets = list(parent), offsets
        self.ibm = from_col_major(inverse_bind_cm)
        self.vertices, self.joints, self.weights = vertices, joints, weights
        self.tri_idx, self.static_tri_pos, self.relative, self.pairs = tri_idx, static_tri_pos, relative, pairs

    def __call__(self, aa: torch.Tensor, mw: torch.Tensor) -> torch.Tensor:
        G = pose(aa, self.parent, self.offsets)
        pos = deform(G, self.ibm, self.vertices, mw, self.joints, self.weights)
        return energy(pos, self.tri_idx, self.static_tri_pos, self.relative, self.pairs)

    def value_and_grad(self, aa, mw):
        a = torch.as_tensor(np.asarray(aa, np.float64), dtype=F64).clone().requires_grad_(True)
        w = torch.as_tensor(np.asarray(mw, np.float64), dtype=F64).clone().requires_grad_(True)
        e = self(a, w)
        ga, gw = torch.autograd.grad(e, (a, w))
        return float(e.detach()), ga.numpy(), gw.numpy()

    def central_difference(self, aa, mw, which: str, index, h: float = 1e-4) -> float:
        """(E(x + h e_i) - E(x - h e_i)) / 2h for one coordinate of `which`
        ("axis_angles" or "morph_weights")."""
        vals = []
        for sgn in (1.0, -1.0):
            a = np.array(aa, np.float64, copy=True)
            w = np.array(mw, np.float64, copy=True)
            (a if which == "axis_angles" else w)[index] += sgn * h
            with torch.no_grad():
                vals.append(float(self(torch.as_tensor(a), torch.as_tensor(w))))
        return (vals[0] - vals[1]) / (2.0 * h)
