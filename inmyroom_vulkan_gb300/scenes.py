"""Seeded synthetic collision workloads (numpy PCG64; workload k uses seed 1000+k).

The reference publishes no collision benchmark or dataset, so every workload is
synthetic. Meshes are indexed triangle lists with per-vertex normals, the form
the reference's tree builder consumes (inMyRoom_vulkan/src/Geometry/Triangle.cpp
Triangle::CreateTriangleList, glTF "triangles" mode). Poses are 4x4 column-major
float32 matrices, the layout of glm::mat4 (CollisionDetectionEntry::
currentGlobalMatrix, include/ECS/ECStypes.h:149-156).

Workloads:
  rigid_pair      two 2,048-triangle jittered spheres (octahedron subdivided 4
                  times, radius 1, vertex jitter N(0, 0.01)) and 1,000 pose
                  pairs: rotations uniform on SO(3), translation uniform in a
                  ball of radius 1.5.
  scene           256 rigid entities, triangle counts log-uniform in
                  [500, 20000]: half jittered UV spheres, half convex-hull blobs;
                  radius U[0.5, 2] m; positions U[0, 20]^3 m; uniform SO(3)
                  orientations; queries are the entity pairs whose world AABBs
                  overlap, ordered (lower id, higher id).
  batch_sweep     a pool of meshes with log-uniform triangle counts in
                  [256, 65536] and 10,000 pair queries drawn from it, poses
                  rejection-sampled so that about half the root boxes overlap.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

SEED_BASE = 1000


@dataclass
class Mesh:
    points: np.ndarray  # (V,3) float32
    normals: np.ndarray  # (V,3) float32
    indices: np.ndarray  # (T*3,) uint32

    @property
    def n_tris(self) -> int:
        return self.indices.size // 3


def vertex_normals(points: np.ndarray, indices: np.ndarray) -> np.ndarray:
    """Area-weighted vertex normals, unit length."""
    p = points.astype(np.float64)
    tri = indices.reshape(-1, 3)
    fn = np.cross(p[tri[:, 1]] - p[tri[:, 0]], p[tri[:, 2]] - p[tri[:, 0]])
    n = np.zeros_like(p)
    for k in range(3):
        np.add.at(n, tri[:, k], fn)
    ln = np.linalg.norm(n, axis=1, keepdims=True)
    ln[ln == 0] = 1.0
    return (n / ln).astype(np.float32)


def octa_sphere(subdiv: int, radius: float, jitter: float, rng: np.random.Generator) -> Mesh:
    """Octahedron subdivided `subdiv` times (8*4^subdiv triangles), projected to
    the sphere, vertices jittered by N(0, jitter)."""
    verts = [np.array(v, np.float64) for v in
             [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]]
    faces = [(0, 2, 4), (2, 1, 4), (1, 3, 4), (3, 0, 4), (2, 0, 5), (1, 2, 5), (3, 1, 5), (0, 3, 5)]
    for _ in range(subdiv):
        mid = {}

        def midpoint(a, b):
            key = (min(a, b), max(a, b))
            if key not in mid:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                mid[key] = len(verts) - 1
            return mid[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            nf += [(a, ab, ca), (ab, b, bc), (ca, bc, c), (ab, bc, ca)]
        faces = nf
    p = np.array(verts) * radius
    p = p + rng.normal(0.0, jitter, size=p.shape)
    idx = np.array(faces, np.uint32).reshape(-1)
    p = p.astype(np.float32)
    return Mesh(p, vertex_normals(p, idx), idx)


def uv_sphere(target_tris: int, radius: float, jitter: float, rng: np.random.Generator) -> Mesh:
    """UV sphere with about `target_tris` triangles: nlon*(2*nlat-2)."""
    nlat = max(3, int(round(math.sqrt(target_tris / 4.0))) + 1)
    nlon = max(3, int(round(target_tris / (2.0 * nlat - 2.0))))
    th = np.linspace(0, math.pi, nlat + 1)[1:-1]
    ph = np.linspace(0, 2 * math.pi, nlon, endpoint=False)
    T, P = np.meshgrid(th, ph, indexing="ij")
    ring = np.stack([np.sin(T) * np.cos(P), np.sin(T) * np.sin(P), np.cos(T)], -1).reshape(-1, 3)
    p = np.concatenate([[[0, 0, 1]], ring, [[0, 0, -1]]]) * radius
    p = p + rng.normal(0.0, jitter, size=p.shape)
    tris = []
    top, bot = 0, 1 + ring.shape[0]
    r = lambda i, j: 1 + i * nlon + (j % nlon)  # noqa: E731
    for j in range(nlon):
        tris.append((top, r(0, j), r(0, j + 1)))
    for i in range(nlat - 2):
        for j in range(nlon):
            a, b, c, d = r(i, j), r(i + 1, j), r(i + 1, j + 1), r(i, j + 1)
            tris += [(a, b, c), (a, c, d)]
    for j in range(nlon):
        tris.append((bot, r(nlat - 2, j + 1), r(nlat - 2, j)))
    idx = np.array(tris, np.uint32).reshape(-1)
    p = p.astype(np.float32)
    return Mesh(p, vertex_normals(p, idx), idx)


def hull_blob(target_tris: int, radius: float, rng: np.random.Generator) -> Mesh:
    """Convex hull of n = T/2 + 2 radially perturbed sphere points (2n-4 = T
    triangles when every point lies on the hull), outward winding."""
    from scipy.spatial import ConvexHull

    n = target_tris // 2 + 2
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    # smooth low-frequency radial perturbation keeps the hull blob-shaped
    k = rng.normal(size=(4, 3))
    bumps = 0.15 * np.tanh(d @ k.T).sum(1) / 2.0
    p = d * (radius * (1.0 + bumps))[:, None]
    hull = ConvexHull(p)
    used = np.unique(hull.simplices)
    remap = -np.ones(n, np.int64)
    remap[used] = np.arange(used.size)
    pts = p[used]
    tri = remap[hull.simplices]
    c = pts.mean(0)
    a, b, cc = pts[tri[:, 0]], pts[tri[:, 1]], pts[tri[:, 2]]
    flip = (np.cross(b - a, cc - a) * (a - c)).sum(1) < 0
    tri[flip] = tri[flip][:, [0, 2, 1]]
    idx = tri.astype(np.uint32).reshape(-1)
    pts = pts.astype(np.float32)
    return Mesh(pts, vertex_normals(pts, idx), idx)


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    """Uniform on SO(3): unit quaternion from a normalised 4-D Gaussian."""
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def pose(R: np.ndarray, t) -> np.ndarray:
    """4x4 column-major float32 (16,) from rotation R and translation t."""
    M = np.eye(4)
    M[:3, :3] = R
    M[:3, 3] = t
    return M.T.reshape(16).astype(np.float32)


def ball_point(rng: np.random.Generator, radius: float) -> np.ndarray:
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    return d * radius * rng.uniform() ** (1.0 / 3.0)


# ------------------------------------------------------------------ rigid pair
@dataclass
class RigidPair:
    mesh_a: Mesh
    mesh_b: Mesh
    mats_a: np.ndarray  # (P,16)
    mats_b: np.ndarray  # (P,16)


def rigid_pair(n_poses: int = 1000, seed: int = SEED_BASE + 1, subdiv: int = 4) -> RigidPair:
    rng = np.random.Generator(np.random.PCG64(seed))
    a = octa_sphere(subdiv, 1.0, 0.01, rng)
    b = octa_sphere(subdiv, 1.0, 0.01, rng)
    ma = np.stack([pose(random_rotation(rng), np.zeros(3)) for _ in range(n_poses)])
    mb = np.stack([pose(random_rotation(rng), ball_point(rng, 1.5)) for _ in range(n_poses)])
    return RigidPair(a, b, ma, mb)


# ------------------------------------------------------------------ scene
@dataclass
class Scene:
    meshes: list
    mats: np.ndarray  # (E,16)
    pairs: np.ndarray  # (Q,2) entity ids, lower first
    kinds: list = field(default_factory=list)


def world_aabb(mesh: Mesh, m16: np.ndarray):
    M = m16.reshape(4, 4).T.astype(np.float64)
    w = mesh.points.astype(np.float64) @ M[:3, :3].T + M[:3, 3]
    return w.min(0), w.max(0)


def aabb_pairs(meshes, mats) -> np.ndarray:
    boxes = [world_aabb(m, t) for m, t in zip(meshes, mats)]
    lo = np.array([b[0] for b in boxes])
    hi = np.array([b[1] for b in boxes])
    ov = np.all((lo[:, None, :] <= hi[None, :, :]) & (lo[None, :, :] <= hi[:, None, :]), axis=2)
    i, j = np.nonzero(np.triu(ov, 1))
    return np.stack([i, j], 1).astype(np.uint32)


def scene(n_entities: int = 256, seed: int = SEED_BASE + 2, tri_lo: int = 500, tri_hi: int = 20000,
          cube: float = 20.0) -> Scene:
    rng = np.random.Generator(np.random.PCG64(seed))
    meshes, mats, kinds = [], [], []
    for e in range(n_entities):
        T = int(round(math.exp(rng.uniform(math.log(tri_lo), math.log(tri_hi)))))
        r = rng.uniform(0.5, 2.0)
        if e % 2 == 0:
            m = uv_sphere(T, r, 0.01 * r, rng)
            kinds.append("sphere")
        else:
            m = hull_blob(T, r, rng)
            kinds.append("blob")
        meshes.append(m)
        mats.append(pose(random_rotation(rng), rng.uniform(0.0, cube, size=3)))
    mats = np.stack(mats)
    return Scene(meshes, mats, aabb_pairs(meshes, mats), kinds)


def frame_motion(sc: Scene, seed: int = SEED_BASE + 6, still_every: int = 3, step: float = 0.05,
                 callback_share: float = 0.7) -> tuple[np.ndarray, np.ndarray]:
    """A previous frame for a scene's current one: every still_every-th entity
    stands still, the others moved by up to `step` (a translation and a small
    rotation about their own origin); and should-callback flags for a seeded
    share of the entities. (previous (n, 16), callback (n,) uint8)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = len(sc.meshes)
    prev = sc.mats.copy()
    for i in range(n):
        if i % still_every == 0:
            continue
        M = sc.mats[i].reshape(4, 4).T.astype(np.float64)
        ax = rng.normal(size=3)
        ax *= rng.uniform(0.0, step) / np.linalg.norm(ax)
        R = np.eye(4)
        R[:3, :3] = axis_angle_matrix(ax)
        T = np.eye(4)
        T[:3, 3] = rng.uniform(-step, step, size=3)
        prev[i] = (T @ M @ R).T.reshape(16).astype(np.float32)
    callback = (rng.random(n) < callback_share).astype(np.uint8)
    return prev, callback


# ------------------------------------------------------------------ batch sweep
@dataclass
class BatchSweep:
    meshes: list
    qa: np.ndarray  # (Q,) mesh ids
    qb: np.ndarray
    mats_a: np.ndarray
    mats_b: np.ndarray


def batch_sweep(n_queries: int = 10000, pool: int = 48, seed: int = SEED_BASE + 5, tri_lo: int = 256,
                tri_hi: int = 65536) -> BatchSweep:
    rng = np.random.Generator(np.random.PCG64(seed))
    meshes = []
    for k in range(pool):
        T = int(round(math.exp(rng.uniform(math.log(tri_lo), math.log(tri_hi)))))
        meshes.append(uv_sphere(T, 1.0, 0.01, rng) if k % 2 == 0 else hull_blob(T, 1.0, rng))
    qa = rng.integers(0, pool, n_queries).astype(np.uint32)
    qb = rng.integers(0, pool, n_queries).astype(np.uint32)
    # root boxes of radius ~1 overlap when |t| < ~2: a ball of radius 2.52
    # puts about half the translations inside (2/2.52)^3 ~ 0.5.
    ma = np.stack([pose(random_rotation(rng), np.zeros(3)) for _ in range(n_queries)])
    mb = np.stack([pose(random_rotation(rng), ball_point(rng, 2.52)) for _ in range(n_queries)])
    return BatchSweep(meshes, qa, qb, ma, mb)


# ---------------------------------------------------------------- deforming --
# Skinned, morphed tubes against a static heightfield (the deforming and
# differentiable workloads). Choices of the builder, recorded here: each mesh
# is an open tube along +y, `rings` x `around` quads (two triangles each),
# radius 0.12 m, length 2 m, skinned to a chain of `n_bones` bones of equal
# length along the tube; a vertex's four joints are the bones nearest to its
# height, with Dirichlet(1) weights; 8 morph targets of N(0, 0.02) offsets;
# per mesh, bone rotations as axis-angle vectors N(0, 0.3 rad) per component
# and morph weights U[0, 1]. The heightfield is a `grid` x `grid` vertex grid
# over [0, 20] m x [0, 20] m with fBm heights of amplitude 0.5 m.


def axis_angle_matrix(aa: np.ndarray) -> np.ndarray:
    """3x3 rotation of an axis-angle vector (Rodrigues), float64."""
    th = float(np.linalg.norm(aa))
    if th < 1e-12:
        return np.eye(3)
    k = aa / th
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + math.sin(th) * K + (1 - math.cos(th)) * (K @ K)


def translate(t) -> np.ndarray:
    M = np.eye(4)
    M[:3, 3] = t
    return M


def chain_matrices(aa: np.ndarray, bone_len: float) -> np.ndarray:
    """World matrices (n_bones, 4, 4) of a bone chain along +y: bone 0 at the
    origin rotated by aa[0]; bone j = bone j-1 * T(0, bone_len, 0) * R(aa[j])."""
    out = np.zeros((len(aa), 4, 4))
    G = np.eye(4)
    for j, a in enumerate(aa):
        R = np.eye(4)
        R[:3, :3] = axis_angle_matrix(a)
        G = (G @ translate([0, bone_len, 0]) @ R) if j else R
        out[j] = G
    return out


def col_major(M: np.ndarray) -> np.ndarray:
    """(..., 4, 4) row-major math -> (..., 16) column-major float32."""
    return np.ascontiguousarray(np.swapaxes(M, -1, -2).reshape(M.shape[:-2] + (16,)), np.float32)


def tube(rings: int, around: int, radius: float, length: float) -> Mesh:
    ys = np.linspace(0.0, length, rings + 1)
    ang = np.linspace(0.0, 2 * math.pi, around, endpoint=False)
    pts = np.stack([np.stack([radius * np.cos(ang), np.full(around, y), radius * np.sin(ang)], 1) for y in ys])
    pts = pts.reshape(-1, 3).astype(np.float32)
    idx = []
    for r in range(rings):
        for a in range(around):
            i0, i1 = r * around + a, r * around + (a + 1) % around
            j0, j1 = i0 + around, i1 + around
            idx += [i0, j0, i1, i1, j0, j1]
    idx = np.array(idx, np.uint32)
    return Mesh(pts, vertex_normals(pts, idx), idx)


def fbm_heightfield(grid: int, size: float, amplitude: float, rng: np.random.Generator) -> Mesh:
    from scipy.ndimage import zoom

    h = np.zeros((grid, grid))
    total = 0.0
    for o in range(5):
        res = 4 * 2 ** o
        noise = rng.uniform(-1, 1, size=(res + 1, res + 1))
        up = zoom(noise, grid / (res + 1), order=3)[:grid, :grid]
        h += up * 0.5 ** o
        total += 0.5 ** o
    h *= amplitude / total
    xs = np.linspace(0.0, size, grid)
    X, Z = np.meshgrid(xs, xs, indexing="ij")
    pts = np.stack([X, h, Z], -1).reshape(-1, 3).astype(np.float32)
    idx = []
    for i in range(grid - 1):
        for j in range(grid - 1):
            a, b, c, d = i * grid + j, i * grid + j + 1, (i + 1) * grid + j, (i + 1) * grid + j + 1
            idx += [a, b, c, b, d, c]
    idx = np.array(idx, np.uint32)
    return Mesh(pts, vertex_normals(pts, idx), idx), h


@dataclass
class DeformingScene:
    mesh: Mesh                  # rest tube (shared topology)
    vertices: np.ndarray        # (n_meshes, V, 1 + targets, 4): base (w = 1) then target offsets (w = 0)
    morph_weights: np.ndarray   # (n_meshes, targets)
    joints: np.ndarray          # (V, 1, 4) uint16
    weights: np.ndarray         # (V, 1, 4) float32
    axis_angles: np.ndarray     # (n_meshes, n_bones, 3)
    joint_matrices: np.ndarray  # (n_meshes, n_bones, 16) posed chain
    inverse_bind: np.ndarray    # (n_bones, 16) inverse rest chain
    models: np.ndarray          # (n_meshes, 16) tube placement in the world
    field: Mesh                 # heightfield (identity placement)
    bone_len: float


def deforming(n_meshes: int = 64, seed: int = SEED_BASE + 3, rings: int = 100, around: int = 60, n_bones: int = 50,
              n_targets: int = 8, grid: int = 316) -> DeformingScene:
    rng = np.random.Generator(np.random.PCG64(seed))
    length = 2.0
    mesh = tube(rings, around, 0.12, length)
    V = len(mesh.points)
    bone_len = length / n_bones
    # four nearest bones by height, Dirichlet(1) weights
    centre = (np.arange(n_bones) + 0.5) * bone_len
    near = np.argsort(np.abs(mesh.points[:, 1:2] - centre[None, :]), axis=1)[:, :4]
    joints = near.astype(np.uint16).reshape(V, 1, 4)
    weights = rng.dirichlet(np.ones(4), size=V).astype(np.float32).reshape(V, 1, 4)
    rest = np.stack([translate([0, j * bone_len, 0]) for j in range(n_bones)])
    inverse_bind = col_major(np.linalg.inv(rest))
    verts = np.zeros((n_meshes, V, 1 + n_targets, 4), np.float32)
    verts[:, :, 0, :3] = mesh.points
    verts[:, :, 0, 3] = 1.0
    verts[:, :, 1:, :3] = rng.normal(0.0, 0.02, size=(n_meshes, V, n_targets, 3))
    morph_w = rng.uniform(0.0, 1.0, size=(n_meshes, n_targets)).astype(np.float32)
    aa = rng.normal(0.0, 0.3, size=(n_meshes, n_bones, 3))
    jm = np.stack([col_major(chain_matrices(aa[m], bone_len)) for m in range(n_meshes)])
    field, h = fbm_heightfield(grid, 20.0, 0.5, rng)
    models = []
    for m in range(n_meshes):
        gx, gz = rng.uniform(2.0, 18.0, size=2)
        gi = min(grid - 1, int(round(gx / 20.0 * (grid - 1))))
        gj = min(grid - 1, int(round(gz / 20.0 * (grid - 1))))
        # the tube's root at the ground, its axis tilted into the ground by a random angle
        R = axis_angle_matrix(np.array([0.0, rng.uniform(0, 2 * math.pi), 0.0])) @ \
            axis_angle_matrix(np.array([0.0, 0.0, math.pi / 2 + rng.uniform(-0.4, 0.4)]))
        models.append(pose(R, [gx, h[gi, gj] + 0.05, gz]))
    return DeformingScene(mesh, verts, morph_w, joints, weights, aa, jm, inverse_bind, np.stack(models), field,
                          bone_len)


def chain_skeleton(sc: DeformingScene) -> tuple[np.ndarray, np.ndarray]:
    """(parent, offsets) of the tubes' bone chain in the axis-angle posing
    form G_j = G_parent(j) * T(offset_j) * R(a_j): bone 0 at the origin, bone j
    one bone length up +y from bone j - 1 (chain_matrices)."""
    B = sc.axis_angles.shape[1]
    parent = np.arange(-1, B - 1, dtype=np.int32)
    offsets = np.zeros((B, 3), np.float32)
    offsets[1:, 1] = sc.bone_len
    return parent, offsets
