"""Generates the golden fixtures in tests/golden/ from the reference's own code.

The reference ships no tests or golden vectors for its collision path, so the
fixtures are outputs of the reference sources themselves (inMyRoom_vulkan/src/
Geometry/*.cpp, src/CollisionDetection/*.cpp, eig3/eig3.cpp) compiled in place
against the glm shim by ``make -C oracle ref`` (needs the reference checkout):

    python tests/golden/make_golden.py

Inputs are seeded, so the fixtures are reproducible. The CPU tests check the
oracle restatement against these files; nothing reads the reference at test time.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import frame  # noqa: E402
from inmyroom_vulkan_gb300 import scenes  # noqa: E402


def tri_cases(rng):
    """Hand-built Moller cases (crossing, touching, edge-on-edge, coplanar,
    parallel, near-epsilon) followed by random near-contact pairs."""
    A, B = [], []
    base = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    # crossing
    A.append(base); B.append(np.array([[0.2, 0.2, -0.5], [0.3, 0.2, 0.5], [0.2, 0.4, 0.5]], np.float32))
    # vertex of B touching A's interior from above
    A.append(base); B.append(np.array([[0.25, 0.25, 0.0], [0.3, 0.3, 1.0], [0.1, 0.4, 1.0]], np.float32))
    # edge on edge (B's edge crosses A's hypotenuse in A's plane)
    A.append(base); B.append(np.array([[0.5, 0.5, -0.5], [0.5, 0.5, 0.5], [1.0, 1.0, 0.0]], np.float32))
    # coplanar overlap
    A.append(base); B.append(np.array([[0.1, 0.1, 0.0], [0.8, 0.1, 0.0], [0.1, 0.8, 0.0]], np.float32))
    # coplanar disjoint
    A.append(base); B.append(np.array([[2.0, 2.0, 0.0], [3.0, 2.0, 0.0], [2.0, 3.0, 0.0]], np.float32))
    # separated parallel
    A.append(base); B.append(base + np.float32([0, 0, 0.25]))
    # identical
    A.append(base); B.append(base.copy())
    # shared edge, hinge
    A.append(base); B.append(np.array([[0, 0, 0], [1, 0, 0], [0.5, -0.5, 0.7]], np.float32))
    # degenerate (zero-area) B
    A.append(base); B.append(np.array([[0.2, 0.2, -1], [0.2, 0.2, 0], [0.2, 0.2, 1]], np.float32))
    # B's vertices at distances near the 1e-6 threshold of A's plane (|N1| = 1)
    for d in [1e-6, 0.99999e-6, 1.00001e-6, 9.99999997e-07, 1.0000001e-06, -1e-6, 5e-7, 2e-6]:
        A.append(base)
        B.append(np.array([[0.2, 0.2, d], [0.6, 0.2, -0.5], [0.2, 0.6, 0.5]], np.float32))
        A.append(base)
        B.append(np.array([[0.2, 0.2, d], [0.6, 0.2, d], [0.2, 0.6, 0.5]], np.float32))
    # random near-contact pairs at several scales
    for scale in (1.0, 0.01, 100.0):
        for _ in range(300):
            a = rng.normal(size=(3, 3)) * scale
            b = a.mean(0) + rng.normal(size=(3, 3)) * scale * rng.uniform(0.2, 1.5)
            A.append(a.astype(np.float32)); B.append(b.astype(np.float32))
    # snapped to a coarse grid: exact zeros and shared coordinates
    for _ in range(300):
        a = np.round(rng.uniform(-2, 2, size=(3, 3)) * 4) / 4
        b = np.round(rng.uniform(-2, 2, size=(3, 3)) * 4) / 4
        A.append(a.astype(np.float32)); B.append(b.astype(np.float32))
    return np.array(A, np.float32).reshape(-1, 9), np.array(B, np.float32).reshape(-1, 9)


def near_epsilon_cases(rng):
    """Pairs whose plane distances lie near the Moller test's 1e-6 threshold
    (or near 0) while the FP32 arithmetic that computes them carries errors of
    that size: tilted triangles far from the origin (coordinates up to 1e3,
    so the two dot products of d = n . p - n . a0 cancel), one corner of the
    other triangle placed at a distance within a few 1e-6 of the plane, the
    other two on both sides of it. Half the pairs have the roles swapped."""
    A, B = [], []
    for _ in range(400):
        off = rng.uniform(-1, 1, 3) * 10.0 ** rng.uniform(0, 3)
        edge = 10.0 ** rng.uniform(-2, 0.5)
        R = scenes.random_rotation(rng)
        a = off + (np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]]) @ R.T) * edge
        a = a.astype(np.float32).astype(np.float64)
        e1, e2 = a[1] - a[0], a[2] - a[0]
        n = np.cross(e1, e2)
        target = rng.uniform(-3e-6, 3e-6) if rng.random() < 0.8 else rng.choice([-1e-6, 0.0, 1e-6])
        inplane = a[0] + e1 * rng.uniform(0.1, 0.4) + e2 * rng.uniform(0.1, 0.4)
        p0 = inplane + n * (target / (n @ n))
        u = R[:, 2] * edge * rng.uniform(0.3, 1.0)
        v = (R[:, 0] - R[:, 1]) * edge * rng.uniform(0.2, 0.8)
        b = np.stack([p0, p0 + u + v, p0 - u + v]).astype(np.float32)
        if rng.random() < 0.5:
            A.append(a.astype(np.float32)); B.append(b)
        else:
            A.append(b); B.append(a.astype(np.float32))
    return np.array(A, np.float32).reshape(-1, 9), np.array(B, np.float32).reshape(-1, 9)


def near_epsilon_fixture(R, rng):
    """The reference's verdicts on near_epsilon_cases (the FP32 verdict that
    the GPU library keeps by default; the FP64 recheck is checked against
    exact arithmetic by the tests)."""
    a, b = near_epsilon_cases(rng)
    n = len(a)
    hit = np.zeros(n, np.int32); cop = np.zeros(n, np.int32)
    src = np.zeros((n, 3), np.float32); tgt = np.zeros((n, 3), np.float32)
    for i in range(n):
        h, c, s, t = R.tri_tri(a[i], b[i])
        hit[i], cop[i] = h, c
        if h and not c:
            src[i], tgt[i] = s, t
    np.savez_compressed(os.path.join(HERE, "tritri_near.npz"), a=a, b=b, hit=hit, coplanar=cop, src=src, tgt=tgt)


def box_cases(rng):
    A, B = [], []
    for _ in range(600):
        def rnd():
            R = scenes.random_rotation(rng)
            h = rng.uniform(0.05, 1.5, 3)
            c = rng.normal(size=3) * 1.5
            return np.concatenate([c, R[:, 0] * h[0], R[:, 1] * h[1], R[:, 2] * h[2]]).astype(np.float32)
        A.append(rnd()); B.append(rnd())
    # separate along each of the 15 axes in turn: axis-aligned unit boxes
    # shifted along a face normal or an edge cross direction
    for k in range(15):
        a = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1], np.float32)
        b = a.copy()
        R = scenes.random_rotation(np.random.Generator(np.random.PCG64(k)))
        b[3:6], b[6:9], b[9:12] = R[:, 0] * 0.5, R[:, 1] * 0.5, R[:, 2] * 0.5
        b[:3] = (2.6 if k < 6 else 2.2) * np.eye(3)[k % 3]
        A.append(a); B.append(b)
    # degenerate: parallel edges (zero cross products), flat boxes
    a = np.array([0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1], np.float32)
    A.append(a); B.append(a + np.float32([0.5, 0.5, 0.5] + [0] * 9))
    A.append(a); B.append(np.array([3, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1e-7], np.float32))
    A.append(np.array([0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 1], np.float32)); B.append(a.copy())
    return np.array(A), np.array(B)


def shoot_fixture(R):
    """ShootUncollideRays::ExecuteShootUncollideRays on the rigid_small poses
    with the reference's own rays of each pose (in its order)."""
    g = np.load(os.path.join(HERE, "rigid_small.npz"))

    def tree(tag):
        return R.tree_build(g[f"points_{tag}"], g[f"indices_{tag}"], g[f"normals_{tag}"])

    ta, tb = tree("a"), tree("b")
    deltas = []
    for k in range(len(g["mats_a"])):
        ra = g["rays_a"][g["rays_a"][:, 0] == k, 1:]
        rb = g["rays_b"][g["rays_b"][:, 0] == k, 1:]
        deltas.append(R.shoot_rays(ta, tb, g["mats_a"][k], g["mats_b"][k], ra, rb))
    np.savez_compressed(os.path.join(HERE, "shoot_small.npz"), deltas=np.array(deltas, np.float32))


def sap_fixture(R):
    """SweepAndPrune::ExecuteSweepAndPrune on the 256-entity scene (seed 1002)
    with a seeded 70% of the entities calling back: the pairs as the
    reference orients them."""
    sc = scenes.scene()
    trees = [R.tree_build(m.points, m.indices, m.normals) for m in sc.meshes]
    cb = (np.random.Generator(np.random.PCG64(7)).random(len(trees)) < 0.7).astype(np.uint8)
    pairs = R.sweep_and_prune(trees, sc.mats, cb)
    pairs = pairs[np.lexsort((pairs[:, 1], pairs[:, 0]))]
    np.savez_compressed(os.path.join(HERE, "sap_scene.npz"), callback=cb, pairs=pairs)


def frame_fixture(R):
    """One frame of CollisionDetection::ExecuteCollisionDetection on the
    256-entity scene (seed 1002) with scenes.frame_motion's previous frame and
    callback flags: the (first, second) pairs with rays and their deltas, by
    the reference's own broad phase, mid phase, rays and shooting."""
    sc = scenes.scene()
    prev, cb = scenes.frame_motion(sc)
    trees = [R.tree_build(m.points, m.indices, m.normals) for m in sc.meshes]
    pairs, deltas = frame.as_arrays(frame.collision_frame(R, trees, sc.mats, prev, cb))
    np.savez_compressed(os.path.join(HERE, "frame_scene.npz"), previous=prev, callback=cb, pairs=pairs,
                        deltas=deltas)


def main():
    R = oracle.ref()
    if R is None:
        raise SystemExit("the reference checkout is needed to make the fixtures")
    rng = np.random.Generator(np.random.PCG64(4242))

    # --- Moller
    a, b = tri_cases(rng)
    n = len(a)
    hit = np.zeros(n, np.int32); cop = np.zeros(n, np.int32)
    src = np.zeros((n, 3), np.float32); tgt = np.zeros((n, 3), np.float32)
    for i in range(n):
        h, c, s, t = R.tri_tri(a[i], b[i])
        hit[i], cop[i] = h, c
        if h and not c:
            src[i], tgt[i] = s, t
    mats = np.stack([scenes.pose(scenes.random_rotation(rng), rng.normal(size=3)) for _ in range(64)])
    xt = np.stack([R.transform_tri(mats[i % 64], a[i]) for i in range(n)])
    np.savez_compressed(os.path.join(HERE, "tritri.npz"), a=a, b=b, hit=hit, coplanar=cop, src=src, tgt=tgt,
                        mats=mats, xformed=xt)

    # --- SAT, surface, box transform, relative matrices
    ba, bb = box_cases(rng)
    sat = np.array([R.sat(x, y) for x, y in zip(ba, bb)], np.int32)
    surf = np.array([R.surface(x) for x in ba], np.float32)
    bx = np.stack([R.transform_box(mats[i % 64], ba[i]) for i in range(len(ba))])
    rel = np.stack([R.relative_matrix(mats[i], mats[(i * 7 + 3) % 64]) for i in range(64)])
    np.savez_compressed(os.path.join(HERE, "boxes.npz"), a=ba, b=bb, sat=sat, surface=surf, mats=mats,
                        xformed=bx, relative=rel)

    # --- eig3 and OBB fits
    As = []
    for _ in range(200):
        M = rng.normal(size=(3, 3)); As.append(M @ M.T)
    As += [np.eye(3), np.diag([1.0, 1.0, 2.0]), np.zeros((3, 3)), np.diag([3.0, 2.0, 1.0]),
           np.array([[1, 1e-12, 0], [1e-12, 1, 0], [0, 0, 1]])]
    As = np.array(As).reshape(-1, 9)
    V = np.zeros_like(As); d = np.zeros((len(As), 3))
    for i, A_ in enumerate(As):
        v, dd = R.eig3(A_); V[i] = v.reshape(9); d[i] = dd
    pts_sets = [rng.normal(size=(k, 3)).astype(np.float32) * rng.uniform(0.1, 3, 3).astype(np.float32)
                for k in (2, 3, 4, 5, 7, 12, 33, 100)]
    pts_sets += [np.zeros((0, 3), np.float32), np.ones((1, 3), np.float32), np.ones((5, 3), np.float32),
                 np.array([[0, 0, 0], [1, 0, 0]], np.float32), np.array([[0, 0, 0], [1, 1, 0], [2, 2, 0]], np.float32)]
    lens = np.array([len(p) for p in pts_sets], np.int64)
    allp = np.concatenate([p.reshape(-1, 3) for p in pts_sets]).astype(np.float32)
    boxes = np.stack([R.obb_from_points(p) for p in pts_sets])
    np.savez_compressed(os.path.join(HERE, "fits.npz"), A=As, V=V, d=d, pts=allp, lens=lens, boxes=boxes)

    # --- whole mid + narrow phase on a small rigid pair
    rp = scenes.rigid_pair(n_poses=24, seed=1001, subdiv=3)
    ta = R.tree_build(rp.mesh_a.points, rp.mesh_a.indices, rp.mesh_a.normals)
    tb = R.tree_build(rp.mesh_b.points, rp.mesh_b.indices, rp.mesh_b.normals)
    fa, fb = ta.export(), tb.export()
    out = dict(points_a=rp.mesh_a.points, normals_a=rp.mesh_a.normals, indices_a=rp.mesh_a.indices,
               points_b=rp.mesh_b.points, normals_b=rp.mesh_b.normals, indices_b=rp.mesh_b.indices,
               mats_a=rp.mats_a, mats_b=rp.mats_b)
    for tag, f in (("a", fa), ("b", fb)):
        for k, v in f.arrays().items():
            out[f"tree_{tag}_{k}"] = v
    lps, pairs, segs, rays_a, rays_b, avgs, tests = [], [], [], [], [], [], []
    for k in range(len(rp.mats_a)):
        m = R.mid_phase(ta, tb, rp.mats_a[k], rp.mats_b[k])
        lp = m.leaf_pairs()
        lps.append(np.concatenate([np.full((len(lp), 1), k, np.uint32), lp], 1))
        p, s, t, _ = m.narrow()
        pairs.append(np.concatenate([np.full((len(p), 1), k, np.uint32), p], 1)); segs.append(s); tests.append(t)
        ra, rb, avg = m.rays()
        rays_a.append(np.concatenate([np.full((len(ra), 1), k, np.float32), ra], 1))
        rays_b.append(np.concatenate([np.full((len(rb), 1), k, np.float32), rb], 1))
        avgs.append(avg)
    out.update(leaf_pairs=np.concatenate(lps), pairs=np.concatenate(pairs), segs=np.concatenate(segs),
               rays_a=np.concatenate(rays_a), rays_b=np.concatenate(rays_b), avgs=np.array(avgs),
               tests=np.array(tests, np.uint64))
    np.savez_compressed(os.path.join(HERE, "rigid_small.npz"), **out)
    shoot_fixture(R)
    sap_fixture(R)
    frame_fixture(R)
    near_epsilon_fixture(R, np.random.Generator(np.random.PCG64(4243)))
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
