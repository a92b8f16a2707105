"""The FP64 recheck of the Moller test's plane distances (the GPU library's
CG_RECHECK / CG_ROBUST), pinned on the CPU.

* The filter bound: every plane distance the test evaluates is recomputed
  here in FP32 with the reference's operation order (Triangle.cpp:866-915)
  and exactly, in rational arithmetic, as the orientation determinant
  det[a1 - a0, a2 - a0, p - a0] of the float corners. Outside the band
  (|d| within B = 32 u C |e1|_1 |e2|_1 of 0 or of 1e-6) the FP32 class (zero
  below 1e-6, else the sign) is the exact class, for every distance of the
  golden and near-epsilon pairs.
* The oracle's recheck: its counts equal the number of evaluated distances
  inside the band, its FP64 class is the exact class, and its default verdict
  is the reference's on the near-epsilon golden pairs (where the reference's
  result is defined).
"""
import os
from fractions import Fraction

import numpy as np

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
f32 = np.float32
U32 = f32(32.0) * f32(2.0 ** -24)
EPS = Fraction(1, 10 ** 6)


def sub(a, b):
    return np.array([a[0] - b[0], a[1] - b[1], a[2] - b[2]], f32)


def cross(a, b):
    return np.array([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]], f32)


def dot(a, b):
    return f32(f32(a[0] * b[0] + a[1] * b[1]) + a[2] * b[2])


def norm1(a):
    return f32(f32(abs(a[0]) + abs(a[1])) + abs(a[2]))


def plane(a, p):
    """FP32 distances of p[0..2] to the plane of a (reference order), the
    filter bound and the exact determinants."""
    e1, e2 = sub(a[1], a[0]), sub(a[2], a[0])
    n = cross(e1, e2)
    d0 = -dot(n, a[0])
    ds = [f32(dot(n, q) + d0) for q in p]
    C = max(float(np.max(np.abs(a[0]))), *(float(np.max(np.abs(q))) for q in p))
    B = f32(f32(f32(U32 * f32(C)) * norm1(e1)) * norm1(e2))
    A = [[Fraction(float(x)) for x in v] for v in a]
    E1 = [A[1][k] - A[0][k] for k in range(3)]
    E2 = [A[2][k] - A[0][k] for k in range(3)]
    N = [E1[1] * E2[2] - E1[2] * E2[1], E1[2] * E2[0] - E1[0] * E2[2], E1[0] * E2[1] - E1[1] * E2[0]]
    ex = []
    for q in p:
        Q = [Fraction(float(x)) - A[0][k] for k, x in enumerate(q)]
        ex.append(N[0] * Q[0] + N[1] * Q[1] + N[2] * Q[2])
    return ds, B, ex


def class32(d):
    return 0 if abs(float(d)) < 1e-6 else (1 if d > 0 else -1)


def class_exact(x):
    return 0 if abs(x) < EPS else (1 if x > 0 else -1)


def uncertain(d, B):
    a = f32(abs(d))
    return a < B or f32(abs(f32(a - f32(1e-6)))) < B


def evaluated_planes(a, b):
    """The planes the test evaluates (the second only when the first does
    not separate), as (distances, bound, exact) tuples."""
    du, B1, x1 = plane(a, b)
    out = [(du, B1, x1)]
    c = [0.0 if class32(d) == 0 else float(d) for d in du]
    if not (c[0] * c[1] > 0 and c[0] * c[2] > 0):
        out.append(plane(b, a))
    return out


def cases():
    g = np.load(os.path.join(GOLD, "tritri.npz"))
    h = np.load(os.path.join(GOLD, "tritri_near.npz"))
    a = np.concatenate([g["a"], h["a"]]).reshape(-1, 3, 3)
    b = np.concatenate([g["b"], h["b"]]).reshape(-1, 3, 3)
    return a, b


def test_filter_bound_holds_and_counts_match(port):
    a, b = cases()
    n_unc = n_dis = 0
    for i in range(len(a)):
        planes = evaluated_planes(a[i], b[i])
        unc = 0
        dis = False
        for ds, B, ex in planes:
            for d, x in zip(ds, ex):
                if uncertain(d, B):
                    unc += 1
                    dis |= class32(d) != class_exact(x)
                else:
                    assert class32(d) == class_exact(x), (i, float(d), float(x), float(B))
        hit, cop, fr, checked, disagreed, _, _ = port.tri_tri_recheck(a[i].reshape(9), b[i].reshape(9), 1)
        assert checked == unc, (i, checked, unc)
        assert disagreed == int(dis), i
        n_unc += unc
        n_dis += int(dis)
    # the near-epsilon pairs exercise the band, and in some the FP32 class is wrong
    assert n_unc > 200 and n_dis > 20, (n_unc, n_dis)


def test_near_epsilon_golden_verdicts(port):
    """Default and counted modes keep the reference's verdicts (where it is
    defined); the robust mode changes some of them."""
    g = np.load(os.path.join(GOLD, "tritri_near.npz"))
    changed = 0
    for i in range(len(g["a"])):
        h0, c0, f0, _, _, s0, t0 = port.tri_tri_recheck(g["a"][i], g["b"][i], 0)
        h1, c1, f1, _, _, s1, t1 = port.tri_tri_recheck(g["a"][i], g["b"][i], 1)
        h2, c2, f2, _, _, _, _ = port.tri_tri_recheck(g["a"][i], g["b"][i], 2)
        assert (h0, c0, f0) == (h1, c1, f1) and np.array_equal(s0, s1) and np.array_equal(t0, t1)
        if not f0:
            assert (h0, c0) == (int(g["hit"][i]), int(g["coplanar"][i])), i
            if h0 and not c0:
                assert np.array_equal(s0.view(np.uint32), g["src"][i].view(np.uint32))
                assert np.array_equal(t0.view(np.uint32), g["tgt"][i].view(np.uint32))
        changed += int((h2 and not c2) != (h0 and not c0))
    assert changed > 0
