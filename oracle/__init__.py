"""Oracle test infrastructure for the collision path. NOT part of the product.

Two CPU implementations behind one Python interface:

* ``port`` — ``oracle/port/imr_port.cpp``, a C++ restatement of the reference
  engine's collision path (OBB fit, OBB-tree build, SAT traversal, Moller
  narrow phase, contacts and uncollide rays), bit-identical in operation order.
  It builds anywhere (``make -C oracle port``).
* ``ref`` — the reference's own sources (inMyRoom_vulkan/src/Geometry/*.cpp,
  src/CollisionDetection/*.cpp, eig3/eig3.cpp) compiled in place against the glm
  shim by ``make -C oracle ref`` into ``oracle/_ref/``. Only available where the
  reference checkout is.

Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
may use this package, and only as the checker / baseline.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference checkout: $INMYROOM_REFERENCE, else its usual place in this
# build's container. Absent on machines without it (the compiled reference and
# the tests that read its sources are then skipped).
REF_ROOT_DEFAULT = os.environ.get("INMYROOM_REFERENCE", "/root/reference")

_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")


def build_port() -> None:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)


def build_ref(ref_root: str = REF_ROOT_DEFAULT) -> bool:
    """Compiles the reference's own sources, if present. Returns availability."""
    if not os.path.isdir(os.path.join(ref_root, "inMyRoom_vulkan", "src", "Geometry")):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref_root}"], check=True)
    return True


def _declare(lib: C.CDLL, prefix: str) -> None:
    vp = C.c_void_p
    sz = C.c_size_t
    f = lambda name: getattr(lib, prefix + name)  # noqa: E731
    f("tree_build").restype = vp
    f("tree_build").argtypes = [_f32p, sz, vp, _u32p, sz]
    f("tree_free").argtypes = [vp]
    f("tree_sizes").argtypes = [vp, C.POINTER(sz), C.POINTER(sz)]
    f("tree_export").argtypes = [vp, _f32p, _f32p, _u32p, _u32p, _f32p, _f32p, _u32p]
    f("relative_matrix").argtypes = [_f32p, _f32p, _f32p]
    f("mid_phase").restype = vp
    f("mid_phase").argtypes = [vp, vp, _f32p, _f32p]
    f("mid_free").argtypes = [vp]
    f("mid_count").restype = sz
    f("mid_count").argtypes = [vp]
    f("mid_get").argtypes = [vp, _u32p]
    f("tri_tri").restype = C.c_int
    f("tri_tri").argtypes = [_f32p, _f32p, C.POINTER(C.c_int), _f32p, _f32p]
    f("transform_tri").argtypes = [_f32p, _f32p, _f32p]
    f("sat").restype = C.c_int
    f("sat").argtypes = [_f32p, _f32p]
    f("surface").restype = C.c_float
    f("surface").argtypes = [_f32p]
    f("transform_box").argtypes = [_f32p, _f32p, _f32p]
    f("obb_from_points").argtypes = [_f32p, sz, _f32p]
    f("eig3").argtypes = [_f64p, _f64p, _f64p]
    f("rays").argtypes = [vp, _f32p, _f32p, sz, sz, C.POINTER(sz), _f32p]
    f("shoot_rays").argtypes = [vp, vp, _f32p, _f32p, _f32p, sz, _f32p, sz, vp, _f32p]
    f("sweep_and_prune").restype = sz
    f("sweep_and_prune").argtypes = [vp, _f32p, vp, sz, vp, vp, sz]
    if prefix == "ref_":
        f("narrow").restype = sz
        f("narrow").argtypes = [vp, _u32p, _f32p, sz, C.POINTER(C.c_uint64)]
        f("collide_batch").restype = C.c_uint64
        f("collide_batch").argtypes = [vp, vp, _f32p, _f32p, sz, C.c_int, C.POINTER(C.c_uint64), _u64p]
    else:
        f("narrow").restype = sz
        f("narrow").argtypes = [vp, _u32p, _f32p, sz, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        f("tree_import").restype = vp
        f("tree_import").argtypes = [_f32p, sz, _f32p, _u32p, _u32p, sz, _f32p, vp, vp]
        f("tri_tri_ex").restype = C.c_int
        f("tri_tri_ex").argtypes = [_f32p, _f32p, C.POINTER(C.c_int), C.POINTER(C.c_int), _f32p, _f32p]
        f("contacts").restype = sz
        f("contacts").argtypes = [vp, C.c_int, _u32p, _u32p, _f32p, sz]
        f("contacts_iter").restype = sz
        f("contacts_iter").argtypes = [vp, C.c_int, _u32p, _u32p, _f32p, sz]
        f("collide_batch").restype = C.c_uint64
        f("collide_batch").argtypes = [vp, vp, _f32p, _f32p, sz, C.c_int,
                                       C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), _u64p]
        f("deform").argtypes = [sz, sz, sz, sz, _f32p, _f32p, vp, _f32p, _f32p, _f32p, _f32p]
        f("tree_refit").argtypes = [sz, _u32p, _u32p, sz, _u32p, _f32p, sz, _f32p, _f32p, _f32p]
        f("collide_pairs").restype = sz
        f("collide_pairs").argtypes = [vp, vp, _f32p, _f32p, sz, _u32p, _f32p, sz,
                                       C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        f("collide_pairs_mode").restype = sz
        f("collide_pairs_mode").argtypes = [vp, vp, _f32p, _f32p, sz, _u32p, _f32p, sz,
                                            C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.c_int,
                                            np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")]
        f("tri_tri_recheck").restype = C.c_int
        f("tri_tri_recheck").argtypes = [_f32p, _f32p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), _u32p,
                                         _f32p, _f32p]


class FlatTree:
    """A flattened OBB tree in the reference's node layout (OBBtree.h:61-75)."""

    def __init__(self, root, node_obbs, node_ref, node_cnt, tri_pos, tri_nrm, tri_idx):
        self.root = np.ascontiguousarray(root, np.float32).reshape(12)
        self.node_obbs = np.ascontiguousarray(node_obbs, np.float32).reshape(-1, 2, 12)
        self.node_ref = np.ascontiguousarray(node_ref, np.uint32).reshape(-1, 2)
        self.node_cnt = np.ascontiguousarray(node_cnt, np.uint32).reshape(-1, 2)
        self.tri_pos = np.ascontiguousarray(tri_pos, np.float32).reshape(-1, 9)
        self.tri_nrm = np.ascontiguousarray(tri_nrm, np.float32).reshape(-1, 9)
        self.tri_idx = np.ascontiguousarray(tri_idx, np.uint32).reshape(-1, 3)

    @property
    def n_nodes(self) -> int:
        return self.node_obbs.shape[0]

    @property
    def n_tris(self) -> int:
        return self.tri_pos.shape[0]

    def arrays(self) -> dict:
        return dict(root=self.root, node_obbs=self.node_obbs, node_ref=self.node_ref,
                    node_cnt=self.node_cnt, tri_pos=self.tri_pos, tri_nrm=self.tri_nrm,
                    tri_idx=self.tri_idx)

    def equal(self, other: "FlatTree") -> bool:
        a, b = self.arrays(), other.arrays()
        return all(a[k].shape == b[k].shape and np.array_equal(a[k].view(np.uint32) if a[k].dtype == np.float32 else a[k],
                                                            b[k].view(np.uint32) if b[k].dtype == np.float32 else b[k])
                   for k in a)


class Tree:
    def __init__(self, impl: "Impl", handle: int):
        self.impl, self.h = impl, handle

    def __del__(self):
        try:
            if self.h:
                self.impl.fn("tree_free")(self.h)
                self.h = None
        except Exception:
            pass

    def sizes(self):
        if getattr(self, "_sizes", None) is None:
            n, t = C.c_size_t(), C.c_size_t()
            self.impl.fn("tree_sizes")(self.h, C.byref(n), C.byref(t))
            self._sizes = (n.value, t.value)
        return self._sizes

    def export(self) -> FlatTree:
        n, t = self.sizes()
        root = np.zeros(12, np.float32)
        obbs = np.zeros((max(n, 1), 2, 12), np.float32)
        ref = np.zeros((max(n, 1), 2), np.uint32)
        cnt = np.zeros((max(n, 1), 2), np.uint32)
        pos = np.zeros((max(t, 1), 9), np.float32)
        nrm = np.zeros((max(t, 1), 9), np.float32)
        idx = np.zeros((max(t, 1), 3), np.uint32)
        self.impl.fn("tree_export")(self.h, root, obbs, ref, cnt, pos, nrm, idx)
        return FlatTree(root, obbs[:n], ref[:n], cnt[:n], pos[:t], nrm[:t], idx[:t])


class Mid:
    """A mid + narrow phase result. It reads its trees when asked for
    contacts and rays, so it keeps them alive."""

    def __init__(self, impl: "Impl", handle: int, trees=()):
        self.impl, self.h = impl, handle
        self._trees = tuple(trees)

    def __del__(self):
        try:
            if self.h:
                self.impl.fn("mid_free")(self.h)
                self.h = None
        except Exception:
            pass

    def leaf_pairs(self) -> np.ndarray:
        n = self.impl.fn("mid_count")(self.h)
        out = np.zeros((max(n, 1), 4), np.uint32)
        self.impl.fn("mid_get")(self.h, out)
        return out[:n]

    def narrow(self):
        """Colliding pairs (n,2) [tree-order indices], segments (n,6), tests, fragile."""
        t = C.c_uint64()
        fr = C.c_uint64()
        dummy_p = np.zeros((1, 2), np.uint32)
        dummy_s = np.zeros((1, 6), np.float32)
        args = (C.byref(t),) if self.impl.prefix == "ref_" else (C.byref(t), C.byref(fr))
        n = self.impl.fn("narrow")(self.h, dummy_p, dummy_s, 0, *args)
        pairs = np.zeros((max(n, 1), 2), np.uint32)
        segs = np.zeros((max(n, 1), 6), np.float32)
        self.impl.fn("narrow")(self.h, pairs, segs, n, *args)
        return pairs[:n], segs[:n], t.value, fr.value

    def rays(self):
        counts = (C.c_size_t * 2)()
        avg = np.zeros(6, np.float32)
        z = np.zeros((1, 6), np.float32)
        self.impl.fn("rays")(self.h, z, z, 0, 0, counts, avg)
        na, nb = counts[0], counts[1]
        ra = np.zeros((max(na, 1), 6), np.float32)
        rb = np.zeros((max(nb, 1), 6), np.float32)
        self.impl.fn("rays")(self.h, ra, rb, na, nb, counts, avg)
        return ra[:na], rb[:nb], avg

    def contacts(self, side: int, iteration_order: bool = False):
        """(port only) per-triangle (index, mask, wsum xyz + weight), sorted by
        index, or in the per-triangle map's iteration order (the order its rays
        are made in)."""
        fn = self.impl.fn("contacts_iter" if iteration_order else "contacts")
        z32 = np.zeros(1, np.uint32)
        zf = np.zeros((1, 4), np.float32)
        n = fn(self.h, side, z32, z32, zf, 0)
        idx = np.zeros(max(n, 1), np.uint32)
        mask = np.zeros(max(n, 1), np.uint32)
        f = np.zeros((max(n, 1), 4), np.float32)
        fn(self.h, side, idx, mask, f, n)
        return idx[:n], mask[:n], f[:n]


def _f32(a, n=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a.reshape(-1) if n is None else a.reshape(n)


class Impl:
    def __init__(self, path: str, prefix: str):
        self.lib = C.CDLL(path)
        self.prefix = prefix
        self.path = path
        _declare(self.lib, prefix)

    def fn(self, name):
        return getattr(self.lib, self.prefix + name)

    # --- trees
    def tree_build(self, points, indices, normals=None) -> Tree:
        pts = _f32(points)
        idx = np.ascontiguousarray(indices, np.uint32).reshape(-1)
        nrm = None if normals is None else _f32(normals)
        h = self.fn("tree_build")(pts, pts.size // 3, None if nrm is None else nrm.ctypes.data, idx, idx.size)
        t = Tree(self, h)
        t._keep = nrm
        return t

    def tree_import(self, ft: FlatTree) -> Tree:
        assert self.prefix == "port_"
        h = self.fn("tree_import")(ft.root, ft.n_nodes, ft.node_obbs if ft.n_nodes else np.zeros(24, np.float32),
                                   ft.node_ref if ft.n_nodes else np.zeros(2, np.uint32),
                                   ft.node_cnt if ft.n_nodes else np.zeros(2, np.uint32),
                                   ft.n_tris, ft.tri_pos, ft.tri_nrm.ctypes.data, ft.tri_idx.ctypes.data)
        t = Tree(self, h)
        t._keep = ft
        return t

    # --- queries
    def relative_matrix(self, ma, mb) -> np.ndarray:
        out = np.zeros(16, np.float32)
        self.fn("relative_matrix")(_f32(ma, 16), _f32(mb, 16), out)
        return out

    def mid_phase(self, ta: Tree, tb: Tree, ma, mb) -> Mid:
        return Mid(self, self.fn("mid_phase")(ta.h, tb.h, _f32(ma, 16), _f32(mb, 16)), (ta, tb))

    # --- primitives
    def tri_tri(self, a, b):
        cop = C.c_int()
        s = np.zeros(3, np.float32)
        t = np.zeros(3, np.float32)
        hit = self.fn("tri_tri")(_f32(a, 9), _f32(b, 9), C.byref(cop), s, t)
        return hit, cop.value, s, t

    def deform(self, vertices, morph_weights, joints, weights, joint_matrices, inverse_bind):
        """(port) morph then linear-blend skinning: vertices (n, 1 + targets, 4),
        joints/weights (n, groups, 4), matrices (joints, 16) -> (n, 4)."""
        v = np.ascontiguousarray(vertices, np.float32)
        n, t1 = v.shape[0], v.shape[1]
        jn = np.ascontiguousarray(joints, np.uint16)
        w = np.ascontiguousarray(weights, np.float32)
        groups = jn.shape[1] if jn.ndim == 3 else 0
        jm = np.ascontiguousarray(joint_matrices, np.float32).reshape(-1, 16)
        ib = np.ascontiguousarray(inverse_bind, np.float32).reshape(-1, 16)
        out = np.zeros((n, 4), np.float32)
        self.fn("deform")(n, t1 - 1, groups, jm.shape[0], v.reshape(-1), _f32(morph_weights),
                          jn.ctypes.data, w.reshape(-1), jm.reshape(-1), ib.reshape(-1), out)
        return out

    def tree_refit(self, ft: "FlatTree", positions) -> "FlatTree":
        """(port) the flat tree refitted to positions (n, 4): new corner positions
        and every box fitted again to its subtree's corners in leaf order."""
        pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 4)
        n, t = ft.n_nodes, ft.n_tris
        root = np.zeros(12, np.float32)
        obbs = np.zeros((max(n, 1), 2, 12), np.float32)
        tri = np.zeros((max(t, 1), 9), np.float32)
        self.fn("tree_refit")(n, ft.node_ref.reshape(-1) if n else np.zeros(2, np.uint32),
                              ft.node_cnt.reshape(-1) if n else np.zeros(2, np.uint32), t,
                              ft.tri_idx.reshape(-1), pos.reshape(-1), pos.shape[0], root, obbs.reshape(-1),
                              tri.reshape(-1))
        return FlatTree(root, obbs[:n], ft.node_ref[:n], ft.node_cnt[:n], tri[:t], ft.tri_nrm[:t], ft.tri_idx[:t])

    def transform_tri(self, m, a):
        out = np.zeros(9, np.float32)
        self.fn("transform_tri")(_f32(m, 16), _f32(a, 9), out)
        return out

    def sat(self, a, b) -> int:
        return self.fn("sat")(_f32(a, 12), _f32(b, 12))

    def surface(self, a) -> float:
        return self.fn("surface")(_f32(a, 12))

    def transform_box(self, m, a):
        out = np.zeros(12, np.float32)
        self.fn("transform_box")(_f32(m, 16), _f32(a, 12), out)
        return out

    def obb_from_points(self, pts):
        p = _f32(pts)
        out = np.zeros(12, np.float32)
        self.fn("obb_from_points")(p, p.size // 3, out)
        return out

    def eig3(self, a):
        a = np.ascontiguousarray(a, np.float64).reshape(9)
        v = np.zeros(9, np.float64)
        d = np.zeros(3, np.float64)
        self.fn("eig3")(a, v, d)
        return v.reshape(3, 3), d

    def collide_batch(self, trees_a, trees_b, mats_a, mats_b, threads=1):
        """The whole per-pair path (mid phase, triangle tests, contacts, rays)
        of a batch on `threads` host threads, which take the queries largest
        first (by the product of the trees' triangle counts) from a shared
        counter."""
        n = len(trees_a)
        ha = (C.c_void_p * n)(*[t.h for t in trees_a])
        hb = (C.c_void_p * n)(*[t.h for t in trees_b])
        ma = _f32(mats_a)
        mb = _f32(mats_b)
        cost = np.array([float(a.sizes()[1]) * float(b.sizes()[1]) for a, b in zip(trees_a, trees_b)])
        order = np.ascontiguousarray(np.argsort(-cost, kind="stable"), np.uint64)
        rays = C.c_uint64()
        if self.prefix == "ref_":
            tests = self.fn("collide_batch")(ha, hb, ma, mb, n, threads, C.byref(rays), order)
            return dict(tests=tests, rays=rays.value)
        hits = C.c_uint64()
        tests = self.fn("collide_batch")(ha, hb, ma, mb, n, threads, C.byref(hits), C.byref(rays), order)
        return dict(tests=tests, hits=hits.value, rays=rays.value)

    def shoot_rays(self, ta: "Tree", tb: "Tree", ga, gb, rays_a, rays_b, params=None) -> np.ndarray:
        """ShootUncollideRays::ExecuteShootUncollideRays for one pair: the
        first entity's world-space delta. rays_*: (n, 6) origin + direction in
        the first entity's space; params (start, finish angle in radians,
        bias) or the engine's settings."""
        ra = np.ascontiguousarray(np.asarray(rays_a, np.float32).reshape(-1, 6))
        rb = np.ascontiguousarray(np.asarray(rays_b, np.float32).reshape(-1, 6))
        out = np.zeros(3, np.float32)
        pr = None
        if params is not None:
            pr = np.ascontiguousarray(params, np.float32)
        self.fn("shoot_rays")(ta.h, tb.h, _f32(ga), _f32(gb), ra if len(ra) else np.zeros((1, 6), np.float32),
                              len(ra), rb if len(rb) else np.zeros((1, 6), np.float32), len(rb),
                              pr.ctypes.data if pr is not None else None, out)
        return out

    def sweep_and_prune(self, trees, globals_, callback=None, axes=None) -> np.ndarray:
        """SweepAndPrune::ExecuteSweepAndPrune: (k, 2) [first, second] entity
        indices in no particular order (the engine's axes unless axes (3, 3))."""
        n = len(trees)
        h = (C.c_void_p * n)(*[t.h for t in trees])
        g = _f32(globals_)
        cb = np.ascontiguousarray(np.ones(n, np.uint8) if callback is None else callback, np.uint8)
        ax = None if axes is None else np.ascontiguousarray(axes, np.float32).reshape(9)
        axp = ax.ctypes.data if ax is not None else None
        cnt = self.fn("sweep_and_prune")(h, g, cb.ctypes.data, n, axp, None, 0)
        out = np.zeros((max(cnt, 1), 2), np.uint32)
        self.fn("sweep_and_prune")(h, g, cb.ctypes.data, n, axp, out.ctypes.data, cnt)
        return out[:cnt]

    def collide_pairs(self, trees_a, trees_b, mats_a, mats_b, recheck_mode=None):
        """(port) all colliding pairs of a batch: (n,3) [query, ia, ib], (n,6) segs, tests, leaf pairs.
        With recheck_mode (0 off, 1 counted, 2 FP64 verdict) also (rechecked, disagreements)."""
        n = len(trees_a)
        ha = (C.c_void_p * n)(*[t.h for t in trees_a])
        hb = (C.c_void_p * n)(*[t.h for t in trees_b])
        ma = _f32(mats_a)
        mb = _f32(mats_b)
        t = C.c_uint64()
        lp = C.c_uint64()
        z = np.zeros((1, 3), np.uint32)
        zs = np.zeros((1, 6), np.float32)
        rk = np.zeros(2, np.uint64)
        if recheck_mode is None:
            fn = lambda *a: self.fn("collide_pairs")(*a)  # noqa: E731
        else:
            fn = lambda *a: self.fn("collide_pairs_mode")(*a, int(recheck_mode), rk)  # noqa: E731
        cnt = fn(ha, hb, ma, mb, n, z, zs, 0, C.byref(t), C.byref(lp))
        pairs = np.zeros((max(cnt, 1), 3), np.uint32)
        segs = np.zeros((max(cnt, 1), 6), np.float32)
        fn(ha, hb, ma, mb, n, pairs, segs, cnt, C.byref(t), C.byref(lp))
        if recheck_mode is None:
            return pairs[:cnt], segs[:cnt], t.value, lp.value
        return pairs[:cnt], segs[:cnt], t.value, lp.value, (int(rk[0]), int(rk[1]))

    def tri_tri_recheck(self, a, b, mode):
        """(port) one test with the FP64 recheck: hit, coplanar, fragile, rechecked, disagreed, src, tgt."""
        cop, fr = C.c_int(), C.c_int()
        chk = np.zeros(2, np.uint32)
        s = np.zeros(3, np.float32)
        t = np.zeros(3, np.float32)
        hit = self.fn("tri_tri_recheck")(_f32(a, 9), _f32(b, 9), int(mode), C.byref(cop), C.byref(fr), chk, s, t)
        return hit, cop.value, fr.value, int(chk[0]), int(chk[1]), s, t


_cache: dict = {}


def port(fast: bool = False) -> Impl:
    key = ("port", fast)
    if key not in _cache:
        name = "liboracle_port_fast.so" if fast else "liboracle_port.so"
        path = os.path.join(HERE, "_build", name)
        if not os.path.exists(path):
            build_port()
        _cache[key] = Impl(path, "port_")
    return _cache[key]


def ref(fast: bool = False, ref_root: str = REF_ROOT_DEFAULT):
    """The reference's own code compiled here, or None when the reference is absent."""
    key = ("ref", fast)
    if key not in _cache:
        name = "libimr_ref_fast.so" if fast else "libimr_ref_strict.so"
        path = os.path.join(HERE, "_ref", name)
        if not os.path.exists(path):
            try:
                if not build_ref(ref_root):
                    return None
            except subprocess.CalledProcessError:
                return None
        try:
            _cache[key] = Impl(path, "ref_")
        except OSError:
            return None
    return _cache[key]
