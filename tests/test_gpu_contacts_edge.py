"""Contacts and rays at the edges of the contact stage's paths, bit for bit and
in order against the oracle (as test_gpu_contacts.py):

* a 2-triangle quad against a fine wavy sheet that crosses it about 7,400
  times: each quad triangle has thousands of colliding pairs (slots sorted by
  a warp in global memory), and the sheet's side of the query has about
  7,400 contact triangles (a map ordered in global working memory, with its
  vertex set in the global table);
* chains of triangles at geometrically growing places, so that every box
  split peels one triangle off and the trees are as deep as they are long:
  two 24-triangle chains (descent paths of about 40 splits: two-word sort
  keys) and two 40-triangle chains (about 72 splits: three-word keys); their
  candidate leaf pairs in the reference's depth-first order (CG_DFS_ORDER)
  too."""
import numpy as np
import pytest

from inmyroom_vulkan_gb300 import capi, scenes

pytestmark = pytest.mark.gpu


def chain(n, r, plane):
    """n small triangles at x = r**k, each 0.2 x across: the reference's
    split at the box centre (OBBtree.cpp:45-74) peels the largest one off."""
    pts, idx = [], []
    for k in range(n):
        x, s = r ** k, 0.2 * r ** k
        if plane == "xz":
            pts += [[x - s, 0.0, -s], [x + s, 0.0, -s], [x, 0.0, s]]
        else:
            pts += [[x - s, -s, 0.0], [x + s, -s, 0.0], [x, 0.7 * s, 0.0]]
        idx += [3 * k, 3 * k + 1, 3 * k + 2]
    return scenes.Mesh(np.array(pts, np.float32), None, np.array(idx, np.uint32))


def sheet(g, amp):
    """A g x g grid over [-0.9, 0.9]^2 whose heights cross z = 0 in many
    curves."""
    xs = np.linspace(-0.9, 0.9, g)
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    Z = amp * np.sin(27.0 * X) * np.cos(23.0 * Y) + 0.002
    pts = np.stack([X, Y, Z], -1).reshape(-1, 3).astype(np.float32)
    i, j = np.meshgrid(np.arange(g - 1), np.arange(g - 1), indexing="ij")
    a = (i * g + j).reshape(-1)
    b, c, d = a + 1, a + g, a + g + 1
    idx = np.stack([np.stack([a, b, c], 1), np.stack([b, d, c], 1)], 1).reshape(-1)
    return scenes.Mesh(pts, None, idx.astype(np.uint32))


QUAD = scenes.Mesh(np.array([[-1, -1, 0], [1, -1, 0], [1, 1, 0], [-1, 1, 0]], np.float32), None,
                   np.array([0, 1, 2, 0, 2, 3], np.uint32))


def run(port, pairs_of_meshes):
    from test_gpu_contacts import check_grouped, check_query

    eye = np.eye(4, dtype=np.float32).reshape(16)
    with capi.Context() as ctx:
        trees, ids = [], []
        for a, b in pairs_of_meshes:
            ta, tb = (port.tree_build(m.points, m.indices, m.normals) for m in (a, b))
            trees.append((ta, tb))
            ids.append((ctx.upload_flat(ta.export()), ctx.upload_flat(tb.export())))
        rel = np.stack([capi.relative_matrix(eye, eye)] * len(ids))
        q = capi.make_queries([i for i, _ in ids], [j for _, j in ids], rel)
        st = ctx.collide(q, flags=capi.CG_CONTACTS)
        assert st["status"] == 0
        contacts, rays, averages = ctx.contacts(), ctx.rays(), ctx.ray_averages()
        check_grouped(contacts, rays)
        mids = [port.mid_phase(ta, tb, eye, eye) for ta, tb in trees]
        for k, m in enumerate(mids):
            check_query(port, m, k, contacts, rays, averages)
        # the candidate leaf pairs in the descent's order
        st = ctx.collide(q, flags=capi.CG_KEEP_LEAF_PAIRS | capi.CG_DFS_ORDER | capi.CG_MID_ONLY)
        assert st["status"] == 0
        lp = ctx.leaf_pairs()
        starts = np.searchsorted(lp["query"], np.arange(len(q) + 1))
        for k, m in enumerate(mids):
            g = lp[starts[k]:starts[k + 1]]
            got = np.stack([g["offset_a"], g["count_a"], g["offset_b"], g["count_b"]], 1).astype(np.uint32)
            assert np.array_equal(got, m.leaf_pairs().astype(np.uint32)), k
        return contacts, mids


def test_large_maps_and_slots(port):
    contacts, mids = run(port, [(QUAD, sheet(140, 0.05))])
    ia, _, _ = mids[0].contacts(0)
    ib, _, _ = mids[0].contacts(1)
    p, _, _, _ = mids[0].narrow()
    assert len(ia) == 2 and len(ib) > 4096  # a map beyond shared memory, its vertex set in the global table
    assert np.bincount(p[:, 0]).max() > 512  # a slot sorted in global memory
    assert len(contacts) == len(ia) + len(ib)


def test_deep_descent_paths(port):
    contacts, mids = run(port, [(chain(24, 2.2, "xz"), chain(24, 2.2, "xy")),
                                (chain(40, 2.2, "xz"), chain(40, 2.2, "xy"))])
    for m, n in zip(mids, (24, 40)):
        assert len(m.leaf_pairs()) > n - 8 and len(m.narrow()[0]) >= n - 1
