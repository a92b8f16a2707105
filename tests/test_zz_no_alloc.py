"""cg_collide_static, the collide step that allocates nothing (its scratch is
a static device array in the library), against cg_collide: the same colliding
pairs, bit for bit, and the same counts over two calls in a row. The file is
collected last, so the static scratch is also exercised after every other GPU
test of the session; it passes on its own as well.

The test itself allocates its device buffers (queries, output, counts) with
torch before the calls; the entry point under test does not allocate."""
import numpy as np
import pytest

from inmyroom_vulkan_gb300 import capi, scenes

pytestmark = pytest.mark.gpu


def pair_rows(p):
    t = np.concatenate([np.stack([p["query"], p["tri_a"], p["tri_b"]], 1).astype(np.uint32),
                        np.ascontiguousarray(np.concatenate([p["source"], p["target"]], 1), np.float32).view(np.uint32)],
                       1)
    return t[np.lexsort(t.T[::-1])] if len(t) else t


def test_static_scratch_matches_collide(port):
    torch = pytest.importorskip("torch")
    rp = scenes.rigid_pair(n_poses=64)
    tp = [port.tree_build(m.points, m.indices, m.normals) for m in (rp.mesh_a, rp.mesh_b)]
    with capi.Context() as ctx:
        ids = [ctx.upload_flat(t.export()) for t in tp]
        rel = np.stack([capi.relative_matrix(a, b) for a, b in zip(rp.mats_a, rp.mats_b)])
        q = capi.make_queries(np.full(len(rel), ids[0]), np.full(len(rel), ids[1]), rel)
        st = ctx.collide(q)
        assert st["status"] == 0 and st["tri_pairs"] > 1000
        want = pair_rows(ctx.tri_pairs())

        cap = int(st["tri_pairs"]) + 16
        dev = torch.device("cuda", 0)
        stream = torch.cuda.Stream(device=dev)
        with torch.cuda.stream(stream):
            d_q = torch.from_numpy(q.view(np.uint8).copy()).to(dev)
            d_pairs = torch.zeros(cap * capi.TRI_PAIR_DTYPE.itemsize, dtype=torch.uint8, device=dev)
            d_counts = torch.zeros(C_COUNTS, dtype=torch.uint8, device=dev)
        stream.synchronize()
        for call in range(2):
            d_pairs.zero_()
            d_counts.zero_()
            torch.cuda.synchronize()
            ctx.collide_static(d_q.data_ptr(), len(q), d_pairs.data_ptr(), cap, d_counts.data_ptr(),
                               stream.cuda_stream)
            stream.synchronize()
            counts = capi.cg_static_counts.from_buffer_copy(d_counts.cpu().numpy().tobytes())
            assert counts.status == 0, call
            assert counts.tri_pairs == st["tri_pairs"] and counts.tri_tests == st["tri_tests"], call
            assert counts.leaf_pairs == st["leaf_pairs"], call
            got = d_pairs.cpu().numpy().view(capi.TRI_PAIR_DTYPE)[:counts.tri_pairs]
            assert np.array_equal(pair_rows(got), want), call


def static_call(torch, ctx, q, cap, with_pairs=True):
    """One cg_collide_static call on its own stream: (counts, pairs written)."""
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    d_q = torch.from_numpy(q.view(np.uint8).copy()).to(dev)
    d_pairs = torch.zeros(max(cap, 1) * capi.TRI_PAIR_DTYPE.itemsize, dtype=torch.uint8, device=dev)
    d_counts = torch.zeros(C_COUNTS, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()
    ctx.collide_static(d_q.data_ptr(), len(q), d_pairs.data_ptr() if with_pairs else 0, cap if with_pairs else 0,
                       d_counts.data_ptr(), stream.cuda_stream)
    stream.synchronize()
    counts = capi.cg_static_counts.from_buffer_copy(d_counts.cpu().numpy().tobytes())
    got = d_pairs.cpu().numpy().view(capi.TRI_PAIR_DTYPE)[:min(counts.tri_pairs, cap)]
    return counts, got


def poses(n, subdiv, far_from=None):
    rp = scenes.rigid_pair(n_poses=n, subdiv=subdiv)
    if far_from is not None:  # the poses from far_from on, moved out of reach: no leaf pairs
        rp.mats_b[far_from:, 12:15] += np.float32(100.0)
    return rp


def test_static_limits(port):
    """At CG_STATIC_MAX_QUERIES dense queries within the leaf-pair limit: the
    work queue holds the launch's donations, status 0 and cg_collide's pairs.
    Past the leaf-pair limit: CG_ERR_OUTPUT_OVERFLOW with the exact count.
    A short pair buffer: the exact count, CG_ERR_OUTPUT_OVERFLOW, and the
    pairs written are colliding pairs. Count only (no pair buffer): CG_OK.
    The device's free memory is the same before and after a call."""
    torch = pytest.importorskip("torch")
    with capi.Context() as ctx:
        for subdiv, far, want_status in ((2, 900, 0), (3, None, capi.CG_ERR_OUTPUT_OVERFLOW)):
            rp = poses(capi.CG_STATIC_MAX_QUERIES, subdiv, far)
            ids = [int(t) for t in ctx.build_trees([rp.mesh_a, rp.mesh_b])]
            rel = np.stack([capi.relative_matrix(a, b) for a, b in zip(rp.mats_a, rp.mats_b)])
            q = capi.make_queries(np.full(len(rel), ids[0]), np.full(len(rel), ids[1]), rel)
            assert len(q) == capi.CG_STATIC_MAX_QUERIES
            st = ctx.collide(q)
            assert st["status"] == 0
            assert (st["leaf_pairs"] <= capi.CG_STATIC_MAX_LEAF_PAIRS) == (want_status == 0), st["leaf_pairs"]
            counts, got = static_call(torch, ctx, q, int(st["tri_pairs"]) + 8)
            assert counts.status == want_status and counts.leaf_pairs == st["leaf_pairs"]
            if want_status == 0:
                assert counts.tri_pairs == st["tri_pairs"] and counts.tri_tests == st["tri_tests"]
                want = pair_rows(ctx.tri_pairs())
                assert np.array_equal(pair_rows(got), want)
                # a short buffer, then count only
                short, part = static_call(torch, ctx, q, int(st["tri_pairs"]) // 2)
                assert short.status == capi.CG_ERR_OUTPUT_OVERFLOW and short.tri_pairs == st["tri_pairs"]
                rows = {r.tobytes() for r in want}
                assert len(part) == int(st["tri_pairs"]) // 2 and all(r.tobytes() in rows for r in pair_rows(part))
                only, _ = static_call(torch, ctx, q, 0, with_pairs=False)
                assert only.status == 0 and only.tri_pairs == st["tri_pairs"]
                # nothing allocated: free device memory unchanged across a call
                dev = torch.device("cuda", 0)
                d_q = torch.from_numpy(q.view(np.uint8).copy()).to(dev)
                d_pairs = torch.zeros(int(st["tri_pairs"]) * capi.TRI_PAIR_DTYPE.itemsize, dtype=torch.uint8,
                                      device=dev)
                d_counts = torch.zeros(C_COUNTS, dtype=torch.uint8, device=dev)
                torch.cuda.synchronize()
                free0 = torch.cuda.mem_get_info(dev)[0]
                ctx.collide_static(d_q.data_ptr(), len(q), d_pairs.data_ptr(), int(st["tri_pairs"]),
                                   d_counts.data_ptr(), 0)
                torch.cuda.synchronize()
                assert torch.cuda.mem_get_info(dev)[0] == free0
            for t in ids:
                ctx.free_tree(t)


def test_static_scratch_rejects_too_many_queries():
    with capi.Context() as ctx:
        with pytest.raises(capi.CgError) as e:
            ctx.collide_static(1, capi.CG_STATIC_MAX_QUERIES + 1, 1, 1, 1)
        assert e.value.code == -1 and "CG_STATIC_MAX_QUERIES" in str(e.value)


C_COUNTS = 32  # sizeof(cg_static_counts)
