"""GPU contacts and uncollide rays (CG_CONTACTS) against the oracle's
restatement of CreateUncollideRays::ExecuteCreateUncollideRays
(src/CollisionDetection/CreateUncollideRays.cpp:60-201), bit for bit and in
order: per (query, side) the contact triangles in the order of the
reference's per-triangle unordered_map (GCC's libstdc++, the order its rays
are made in), their "vertex not outside" masks, weights and weighted
averages; the rays in the reference's order; the per-query mean origins.
The records come grouped by query, then side. A side without rays has the
reference's 0 / 0 mean origin (a NaN, whose payload bits are the platform's).
"""
import numpy as np
import pytest

from inmyroom_vulkan_gb300 import capi, scenes

pytestmark = pytest.mark.gpu


def bits(x):
    return np.ascontiguousarray(x, np.float32).view(np.uint32)


def same_bits(got, want, what):
    got = np.ascontiguousarray(got, np.float32)
    want = np.ascontiguousarray(want, np.float32)
    assert got.shape == want.shape, (what, got.shape, want.shape)
    nan = np.isnan(want)
    assert np.array_equal(np.isnan(got), nan), what
    assert np.array_equal(bits(got)[~nan], bits(want)[~nan]), what


def check_query(port, m, q, contacts, rays, averages):
    ra, rb, avg = m.rays()
    for side, want_rays in ((0, ra), (1, rb)):
        idx, mask, f = m.contacts(side, iteration_order=True)
        c = contacts[(contacts["query"] == q) & (contacts["side"] == side)]
        assert np.array_equal(c["tri"], idx), (q, side)
        assert np.array_equal(c["mask"], mask), (q, side)
        same_bits(c["weight"], f[:, 3], (q, side, "weight"))
        with np.errstate(invalid="ignore", divide="ignore"):
            want_avg = (f[:, :3] / f[:, 3:4]).astype(np.float32)
        same_bits(c["weighted_avg"], want_avg, (q, side, "weighted average"))
        r = rays[(rays["query"] == q) & (rays["side"] == side)]
        got_rays = np.concatenate([r["origin"], r["direction"]], 1)
        same_bits(got_rays, want_rays, (q, side, "rays"))
    a = averages[q]
    assert a["rays_first"] == len(ra) and a["rays_second"] == len(rb)
    same_bits(np.concatenate([a["first"], a["second"]]), avg, (q, "mean origins"))


def check_grouped(contacts, rays):
    """Records grouped by query, then side."""
    for rec in (contacts, rays):
        k = rec["query"].astype(np.int64) * 2 + rec["side"]
        assert np.all(np.diff(k) >= 0)


def run_contacts(ctx, port, tp, ids, qa, qb, mats_a, mats_b, flags=capi.CG_CONTACTS):
    rel = np.stack([port.relative_matrix(a, b) for a, b in zip(mats_a, mats_b)])
    q = capi.make_queries(np.asarray(ids)[qa], np.asarray(ids)[qb], rel)
    st = ctx.collide(q, flags=flags)
    return st, ctx.contacts(), ctx.rays(), ctx.ray_averages()


def test_rigid_pair_contacts_and_rays(gpu_ctx, port):
    rp = scenes.rigid_pair(n_poses=200)
    tp = [port.tree_build(m.points, m.indices, m.normals) for m in (rp.mesh_a, rp.mesh_b)]
    ids = [gpu_ctx.upload_flat(t.export()) for t in tp]
    n = len(rp.mats_a)
    st, contacts, rays, averages = run_contacts(gpu_ctx, port, tp, ids, np.zeros(n, int), np.ones(n, int),
                                                rp.mats_a, rp.mats_b)
    assert st["status"] == 0 and len(averages) == n
    assert len(contacts) > 10000 and len(rays) > 10000
    assert st["contacts"] == len(contacts) and st["rays"] == len(rays)
    check_grouped(contacts, rays)
    hit = 0
    for k in range(n):
        m = port.mid_phase(tp[0], tp[1], rp.mats_a[k], rp.mats_b[k])
        check_query(port, m, k, contacts, rays, averages)
        hit += int(averages[k]["rays_first"] > 0)
    assert hit > 50
    for i in ids:
        gpu_ctx.free_tree(i)


def test_scene_contacts_and_rays_repeatable(gpu_ctx, port):
    sc = scenes.scene()
    tp = [port.tree_build(m.points, m.indices, m.normals) for m in sc.meshes]
    ids = [gpu_ctx.upload_flat(t.export()) for t in tp]
    qa, qb = sc.pairs[:, 0], sc.pairs[:, 1]
    st, contacts, rays, averages = run_contacts(gpu_ctx, port, tp, ids, qa, qb, sc.mats[qa], sc.mats[qb])
    assert st["status"] == 0
    check_grouped(contacts, rays)
    for k in range(len(qa)):
        m = port.mid_phase(tp[qa[k]], tp[qb[k]], sc.mats[qa[k]], sc.mats[qb[k]])
        check_query(port, m, k, contacts, rays, averages)
    # a launch without contacts in between, then the same launch again: the
    # tables were emptied, the results are the same, bit for bit
    gpu_ctx.collide(capi.make_queries(np.asarray(ids)[qa], np.asarray(ids)[qb],
                                      np.stack([capi.relative_matrix(sc.mats[i], sc.mats[j]) for i, j in zip(qa, qb)])))
    st2, c2, r2, a2 = run_contacts(gpu_ctx, port, tp, ids, qa, qb, sc.mats[qa], sc.mats[qb])
    assert st2["status"] == 0
    assert np.array_equal(c2.view(np.uint8), contacts.view(np.uint8))
    assert np.array_equal(r2.view(np.uint8), rays.view(np.uint8))
    nan = np.isnan(averages["first"]).any(1) | np.isnan(averages["second"]).any(1)
    assert np.array_equal(a2[~nan].view(np.uint8), averages[~nan].view(np.uint8))
    for i in ids:
        gpu_ctx.free_tree(i)


def test_zero_length_segment_keeps_its_mask_bits(gpu_ctx, port):
    """One leaf pair: the second tree's first triangle touches the first's
    plane in a single point (a colliding pair of zero length), the second
    crosses it. The touching pair adds no weight, but its plane test still
    clears a vertex bit of the first triangle, as in the reference."""
    pa = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    pb = np.array([[0.25, 0.25, 0], [1, 1, 1], [-1, 1, 1], [0.5, -0.5, -1], [0.5, 1.5, -1], [0.25, 0.5, 1]],
                  np.float32)
    ta = port.tree_build(pa, np.arange(3, dtype=np.uint32))
    tb = port.tree_build(pb, np.arange(6, dtype=np.uint32))
    eye = np.eye(4, dtype=np.float32).reshape(-1)
    pairs, segs, _, _ = port.collide_pairs([ta], [tb], [eye], [eye])
    w = np.linalg.norm(segs[:, :3] - segs[:, 3:], axis=1)
    assert (w == 0).sum() == 1 and (w > 0).sum() == 1
    fa, fb = ta.export(), tb.export()
    # the first tree goes up without vertex normals: the face normal is used, as the oracle's build does
    ida = gpu_ctx.upload_tree(fa.root, fa.node_obbs, fa.node_ref, fa.node_cnt, fa.tri_pos, None, fa.tri_idx)
    idb = gpu_ctx.upload_flat(fb)
    st, contacts, rays, averages = run_contacts(gpu_ctx, port, [ta, tb], [ida, idb], [0], [1], [eye], [eye])
    assert st["status"] == 0
    m = port.mid_phase(ta, tb, eye, eye)
    assert m.contacts(0)[1].tolist() == [4]  # bit 0 cleared by the zero-length pair alone
    check_query(port, m, 0, contacts, rays, averages)
    gpu_ctx.free_tree(ida)
    gpu_ctx.free_tree(idb)


def test_contacts_flag_combinations_and_overflow(port):
    sc = scenes.scene()
    tp = [port.tree_build(m.points, m.indices, m.normals) for m in sc.meshes[:64]]
    keep = (sc.pairs[:, 0] < 64) & (sc.pairs[:, 1] < 64)
    qa, qb = sc.pairs[keep, 0], sc.pairs[keep, 1]
    with capi.Context(max_contacts=16) as ctx:
        ids = [ctx.upload_flat(t.export()) for t in tp]
        rel = np.stack([capi.relative_matrix(sc.mats[i], sc.mats[j]) for i, j in zip(qa, qb)])
        q = capi.make_queries(np.asarray(ids)[qa], np.asarray(ids)[qb], rel)
        for bad in (capi.CG_CONTACTS | capi.CG_MID_ONLY, capi.CG_CONTACTS | capi.CG_NO_TRI_PAIRS):
            with pytest.raises(capi.CgError) as e:
                ctx.collide(q, flags=bad)
            assert e.value.code == -1
        st = ctx.collide(q, flags=capi.CG_CONTACTS, check=False)
        assert st["rc"] == -5  # more contacts than max_contacts
        ctx.reconfigure(max_contacts=1 << 18)
        st = ctx.collide(q, flags=capi.CG_CONTACTS)
        assert st["status"] == 0 and len(ctx.contacts()) > 16


def test_host_outputs_match_the_read_calls(port):
    """cg_set_host_outputs: one cg_collide writes the pairs, rays and
    averages into page-locked host arrays; they equal what the read calls
    return. A smaller capacity takes the first records."""
    import torch

    sc = scenes.scene()
    tp = [port.tree_build(m.points, m.indices, m.normals) for m in sc.meshes[:96]]
    keep = (sc.pairs[:, 0] < 96) & (sc.pairs[:, 1] < 96)
    qa, qb = sc.pairs[keep, 0], sc.pairs[keep, 1]

    def pinned(count, dtype):
        return torch.empty(count * dtype.itemsize, dtype=torch.uint8, pin_memory=True).numpy().view(dtype)

    with capi.Context() as ctx:
        ids = [ctx.upload_flat(t.export()) for t in tp]
        rel = np.stack([capi.relative_matrix(sc.mats[i], sc.mats[j]) for i, j in zip(qa, qb)])
        q = capi.make_queries(np.asarray(ids)[qa], np.asarray(ids)[qb], rel)
        st = ctx.collide(q, flags=capi.CG_CONTACTS)
        n_p, n_r = st["tri_pairs"], st["rays"]
        assert n_p > 1000 and n_r > 1000
        hp, hr, ha = pinned(n_p + 7, capi.TRI_PAIR_DTYPE), pinned(n_r, capi.RAY_DTYPE), pinned(len(q),
                                                                                            capi.RAY_AVERAGE_DTYPE)
        ctx.set_host_outputs(hp, hr, ha)
        st2 = ctx.collide(q, flags=capi.CG_CONTACTS)
        assert st2["tri_pairs"] == n_p and st2["rays"] == n_r
        assert np.array_equal(hp[:n_p].view(np.uint8), ctx.tri_pairs().view(np.uint8))
        assert np.array_equal(hr.view(np.uint8), ctx.rays().view(np.uint8))
        assert np.array_equal(ha.view(np.uint8), ctx.ray_averages().view(np.uint8))
        small = pinned(100, capi.TRI_PAIR_DTYPE)
        ctx.set_host_outputs(small)
        ctx.collide(q)
        assert np.array_equal(small.view(np.uint8), ctx.tri_pairs()[:100].view(np.uint8))
        # smaller ray and average buffers take the first ones
        small_r, small_a = pinned(100, capi.RAY_DTYPE), pinned(3, capi.RAY_AVERAGE_DTYPE)
        ctx.set_host_outputs(None, small_r, small_a)
        st3 = ctx.collide(q, flags=capi.CG_CONTACTS)
        assert st3["rays"] == n_r
        assert np.array_equal(small_r.view(np.uint8), ctx.rays()[:100].view(np.uint8))
        assert np.array_equal(small_a.view(np.uint8), ctx.ray_averages()[:3].view(np.uint8))
        # pageable memory: refused, unless the device writes pageable host
        # memory directly (as on Grace), and then the results land there too
        pageable = np.zeros(100, capi.TRI_PAIR_DTYPE)
        try:
            ctx.set_host_outputs(pageable)
        except capi.CgError:
            pass
        else:
            ctx.collide(q)
            assert np.array_equal(pageable.view(np.uint8), ctx.tri_pairs()[:100].view(np.uint8))
        ctx.set_host_outputs()
