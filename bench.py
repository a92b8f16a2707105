"""Benchmark of the GB300 collision path on the 256-entity scene.

One step = one batched collide launch (CUDA graph: counter reset, query
packing, persistent traversal, persistent triangle-pair narrow phase with the
FP64 recheck of near-threshold plane distances, then per-triangle contacts,
uncollide rays and their mean origins in the reference's order) over every
entity pair of the scene whose world AABBs overlap, the work the reference's
mid phase + CreateUncollideRays does per pair. The metric is triangle-pair
tests per second (Moller calls on candidate leaf pairs), with collision
queries per second beside it.

  python bench.py [--gpus N --steps K --warmup W]      # GPU arm
  python bench.py --impl reference [...]                # the reference's CPU path

value: device-resident inputs, each step timed with CUDA events on the
launching stream, L2 flushed (a 512 MB write) between steps.
e2e: the public host API: one cg_collide call with host queries, whose step
also writes the colliding pairs, the rays and the per-query mean origins into
pinned host buffers (cg_set_host_outputs); host-timed around the call.
roofline: the traversal kernel (the dominant one), algorithmic bytes (node
pairs x 96 B of box data) per launch over its event-timed duration, against the
measured copy bandwidth, with the FP32 view beside it; roofline_narrow: the
same for the narrow-phase kernel (triangle tests x 72 B of triangle data).
cpu_baseline: the oracle restatement of the reference's CPU path (release
flags) on all host cores over a bounded number of scene steps.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "tri-pair tests/s & collision queries/s, 1 GB300 (batched vs plain), bwd ms"
UNIT = "tri-pair tests/s"
WORKLOAD = "scene: 256 rigid entities (500-20,000 tris, log-uniform), AABB-overlap pairs, batched launch"
# per-unit algorithmic figures (source-level op counts of the reference path)
NODE_PAIR_BYTES = 2 * 48   # two boxes
TRI_TEST_BYTES = 2 * 36    # two triangles
NODE_PAIR_FLOPS = 714      # SAT worst case ~650 + B-box transform 64
TRI_TEST_FLOPS = 147       # full non-coplanar Moller path
COUNTERS_BYTES = 152       # the launch counters, read back by cg_collide and by each result read
# init, pack, traverse, narrow; contacts: pairs, paths, alloc, scatter, fold, order, emit
STEP_KERNELS = 11
STEP_FLAGS_DOC = ("CUDA graph: init + pack + persistent traversal + persistent narrow phase (FP64 recheck counted) "
                  "+ contacts in the reference's order (pairs; alloc, scatter beside the descent paths; fold and "
                  "rank; order and placement; emit)")
CACHE_DOC = "L2 flushed (512 MB write) between timed GPU steps"


def scene_config(n_queries: int, n_tris: int) -> dict:
    """The workload's description, the same keys and values in both arms (the
    work each arm counts per step is reported beside it, in work_per_step: the
    reference's release build, -ffast-math, classifies a few pairs
    differently)."""
    return {"workload": WORKLOAD, "queries_per_step": int(n_queries), "triangles": int(n_tris), "seed": 1002,
            "cache": CACHE_DOC}


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": d.get("hbm_gbs", 6800.0), "sm_max_mhz": d.get("sm_max_mhz", 2070.0), "source": "measured"}
    return {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0, "source": "fallback"}


def profiled_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` from its committed ncu summary
    (profiles/<kernel>_scene256.md, the row marked 'traffic per launch'), or
    None when there is none."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_scene256.md")
    if not os.path.exists(path):
        return None
    scale = {"B": 1, "KB": 1e3, "MB": 1e6, "GB": 1e9}
    for line in open(path):
        if "traffic per launch" in line:
            cell = line.split("|")[2].split()
            return int(float(cell[0]) * scale[cell[1]])
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int = 0):
        self.device = device
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # sampling is live before the timed region starts
            t0 = time.perf_counter()
            while not self.rows and time.perf_counter() - t0 < 5.0:
                time.sleep(0.005)
            self.rows.clear()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows if len(r) >= 9 for k in range(4) if r[5 + k] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def run_tree_build(ctx, sc, cpu_seconds: float, reps: int = 10, device: int = 0) -> tuple[np.ndarray, dict]:
    """OBB trees of the scene's meshes built on the device (cg_tree_build, one
    call for all 256, trees uploaded); host-timed around the synchronous call,
    the median of `reps` builds after one untimed build, with the SM clocks
    sampled meanwhile. Beside it the oracle's builder on all host cores.
    Returns the trees' ids and the line."""
    ids = ctx.build_trees(sc.meshes)
    times = []
    with ClockSampler(device) as clocks:
        for _ in range(reps):
            for tid in ids:
                ctx.free_tree(int(tid))
            t0 = time.perf_counter()
            ids = ctx.build_trees(sc.meshes)
            times.append(1e3 * (time.perf_counter() - t0))
    ms = float(np.median(times))
    tris = int(sum(m.n_tris for m in sc.meshes))
    line = {"workload": f"OBB trees of the scene's {len(sc.meshes)} meshes ({tris} triangles), one cg_tree_build",
            "ms": ms, "ms_min": float(np.min(times)), "ms_max": float(np.max(times)), "builds": reps,
            "triangles_per_s": tris / (ms / 1e3), "clocks": clocks.summary(),
            "timing": "host perf_counter around the synchronous call (meshes read from host memory, trees written to the arenas); median of "
                      f"{reps} builds"}
    if cpu_seconds > 0:
        from concurrent.futures import ThreadPoolExecutor

        import oracle

        fast = oracle.port(fast=True)
        cores = os.cpu_count() or 1
        pool = ThreadPoolExecutor(cores)
        runs, t0 = 0, time.perf_counter()
        while True:
            list(pool.map(lambda m: fast.tree_build(m.points, m.indices, m.normals), sc.meshes))
            runs += 1
            if time.perf_counter() - t0 >= cpu_seconds:
                break
        el = time.perf_counter() - t0
        line["cpu_baseline"] = {"ms": 1e3 * el / runs, "cores": cores, "kind": "port",
                                "sample": f"{runs} builds of all the scene's trees, {el:.1f} s, release flags"}
    return ids, line


def cpu_baseline(sc, seconds: float = 10.0) -> dict:
    """The oracle restatement (release flags) on all host cores over whole scene steps."""
    import oracle

    fast = oracle.port(fast=True)
    trees = [fast.tree_build(m.points, m.indices, m.normals) for m in sc.meshes]
    qa, qb = sc.pairs[:, 0], sc.pairs[:, 1]
    ta, tb = [trees[i] for i in qa], [trees[j] for j in qb]
    ma, mb = sc.mats[qa], sc.mats[qb]
    cores = os.cpu_count() or 1
    fast.collide_batch(ta, tb, ma, mb, threads=cores)  # warm
    steps, tests, t0 = 0, 0, time.perf_counter()
    while True:
        r = fast.collide_batch(ta, tb, ma, mb, threads=cores)
        steps += 1
        tests += r["tests"]
        el = time.perf_counter() - t0
        if el >= seconds or steps >= 5000:
            break
    t1 = time.perf_counter()
    r1 = fast.collide_batch(ta, tb, ma, mb, threads=1)
    single = time.perf_counter() - t1
    v1 = r1["tests"] / single
    return {"value": tests / el, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{steps} whole scene steps ({len(qa)} queries each), {el:.1f} s, release flags, queries "
                      "largest first from a shared counter",
            "single_thread_value": v1, "efficiency": tests / el / v1 / cores, "steps": steps}


def run_reference(args) -> dict:
    """`--impl reference`: the reference's CPU path on the host cores. The
    reference compiled from its own sources (oracle/_ref) where it exists,
    else the oracle restatement of it."""
    import oracle
    from inmyroom_vulkan_gb300 import scenes

    sc = scenes.scene(seed=1002)
    impl, kind = oracle.ref(fast=True), "reference"
    if impl is None:
        impl, kind = oracle.port(fast=True), "port"
    trees = [impl.tree_build(m.points, m.indices, m.normals) for m in sc.meshes]
    qa, qb = sc.pairs[:, 0], sc.pairs[:, 1]
    ta, tb = [trees[i] for i in qa], [trees[j] for j in qb]
    ma, mb = sc.mats[qa], sc.mats[qb]
    cores = os.cpu_count() or 1
    first = None
    for _ in range(args.warmup):
        first = impl.collide_batch(ta, tb, ma, mb, threads=cores)
    tests, t0 = 0, time.perf_counter()
    for _ in range(args.steps):
        r = impl.collide_batch(ta, tb, ma, mb, threads=cores)
        tests += r["tests"]
    el = time.perf_counter() - t0
    v = tests / el
    r = first or r
    return {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded PCG64, seed 1002)",
            "config": scene_config(len(qa), sum(m.n_tris for m in sc.meshes)),
            "work_per_step": {"tri_tests": int(r["tests"]), "rays": int(r["rays"])},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": kind,
                             "sample": f"{args.steps} whole scene steps, release flags, queries largest first from a "
                                       "shared counter"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_shoot(args, ctx, sc, ids, q, cpu_seconds: float) -> dict:
    """Uncollide-ray shooting of the scene step: ShootUncollideRays for every
    AABB-overlap pair with the rays the step's contact kernels made (grouped
    per pair and side). Host-timed around the synchronous cg_shoot_rays call
    (rays and queries uploaded, deltas read back, inside the timing); beside
    it the oracle restatement on all host cores over the same rays."""
    from concurrent.futures import ThreadPoolExecutor

    import oracle
    from inmyroom_vulkan_gb300 import capi

    assert ctx.collide(q, flags=capi.CG_CONTACTS)["status"] == 0
    rays = ctx.rays()
    rays = rays[np.lexsort((rays["side"], rays["query"]))]
    qa, qb = sc.pairs[:, 0], sc.pairs[:, 1]
    n = len(qa)
    starts = np.searchsorted(rays["query"], np.arange(n + 1))
    ra, rb = [], []
    for k in range(n):
        mine = rays[starts[k]:starts[k + 1]]
        for side, out in ((0, ra), (1, rb)):
            m = mine[mine["side"] == side]
            out.append(np.concatenate([m["origin"], m["direction"]], 1))
    ga, gb = sc.mats[qa], sc.mats[qb]
    ta, tb = [int(ids[i]) for i in qa], [int(ids[j]) for j in qb]
    packed_q, packed_rays = ctx.pack_shoot(ta, tb, ga, gb, ra, rb)
    out = np.zeros((n, 3), np.float32)
    for _ in range(max(args.warmup, 3)):
        deltas = ctx.shoot_packed(packed_q, packed_rays, out=out)
    times = []
    for _ in range(max(args.steps, 5)):
        t0 = time.perf_counter()
        deltas = ctx.shoot_packed(packed_q, packed_rays, out=out)
        times.append(time.perf_counter() - t0)
    ms = 1e3 * float(np.median(times))
    res = {"workload": f"ShootUncollideRays for the scene step's {n} pairs with its {len(rays)} uncollide rays",
           "rays": int(len(rays)), "pairs": int(n), "pairs_moved": int((np.abs(deltas).sum(1) > 0).sum()),
           "ms_per_step": ms, "rays_per_s": len(rays) / (ms / 1e3),
           "timing": "host perf_counter around the synchronous cg_shoot_rays (uploads and read-back included)"}
    if cpu_seconds > 0:
        fast = oracle.port(fast=True)
        trees = [fast.tree_build(m.points, m.indices, m.normals) for m in sc.meshes]
        cores = os.cpu_count() or 1
        pool = ThreadPoolExecutor(cores)
        work = [k for k in range(n) if len(ra[k]) or len(rb[k])]

        def one(k):
            return fast.shoot_rays(trees[qa[k]], trees[qb[k]], ga[k], gb[k], ra[k], rb[k])

        runs, t0 = 0, time.perf_counter()
        while True:
            list(pool.map(one, work))
            runs += 1
            if time.perf_counter() - t0 >= cpu_seconds:
                break
        el = time.perf_counter() - t0
        res["cpu_baseline"] = {"ms_per_step": 1e3 * el / runs, "cores": cores, "kind": "port",
                               "sample": f"{runs} whole steps of shooting, {el:.1f} s, release flags"}
    return res


def run_frame(args, ctx, sc, ids, cpu_seconds: float) -> dict:
    """One collision frame of the 256-entity scene (cg_collision_frame): the
    engine's whole per-frame pipeline (broad phase, OBB-tree collide with
    contacts and rays, shooting for pairs where an entity moved, the delta
    split) from the entities' current and previous matrices to one record per
    pair with rays. A third of the entities stand still, the rest moved up to
    0.05; 70% call back. Host-timed around the synchronous call (entities in,
    results out); beside it the oracle's frame on all host cores."""
    from concurrent.futures import ThreadPoolExecutor

    import oracle
    from inmyroom_vulkan_gb300 import scenes
    from oracle import frame

    prev, cb = scenes.frame_motion(sc)
    for _ in range(max(args.warmup, 3)):
        res = ctx.collision_frame(ids, sc.mats, prev, cb)
    times = []
    for _ in range(max(args.steps, 5)):
        t0 = time.perf_counter()
        res = ctx.collision_frame(ids, sc.mats, prev, cb)
        times.append(time.perf_counter() - t0)
    ms = 1e3 * float(np.median(times))
    out = {"workload": "one collision frame of the 256-entity scene (SweepAndPrune, OBB trees, uncollide rays, "
                       "ShootUncollideRays, delta split)",
           "entities": len(ids), "pairs_with_rays": int(len(res)),
           "pairs_moved": int((np.abs(res["first_delta"]).sum(1) + np.abs(res["second_delta"]).sum(1) > 0).sum()),
           "ms_per_frame": ms, "frames_per_s": 1e3 / ms,
           "timing": "host perf_counter around the synchronous cg_collision_frame (entity upload and result "
                     "read-back included); median of the steps"}
    if cpu_seconds > 0:
        fast = oracle.port(fast=True)
        trees = [fast.tree_build(m.points, m.indices, m.normals) for m in sc.meshes]
        cores = os.cpu_count() or 1
        pool = ThreadPoolExecutor(cores)
        runs, t0 = 0, time.perf_counter()
        while True:
            frame.collision_frame(fast, trees, sc.mats, prev, cb, map_fn=pool.map)
            runs += 1
            if time.perf_counter() - t0 >= cpu_seconds:
                break
        el = time.perf_counter() - t0
        out["cpu_baseline"] = {"ms_per_frame": 1e3 * el / runs, "cores": cores, "kind": "port",
                               "sample": f"{runs} whole frames, {el:.1f} s, release flags, pairs over a thread pool"}
    return out


def run_sweep(args, local: int, flush, stream, cpu_seconds: float) -> dict:
    """Autotuned batch sweep: 10,000 uneven rigid mesh-pair queries (a pool of
    48 meshes of 256..65,536 triangles, log-uniform; random SO(3) poses with
    root-box overlap probability about 0.5) resolved in one launch. Timed with
    the context's starting settings, then tuned (autotune.tune_collide) and
    timed again as a captured CUDA graph; beside it the plain path (one query
    per launch) over the first 1,000 queries and the CPU restatement on the
    host cores. L2 flushed before every timed launch."""
    import torch

    import oracle
    from inmyroom_vulkan_gb300 import autotune, capi, scenes

    bs = scenes.batch_sweep()
    ctx = capi.Context(device=local, max_queries=16384, max_tri_pairs=1 << 23, max_leaf_pairs=1 << 24)
    ids = ctx.build_trees(bs.meshes)
    rel = np.stack([capi.relative_matrix(a, b) for a, b in zip(bs.mats_a, bs.mats_b)])
    q = capi.make_queries(ids[bs.qa], ids[bs.qb], rel)
    n = len(q)
    d_q = torch.from_numpy(q.view(np.uint8).copy()).cuda()
    flags = 0
    sp = stream.cuda_stream
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(launch, reps):
        ms = []
        for k in range(reps):
            flush.fill_(k & 0xff)
            e0.record(stream)
            launch()
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return float(np.median(ms))

    batched = lambda: ctx.collide_async(d_q.data_ptr(), n, flags, sp)  # noqa: E731
    for _ in range(max(args.warmup, 3)):
        batched()
    st = ctx.sync_stats()
    start_ms = timed(batched, max(args.steps, 5))
    tune = autotune.tune_collide(ctx, d_q.data_ptr(), n, flags, flush=flush)
    ctx.graph_capture(d_q.data_ptr(), n, flags)
    graph = lambda: ctx.graph_launch(sp)  # noqa: E731
    for _ in range(max(args.warmup, 3)):
        graph()
    tuned_ms = timed(graph, max(args.steps, 5))
    st2 = ctx.sync_stats()
    assert st2["status"] == 0 and st2["tri_tests"] == st["tri_tests"] and st2["tri_pairs"] == st["tri_pairs"]
    tests, node_pairs = st["tri_tests"], st["node_pairs"]
    # plain path: one query per launch
    P = min(1000, n)
    qsz = capi.QUERY_DTYPE.itemsize
    plain = lambda: [ctx.collide_async(d_q.data_ptr() + i * qsz, 1, flags, sp) for i in range(P)]  # noqa: E731
    plain()
    plain_ms = timed(plain, 3)
    ctx.collide(q[:P], flags=flags)
    ptests = ctx.sync_stats()["tri_tests"]
    res = {"workload": f"{n} rigid mesh-pair queries over a pool of {len(bs.meshes)} meshes "
                       f"({min(m.n_tris for m in bs.meshes)}..{max(m.n_tris for m in bs.meshes)} triangles, "
                       "log-uniform), root-box overlap ~0.5, one launch (colliding pairs out)",
           "tri_tests_per_launch": int(tests), "tri_pairs_per_launch": int(st["tri_pairs"]),
           "leaf_pairs_per_launch": int(st["leaf_pairs"]), "node_pairs_per_launch": int(node_pairs),
           "start_ms": start_ms, "tuned_ms": tuned_ms, "tri_tests_per_s": tests / (tuned_ms / 1e3),
           "queries_per_s": n / (tuned_ms / 1e3),
           "operand_gbs": (node_pairs * NODE_PAIR_BYTES + tests * TRI_TEST_BYTES) / (tuned_ms / 1e3) / 1e9,
           "autotune": tune.as_dict(),
           "plain": {"queries": P, "ms_per_query": plain_ms / P, "queries_per_s": P / (plain_ms / 1e3),
                     "tri_tests_per_s": ptests / (plain_ms / 1e3)},
           "cache": "L2 flushed (512 MB write) before every timed launch", "launch": "CUDA graph after tuning"}
    ctx.close()
    if cpu_seconds > 0:
        port = oracle.port(fast=True)
        trees = [port.tree_build(m.points, m.indices, m.normals) for m in bs.meshes]
        cores = os.cpu_count() or 1
        ta = [trees[i] for i in bs.qa[:P]]
        tb = [trees[i] for i in bs.qb[:P]]
        runs, ctests, t0 = 0, 0, time.perf_counter()
        while True:
            ctests += port.collide_batch(ta, tb, bs.mats_a[:P], bs.mats_b[:P], threads=cores)["tests"]
            runs += 1
            if time.perf_counter() - t0 >= cpu_seconds:
                break
        el = time.perf_counter() - t0
        res["cpu_baseline"] = {"tri_tests_per_s": ctests / el, "cores": cores, "kind": "port",
                               "sample": f"the first {P} queries x {runs}, {el:.1f} s, release flags"}
    return res


def run_differentiable(args, ctx_factory, flush, stream, cpu_seconds: float) -> dict:
    """Differentiable workload on the deforming scene: forward = pose the 64
    skeletons from axis angles, morph + skin, refit, collide, penetration
    energy; backward = the energy's adjoint to the axis angles and morph
    weights (recomputing deformed vertices). Both event-timed on `stream`, L2
    flushed before each forward. Beside it, the FP64 reference gradient of the
    same pair set on the host (torch autograd on the CPU)."""
    import torch

    from inmyroom_vulkan_gb300 import capi, scenes
    from inmyroom_vulkan_gb300.energy import DeformingCollider, penetration_energy

    sc = scenes.deforming()
    n = sc.vertices.shape[0]
    parent, offsets = scenes.chain_skeleton(sc)
    ctx = ctx_factory()
    rid, fid = (int(t) for t in ctx.build_trees([sc.mesh, sc.field]))
    rf, ff = ctx.export_tree(rid), ctx.export_tree(fid)
    ctx.free_tree(rid)
    eye = np.eye(4, dtype=np.float32).reshape(16)
    rel = np.stack([capi.relative_matrix(m, eye) for m in sc.models])
    col = DeformingCollider(ctx, rf, capi.Skeleton(parent, offsets), sc.vertices, sc.joints, sc.weights,
                            sc.inverse_bind, fid, rel)
    aa = torch.tensor(sc.axis_angles, dtype=torch.float32, device="cuda", requires_grad=True)
    mw = torch.tensor(sc.morph_weights, dtype=torch.float32, device="cuda", requires_grad=True)
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    with torch.cuda.stream(stream):
        for _ in range(max(args.warmup, 3)):
            aa.grad = mw.grad = None
            penetration_energy(aa, mw, col).backward()
        fwd, bwd = [], []
        for k in range(args.steps):
            aa.grad = mw.grad = None
            flush.fill_(k & 0xff)
            e0.record(stream)
            E = penetration_energy(aa, mw, col)
            e1.record(stream)
            E.backward()
            e2.record(stream)
            e2.synchronize()
            fwd.append(e0.elapsed_time(e1))
            bwd.append(e1.elapsed_time(e2))
    st = ctx.sync_stats()
    assert st["status"] == 0
    pairs = col.tri_pairs()
    f_ms, b_ms = float(np.mean(fwd)), float(np.mean(bwd))
    res = {"workload": f"{n} tubes ({sc.mesh.n_tris} tris, 50 bones, 8 targets) vs a {sc.field.n_tris}-triangle "
                       "heightfield; E = sum of squared plane-penetration depths over colliding pairs; "
                       "gradients to 64x50x3 axis angles and 64x8 morph weights",
           "forward_ms": f_ms, "backward_ms": b_ms, "backward_over_forward": b_ms / f_ms,
           "energy": float(E.item()), "colliding_pairs": int(len(pairs)), "steps": args.steps,
           "forward": "pose + deform + refit + collide + energy kernels", "backward":
           "vertex-gradient + skin-adjoint + pose-adjoint kernels (deformed vertices recomputed)"}
    col.close()
    ctx.free_tree(fid)
    ctx.close()
    if cpu_seconds > 0:
        from oracle import energy as oe

        arr = np.stack([pairs["query"], pairs["tri_a"], pairs["tri_b"]], 1).astype(np.int64)
        pr = oe.Problem(parent, offsets.astype(np.float64), sc.inverse_bind, sc.vertices, sc.joints, sc.weights,
                        rf.tri_idx, ff.tri_pos, rel, arr)
        runs, t0 = 0, time.perf_counter()
        while True:
            pr.value_and_grad(sc.axis_angles, sc.morph_weights.astype(np.float64))
            runs += 1
            if time.perf_counter() - t0 >= cpu_seconds:
                break
        el = time.perf_counter() - t0
        res["cpu_baseline"] = {"ms_forward_backward": 1e3 * el / runs, "cores": torch.get_num_threads(),
                               "kind": "port", "sample": f"{runs} FP64 torch-autograd energy + gradient evaluations "
                                                         "on the host (same pair set, no collide)"}
    return res


def run_deforming(args, ctx_factory, flush, stream, cpu_seconds: float) -> dict:
    """Deforming workload: per frame, morph + skin all tubes (one batched
    launch), refit their trees (one batched launch of each refit kernel), and
    collide every tube with the static heightfield with contacts and rays.
    Event-timed per phase on `stream`, L2 flushed between frames; beside it the
    oracle restatement of the same frame on the host cores."""
    import torch

    import oracle
    from inmyroom_vulkan_gb300 import capi, scenes

    sc = scenes.deforming()
    n = sc.vertices.shape[0]
    V = sc.vertices.shape[1]
    ctx = ctx_factory()
    rid, fid = (int(t) for t in ctx.build_trees([sc.mesh, sc.field]))
    rest_arrays = ctx.export_tree(rid)
    ctx.free_tree(rid)
    ids = [ctx.upload_flat(rest_arrays) for _ in range(n)]
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    j, w, ib = dev(sc.joints.view(np.int16)), dev(sc.weights), dev(sc.inverse_bind)
    keep, views, outs = [j, w, ib], [], []
    for m in range(n):
        v, mw, jm = dev(sc.vertices[m]), dev(sc.morph_weights[m]), dev(sc.joint_matrices[m])
        out = torch.zeros((V, 4), dtype=torch.float32, device="cuda")
        keep += [v, mw, jm]
        outs.append(out)
        views.append(capi.cg_deform_view(V, sc.vertices.shape[2] - 1, 1, sc.joint_matrices.shape[1], v.data_ptr(),
                                         mw.data_ptr(), j.data_ptr(), w.data_ptr(), jm.data_ptr(), ib.data_ptr()))
    out_ptrs = [o.data_ptr() for o in outs]
    eye = np.eye(4, dtype=np.float32).reshape(16)
    q = capi.make_queries(ids, [fid] * n, np.stack([capi.relative_matrix(sc.models[m], eye) for m in range(n)]))
    d_q = torch.from_numpy(q.view(np.uint8).copy()).cuda()
    flags = capi.CG_CONTACTS
    sp = stream.cuda_stream

    def frame():
        ctx.deform_batch(views, out_ptrs, sp)
        e1.record(stream)
        ctx.tree_refit_batch(ids, out_ptrs, [V] * n, sp)
        e2.record(stream)
        ctx.collide_async(d_q.data_ptr(), n, flags, sp)

    e0, e1, e2, e3 = (torch.cuda.Event(enable_timing=True) for _ in range(4))
    for _ in range(max(args.warmup, 3)):
        frame()
    st = ctx.sync_stats()
    ms, parts = [], []
    for k in range(args.steps):
        flush.fill_(k & 0xff)
        e0.record(stream)
        frame()
        e3.record(stream)
        e3.synchronize()
        ms.append(e0.elapsed_time(e3))
        parts.append((e0.elapsed_time(e1), e1.elapsed_time(e2), e2.elapsed_time(e3)))
    st = ctx.sync_stats()
    assert st["status"] == 0
    frame_ms = float(np.mean(ms))
    tests = st["tri_tests"]
    res = {"workload": f"{n} skinned + morphed tubes ({sc.mesh.n_tris} tris, 50 bones, 8 targets) vs a "
                       f"{sc.field.n_tris}-triangle heightfield; per frame deform + refit + collide with contacts",
           "ms_per_frame": frame_ms, "deform_ms": float(np.mean([p[0] for p in parts])),
           "refit_ms": float(np.mean([p[1] for p in parts])), "collide_ms": float(np.mean([p[2] for p in parts])),
           "tri_tests_per_frame": int(tests), "tri_pairs_per_frame": int(st["tri_pairs"]),
           "tri_tests_per_s": tests / (frame_ms / 1e3), "frames": args.steps}
    ctx.close()
    if cpu_seconds > 0:
        from concurrent.futures import ThreadPoolExecutor

        port = oracle.port(fast=True)
        rest_flat = port.tree_build(sc.mesh.points, sc.mesh.indices, sc.mesh.normals).export()
        field = port.tree_build(sc.field.points, sc.field.indices, sc.field.normals)
        cores = os.cpu_count() or 1
        pool = ThreadPoolExecutor(cores)

        def cpu_mesh(m):
            pos = port.deform(sc.vertices[m], sc.morph_weights[m], sc.joints, sc.weights, sc.joint_matrices[m],
                              sc.inverse_bind)
            return port.tree_import(port.tree_refit(rest_flat, pos))

        frames, t0 = 0, time.perf_counter()
        while True:
            trees = list(pool.map(cpu_mesh, range(n)))
            port.collide_batch(trees, [field] * n, sc.models, [eye] * n, threads=cores)
            frames += 1
            if time.perf_counter() - t0 >= cpu_seconds:
                break
        el = time.perf_counter() - t0
        res["cpu_baseline"] = {"ms_per_frame": 1e3 * el / frames, "cores": cores, "kind": "port",
                               "sample": f"{frames} whole frames, {el:.1f} s (deform, refit, collide with rays)"}
    return res


def run_sharded(args, dist, rank, world, local, dev, stream, flush) -> dict:
    """Strong scaling: the one 256-entity frame (seed 1002) split over the
    ranks by cost (LPT, every rank computing the same partition); each rank
    builds the trees its queries use and collides its share, event-timed; the
    frame's time is the slowest rank's. The colliding pairs are then gathered
    to every rank (fixed-width rows, all_gather_into_tensor), outside the
    timed steps and timed on their own."""
    import torch

    from inmyroom_vulkan_gb300 import capi, scenes, shard

    sc = scenes.scene(seed=1002)
    pa, pb = sc.pairs[:, 0], sc.pairs[:, 1]
    costs = shard.query_costs([sc.meshes[i].n_tris for i in pa], [sc.meshes[j].n_tris for j in pb])
    parts = shard.lpt_partition(costs, world)
    mine = parts[rank]
    used = np.unique(sc.pairs[mine])
    ctx = capi.Context(device=local, max_queries=max(4096, len(mine)), max_tri_pairs=1 << 22)
    ids = np.zeros(len(sc.meshes), np.uint32)
    ids[used] = ctx.build_trees([sc.meshes[i] for i in used])
    qa, qb = pa[mine], pb[mine]
    rel = np.stack([capi.relative_matrix(sc.mats[i], sc.mats[j]) for i, j in zip(qa, qb)])
    q = capi.make_queries(ids[qa], ids[qb], rel)
    d_q = torch.from_numpy(q.view(np.uint8).copy()).to(dev)
    flags = capi.CG_CONTACTS | capi.CG_RECHECK
    ctx.graph_capture(d_q.data_ptr(), len(q), flags)
    for _ in range(max(args.warmup, 3)):
        ctx.graph_launch(stream.cuda_stream)
    torch.cuda.synchronize()
    shard.barrier(dist)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for k in range(args.steps):
        flush.fill_(k & 0xff)
        ev[k][0].record(stream)
        ctx.graph_launch(stream.cuda_stream)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    ms = float(np.sum([a.elapsed_time(b) for a, b in ev]))
    st = ctx.sync_stats()
    frame_ms = shard.max_over_ranks(ms, dist, dev) / args.steps
    mine_tests = torch.tensor([float(st["tri_tests"])], dtype=torch.float64, device=dev)
    dist.all_reduce(mine_tests)
    tests = float(mine_tests.item())
    rows = ctx.tri_pairs()
    out_rows = np.zeros(len(rows), shard.PAIR_ROW_DTYPE)
    out_rows["query"], out_rows["tri_a"], out_rows["tri_b"] = rows["query"], rows["tri_a"], rows["tri_b"]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    gathered = shard.gather_rows(out_rows, mine, dist, device=dev)
    gather_ms = 1e3 * (time.perf_counter() - t0)
    ctx.close()
    loads = np.array([costs[p].sum() for p in parts])
    return {"workload": "the scene of 256 rigid entities (seed 1002) split over the ranks by cost (LPT)",
            "scaling": "strong", "value": tests / (frame_ms / 1e3), "unit": UNIT, "ms_per_frame": frame_ms,
            "queries_per_rank": [int(len(p)) for p in parts], "load_spread": float(loads.max() / loads.min()),
            "gathered_pairs": int(len(gathered)), "gather_ms": gather_ms,
            "note": "unmeasured on hardware until a several-GPU run exists"}


def run_gpu(args) -> dict:
    import torch

    from inmyroom_vulkan_gb300 import capi, scenes, shard

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    # each rank collides its own scene replica (weak scaling, no data exchange)
    sc = scenes.scene(seed=1002 + 1000 * rank)
    ctx = capi.Context(device=local, max_queries=max(4096, len(sc.pairs)), max_tri_pairs=1 << 22)
    ids, tree_build = run_tree_build(ctx, sc, min(args.cpu_seconds, 5.0) if rank == 0 else 0.0, device=local)
    qa, qb = sc.pairs[:, 0], sc.pairs[:, 1]
    rel = np.stack([capi.relative_matrix(sc.mats[i], sc.mats[j]) for i, j in zip(qa, qb)])
    q = capi.make_queries(ids[qa], ids[qb], rel)
    n = len(q)

    d_q = torch.from_numpy(q.view(np.uint8).copy()).to(dev)
    torch.cuda.synchronize()
    # the scene with the FP64 determinant filter: near-threshold plane
    # distances rechecked in FP64 and counted, the reference's verdicts kept
    flags = capi.CG_CONTACTS | capi.CG_RECHECK
    # a dedicated stream: its handle is never 0, which the C ABI reads as
    # "the context's own stream"
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    tune = None
    if not args.no_tune:
        from inmyroom_vulkan_gb300 import autotune

        tune = autotune.tune_collide(ctx, d_q.data_ptr(), n, flags, flush=flush).as_dict()
    ctx.graph_capture(d_q.data_ptr(), n, flags)

    st = None
    for _ in range(max(args.warmup, 3)):
        ctx.graph_launch(stream.cuda_stream)
    st = ctx.sync_stats()
    tests_per_step, pairs_per_step, rays_per_step = st["tri_tests"], st["tri_pairs"], st["rays"]

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    trav_ms, narrow_ms = [], []
    torch.cuda.synchronize()
    shard.barrier(dist)
    with ClockSampler(local) as clocks:
        for k in range(args.steps):
            flush.fill_(k & 0xff)
            starts[k].record(stream)
            ctx.graph_launch(stream.cuda_stream)
            ends[k].record(stream)
            trav_ms.append(ctx.traversal_ms())
            narrow_ms.append(ctx.narrow_ms())
        torch.cuda.synchronize()
        shard.barrier(dist)
        step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
        st = ctx.sync_stats()
        assert st["tri_tests"] == tests_per_step and st["status"] == 0 and st["rays"] == rays_per_step

        # end to end through the public host API: host queries in; pairs, rays
        # and mean origins out, into pinned host memory, in one cg_collide call
        def pinned(count, dtype):
            return torch.empty(count * dtype.itemsize, dtype=torch.uint8).pin_memory().numpy().view(dtype)

        out_pairs = pinned(pairs_per_step, capi.TRI_PAIR_DTYPE)
        out_rays = pinned(rays_per_step, capi.RAY_DTYPE)
        out_avg = pinned(n, capi.RAY_AVERAGE_DTYPE)
        # the step graph itself writes the results into these buffers
        ctx.set_host_outputs(out_pairs, out_rays, out_avg)
        ctx.collide(q, flags=flags)  # captures cg_collide's step graph outside the timed region
        e2e_times = []
        for k in range(args.steps):
            flush.fill_(k & 0xff)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            st_e = ctx.collide(q, flags=flags)
            pairs = out_pairs[:st_e["tri_pairs"]]
            rays = out_rays[:st_e["rays"]]
            avgs = out_avg[:n]
            e2e_times.append(time.perf_counter() - t0)
        assert len(pairs) == pairs_per_step and len(rays) == rays_per_step and len(avgs) == n
        assert np.array_equal(pairs.view(np.uint8), ctx.tri_pairs().view(np.uint8))
    ctx.set_host_outputs()

    # the recheck's cost: the same step without it, event-timed the same way
    recheck = {"rechecked_per_step": int(st["rechecked"]), "disagreements_per_step": int(st["disagreements"]),
               "ms_per_step_with": float(np.mean(step_ms))}
    ctx.graph_capture(d_q.data_ptr(), n, capi.CG_CONTACTS)
    for _ in range(3):
        ctx.graph_launch(stream.cuda_stream)
    plain_steps = []
    for k in range(args.steps):
        flush.fill_(k & 0xff)
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        ctx.graph_launch(stream.cuda_stream)
        s1.record(stream)
        s1.synchronize()
        plain_steps.append(s0.elapsed_time(s1))
    st_plain = ctx.sync_stats()
    assert st_plain["tri_pairs"] == pairs_per_step and st_plain["rays"] == rays_per_step
    recheck["ms_per_step_without"] = float(np.mean(plain_steps))
    recheck["cost_ms"] = recheck["ms_per_step_with"] - recheck["ms_per_step_without"]
    # the slowest rank's times (every rank does a replica's fixed work)
    total_ms = shard.max_over_ranks(float(np.sum(step_ms)), dist, dev)
    value = world * tests_per_step * args.steps / (total_ms / 1e3)
    e2e_s = shard.max_over_ranks(float(np.sum(e2e_times)), dist, dev)
    e2e_value = world * tests_per_step * args.steps / e2e_s

    peaks = measured_peaks()
    sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
    fp32_peak = sm_count * 128 * 2 * peaks["sm_max_mhz"] * 1e6 / 1e12

    def kernel_roofline(name, ms, units, unit_bytes, unit_flops):
        by, fl = units * unit_bytes, units * unit_flops
        ach = by / (ms / 1e3) / 1e9
        return {"bound": "hbm", "achieved": ach, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": ach / peaks["hbm_gbs"], "traffic": profiled_traffic(name), "kernel": name, "kernel_ms": ms,
                "algorithmic_bytes": int(by), "peak_source": peaks["source"],
                "fp32": {"achieved_tflops": fl / (ms / 1e3) / 1e12, "peak_tflops": fp32_peak,
                         "frac": fl / (ms / 1e3) / 1e12 / fp32_peak}}

    roof_trav = kernel_roofline("traverse_kernel", float(np.mean(trav_ms)), st["node_pairs"], NODE_PAIR_BYTES,
                                NODE_PAIR_FLOPS)
    roof_narrow = kernel_roofline("narrow_kernel", float(np.mean(narrow_ms)), st["tri_tests"], TRI_TEST_BYTES,
                                  TRI_TEST_FLOPS)

    # plain path: the rigid pair, one query per launch (the reference's unit of work)
    rp = scenes.rigid_pair(n_poses=200)
    pid = [int(t) for t in ctx.build_trees([rp.mesh_a, rp.mesh_b])]
    prel = np.stack([capi.relative_matrix(a, b) for a, b in zip(rp.mats_a, rp.mats_b)])
    pq = capi.make_queries(np.full(200, pid[0]), np.full(200, pid[1]), prel)
    d_pq = torch.from_numpy(pq.view(np.uint8).copy()).to(dev)
    qsz = capi.QUERY_DTYPE.itemsize
    # one-query launches get settings of their own from the autotuner (the
    # scene's are put back afterwards)
    plain_tune = None
    if not args.no_tune:
        from inmyroom_vulkan_gb300 import autotune

        scene_settings = {k: int(getattr(ctx.config(), k)) for k in autotune.SPACE}
        plain_tune = autotune.tune_collide(ctx, d_pq.data_ptr(), 1, flags, flush=flush).as_dict()
    for i in range(5):
        ctx.collide_async(d_pq.data_ptr() + i * qsz, 1, flags, stream.cuda_stream)
    torch.cuda.synchronize()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    ptests = 0
    for i in range(200):
        ctx.collide_async(d_pq.data_ptr() + i * qsz, 1, flags, stream.cuda_stream)
    s1.record(stream)
    torch.cuda.synchronize()
    plain_ms = s0.elapsed_time(s1)
    ctx.collide(pq, flags=flags)
    ptests = ctx.sync_stats()["tri_tests"]
    if plain_tune:
        ctx.reconfigure(**scene_settings)

    shoot = None
    if rank == 0 and not args.skip_shoot:
        shoot = run_shoot(args, ctx, sc, ids, q, min(args.cpu_seconds, 5.0))
    frame_line = None
    if rank == 0 and not args.skip_frame:
        frame_line = run_frame(args, ctx, sc, ids, min(args.cpu_seconds, 5.0))
    cpu = cpu_baseline(sc, seconds=args.cpu_seconds) if rank == 0 and args.cpu_seconds > 0 else None
    deforming = None
    if rank == 0 and not args.skip_deforming:
        deforming = run_deforming(args, lambda: capi.Context(device=local, max_queries=4096, max_tri_pairs=1 << 22),
                                  flush, stream, min(args.cpu_seconds, 5.0))
    differentiable = None
    if rank == 0 and not args.skip_deforming:
        differentiable = run_differentiable(
            args, lambda: capi.Context(device=local, max_queries=4096, max_tri_pairs=1 << 22), flush, stream,
            min(args.cpu_seconds, 5.0))
    sweep = None
    if rank == 0 and not args.skip_sweep:
        sweep = run_sweep(args, local, flush, stream, min(args.cpu_seconds, 5.0))
    sharded = run_sharded(args, dist, rank, world, local, dev, stream, flush) if world > 1 else None
    clk = clocks.summary()
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded PCG64, seed 1002 + 1000*rank)",
        "config": scene_config(n, sum(m.n_tris for m in sc.meshes)),
        "work_per_step": {"tri_tests": int(tests_per_step), "rays": int(rays_per_step)},
        "step": {"launch": STEP_FLAGS_DOC, "colliding_pairs": int(pairs_per_step), "contacts": int(st["contacts"]),
                 "node_pairs": int(st["node_pairs"]), "lanes_per_traversal_step": st["node_pairs"] / max(1, st["warp_steps"]),
                 "autotune": tune},
        "recheck": recheck,
        "queries_per_s": world * n * args.steps / (total_ms / 1e3),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(n * capi.QUERY_DTYPE.itemsize),
                "d2h_bytes_per_step": int(COUNTERS_BYTES + pairs_per_step * capi.TRI_PAIR_DTYPE.itemsize
                                          + rays_per_step * capi.RAY_DTYPE.itemsize
                                          + n * capi.RAY_AVERAGE_DTYPE.itemsize),
                "ms_per_step": 1e3 * e2e_s / args.steps,
                "timing": "host perf_counter around one synchronous cg_collide (results written to pinned "
                          "host buffers by the step)"},
        "roofline": roof_trav,
        "roofline_narrow": roof_narrow,
        "plain": {"workload": "rigid pair, 2x2048 tris, 200 poses, one query per launch (with contacts and rays)",
                  "queries_per_s": 200 / (plain_ms / 1e3), "tri_tests_per_s": ptests / (plain_ms / 1e3),
                  "ms_per_query": plain_ms / 200, "autotune": plain_tune},
        "gpu_launches": STEP_KERNELS * args.steps,
        "clocks": clk,
    }
    if cpu:
        out["cpu_baseline"] = cpu
    if deforming:
        out["deforming"] = deforming
    if differentiable:
        out["differentiable"] = differentiable
    if sweep:
        out["batch_sweep"] = sweep
    if shoot:
        out["shoot"] = shoot
    if rank == 0:
        out["tree_build"] = tree_build
    if frame_line:
        out["frame"] = frame_line
    if sharded:
        out["sharded"] = sharded
    ctx.close()
    if dist:
        dist.destroy_process_group()
    return out if rank == 0 else None


def run_only(args) -> dict:
    """One secondary workload alone (for profiling it): its JSON object."""
    import torch

    from inmyroom_vulkan_gb300 import capi

    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    factory = lambda: capi.Context(max_queries=4096, max_tri_pairs=1 << 22)  # noqa: E731
    if args.only in ("shoot", "frame", "build"):
        from inmyroom_vulkan_gb300 import scenes

        sc = scenes.scene(seed=1002)
        ctx = capi.Context(max_queries=max(4096, len(sc.pairs)), max_tri_pairs=1 << 22)
        ids, line = run_tree_build(ctx, sc, 0.0)
        if args.only == "build":
            return line
        if args.only == "frame":
            return run_frame(args, ctx, sc, ids, 0.0)
        qa, qb = sc.pairs[:, 0], sc.pairs[:, 1]
        rel = np.stack([capi.relative_matrix(sc.mats[i], sc.mats[j]) for i, j in zip(qa, qb)])
        return run_shoot(args, ctx, sc, ids, capi.make_queries(ids[qa], ids[qb], rel), 0.0)
    if args.only == "deforming":
        return run_deforming(args, factory, flush, stream, 0.0)
    if args.only == "differentiable":
        return run_differentiable(args, factory, flush, stream, 0.0)
    return run_sweep(args, 0, flush, stream, 0.0)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--skip-deforming", action="store_true", help="leave out the deforming and differentiable lines")
    ap.add_argument("--skip-sweep", action="store_true", help="leave out the autotuned batch-sweep line")
    ap.add_argument("--no-tune", action="store_true", help="time the scene step with the default launch settings")
    ap.add_argument("--skip-shoot", action="store_true", help="leave out the uncollide-ray shooting line")
    ap.add_argument("--skip-frame", action="store_true", help="leave out the collision-frame line")
    ap.add_argument("--only", choices=["deforming", "differentiable", "sweep", "shoot", "frame", "build"],
                    help="run one secondary workload alone and print its object (for profiling)")
    args = ap.parse_args()
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        print(json.dumps(run_reference(args)))
        return
    if args.only:
        print(json.dumps(run_only(args)))
        return
    res = run_gpu(args)
    if res is not None:
        print(json.dumps(res))


if __name__ == "__main__":
    main()
