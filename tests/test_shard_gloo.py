"""The several-GPU path's host logic on the CPU: two ranks over gloo shard the
256-entity scene's queries by cost (LPT), each collides its shard with the
oracle standing in for its device, and the gathered colliding pairs (fixed
rows through all_gather_into_tensor) equal the whole frame's; the loads are
within LPT's bound; the timing rule takes the slowest rank. No device
involved."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from inmyroom_vulkan_gb300 import shard


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


PAIR_DTYPE = shard.PAIR_ROW_DTYPE


def scene_queries():
    from inmyroom_vulkan_gb300 import scenes

    sc = scenes.scene()
    keep = (sc.pairs[:, 0] < 96) & (sc.pairs[:, 1] < 96)
    return sc, sc.pairs[keep]


def collide_rows(port, trees, sc, pairs) -> np.ndarray:
    qa, qb = pairs[:, 0], pairs[:, 1]
    got, _, _, _ = port.collide_pairs([trees[i] for i in qa], [trees[j] for j in qb], sc.mats[qa], sc.mats[qb])
    rows = np.zeros(len(got), PAIR_DTYPE)
    rows["query"], rows["tri_a"], rows["tri_b"] = got[:, 0], got[:, 1], got[:, 2]
    return rows


def rank_main(rank, world, port_no, out_dir):
    import torch.distributed as dist

    import oracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port_no)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sc, pairs = scene_queries()
    port = oracle.port()
    used = np.unique(pairs)
    trees = {int(i): port.tree_build(sc.meshes[i].points, sc.meshes[i].indices, sc.meshes[i].normals) for i in used}
    costs = shard.query_costs([sc.meshes[i].n_tris for i in pairs[:, 0]], [sc.meshes[j].n_tris for j in pairs[:, 1]])
    parts = shard.lpt_partition(costs, world)
    mine = parts[rank]
    rows = collide_rows(port, trees, sc, pairs[mine])
    shard.barrier(dist)
    allrows = shard.gather_rows(rows, mine, dist)
    slowest = shard.max_over_ranks(float(rank + 1), dist)
    if rank == 0:
        np.save(os.path.join(out_dir, "gathered.npy"), allrows)
        np.save(os.path.join(out_dir, "slowest.npy"), np.array([slowest]))
        np.save(os.path.join(out_dir, "loads.npy"), np.array([costs[p].sum() for p in parts]))
    dist.destroy_process_group()


def test_lpt_partition_covers_and_balances():
    rng = np.random.default_rng(0)
    costs = rng.lognormal(size=1000)
    for world in (1, 2, 3, 8):
        parts = shard.lpt_partition(costs, world)
        assert np.array_equal(np.sort(np.concatenate(parts)), np.arange(1000))
        loads = np.array([costs[p].sum() for p in parts])
        assert loads.max() - loads.min() <= costs.max() + 1e-9  # LPT's bound: within one job
        assert all(np.array_equal(a, b) for a, b in zip(parts, shard.lpt_partition(costs, world)))
    assert [len(p) for p in shard.lpt_partition([], 2)] == [0, 0]


def test_two_ranks_gloo(tmp_path):
    port_no = free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=rank_main, args=(r, 2, port_no, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    import oracle

    sc, pairs = scene_queries()
    port = oracle.port()
    used = np.unique(pairs)
    trees = {int(i): port.tree_build(sc.meshes[i].points, sc.meshes[i].indices, sc.meshes[i].normals) for i in used}
    want = collide_rows(port, trees, sc, pairs)
    got = np.load(tmp_path / "gathered.npy")
    key = lambda r: np.lexsort((r["tri_b"], r["tri_a"], r["query"]))  # noqa: E731
    assert len(want) > 1000 and np.array_equal(got[key(got)], want[key(want)])
    assert float(np.load(tmp_path / "slowest.npy")[0]) == 2.0
    loads = np.load(tmp_path / "loads.npy")
    costs = shard.query_costs([sc.meshes[i].n_tris for i in pairs[:, 0]], [sc.meshes[j].n_tris for j in pairs[:, 1]])
    assert loads.max() - loads.min() <= costs.max()  # LPT's bound: the ranks' loads differ by at most one query
