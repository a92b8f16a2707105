"""Several GPUs, one process each: the collide path's queries are independent
(entity pairs or poses, no exchange step), so a frame shards by query.

* `lpt_partition`: queries to ranks by estimated cost, longest first onto the
  least-loaded rank (cost = triangles of A x triangles of B, the bound on its
  triangle tests); every rank computes the same partition from the same
  inputs, so no message is needed to agree on it.
* `gather_rows`: the ranks' result rows (colliding pairs, rays) to every rank
  once per frame, in rank order, with the query indices mapped back to the
  frame's numbering: fixed-width rows as bytes through
  all_gather_into_tensor (the counts first, then the rows padded to the
  largest count).
* `max_over_ranks` / `barrier`: the timing rule of the bench (the slowest
  rank's time).

The trees a shard needs are built on its own device (`Context.build_trees`);
nothing on the data path is exchanged.
"""
from __future__ import annotations

import heapq

import numpy as np


def query_costs(tris_a, tris_b) -> np.ndarray:
    """Cost of each query: |A| x |B| triangles."""
    return np.asarray(tris_a, np.float64) * np.asarray(tris_b, np.float64)


def lpt_partition(costs, world: int) -> list[np.ndarray]:
    """Longest-processing-time-first: query indices per rank, each in
    ascending order. Ties (equal costs, equal loads) go by query index and
    rank index, so the result is deterministic."""
    costs = np.asarray(costs, np.float64)
    order = np.lexsort((np.arange(len(costs)), -costs))
    heap = [(0.0, r) for r in range(world)]
    parts: list[list[int]] = [[] for _ in range(world)]
    for q in order:
        load, r = heapq.heappop(heap)
        parts[r].append(int(q))
        heapq.heappush(heap, (load + float(costs[q]), r))
    return [np.array(sorted(p), np.int64) for p in parts]


PAIR_ROW_DTYPE = np.dtype([("query", "<i8"), ("tri_a", "<u4"), ("tri_b", "<u4")])


def gather_rows(rows: np.ndarray, shard: np.ndarray, dist, query_field: str = "query", device=None) -> np.ndarray:
    """All ranks' structured result rows (one fixed dtype), rank by rank; each
    rank's `query_field` (an index into its shard) becomes the frame's query
    index. `device`: where the collective's tensors live (the rank's GPU for
    NCCL, None for gloo)."""
    import torch

    rows = np.ascontiguousarray(rows).copy()
    if len(rows):
        rows[query_field] = shard[rows[query_field]]
    if dist is None:
        return rows
    world = dist.get_world_size()
    width = rows.dtype.itemsize
    counts = torch.empty(world, dtype=torch.int64, device=device)
    dist.all_gather_into_tensor(counts, torch.tensor([len(rows)], dtype=torch.int64, device=device))
    counts = counts.cpu().numpy()
    cap = max(int(counts.max()), 1)
    buf = np.zeros(cap * width, np.uint8)
    buf[:len(rows) * width] = rows.view(np.uint8).reshape(-1)
    out = torch.empty(world * cap * width, dtype=torch.uint8, device=device)
    dist.all_gather_into_tensor(out, torch.from_numpy(buf).to(device))
    out = out.cpu().numpy().reshape(world, cap * width)
    return np.concatenate([out[r, :int(counts[r]) * width].view(rows.dtype) for r in range(world)])


def max_over_ranks(x: float, dist, device=None) -> float:
    """The largest value over the ranks (the bench's timing rule)."""
    if dist is None:
        return float(x)
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist) -> None:
    if dist is not None:
        dist.barrier()
