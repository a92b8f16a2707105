"""Failure paths of the collide step on the GPU, each ending in a normal
return with the error status and a context that stays usable.

* CG_ERR_TIMEOUT: every device-side wait is bounded by wait_limit_ms. One
  heavy query (two overlapping 32,768-triangle spheres) whose first warp never
  donates work (donate_min at its maximum) keeps that warp busy for several
  milliseconds while every other warp waits for work: with wait_limit_ms = 1
  their waits run out, they record the timeout and return; the busy warp
  finishes its own work and returns.
* CG_ERR_QUEUE_OVERFLOW: the same query with a 256-entry warp stack and the
  smallest work queue (64 chunks): a warp whose stack fills must donate, the
  queue runs out of chunks, the warp records the overflow and stops.
After each, the next call on the same context (a light batch) returns the
oracle's colliding pairs bit for bit, and so does the heavy query once the
settings are back to the defaults."""
import numpy as np
import pytest

from inmyroom_vulkan_gb300 import capi, scenes

pytestmark = pytest.mark.gpu


def rows(p):
    t = np.concatenate([np.stack([p["query"], p["tri_a"], p["tri_b"]], 1).astype(np.uint32),
                        np.ascontiguousarray(np.concatenate([p["source"], p["target"]], 1), np.float32).view(np.uint32)],
                       1)
    return t[np.lexsort(t.T[::-1])] if len(t) else t


def port_rows(pairs, segs):
    t = np.concatenate([pairs.astype(np.uint32), np.ascontiguousarray(segs, np.float32).view(np.uint32)], 1)
    return t[np.lexsort(t.T[::-1])] if len(t) else t


@pytest.fixture(scope="module")
def workloads(port):
    rng = np.random.Generator(np.random.PCG64(5))
    big = [scenes.octa_sphere(6, 1.0, 0.01, rng) for _ in range(2)]
    small = scenes.rigid_pair(n_poses=32, subdiv=3)
    return big, small


def check_light(ctx, port, small, ids):
    rel = np.stack([capi.relative_matrix(a, b) for a, b in zip(small.mats_a, small.mats_b)])
    st = ctx.collide(capi.make_queries(np.full(len(rel), ids[0]), np.full(len(rel), ids[1]), rel))
    assert st["status"] == 0
    ta, tb = (port.tree_build(m.points, m.indices, m.normals) for m in (small.mesh_a, small.mesh_b))
    pairs, segs, tests, _ = port.collide_pairs([ta] * len(rel), [tb] * len(rel), small.mats_a, small.mats_b)
    assert st["tri_tests"] == tests and len(pairs) > 100
    assert np.array_equal(rows(ctx.tri_pairs()), port_rows(pairs, segs))


@pytest.mark.parametrize("case", ["timeout", "queue"])
def test_bounded_failure_then_usable(port, workloads, case):
    big, small = workloads
    if case == "timeout":
        settings = dict(wait_limit_ms=1, stack_entries=4096, donate_min=4096)
        want = capi.CG_ERR_TIMEOUT
    else:
        settings = dict(stack_entries=256, queue_capacity=1024)
        want = capi.CG_ERR_QUEUE_OVERFLOW
    with capi.Context(**settings) as ctx:
        bid = [int(t) for t in ctx.build_trees(big)]
        sid = [int(t) for t in ctx.build_trees([small.mesh_a, small.mesh_b])]
        eye = np.eye(4, dtype=np.float32).reshape(16)
        heavy = capi.make_queries([bid[0]], [bid[1]], capi.relative_matrix(eye, eye)[None])
        st = ctx.collide(heavy, flags=capi.CG_MID_ONLY, check=False)
        assert st["rc"] == want, (st, ctx.last_error())
        assert st["status"] == want
        # the same context, a light batch: the oracle's pairs
        check_light(ctx, port, small, sid)
        # defaults again: the heavy query completes
        d = capi.default_config()
        ctx.reconfigure(**{k: getattr(d, k) for k in settings})
        st = ctx.collide(heavy, flags=capi.CG_MID_ONLY)
        assert st["status"] == 0 and st["leaf_pairs"] > 50000
        ta, tb = (port.tree_build(m.points, m.indices, m.normals) for m in big)
        assert st["leaf_pairs"] == len(port.mid_phase(ta, tb, eye, eye).leaf_pairs())
