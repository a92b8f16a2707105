"""Oracle (test infrastructure, NOT part of the product): one frame of
CollisionDetection::ExecuteCollisionDetection
(inMyRoom_vulkan/src/CollisionDetection/CollisionDetection.cpp:38-103) composed
from an implementation's pieces (the port's or the compiled reference's):
SweepAndPrune, the OBB-tree mid phase, CreateUncollideRays and
ShootUncollideRays, then the split of the delta by each entity's movement
between frames. The ancestor fan-out (:106-124) needs the engine's entity
tree and is left out: the result is one record per broad pair with rays.
"""
from __future__ import annotations

import numpy as np

f32 = np.float32


def _xform(m, p):
    """glm mat4 * vec4(p, 1) in the shim's order ((c0 x + c1 y) + (c2 z + c3))."""
    c = np.asarray(m, f32).reshape(4, 4)
    return ((c[0, :3] * p[0] + c[1, :3] * p[1]) + (c[2, :3] * p[2] + c[3, :3] * f32(1.0))).astype(f32)


def point_movement(p, current, previous) -> np.float32:
    """CollisionDetection::PointMovementBetweenFrames (CollisionDetection.cpp:143-151)."""
    p = np.asarray(p, f32)
    d = (_xform(current, p) - _xform(previous, p)).astype(f32)
    return np.sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2], dtype=f32)


def collision_frame(impl, trees, current, previous, callback=None, params=None, map_fn=map):
    """Records (first, second, first_delta (3,), second_delta (3,)) for every
    broad pair whose mid phase collides and which makes rays
    (CollisionDetection.cpp:44-66), deltas per :74-103. map_fn runs the
    per-pair work (a thread pool's map spreads it over host cores)."""
    n = len(trees)
    if n < 2:  # CollisionDetection.cpp:40
        return []
    current = np.asarray(current, f32).reshape(n, 16)
    previous = np.asarray(previous, f32).reshape(n, 16)
    pairs = impl.sweep_and_prune(trees, current, callback)

    def one(pair):
        a, b = int(pair[0]), int(pair[1])
        mid = impl.mid_phase(trees[a], trees[b], current[a], current[b])
        if not len(mid.leaf_pairs()):
            return None
        ra, rb, avg = mid.rays()
        if not len(ra) and not len(rb):
            return None
        moved = not (np.array_equal(current[a], previous[a]) and np.array_equal(current[b], previous[b]))
        d1 = d2 = np.zeros(3, f32)
        if moved:
            delta = impl.shoot_rays(trees[a], trees[b], current[a], current[b], ra, rb,
                                    None if params is None else np.asarray(params, f32))
            with np.errstate(invalid="ignore", divide="ignore"):
                m1 = point_movement(avg[:3], current[a], previous[a])
                m2 = point_movement(avg[3:], current[b], previous[b])
                total = f32(m1 + m2)
                d1 = (-delta * f32(m1 / total)).astype(f32)
                d2 = (delta * f32(m2 / total)).astype(f32)
        return a, b, d1, d2

    return [r for r in map_fn(one, list(pairs)) if r is not None]


def as_arrays(records):
    """(k, 2) uint32 pairs and (k, 6) float32 deltas, sorted by pair."""
    if not records:
        return np.zeros((0, 2), np.uint32), np.zeros((0, 6), f32)
    p = np.array([(r[0], r[1]) for r in records], np.uint32)
    d = np.array([np.concatenate([r[2], r[3]]) for r in records], f32)
    o = np.lexsort((p[:, 1], p[:, 0]))
    return p[o], d[o]


def ancestors(entity: int, parent) -> list:
    """EntitiesHandler::GetEntityAncestors (src/ECS/EntitiesHandler.cpp:186-204):
    the root (entity 0) down to the entity."""
    out = [entity]
    while entity != 0:
        entity = int(parent[entity])
        out.append(entity)
    return out[::-1]


def fan_out(records, entity_ids, parent) -> dict:
    """CollisionDetection.cpp:104-124: receiver -> [(family, collide_with,
    delta)] in record order, for records (first, second, first_delta,
    second_delta) over frame entity indices."""
    calls: dict = {}
    for a, b, d1, d2 in records:
        fa, fb = int(entity_ids[a]), int(entity_ids[b])
        A, B = ancestors(fa, parent), ancestors(fb, parent)
        for mine, other, fam, with_, d in ((A, B, fa, fb, d1), (B, A, fb, fa, d2)):
            for i, e in enumerate(mine):
                if i >= len(other) or other[i] != e:
                    calls.setdefault(e, []).append((fam, with_, tuple(np.asarray(d, f32).tolist())))
    return calls
