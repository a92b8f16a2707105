"""The method of the tree build's large-node coordinate sums, restated on the
CPU (build_sums_big_kernel in csrc/cg_build.cu): the sequential FP64 sum of
float terms (OBB.cpp:53-55, std::accumulate from +0) replayed exactly in
integer counts of 2^q, q the smallest exponent of the terms' ulps. The running
sums are exact until the first one that is not a double; that add is the
first that rounds, and its rounded value (to nearest, ties to even) is the
next start. A sum whose exponents span too far for 64-bit counts, or that
rounds more than 64 times, is left to the sequential chain.

Checked against numpy's sequential float64 accumulation (bit for bit, the
sign of zero included) on terms that round never, a few times and too often,
on signed zeros, and on the 256-entity scene's three coordinates whose root
sums do round. The device kernel itself is pinned by
tests/test_gpu_build.py (whole trees bit-identical to the reference's)."""
import numpy as np
import pytest

MAX_ROUNDS = 64


def fits_double(count: int) -> bool:
    if count == 0:
        return True
    m = abs(count)
    return m.bit_length() - ((m & -m).bit_length() - 1) <= 53


def round_double(count: int) -> int:
    if fits_double(count):
        return count
    m = abs(count)
    d = m.bit_length() - 53
    k, rem, half = m >> d, m & ((1 << d) - 1), 1 << (d - 1)
    if rem > half or (rem == half and k & 1):
        k += 1
    return (k << d) * (-1 if count < 0 else 1)


def replayed_sum(terms: np.ndarray):
    """(sum, roundings) as the kernel computes it, or (None, reason)."""
    x = terms.astype(np.float32).astype(np.float64)
    nz = x[x != 0]
    if len(nz) == 0:
        return 0.0, 0
    bits = nz.view(np.int64)
    e = ((bits >> 52) & 0x7FF) - 1023
    q = int((np.maximum(e, -126) - 23).min())
    emax = int(e.max())
    lg = int(np.ceil(np.log2(len(x)))) if len(x) > 1 else 0
    if not (emax < 1024 and lg + emax + 1 - q <= 62):
        return None, "span"
    units = [0 if v == 0 else int(np.ldexp(v, -q)) for v in x.tolist()]  # exact: integers below 2^62
    start, k0, rounds = 0, 0, 0
    while k0 < len(units):
        r, hit = start, None
        for j in range(k0, len(units)):
            r += units[j]
            if not fits_double(r):
                hit = j
                break
        if hit is None:
            start = r
            break
        start, k0, rounds = round_double(r), hit + 1, rounds + 1
        if rounds > MAX_ROUNDS:
            return None, "rounds"
    return float(np.ldexp(float(start), q)), rounds


def sequential(terms: np.ndarray) -> float:
    return float(np.add.accumulate(terms.astype(np.float32).astype(np.float64), dtype=np.float64)[-1] + 0.0)


def same(a: float, b: float) -> bool:
    return a == b and np.signbit(a) == np.signbit(b)


def test_rounding_cases():
    rng = np.random.default_rng(7)
    seen = {"exact": 0, "rounded": 0, "span": 0, "rounds": 0}
    for t in range(240):
        n = int(rng.integers(300, 3000))
        x = rng.standard_normal(n)
        if t % 3 == 0:  # values near 20 and a few near 2^-20: the sum rounds now and then
            x = x + 20.0
            sel = rng.random(n) < rng.choice([0.002, 0.01, 0.05])
            x[sel] = (1.0 + rng.random(sel.sum())) * 2.0 ** -20
        elif t % 3 == 1:  # magnitudes 2^-30 .. 2^30 apart: counts would not fit 64 bits
            x = x * 2.0 ** rng.uniform(-30, 30, n)
        x = x.astype(np.float32)
        s, info = replayed_sum(x)
        if s is None:
            seen[info] += 1
            continue
        seen["rounded" if info else "exact"] += 1
        assert same(s, sequential(x)), (t, info)
    assert all(v > 0 for v in seen.values()), seen


def test_zeros_and_signs():
    for x in ([0.0, -0.0, 0.0], [-0.0, -0.0], [1.5, -1.5], [-2.0 ** -149, 2.0 ** -149, -0.0]):
        x = np.array(x, np.float32)
        s, _ = replayed_sum(x)
        assert same(s, sequential(x)), x


@pytest.mark.parametrize("mesh,coord", [(88, 2), (106, 2), (169, 1)])
def test_scene_sums_that_round(mesh, coord):
    """The scene's root sums that round (6, 6 and 11 times): replayed, not
    chained, and equal to the sequential sum."""
    from inmyroom_vulkan_gb300 import scenes

    m = scenes.scene().meshes[mesh]
    x = m.points[m.indices.reshape(-1)][:, coord]
    s, rounds = replayed_sum(x)
    assert s is not None and 0 < rounds <= MAX_ROUNDS
    assert same(s, sequential(x))
