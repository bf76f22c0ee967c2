"""Validated rotations in the oracle (orc_rotate_enclosed): the restatement
of rotate_product with validated = 1 and caller-supplied c, s, rc, rs.

The reference runs validated mode only with MPFR (engine/src/tpgp_rev.c:
484-527), which this image lacks, so its validated outputs cannot be
produced here.  The restatement is anchored on the pinned pieces instead:
keys, values and the dropped sums equal the plain rotation's (orc_rotate,
pinned to the reference engine's golden rotations), and each child's radius
is the one the reference's CUDA branch computes with enclose = 1 (orc_branches,
pinned to the reference's test_cuda_rev.c cases); what is left, the merge of
radii and the upper L2 of the merged radii (tpgp_rev.c:57-62, 699-712), is
checked here on maps whose merged radii can be written down.
"""
import math

import numpy as np
import pytest

from ddevol_gb300 import hamiltonians as H

pytest.importorskip("ctypes")


def up_add(a, b):
    if a == 0.0:
        return b
    if b == 0.0:
        return a
    return math.nextafter(a + b, math.inf)


def up_mul(a, b):
    if a == 0.0 or b == 0.0:
        return 0.0
    return math.nextafter(a * b, math.inf)


def upper_l2(values):
    s = 0.0
    for v in values:
        s = up_add(s, up_mul(v, v))
    return 0.0 if s == 0.0 else math.nextafter(math.sqrt(s), math.inf)


def random_map(rng, n, count):
    words = (n + 31) // 32
    keys = set()
    while len(keys) < count:
        k = 0
        for s in rng.choice(n, size=int(rng.integers(1, 6)), replace=False):
            k |= int(rng.integers(1, 4)) << (2 * int(s))
        keys.add(k)
    keys = sorted(keys)
    arr = np.array([[(k >> (64 * w)) & ((1 << 64) - 1) for w in range(words)] for k in keys],
                   dtype=np.uint64).reshape(-1)
    vals = rng.standard_normal(len(keys)) * 10.0 ** rng.uniform(-4, 0, len(keys))
    return arr, vals


@pytest.mark.parametrize("n", [16, 40, 70])
def test_keys_values_and_dropped_sums_are_the_plain_rotations(oracle, n):
    rng = np.random.default_rng(n)
    keys, vals = random_map(rng, n, 400)
    for _ in range(6):
        i, j = (int(x) for x in rng.choice(n, 2, replace=False))
        qi, qj = int(rng.integers(0, 4)), int(rng.integers(0, 4))
        h, dur = float(rng.uniform(-1, 1)), 0.05
        c, s = oracle.trig(h, dur)
        st_a, ka, va, la = oracle.rotate(keys, vals, n, i, j, qi, qj, h, dur, threshold=1e-4)
        st_b, kb, vb, lb = oracle.rotations_enclosed(keys, vals, n, [(i, j, qi, qj, c, s, 3e-17, 2e-17)],
                                                     threshold=1e-4)
        assert st_a == st_b == 0
        assert np.array_equal(ka, kb) and np.array_equal(va.view(np.uint64), vb.view(np.uint64))
        for f in ("dropped_l1", "dropped_l2", "dropped_l2_squared", "rotations", "removal_events",
                  "peak_terms"):
            assert getattr(la, f) == getattr(lb, f), f
        keys, vals = kb, vb
    assert lb.arithmetic_l2 > 0 and lb.arithmetic_enclosed == 0


def test_single_pair_merged_radii(oracle):
    """One anticommuting key alone: each output key has one contribution, so
    the merged radii are the two child radii of the CUDA branch (enclose = 1)
    and arithmetic_l2 is their upper L2 in key order."""
    n = 8
    keys = np.array([1 << 2], dtype=np.uint64)      # X on site 1
    vals = np.array([0.7])
    c, s, rc, rs = 0.8, 0.6, 1e-16, 3e-16
    # generator Z0 Z1: anticommutes with X1 (site 1), commutes on site 0
    st, ok, ov, orad = oracle.branches(keys, vals, n, 0, 1, 3, 3, c, s, rc, rs, enclose=1)
    assert st == 0
    st, k, v, led = oracle.rotations_enclosed(keys, vals, n, [(0, 1, 3, 3, c, s, rc, rs)])
    assert st == 0
    order = np.argsort(ok.astype(np.uint64))  # one word: key order
    assert led.arithmetic_l2 == upper_l2([float(orad[p]) for p in order])


def test_two_contributions_add_the_sum_radius(oracle):
    """A pair of live keys K, P = K xor Q: each output key gets its cos child
    and the partner's sin child; the merged radius adds the two child radii
    and the rounding radius of the sum."""
    n = 8
    K, P = (1 << 2), (1 << 2) ^ (3 | (3 << 2))  # X1 and K xor (Z0 Z1)
    keys = np.array(sorted([K, P]), dtype=np.uint64)
    vals = np.array([0.7, -0.3] if keys[0] == K else [-0.3, 0.7])
    c, s, rc, rs = 0.8, 0.6, 1e-16, 3e-16
    st, ok, ov, orad = oracle.branches(keys, vals, n, 0, 1, 3, 3, c, s, rc, rs, enclose=1)
    assert st == 0
    merged = {}
    for p in range(4):
        key = int(ok[p])
        if key not in merged:
            merged[key] = [float(ov[p]), float(orad[p]), 1]
        else:
            prev = merged[key][0]
            merged[key][0] = prev + float(ov[p])
            merged[key][1] = up_add(merged[key][1], float(orad[p]))
            if prev != 0 and float(ov[p]) != 0:
                x = merged[key][0]
                rr = max(abs(math.nextafter(x, math.inf) - x), abs(x - math.nextafter(x, -math.inf)))
                merged[key][1] = up_add(merged[key][1], rr)
    want = upper_l2([merged[k][1] for k in sorted(merged)])
    st, k, v, led = oracle.rotations_enclosed(keys, vals, n, [(0, 1, 3, 3, c, s, rc, rs)])
    assert st == 0 and led.arithmetic_l2 == want


def test_statuses(oracle):
    k0, v0 = H.global_x_operator(8)
    good = (0, 1, 3, 3, 0.8, 0.6, 1e-16, 1e-16)
    assert oracle.rotations_enclosed(k0, v0, 8, [good, (0, 0, 3, 3, 0.8, 0.6, 0, 0)])[0] == 1
    assert oracle.rotations_enclosed(k0, v0, 8, [(0, 1, 3, 3, 0.8, 0.6, -1e-16, 0)])[0] == 1
    assert oracle.rotations_enclosed(k0, v0, 8, [(0, 1, 3, 3, 0.8, 0.6, 1e100, 0)])[0] == 0
    # finite radii whose squares overflow: the ledger's upper L2 is not finite
    assert oracle.rotations_enclosed(k0, v0, 8, [(0, 1, 3, 3, 0.8, 0.6, 1e300, 0)])[0] == 4
    big = np.full(len(v0), 1e300)
    assert oracle.rotations_enclosed(k0, big, 8, [(0, 1, 3, 3, 0.8, 0.6, 1e300, 0)])[0] == 4
    st, k, v, led = oracle.rotations_enclosed(k0[:0], v0[:0], 8, [good])
    assert st == 0 and led.rotations == 0
