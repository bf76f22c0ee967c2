"""The warp-parallel upward sum (tpgp_gb_upward_sums) against the sequential
upadd chain of the reference (engine/src/tpgp_rev.c:25-36: nextafter(a + b,
+inf), a zero operand returning the other), bit for bit.

The device computes a chain 32 addends at a time as integer grid steps
within a binade and falls back to a sequential step at binade crossings,
ties (an addend of exactly half a grid step), subnormal or zero running
sums and nonfinite values; these cases are planted here: half-ulp addends,
subnormals, zeros, magnitudes across the whole exponent range, overflow to
infinity and chains of every length around the warp width.  This kernel
carries the exact ledger's per-rotation sums and the step's ledger commit.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def up_add(a, b):
    if a == 0.0:
        return b
    if b == 0.0:
        return a
    return math.nextafter(a + b, math.inf)


def chains(x, chain):
    out = []
    for c in range(0, len(x), chain):
        s = 0.0
        for v in x[c:c + chain]:
            s = up_add(s, float(v))
        out.append(s)
    return np.array(out)


def mixed(rng, n):
    kind = rng.integers(0, 7, n)
    x = np.empty(n)
    x[kind == 0] = rng.uniform(1e-12, 1e-5, (kind == 0).sum())
    x[kind == 1] = 2.0 ** rng.integers(-80, -5, (kind == 1).sum())
    x[kind == 2] = 3 * 2.0 ** rng.integers(-90, -20, (kind == 2).sum())
    x[kind == 3] = rng.integers(1, 5000, (kind == 3).sum()) * 5e-324  # subnormals
    x[kind == 4] = 0.0
    x[kind == 5] = 10.0 ** rng.uniform(-300, 300, (kind == 5).sum())
    x[kind == 6] = rng.uniform(0, 1, (kind == 6).sum()) ** 8
    return x


@pytest.mark.parametrize("chain", [1, 31, 32, 33, 64, 1000, 4096])
def test_mixed_chains(engine, chain):
    rng = np.random.default_rng(chain)
    x = mixed(rng, 40 * chain + 7)
    got = engine.upward_sums(x, chain)
    want = chains(x, chain)
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))


def test_half_ulp_ties(engine):
    """Sums sitting on a binade with addends of exactly half a grid step (or
    odd multiples of it): round-half-even decides by the sum's last bit."""
    rng = np.random.default_rng(7)
    chain = 96
    x = []
    for c in range(200):
        x.append(1.0 + int(rng.integers(0, 1 << 30)) * 2.0 ** -52)
        x += list(2.0 ** -53 * rng.choice([1, 3, 5, 0.5, 1.5, 2, 7], chain - 1))
    x = np.array(x)
    got = engine.upward_sums(x, chain)
    assert np.array_equal(got.view(np.uint64), chains(x, chain).view(np.uint64))


def test_removed_weights_like_the_ledger(engine):
    """Addends like the threshold's removed |v| (below 1e-5, long chains):
    the case the exact ledger runs at scale."""
    rng = np.random.default_rng(11)
    x = np.abs(rng.standard_normal(300_000)) * 10.0 ** rng.uniform(-12, -5, 300_000)
    got = engine.upward_sums(x, 60_000)
    assert np.array_equal(got.view(np.uint64), chains(x, 60_000).view(np.uint64))


def test_overflow_to_infinity(engine):
    x = np.array([1e308, 1e308, 1.0, 1e300] * 20)
    got = engine.upward_sums(x, 40)
    want = chains(x, 40)
    assert np.all(np.isinf(got)) and np.array_equal(got.view(np.uint64), want.view(np.uint64))
