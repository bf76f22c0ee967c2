"""Validated rotations on the device (tpgp_gb_rotate_enclosed) against the
oracle's restatement (orc_rotations_enclosed), bitwise: keys, values and
every ledger field, arithmetic_l2 included.

The merged radii are logged per rotation with the exact ledger's removed
terms (tagged), sorted by key with them and added in key order, so the
cases cover maps of one to four key words, pairs with both members live,
children that are exactly zero (c = 0), pure radius growth (c = 1, s = 0),
zero factor radii (rounding radii only), a 10^5-term map whose segments run
past one shared-memory tile, and the statuses (invalid rotation after valid
ones, nonfinite radii, empty map).
"""
import os

import numpy as np
import pytest

from ddevol_gb300.engine import GbLedger, options
from gpu_helpers import bits, ledger_vec, random_map

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def random_rotations(rng, n, count, c_s=None):
    out = []
    for _ in range(count):
        i, j = (int(x) for x in rng.choice(n, 2, replace=False))
        qi, qj = int(rng.integers(1, 4)), int(rng.integers(0, 4))
        if c_s is None:
            x = float(rng.uniform(-0.2, 0.2))
            c, s = float(np.cos(x)), float(np.sin(x))
        else:
            c, s = c_s
        rc = float(rng.choice([0.0, 1.1e-16, 3e-17]))
        rs = float(rng.choice([0.0, 2.2e-16, 5e-18]))
        out.append((i, j, qi, qj, c, s, rc, rs))
    return out


def check(engine, oracle, n, keys, vals, rots, threshold):
    m = engine.map(n, keys, vals)
    st, led, msg = m.rotate_enclosed(rots, options(threshold))
    k, v = m.download()
    m.close()
    ost, ok, ov, oled = oracle.rotations_enclosed(keys, vals, n, rots, threshold=threshold)
    assert st == ost, (st, ost, msg)
    if st == 0:
        assert np.array_equal(k, ok)
        assert np.array_equal(bits(v), bits(ov))
        assert np.array_equal(bits(ledger_vec(led)), bits(ledger_vec(oled)))
    return st, led


@pytest.mark.parametrize("n_spins", [24, 60, 90, 120])
def test_random_maps_match_the_oracle(engine, oracle, n_spins):
    rng = np.random.default_rng(7 + n_spins)
    keys, vals = random_map(rng, n_spins, 3000)
    st, led = check(engine, oracle, n_spins, keys, vals, random_rotations(rng, n_spins, 24), 1e-4)
    assert st == 0 and led.arithmetic_l2 > 0 and led.removal_events > 0


@pytest.mark.parametrize("c_s", [(0.0, 1.0), (1.0, 0.0), (-0.6, 0.8)])
def test_edge_factors(engine, oracle, c_s):
    rng = np.random.default_rng(3)
    keys, vals = random_map(rng, 40, 2000)
    st, led = check(engine, oracle, 40, keys, vals, random_rotations(rng, 40, 10, c_s), 1e-5)
    assert st == 0


def test_window_map(engine, oracle):
    """The 10^5-term ring64 window state, six all-pairs rotations."""
    z = np.load(os.path.join(GOLDEN, "ring64_window.npz"))
    rng = np.random.default_rng(5)
    rots = []
    for _ in range(6):
        i, j = (int(x) for x in rng.choice(64, 2, replace=False))
        q = int(rng.integers(1, 4))
        rots.append((i, j, q, q, float(np.cos(0.01)), float(np.sin(0.01)), 1.1e-16, 1.1e-16))
    st, led = check(engine, oracle, 64, z["keys"], z["values"], rots, 1e-5)
    assert st == 0 and led.arithmetic_l2 > 0


def test_statuses_and_transactions(engine, oracle):
    rng = np.random.default_rng(9)
    keys, vals = random_map(rng, 30, 500)
    good = random_rotations(rng, 30, 4)
    bad = (0, 0, 1, 1, 1.0, 0.0, 0.0, 0.0)
    for rots in (good + [bad], good + [(1, 2, 1, 1, 1.0, 0.0, -1e-16, 0.0)],
                 good + [(1, 2, 1, 1, float("nan"), 0.0, 0.0, 0.0)]):
        m = engine.map(30, keys, vals)
        led0 = GbLedger()
        led0.dropped_l1 = 0.5
        st, led, _ = m.rotate_enclosed(rots, options(1e-4), led0)
        k, v = m.download()
        m.close()
        assert st == 1 and oracle.rotations_enclosed(keys, vals, 30, rots, threshold=1e-4)[0] == 1
        assert np.array_equal(k, keys) and np.array_equal(bits(v), bits(vals))
        assert led.dropped_l1 == 0.5 and led.rotations == 0
    # radii whose squares overflow: ENUMERIC from the ledger, map untouched
    big = np.full(len(vals), 1e300) * np.sign(vals)
    st, _ = check(engine, oracle, 30, keys, big, [(0, 1, 1, 1, 0.8, 0.6, 1e300, 0.0)] * 2, 0.0)
    assert st == 4
    # empty map: no-op
    m = engine.map(30)
    st, led, _ = m.rotate_enclosed(good, options(1e-4))
    assert st == 0 and led.rotations == 0
    m.close()
