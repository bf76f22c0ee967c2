"""Device-resident rotation (tpgp_gb_rotate) against the reference and the oracle.

* every golden case produced by the reference engine itself, bitwise: keys,
  values, statuses and (exact-ledger mode) every ledger field;
* the reference's local_dense known answers (256 two-site conjugations);
* random maps up to 10^6 terms against the oracle, bitwise, on site pairs that
  make the flipped-key segments span many tiles, single tiles, or straddle
  word boundaries;
* upload validation and transactional failures.
"""
import math

import numpy as np
import pytest

from gpu_helpers import (bits, fast_random_map, gpu_rotate, ledger_vec, random_map,
                         sparse_random_map)
from test_local_dense import check_local_dense

pytestmark = pytest.mark.gpu


def test_golden_rotations_exact_ledger(engine, golden_rotations):
    g = golden_rotations
    for idx in range(int(g["count"])):
        p = f"c{idx:03d}_"
        n = int(g[p + "n"])
        keys, vals = g[p + "in_keys"], g[p + "in_values"]
        if not np.all(np.isfinite(vals)):
            # a nonfinite stored coefficient violates the map invariants: the
            # device map refuses it at upload instead of failing the rotation
            m = engine.map(n)
            st, _ = m.upload(keys, vals)
            m.close()
            assert st == 1
            continue
        i, j, qi, qj = (int(x) for x in g[p + "params"])
        st, k, v, led, msg = gpu_rotate(engine, keys, vals, n, i, j, qi, qj, float(g[p + "theta"]),
                                        float(g[p + "threshold"]), int(g[p + "max_terms"]),
                                        float(g[p + "max_drop_l2"]))
        assert st == int(g[p + "status"]), (idx, msg)
        if st == 0:
            assert np.array_equal(k, g[p + "out_keys"]), idx
            assert np.array_equal(bits(v), bits(g[p + "out_values"])), idx
            assert np.array_equal(bits(ledger_vec(led)), bits(g[p + "ledger"])), idx
        else:
            # transactional: map and ledger unchanged
            assert np.array_equal(k, keys) and np.array_equal(bits(v), bits(vals)), idx
            assert not np.any(ledger_vec(led)), idx


def test_golden_rotations_bound_ledger(engine, golden_rotations):
    """Fast ledger: same keys/values; the removed-weight sums are exact 128-bit
    fixed-point sums of addends rounded up to multiples of 2^(et-96) (et the
    exponent just above the threshold), so they bound the exact sums from
    above within k 2^(et-96) + 1 ulp; the reference's sequential upward sums
    bound them within 3 k 2^-53 relative."""
    g = golden_rotations
    for idx in range(int(g["count"])):
        p = f"c{idx:03d}_"
        if int(g[p + "status"]) != 0 or not np.all(np.isfinite(g[p + "in_values"])):
            continue
        i, j, qi, qj = (int(x) for x in g[p + "params"])
        st, k, v, led, _ = gpu_rotate(engine, g[p + "in_keys"], g[p + "in_values"],
                                      int(g[p + "n"]), i, j, qi, qj, float(g[p + "theta"]),
                                      float(g[p + "threshold"]), exact_ledger=False)
        assert st == 0
        assert np.array_equal(k, g[p + "out_keys"])
        assert np.array_equal(bits(v), bits(g[p + "out_values"]))
        want = g[p + "ledger"]
        got = ledger_vec(led)
        k = 2 * len(g[p + "in_values"]) + 2
        thr = float(g[p + "threshold"])
        et = math.frexp(thr)[1] if thr > 0 else 1
        for f, unit in ((0, et - 96), (1, et - 96), (2, 2 * et - 96)):
            tol = 3.0 * k * 2.0 ** -53 * abs(want[f]) + k * 2.0 ** unit + 2.0 ** -1000
            assert abs(got[f] - want[f]) <= tol, (idx, f, got[f], want[f])
        assert np.array_equal(got[3:], want[3:])


def test_local_dense_gpu(engine):
    def rotate(keys, values, qa, qb, theta):
        st, k, v, _, msg = gpu_rotate(engine, keys, values, 2, 0, 1, qa, qb, theta)
        assert st == 0, msg
        return {int(a): float(b) for a, b in zip(k, v)}
    check_local_dense(rotate)


CASES = [
    # (n_spins, count, sites list, threshold, dense)
    (16, 200_000, [(15, 14), (0, 1), (7, 3), (15, 0)], 1e-4, True),
    (64, 150_000, [(63, 62), (31, 32), (0, 63), (5, 40)], 1e-5, False),
    (96, 100_000, [(95, 0), (63, 64), (31, 95), (10, 11)], 1e-5, False),
    (100, 50_000, [(99, 98), (0, 64), (96, 97)], 0.0, False),
]


@pytest.mark.parametrize("n_spins,count,pairs,threshold,dense", CASES)
def test_random_maps_vs_oracle(engine, oracle, n_spins, count, pairs, threshold, dense):
    rng = np.random.default_rng(n_spins * 7919 + count)
    if dense:
        keys, vals = fast_random_map(rng, n_spins, count)
    else:
        keys, vals = sparse_random_map(rng, n_spins, count)
    for (i, j) in pairs:
        for qi, qj in ((3, 3), (1, 1), (2, 2), (1, 3), (0, 2)):
            theta = float(rng.uniform(-1, 1))
            ost, ok, ov, oled = oracle.rotate(keys, vals, n_spins, i, j, qi, qj, theta, 1.0,
                                              threshold=threshold)
            st, k, v, led, msg = gpu_rotate(engine, keys, vals, n_spins, i, j, qi, qj, theta,
                                            threshold)
            assert st == ost == 0, msg
            assert len(v) == len(ov), (i, j, qi, qj)
            assert np.array_equal(k, ok), (i, j, qi, qj)
            assert np.array_equal(bits(v), bits(ov)), (i, j, qi, qj)
            want = np.array([oled.dropped_l1, oled.dropped_l2, oled.dropped_l2_squared,
                             oled.arithmetic_l2, oled.rotations, oled.removal_events,
                             oled.peak_terms, 0], np.float64)
            assert np.array_equal(bits(ledger_vec(led)), bits(want)), (i, j, qi, qj)


def test_structured_map_multi_tile(engine, oracle):
    """A propagated-operator-like map: few active sites per key, many terms."""
    rng = np.random.default_rng(5)
    keys, vals = random_map(rng, 64, 20_000, active_sites=range(0, 64, 3))
    for (i, j) in ((0, 3), (63, 60), (30, 33)):
        for q in (1, 2, 3):
            ost, ok, ov, _ = oracle.rotate(keys, vals, 64, i, j, q, q, 0.3, 1.0, threshold=1e-6)
            st, k, v, _, msg = gpu_rotate(engine, keys, vals, 64, i, j, q, q, 0.3, 1e-6)
            assert st == ost == 0, msg
            assert np.array_equal(k, ok) and np.array_equal(bits(v), bits(ov))


def test_upload_validation(engine):
    m = engine.map(16)
    ok_keys = np.array([1, 4, 16], np.uint64)
    assert m.upload(ok_keys, np.array([1.0, 2.0, 3.0]))[0] == 0
    for keys, vals in (
            (np.array([4, 1, 16], np.uint64), np.array([1.0, 2.0, 3.0])),   # unsorted
            (np.array([1, 1, 16], np.uint64), np.array([1.0, 2.0, 3.0])),   # duplicate
            (np.array([1, 4, 1 << 40], np.uint64), np.array([1.0, 2.0, 3.0])),  # padding
            (ok_keys, np.array([1.0, 0.0, 3.0])),                           # stored zero
            (ok_keys, np.array([1.0, np.inf, 3.0]))):                       # nonfinite
        assert m.upload(keys, vals)[0] == 1
    k, v = m.download()
    assert list(k) == [1, 4, 16] and list(v) == [1.0, 2.0, 3.0]
    m.close()


def test_empty_and_noop(engine):
    m = engine.map(8)
    st, led, _ = m.rotate(0, 1, 3, 3, 0.4)
    assert st == 0 and led.rotations == 0  # empty map: no ledger change
    m.upload(np.array([1], np.uint64), np.array([1.0]))
    st, led, _ = m.rotate(0, 1, 3, 3, 0.0)  # h == 0: no-op
    assert st == 0 and led.rotations == 0 and len(m) == 1
    st, led, _ = m.rotate(0, 1, 0, 0, 0.4)  # identity generator: every term commutes
    assert st == 0 and led.rotations == 1 and len(m) == 1
    m.close()
