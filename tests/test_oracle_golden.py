"""The CPU oracle against the reference engine's own outputs (golden fixtures).

The fixtures were produced by running DDevol's engine/src/tpgp_rev.c itself
(tests/golden/make_golden.py).  Every comparison is bitwise: keys, values,
statuses and all ledger fields.
"""
import numpy as np
import pytest

from oracle.oracle import LedgerStruct

LEDGER_FIELDS = [name for name, _ in LedgerStruct._fields_]


def ledger_vec(led):
    return np.array([float(getattr(led, f)) for f in LEDGER_FIELDS], np.float64)


def test_rotation_fixtures(oracle, golden_rotations):
    g = golden_rotations
    count = int(g["count"])
    assert count > 100
    for idx in range(count):
        p = f"c{idx:03d}_"
        i, j, qi, qj = (int(x) for x in g[p + "params"])
        st, k, v, led = oracle.rotate(g[p + "in_keys"], g[p + "in_values"], int(g[p + "n"]), i, j,
                                      qi, qj, float(g[p + "theta"]), 1.0,
                                      threshold=float(g[p + "threshold"]),
                                      max_terms=int(g[p + "max_terms"]),
                                      max_drop_l2=float(g[p + "max_drop_l2"]))
        assert st == int(g[p + "status"]), idx
        if st == 0:
            assert np.array_equal(k, g[p + "out_keys"]), idx
            assert np.array_equal(v.view(np.uint64), g[p + "out_values"].view(np.uint64)), idx
            assert np.array_equal(ledger_vec(led).view(np.uint64),
                                  g[p + "ledger"].view(np.uint64)), idx


def test_fixture_statuses_cover_every_failure(golden_rotations):
    g = golden_rotations
    statuses = {int(g[f"c{i:03d}_status"]) for i in range(int(g["count"]))}
    # ok, einval, ecap, enumeric, ebudget all appear
    assert {0, 1, 3, 4, 6} <= statuses


@pytest.mark.parametrize("name", ["ring16", "n6_thr0", "n6_thr1e-5", "ring64_allpairs", "cubic4",
                                  "chain96"])
def test_trajectory_fixtures(oracle, golden_trajectories, name):
    g = golden_trajectories
    p = name + "__"
    terms = [(int(a), int(b), int(c), int(d), float(h))
             for (a, b, c, d), h in zip(g[p + "terms"], g[p + "h"])]
    fids, lens = [], []
    st, k, v, led = oracle.strang_step(g[p + "in_keys"], g[p + "in_values"], int(g[p + "n"]),
                                       terms, float(g[p + "dt"]),
                                       threshold=float(g[p + "threshold"]),
                                       steps=int(g[p + "steps"]),
                                       on_step=lambda s, f, n: (fids.append(f), lens.append(n)))
    assert st == 0
    assert np.array_equal(k, g[p + "out_keys"])
    assert np.array_equal(v.view(np.uint64), g[p + "out_values"].view(np.uint64))
    assert np.array_equal(ledger_vec(led).view(np.uint64), g[p + "ledger"].view(np.uint64))
    assert np.array_equal(np.array(fids).view(np.uint64), g[p + "fid_sum"].view(np.uint64))
    assert lens == list(g[p + "len"])
