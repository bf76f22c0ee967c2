"""The hash-table Strang step (bound ledger) against the sorted path.

The bound ledger runs multi-rotation lists through the hash-table step by
default; TPGP_GB_HASH=0 selects the sorted per-rotation kernels.  Both must
give bitwise the same keys, values, FIDs and ledgers (the bound ledger's
fixed-point sums are order-independent), including maps whose keys span one
to four words, maps that empty mid-step, steps that outgrow the table and
the arena, and a cap hit mid-step.
"""
import os

import numpy as np
import pytest

from ddevol_gb300 import hamiltonians as H
from ddevol_gb300.engine import Engine, GbLedger, options
from gpu_helpers import bits, ledger_vec, random_map

pytestmark = pytest.mark.gpu


def evolve(hash_on, n, keys, vals, terms, dt, steps, opts, ledger=None):
    os.environ["TPGP_GB_HASH"] = "1" if hash_on else "0"
    try:
        eng = Engine(0)
        m = eng.map(n, keys, vals)
        st, fids, led, msg = m.evolve(terms, dt, steps, opts, ledger or GbLedger())
        k, v = m.download()
        m.close()
        eng.close()
    finally:
        os.environ.pop("TPGP_GB_HASH", None)
    return st, k, v, fids, led, msg


@pytest.mark.parametrize("n_spins", [24, 60, 90, 120])
def test_exact_ledger_hash_matches_sorted(n_spins):
    """The exact ledger through the hash-table step (removed terms logged,
    sorted per rotation, added in key order) against the sorted kernels'
    in-order sums, W = 1..4: maps, FIDs and every ledger field bitwise."""
    rng = np.random.default_rng(100 + n_spins)
    keys, vals = random_map(rng, n_spins, 3000)
    terms = H.ring_j1j2(n_spins, 1.0, 0.3)
    opts = options(1e-3, exact_ledger=True)
    a = evolve(True, n_spins, keys, vals, terms, 0.03, 3, opts)
    b = evolve(False, n_spins, keys, vals, terms, 0.03, 3, opts)
    assert a[0] == b[0] == 0, (a[5], b[5])
    assert a[4].removal_events > 0
    assert np.array_equal(a[1], b[1])
    assert np.array_equal(bits(a[2]), bits(b[2]))
    assert np.array_equal(bits(a[3]), bits(b[3]))
    assert np.array_equal(bits(ledger_vec(a[4])), bits(ledger_vec(b[4])))


@pytest.mark.parametrize("n_spins", [24, 60, 90, 120])
def test_exact_ledger_multi_tile_segments(n_spins):
    """Maps of 4·10^4 terms with values spread over six decades and a high
    threshold, so a rotation removes thousands of terms: the per-rotation
    segment sort runs its multi-tile passes at every key width (W = 1..4).
    Hash-table step against the sorted kernels, everything bitwise."""
    rng = np.random.default_rng(500 + n_spins)
    keys, vals = random_map(rng, n_spins, 40000)
    terms = H.ring_j1j2(n_spins, 1.0, 0.3)[:6]
    opts = options(3e-3, exact_ledger=True)
    a = evolve(True, n_spins, keys, vals, terms, 0.2, 1, opts)
    b = evolve(False, n_spins, keys, vals, terms, 0.2, 1, opts)
    assert a[0] == b[0] == 0, (a[5], b[5])
    assert a[4].removal_events > 0 and len(a[2]) < len(vals)
    assert np.array_equal(a[1], b[1])
    assert np.array_equal(bits(a[2]), bits(b[2]))
    assert np.array_equal(bits(ledger_vec(a[4])), bits(ledger_vec(b[4])))


@pytest.mark.parametrize("n_spins", [24, 60, 90, 120])
def test_hash_matches_sorted_random_maps(n_spins):
    """Random multi-site maps (W = 1..4) under three steps of a ring with
    next-nearest couplings: hash and sorted paths bitwise equal."""
    rng = np.random.default_rng(n_spins)
    keys, vals = random_map(rng, n_spins, 3000)
    terms = H.ring_j1j2(n_spins, 1.0, 0.3)
    opts = options(1e-4, exact_ledger=False)
    a = evolve(True, n_spins, keys, vals, terms, 0.03, 3, opts)
    b = evolve(False, n_spins, keys, vals, terms, 0.03, 3, opts)
    assert a[0] == b[0] == 0, (a[5], b[5])
    assert np.array_equal(a[1], b[1])
    assert np.array_equal(bits(a[2]), bits(b[2]))
    assert np.array_equal(bits(a[3]), bits(b[3]))
    assert np.array_equal(bits(ledger_vec(a[4])), bits(ledger_vec(b[4])))


def test_map_that_empties_mid_step(oracle):
    """A threshold above every value removes the whole map in the first
    anticommuting rotation; the remaining rotations are no-ops (no ledger
    change), as in the reference."""
    terms = H.ring_j1j2(8)
    k0, v0 = H.single_site_operator(8)
    a = evolve(True, 8, k0, v0, terms, 0.05, 1, options(10.0, exact_ledger=False))
    b = evolve(False, 8, k0, v0, terms, 0.05, 1, options(10.0, exact_ledger=False))
    ost, ok, ov, oled = oracle.strang_step(k0, v0, 8, terms, 0.05, threshold=10.0, steps=1)
    assert a[0] == b[0] == ost == 0
    assert len(a[2]) == len(ov) == 0
    assert a[4].rotations == b[4].rotations == oled.rotations
    assert np.array_equal(bits(ledger_vec(a[4])), bits(ledger_vec(b[4])))


def test_table_and_arena_growth_in_one_step(oracle):
    """Eight spins, global X, threshold 0: the map grows from 8 terms to
    thousands within a step, past the initial table and arena."""
    terms = H.ring_j1j2(8)
    k0, v0 = H.global_x_operator(8)
    ost, ok, ov, _ = oracle.strang_step(k0, v0, 8, terms, 0.05, threshold=0.0, steps=3)
    a = evolve(True, 8, k0, v0, terms, 0.05, 3, options(0.0, exact_ledger=False))
    assert a[0] == ost == 0, a[5]
    assert len(a[2]) > 4096
    assert np.array_equal(a[1], ok) and np.array_equal(bits(a[2]), bits(ov))


def test_cap_mid_step_is_transactional():
    terms = H.ring_j1j2(16)
    k0, v0 = H.single_site_operator(16)
    base = evolve(True, 16, k0, v0, terms, 0.01, 20, options(1e-6, exact_ledger=False))
    assert base[0] == 0
    n20 = len(base[2])
    a = evolve(True, 16, base[1], base[2], terms, 0.01, 1,
               options(1e-6, max_terms=n20 + 3, exact_ledger=False))
    b = evolve(False, 16, base[1], base[2], terms, 0.01, 1,
               options(1e-6, max_terms=n20 + 3, exact_ledger=False))
    assert a[0] == b[0] == 3  # ECAP
    assert np.array_equal(a[1], base[1]) and np.array_equal(bits(a[2]), bits(base[2]))


def test_persistent_hash_step(golden_trajectories):
    """TPGP_GB_HASH_PERSISTENT=1 runs a step's rotations in one cooperative
    launch with grid barriers: same results as the per-rotation launches."""
    g = golden_trajectories
    p = "ring16__"
    terms = [(int(a), int(b), int(c), int(d), float(h))
             for (a, b, c, d), h in zip(g[p + "terms"], g[p + "h"])]
    opts = options(float(g[p + "threshold"]), exact_ledger=False)
    args = (int(g[p + "n"]), g[p + "in_keys"], g[p + "in_values"], terms, float(g[p + "dt"]),
            int(g[p + "steps"]), opts)
    os.environ["TPGP_GB_HASH_PERSISTENT"] = "1"
    try:
        a = evolve(True, *args)
        rng = np.random.default_rng(60)
        keys, vals = random_map(rng, 60, 3000)
        ra = evolve(True, 60, keys, vals, H.ring_j1j2(60, 1.0, 0.3), 0.03, 2,
                    options(1e-4, exact_ledger=False))
    finally:
        os.environ.pop("TPGP_GB_HASH_PERSISTENT", None)
    assert a[0] == 0, a[5]
    assert np.array_equal(a[1], g[p + "out_keys"])
    assert np.array_equal(bits(a[2]), bits(g[p + "out_values"]))
    assert np.array_equal(bits(a[3]), bits(g[p + "fid_sum"]))
    rb = evolve(False, 60, keys, vals, H.ring_j1j2(60, 1.0, 0.3), 0.03, 2,
                options(1e-4, exact_ledger=False))
    assert ra[0] == rb[0] == 0
    assert np.array_equal(ra[1], rb[1]) and np.array_equal(bits(ra[2]), bits(rb[2]))
    assert np.array_equal(bits(ledger_vec(ra[4])), bits(ledger_vec(rb[4])))


def _fused(*args):
    os.environ["TPGP_GB_HASH_FUSE"] = "1"
    try:
        return evolve(True, *args)
    finally:
        os.environ.pop("TPGP_GB_HASH_FUSE", None)


def _same(a, b):
    assert a[0] == b[0] == 0, (a[5], b[5])
    assert np.array_equal(a[1], b[1])
    assert np.array_equal(bits(a[2]), bits(b[2]))
    assert np.array_equal(bits(a[3]), bits(b[3]))
    assert np.array_equal(bits(ledger_vec(a[4])), bits(ledger_vec(b[4])))


@pytest.mark.parametrize("n_spins", [16, 40, 64, 100, 120])
def test_fused_runs_match(n_spins):
    """TPGP_GB_HASH_FUSE=1: one pass per run of rotations on a site pair
    (each coset evolved through the run) instead of one pass per rotation;
    same maps, FIDs and ledgers as the sorted path, for one- to four-word
    keys.  A Strang step's middle run is six rotations on one edge (the
    longest run the pass takes)."""
    rng = np.random.default_rng(42 + n_spins)
    keys, vals = random_map(rng, n_spins, 3000)
    terms = H.ring_j1j2(n_spins, 1.0, 0.3)
    opts = options(1e-4, exact_ledger=False)
    _same(_fused(n_spins, keys, vals, terms, 0.03, 2, opts),
          evolve(False, n_spins, keys, vals, terms, 0.03, 2, opts))


def test_fused_runs_single_generator_and_cubic():
    """Runs whose group has one mask (an Ising-only edge list: every run is
    ZZ on one pair, a two-member coset) and the cubic lattice's edge list."""
    rng = np.random.default_rng(7)
    keys, vals = random_map(rng, 24, 3000)
    zz = [t for t in H.ring_j1j2(24, 1.0, 0.3) if t[2] == 3 and t[3] == 3]
    opts = options(1e-4, exact_ledger=False)
    _same(_fused(24, keys, vals, zz, 0.05, 2, opts), evolve(False, 24, keys, vals, zz, 0.05, 2, opts))
    k0, v0 = H.single_site_operator(64, 0)
    cubic = H.cubic_111(4)
    copts = options(1e-5, exact_ledger=False)
    _same(_fused(64, k0, v0, cubic, 0.005, 3, copts), evolve(False, 64, k0, v0, cubic, 0.005, 3, copts))


def test_fused_runs_table_retry(oracle):
    """A map that outgrows its table inside a step (8 spins, global X,
    threshold 0): the fused passes report the full table, the step is re-run
    on a larger one, and the result is the oracle's."""
    terms = H.ring_j1j2(8)
    k0, v0 = H.global_x_operator(8)
    ost, ok, ov, _ = oracle.strang_step(k0, v0, 8, terms, 0.05, threshold=0.0, steps=3)
    a = _fused(8, k0, v0, terms, 0.05, 3, options(0.0, exact_ledger=False))
    assert a[0] == ost == 0, a[5]
    assert np.array_equal(a[1], ok) and np.array_equal(bits(a[2]), bits(ov))
