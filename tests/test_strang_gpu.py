"""Strang steps and trajectories on the device against the reference and the oracle.

* every golden trajectory from the reference engine (ring16 J1-J2, the
  reference's own N=6 CUDA-trajectory case, 64-site all-pairs ring, 4x4x4
  cubic, 96-site chain): final keys, values and ledger bitwise, the per-step
  FID sum (tpgp_map_single_sum) bitwise, the per-step term count;
* graph replay and plain launches give identical results;
* the bound (fixed-point) ledger keeps keys/values bitwise and stays within its bound;
* transactional failures: a cap or budget hit mid-step, an invalid term after
  valid ones, leave map and ledger untouched.
"""
import numpy as np
import pytest

from ddevol_gb300 import hamiltonians as H
from ddevol_gb300.engine import GbLedger, options
from gpu_helpers import bits, ledger_vec

pytestmark = pytest.mark.gpu

NAMES = ["ring16", "n6_thr0", "n6_thr1e-5", "ring64_allpairs", "cubic4", "chain96"]


def load_traj(g, name):
    p = name + "__"
    terms = [(int(a), int(b), int(c), int(d), float(h))
             for (a, b, c, d), h in zip(g[p + "terms"], g[p + "h"])]
    return p, terms


@pytest.mark.parametrize("use_graphs", [True, False])
@pytest.mark.parametrize("name", NAMES)
def test_golden_trajectories(engine, golden_trajectories, name, use_graphs):
    g = golden_trajectories
    p, terms = load_traj(g, name)
    m = engine.map(int(g[p + "n"]), g[p + "in_keys"], g[p + "in_values"])
    st, fids, led, msg = m.evolve(terms, float(g[p + "dt"]), int(g[p + "steps"]),
                                  options(float(g[p + "threshold"]), use_graphs=use_graphs))
    assert st == 0, msg
    k, v = m.download()
    m.close()
    assert np.array_equal(k, g[p + "out_keys"])
    assert np.array_equal(bits(v), bits(g[p + "out_values"]))
    assert np.array_equal(bits(ledger_vec(led)), bits(g[p + "ledger"]))
    assert np.array_equal(bits(fids), bits(g[p + "fid_sum"]))


@pytest.mark.parametrize("name", NAMES)
def test_bound_ledger_trajectory(engine, golden_trajectories, name):
    """Fast (bound) ledger: this mode runs the persistent one-launch-per-step
    kernel; keys, values and FID stay bitwise."""
    g = golden_trajectories
    p, terms = load_traj(g, name)
    m = engine.map(int(g[p + "n"]), g[p + "in_keys"], g[p + "in_values"])
    st, fids, led, msg = m.evolve(terms, float(g[p + "dt"]), int(g[p + "steps"]),
                                  options(float(g[p + "threshold"]), exact_ledger=False))
    assert st == 0, msg
    k, v = m.download()
    m.close()
    assert np.array_equal(k, g[p + "out_keys"])
    assert np.array_equal(bits(v), bits(g[p + "out_values"]))
    assert np.array_equal(bits(fids), bits(g[p + "fid_sum"]))
    got, want = ledger_vec(led), g[p + "ledger"]
    # each rotation's tree sum and the sequential sum both bound the exact sum
    # from above within 3 k 2^-53 (k <= 2n upward additions); 1e-11 covers
    # thousands of rotations of these sizes
    for f in range(3):
        assert abs(got[f] - want[f]) <= 1e-11 * want[f]
    assert np.array_equal(got[3:], want[3:])


def test_strang_step_matches_evolve(engine, golden_trajectories):
    g = golden_trajectories
    p, terms = load_traj(g, "ring16")
    m = engine.map(16, g[p + "in_keys"], g[p + "in_values"])
    led = GbLedger()
    opts = options(float(g[p + "threshold"]))
    for _ in range(int(g[p + "steps"])):
        st, led, msg = m.strang_step(terms, float(g[p + "dt"]), opts, led)
        assert st == 0, msg
    k, v = m.download()
    assert np.array_equal(k, g[p + "out_keys"])
    assert np.array_equal(bits(v), bits(g[p + "out_values"]))
    assert np.array_equal(bits(ledger_vec(led)), bits(g[p + "ledger"]))
    assert m.single_sum(1) == float(g[p + "fid_sum"][-1])
    m.close()


@pytest.fixture(scope="module")
def ring16_60_oracle(oracle):
    terms = H.ring_j1j2(16)
    k0, v0 = H.single_site_operator(16)
    fids_o = []
    ost, ok, ov, oled = oracle.strang_step(k0, v0, 16, terms, 0.01, threshold=1e-6, steps=60,
                                           threads=8, on_step=lambda s, f, n: fids_o.append(f))
    assert ost == 0
    return terms, k0, v0, ok, ov, oled, np.array(fids_o)


@pytest.mark.parametrize("exact", [True, False])
def test_longer_ring16_vs_oracle(engine, ring16_60_oracle, exact):
    """60 steps of the benchmark ring (map ~45k terms): multi-tile every rotation;
    the bound ledger runs the persistent kernel, the exact one the per-kernel path."""
    terms, k0, v0, ok, ov, oled, fids_o = ring16_60_oracle
    m = engine.map(16, k0, v0)
    st, fids, led, msg = m.evolve(terms, 0.01, 60, options(1e-6, exact_ledger=exact))
    assert st == 0, msg
    k, v = m.download()
    m.close()
    assert len(v) > 20000
    assert np.array_equal(k, ok) and np.array_equal(bits(v), bits(ov))
    assert np.array_equal(bits(fids), bits(fids_o))
    if exact:
        assert led.dropped_l2 == oled.dropped_l2 and led.dropped_l1 == oled.dropped_l1
    else:
        assert abs(led.dropped_l2 - oled.dropped_l2) <= 1e-11 * oled.dropped_l2
        assert led.removal_events == oled.removal_events


@pytest.fixture(scope="module")
def cubic30_oracle(oracle):
    terms = H.cubic_111(4)
    k0, v0 = H.single_site_operator(64)
    fids_o = []
    ost, ok, ov, oled = oracle.strang_step(k0, v0, 64, terms, 0.005, threshold=1e-5, steps=30,
                                           threads=16, on_step=lambda s, f, n: fids_o.append(f))
    assert ost == 0
    return terms, k0, v0, ok, ov, oled, np.array(fids_o)


@pytest.mark.parametrize("exact", [True, False])
def test_cubic_30_steps_vs_oracle(engine, cubic30_oracle, exact):
    """30 steps of the 4x4x4 cubic lattice (64 spins, two-word keys, 3840
    rotations per step) from X on site 0: keys, values and every step's FID
    bitwise; the exact ledger bitwise (through the hash-table step's
    per-rotation segment sums), the bound ledger within its bound."""
    terms, k0, v0, ok, ov, oled, fids_o = cubic30_oracle
    m = engine.map(64, k0, v0)
    st, fids, led, msg = m.evolve(terms, 0.005, 30, options(1e-5, exact_ledger=exact))
    assert st == 0, msg
    k, v = m.download()
    m.close()
    assert np.array_equal(k, ok) and np.array_equal(bits(v), bits(ov))
    assert np.array_equal(bits(fids), bits(fids_o))
    if exact:
        assert np.array_equal(bits(ledger_vec(led)), bits(ledger_vec(oled)))
    else:
        assert abs(led.dropped_l2 - oled.dropped_l2) <= 1e-11 * oled.dropped_l2
        assert led.removal_events == oled.removal_events


@pytest.mark.parametrize("exact", [True, False])
def test_transactional_cap_and_budget(engine, golden_trajectories, exact):
    g = golden_trajectories
    p, terms = load_traj(g, "ring16")
    m = engine.map(16, g[p + "in_keys"], g[p + "in_values"])
    k0, v0 = m.download()
    led0 = GbLedger()
    led0.dropped_l1 = 0.25
    st, led, _ = m.strang_step(terms, 0.01, options(1e-6, max_terms=len(v0) + 5,
                                                      exact_ledger=exact), led0)
    assert st == 3  # ECAP part-way through the step
    k, v = m.download()
    assert np.array_equal(k, k0) and np.array_equal(bits(v), bits(v0))
    assert led.dropped_l1 == 0.25 and led.rotations == 0
    st, led, _ = m.strang_step(terms, 0.01, options(1e-6, max_drop_l2=1e-12, exact_ledger=exact),
                               led0)
    assert st == 6  # EBUDGET
    k, v = m.download()
    assert np.array_equal(k, k0) and np.array_equal(bits(v), bits(v0))
    # an invalid term after valid ones: the valid prefix runs, the step fails
    bad = list(terms[:5]) + [(3, 3, 1, 1, 0.1)]
    st, led, _ = m.strang_step(bad, 0.01, options(1e-6, exact_ledger=exact), GbLedger())
    assert st == 1
    k, v = m.download()
    assert np.array_equal(k, k0) and np.array_equal(bits(v), bits(v0))
    st, led, _ = m.strang_step(terms, 3 * 2.0 ** -1074, options(), GbLedger())
    assert st == 4  # dt/2 inexact
    m.close()


def test_invalid_term_after_buffer_allocation(engine, golden_trajectories):
    """A step on a map that has already stepped (its current buffer is not
    the first) which allocates device buffers (the exact ledger's log, a
    longer parameter list) and then reaches an invalid term restores the
    committed map, not the arena's first buffer."""
    g = golden_trajectories
    p, terms = load_traj(g, "ring16")
    m = engine.map(16, g[p + "in_keys"], g[p + "in_values"])
    st, led, msg = m.strang_step(terms, 0.01, options(1e-6, exact_ledger=False), GbLedger())
    assert st == 0, msg
    k0, v0 = m.download()
    bad = list(terms[:5]) + [(3, 3, 1, 1, 0.1)]
    st, _, _ = m.strang_step(bad, 0.01, options(1e-6, exact_ledger=True), GbLedger())
    assert st == 1
    k, v = m.download()
    m.close()
    assert np.array_equal(k, k0) and np.array_equal(bits(v), bits(v0))


@pytest.mark.parametrize("exact", [True, False])
def test_growth_across_arena_resize(engine, oracle, exact):
    """Start from a tiny arena and grow through several reallocations in one call."""
    terms = H.ring_j1j2(8)
    k0, v0 = H.global_x_operator(8)
    ost, ok, ov, _ = oracle.strang_step(k0, v0, 8, terms, 0.05, threshold=0.0, steps=2)
    m = engine.map(8, k0, v0)
    st, _, _, msg = m.evolve(terms, 0.05, 2, options(0.0, exact_ledger=exact))
    assert st == ost == 0, msg
    k, v = m.download()
    m.close()
    assert len(v) > 4096
    assert np.array_equal(k, ok) and np.array_equal(bits(v), bits(ov))


def test_persistent_step_kernel(golden_trajectories, oracle):
    """The opt-in cooperative one-launch-per-step kernel gives the same maps."""
    import os
    from ddevol_gb300.engine import Engine
    os.environ["TPGP_GB_PERSISTENT"] = "1"
    try:
        eng = Engine(0)
        g = golden_trajectories
        for name in ("ring16", "cubic4", "chain96"):
            p, terms = load_traj(g, name)
            m = eng.map(int(g[p + "n"]), g[p + "in_keys"], g[p + "in_values"])
            st, fids, led, msg = m.evolve(terms, float(g[p + "dt"]), int(g[p + "steps"]),
                                          options(float(g[p + "threshold"]), exact_ledger=False))
            assert st == 0, msg
            assert m.last_launches() <= int(g[p + "steps"])  # one launch per step
            k, v = m.download()
            m.close()
            assert np.array_equal(k, g[p + "out_keys"])
            assert np.array_equal(bits(v), bits(g[p + "out_values"]))
            assert np.array_equal(bits(fids), bits(g[p + "fid_sum"]))
        eng.close()
    finally:
        os.environ.pop("TPGP_GB_PERSISTENT", None)


def test_with_programmatic_launch(ring16_60_oracle):
    """TPGP_GB_PDL=1 (programmatic dependent launch between the rotation
    kernels) gives the same maps and FIDs as plain stream-ordered launches."""
    import os
    from ddevol_gb300.engine import Engine
    terms, k0, v0, ok, ov, oled, fids_o = ring16_60_oracle
    os.environ["TPGP_GB_PDL"] = "1"
    try:
        eng = Engine(0)
        m = eng.map(16, k0, v0)
        st, fids, _, msg = m.evolve(terms, 0.01, 60, options(1e-6, exact_ledger=False))
        assert st == 0, msg
        k, v = m.download()
        m.close()
        eng.close()
        assert np.array_equal(k, ok) and np.array_equal(bits(v), bits(ov))
        assert np.array_equal(bits(fids), bits(fids_o))
    finally:
        os.environ.pop("TPGP_GB_PDL", None)


@pytest.mark.parametrize("exact", [True, False])
def test_first_failure_in_rotation_order(engine, oracle, exact):
    """A step whose drop budget runs out at one rotation and whose term cap
    would be hit at a later one reports the earlier failure, as the reference
    does (its step stops at the first failing rotation); with the cap first,
    ECAP.  The exact ledger's sums run after the rotations, so this checks
    that the deferred walk puts the failures back in rotation order."""
    g_terms = H.ring_j1j2(16)
    k0, v0 = H.single_site_operator(16)
    st, k20, v20, led20 = oracle.strang_step(k0, v0, 16, g_terms, 0.01, threshold=1e-6, steps=20)
    assert st == 0
    st, k21, v21, led21 = oracle.strang_step(k20, v20, 16, g_terms, 0.01, threshold=1e-6, steps=1)
    grown = max(len(v21), len(v20))
    step_drop = led21.dropped_l2  # the 21st step's total removed weight (from zero)
    cases = [
        # budget runs out early in the step, the cap only at its largest map
        dict(max_drop_l2=step_drop * 0.05, max_terms=grown - 1),
        # the cap is hit almost at once, the budget only near the end
        dict(max_drop_l2=step_drop * 0.95, max_terms=len(v20) + 1),
    ]
    for lim in cases:
        ost, _, _, _ = oracle.strang_step(k20, v20, 16, g_terms, 0.01, threshold=1e-6,
                                          max_terms=lim["max_terms"], max_drop_l2=lim["max_drop_l2"])
        assert ost in (3, 6)
        m = engine.map(16, k20, v20)
        st, led, msg = m.strang_step(g_terms, 0.01, options(1e-6, exact_ledger=exact, **lim),
                                     GbLedger())
        k, v = m.download()
        m.close()
        assert st == ost, (lim, st, ost, msg)
        assert np.array_equal(k, k20) and np.array_equal(bits(v), bits(v20))
