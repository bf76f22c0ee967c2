"""Serving with continuous batching (tpgp_gb_serve).

Requests of different spin counts (all three key widths), couplings,
thresholds and lengths arrive staggered and outnumber the slots, so they
queue, take slots as earlier solves finish, and run interleaved with each
other.  Each request's FID sequence must be the same (bitwise) in the mix,
served alone, and as a plain single-map evolve at its slot's width.
"""
import numpy as np
import pytest

from ddevol_gb300 import hamiltonians as H
from ddevol_gb300.engine import options

pytestmark = pytest.mark.gpu


def make_requests(count, seed=11, gap=0.005):
    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(count):
        n, terms, thr, steps, dt = H.serving_request(rng, steps_range=(3, 6))
        keys, vals = H.single_site_operator(n, 0)
        reqs.append(dict(arrival=k * gap, n_spins=n, terms=terms, dt=dt, steps=steps,
                         options=options(thr, exact_ledger=False), keys=keys, values=vals))
    return reqs


def test_same_result_alone_and_in_the_mix(engine):
    reqs = make_requests(10)
    assert {(q["n_spins"] + 31) // 32 for q in reqs} == {1, 2, 3}
    resp, fids, stats = engine.serve(reqs, slots=(2, 2, 2))
    assert 0 < stats["busy_seconds"] <= stats["wall_seconds"]
    assert stats["ticks"] >= max(q["steps"] for q in reqs) and stats["terms"] > 0
    assert 1 <= stats["max_active"] <= 6
    for r, q in enumerate(reqs):
        x = resp[r]
        assert x["status"] == 0
        assert x["admitted"] >= q["arrival"] - 1e-9 and x["finished"] >= x["admitted"]
        assert len(fids[r]) == q["steps"] and np.all(np.isfinite(fids[r]))
        # alone through the server
        resp1, fids1, _ = engine.serve([dict(q, arrival=0.0)], slots=(1, 1, 1))
        assert np.array_equal(fids1[0].view(np.uint64), fids[r].view(np.uint64)), r
        # alone as a plain map at the slot's width
        width = x["slot_spins"]
        words = width // 32
        k0 = np.zeros(words, np.uint64)
        k0[: (q["n_spins"] + 31) // 32] = q["keys"]
        m = engine.map(width, k0, q["values"])
        st, f2, _, msg = m.evolve(q["terms"], q["dt"], q["steps"], q["options"])
        m.close()
        assert st == 0, msg
        assert np.array_equal(f2.view(np.uint64), fids[r].view(np.uint64)), r


def test_queueing_reuses_slots(engine):
    reqs = make_requests(7, seed=12, gap=0.0)
    resp, fids, _ = engine.serve(reqs, slots=(1, 1, 1))
    assert all(x["status"] == 0 for x in resp)
    # with one slot per width, some request had to wait for a slot
    assert max(x["admitted"] - q["arrival"] for x, q in zip(resp, reqs)) > 0


def test_served_fids_match_oracle_at_true_size(engine, oracle):
    """Each served request against the CPU oracle run at the request's own
    spin count (the server widens a request to its slot's 32/64/96 spins):
    per-step FIDs bitwise, requests of all three key widths, one of them
    run for 30 steps."""
    reqs = make_requests(9, seed=14)
    reqs[0]["steps"] = 30
    assert {(q["n_spins"] + 31) // 32 for q in reqs} == {1, 2, 3}
    resp, fids, _ = engine.serve(reqs, slots=(2, 2, 2))
    for r, q in enumerate(reqs):
        assert resp[r]["status"] == 0
        fo = []
        st, _, _, _ = oracle.strang_step(q["keys"], q["values"], q["n_spins"], q["terms"], q["dt"],
                                         threshold=q["options"].threshold, steps=q["steps"],
                                         on_step=lambda s, f, n: fo.append(f))
        assert st == 0
        assert np.array_equal(fids[r].view(np.uint64), np.array(fo).view(np.uint64)), r
