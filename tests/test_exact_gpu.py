"""The benchmark ring's FID on the device against the exact references.

The 16-spin J1-J2 ring (d(nn) = 1, d(nnn) = 1/8, X_0, dt = 0.01, threshold
1e-6) is evolved on the GPU for its whole 400-step horizon.  Every step:

* containment, as the reference CLI states it (engine/src/cli_rev.c:549-587):
  |F_gpu - F_exact| <= pf * norm0 * dual + dropped_l2 * dual, with pf the
  upward sum of the per-step Strang bound (tpgp_strang_bound,
  engine/src/tpgp_rev.c:902-961, restated in the oracle), norm0 = 1 and
  dual = sqrt(16) for a local X_0 start; F_exact from the momentum-resolved
  sector diagonalisation (tests/golden/exact.npz);
* agreement with the stochastic Krylov reference within its 95% interval
  plus the same allowance, at t = 0.04 k;
* an empirical band: the propagated FID stays within 1e-3 of the exact one
  (7.5e-4 is the measured worst case over the 400 steps; the trajectory is
  deterministic, so a larger deviation means the propagation changed).
"""
import math
import os
import time

import numpy as np
import pytest

from ddevol_gb300 import hamiltonians as H
from ddevol_gb300.engine import GbLedger, options

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "exact.npz")


def up_add(a, b):
    """tpgp_bound_add_up for finite non-negative operands: nextUp(a + b)."""
    if a == 0:
        return b
    if b == 0:
        return a
    return math.nextafter(a + b, math.inf)


@pytest.mark.parametrize("exact_ledger", [False])
def test_ring16_enclosed_by_exact_fid(engine, oracle, exact_ledger):
    ex = dict(np.load(GOLDEN))
    exact = ex["ring16_exact"]
    terms = H.ring_j1j2(16)
    dt, steps = 0.01, 400
    per_step = oracle.strang_bound(terms, dt)
    assert 0 < per_step < 1e-3
    dual, norm0 = math.sqrt(16.0) / 1.0, math.sqrt(1.0)
    m = engine.map(16, *H.single_site_operator(16))
    opts = options(1e-6, exact_ledger=exact_ledger)
    led = GbLedger()
    pf = 0.0
    fids, allowance = np.zeros(steps), np.zeros(steps)
    t0 = time.perf_counter()
    for k in range(steps):
        st, f, led, msg = m.evolve(terms, dt, 1, opts, led)
        assert st == 0, (k, msg)
        pf = up_add(pf, per_step)
        fids[k] = f[0]
        allowance[k] = pf * norm0 * dual + (led.dropped_l2 + led.arithmetic_l2) * dual
    elapsed = time.perf_counter() - t0
    peak = led.peak_terms
    m.close()
    dev = np.abs(fids - exact[1:steps + 1])
    assert np.all(dev <= allowance), int(np.argmax(dev - allowance))
    assert dev.max() < 1e-3, dev.max()
    # Krylov reference at t = 0.04 k (k >= 1)
    t = ex["ring16_lanczos_times"]
    idx = np.rint(t / dt).astype(int)
    sel = (idx >= 1) & (idx <= steps)
    kry = np.abs(fids[idx[sel] - 1] - ex["ring16_lanczos_mean"][sel])
    assert np.all(kry <= ex["ring16_lanczos_ci95"][sel] + allowance[idx[sel] - 1])
    print(f"ring16 400 steps in {elapsed:.1f} s, peak {peak} terms, max |F - F_exact| "
          f"{dev.max():.3e}, final allowance {allowance[-1]:.3e}")
