"""Bounded device-side waits.  TPGP_GB_WAIT_TEST=1 makes the persistent
kernels' grid barriers wait for one participant that does not exist, so
every barrier wait runs out its poll limit (options.wait_polls, here 2000
polls of ~32 ns): the call must return EBACKEND with the committed map
unchanged, nothing may hang, and the context must stay usable.  No fault is
involved: the wait ends by its own limit."""
import os

import numpy as np
import pytest

from ddevol_gb300 import hamiltonians as H
from ddevol_gb300.engine import STATUS_NAMES, Engine, GbLedger, options
from gpu_helpers import bits, random_map

pytestmark = pytest.mark.gpu

EBACKEND = STATUS_NAMES.index("ebackend")


def _with_env(env, fn):
    old = {k: os.environ.get(k) for k in env}
    os.environ.update(env)
    try:
        return fn()
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


# the persistent sorted-path kernel (bound ledger, hash step off) and the
# persistent hash-table step
@pytest.mark.parametrize("kernel,extra", [("TPGP_GB_PERSISTENT", {"TPGP_GB_HASH": "0"}),
                                          ("TPGP_GB_HASH_PERSISTENT", {})])
def test_barrier_wait_gives_up_and_the_map_is_unchanged(kernel, extra):
    rng = np.random.default_rng(11)
    keys, vals = random_map(rng, 40, 3000)
    terms = H.ring_j1j2(40, 1.0, 0.3)

    def run(polls):
        eng = Engine(0)
        m = eng.map(40, keys, vals)
        led = GbLedger()
        st, fids, led2, msg = m.evolve(terms, 0.02, 1, options(1e-4, exact_ledger=False,
                                                              wait_polls=polls), led)
        k, v = m.download()
        m.close()
        eng.close()
        return st, msg, k, v, led2

    st, msg, k, v, led = _with_env({kernel: "1", "TPGP_GB_WAIT_TEST": "1", **extra},
                                   lambda: run(2000))
    assert st == EBACKEND, (st, msg)
    assert "timed out" in msg
    assert np.array_equal(k, keys) and np.array_equal(bits(v), bits(vals))
    assert led.rotations == 0
    # the same kernels work again without the phantom participant (default limit)
    st2, msg2, k2, v2, led2 = _with_env({kernel: "1", **extra}, lambda: run(0))
    assert st2 == 0, msg2
    assert led2.rotations == 2 * len(terms)
