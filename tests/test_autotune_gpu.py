"""The single-map autotuner (tpgp_gb_map_autotune) and the engine
configurations it chooses among.

Every configuration (sorted kernels with or without dependent launch; the
hash-table step at 2 or 4 CTAs per SM, with or without dependent launch and
fusion) gives the reference engine's golden trajectories bit for bit; the
autotuner leaves the map's contents as they were, times every candidate and
applies the fastest.
"""
import numpy as np
import pytest

from ddevol_gb300.engine import GbLedger, options
from gpu_helpers import bits, ledger_vec

pytestmark = pytest.mark.gpu

CONFIGS = [dict(hash_step=0, sorted_pdl=0), dict(hash_step=0, sorted_pdl=1),
           dict(hash_step=1, hash_ctas=2, hash_pdl=0, hash_fuse=0),
           dict(hash_step=1, hash_ctas=4, hash_pdl=1, hash_fuse=0),
           dict(hash_step=1, hash_ctas=3, hash_pdl=1, hash_fuse=1)]


def load(g, name):
    p = name + "__"
    terms = [(int(a), int(b), int(c), int(d), float(h))
             for (a, b, c, d), h in zip(g[p + "terms"], g[p + "h"])]
    return p, terms


@pytest.mark.parametrize("cfg", CONFIGS)
@pytest.mark.parametrize("name", ["ring16", "cubic4"])
def test_every_configuration_gives_the_golden_trajectory(engine, golden_trajectories, name, cfg):
    g = golden_trajectories
    p, terms = load(g, name)
    m = engine.map(int(g[p + "n"]), g[p + "in_keys"], g[p + "in_values"])
    m.set_engine_config(**cfg)
    got = m.engine_config()
    assert all(got[k] == v for k, v in cfg.items())
    exact = not cfg.get("hash_fuse", 0)  # fusion applies to the bound ledger
    st, fids, led, msg = m.evolve(terms, float(g[p + "dt"]), int(g[p + "steps"]),
                                  options(float(g[p + "threshold"]), exact_ledger=exact))
    assert st == 0, msg
    k, v = m.download()
    m.close()
    assert np.array_equal(k, g[p + "out_keys"])
    assert np.array_equal(bits(v), bits(g[p + "out_values"]))
    assert np.array_equal(bits(fids), bits(g[p + "fid_sum"]))
    if exact:
        assert np.array_equal(bits(ledger_vec(led)), bits(g[p + "ledger"]))


@pytest.mark.parametrize("exact", [True, False])
def test_autotune_keeps_the_map_and_applies_the_fastest(engine, golden_trajectories, exact):
    g = golden_trajectories
    p, terms = load(g, "ring16")
    m = engine.map(16, g[p + "in_keys"], g[p + "in_values"])
    opts = options(float(g[p + "threshold"]), exact_ledger=exact)
    st, _, led, msg = m.evolve(terms, float(g[p + "dt"]), 3, opts)
    assert st == 0, msg
    k0, v0 = m.download()
    t = m.autotune(terms, float(g[p + "dt"]), opts)
    k1, v1 = m.download()
    assert np.array_equal(k0, k1) and np.array_equal(bits(v0), bits(v1))
    tried = t["tried"]
    assert len(tried) >= 3 and all(c["step_ms"] > 0 for c in tried)
    assert t["chosen"]["step_ms"] == min(c["step_ms"] for c in tried)
    chosen = {k: v for k, v in t["chosen"].items() if k != "step_ms"}
    now = m.engine_config()
    assert all(now[k] == v for k, v in chosen.items())
    # the tuned map continues the trajectory exactly as an untuned one
    ref = engine.map(16, k0, v0)
    st_a, f_a, led_a, _ = m.evolve(terms, float(g[p + "dt"]), 3, opts, GbLedger.from_buffer_copy(led))
    st_b, f_b, led_b, _ = ref.evolve(terms, float(g[p + "dt"]), 3, opts, GbLedger.from_buffer_copy(led))
    assert st_a == st_b == 0
    ka, va = m.download()
    kb, vb = ref.download()
    m.close()
    ref.close()
    assert np.array_equal(ka, kb) and np.array_equal(bits(va), bits(vb))
    assert np.array_equal(bits(f_a), bits(f_b))
    assert np.array_equal(bits(ledger_vec(led_a)), bits(ledger_vec(led_b)))
