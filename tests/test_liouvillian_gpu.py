"""The device generator -i[H, A] (tpgp_gb_liouvillian) bitwise against the
reference engine's tpgp_liouvillian on the golden cases, the oracle on
larger maps, and its transactional contract."""
import numpy as np
import pytest

from ddevol_gb300 import hamiltonians as H
from gpu_helpers import bits, random_map
from test_liouvillian_cpu import golden_cases

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", list(golden_cases()), ids=lambda c: c[0])
def test_device_generator_matches_reference(engine, case):
    name, n, k, v, terms, st, ok, ov = case
    src = engine.map(n, k, v) if len(v) else engine.map(n)
    # the output map starts holding something, which must survive a failure
    keep_k, keep_v = H.single_site_operator(n, 1)
    out = engine.map(n, keep_k, keep_v)
    got, out, msg = src.liouvillian(terms, out)
    assert got == st, (name, msg)
    k2, v2 = out.download()
    if st == 0:
        assert np.array_equal(k2, ok), name
        assert np.array_equal(bits(v2), bits(ov)), name
    else:
        assert np.array_equal(k2, keep_k) and np.array_equal(bits(v2), bits(keep_v)), name
    sk, sv = src.download()
    assert np.array_equal(sv.view(np.uint64), np.asarray(v, np.float64).view(np.uint64))
    out.close()
    src.close()


@pytest.mark.parametrize("n_spins,count", [(16, 60000), (64, 30000), (100, 20000)])
def test_device_generator_matches_oracle_on_larger_maps(engine, oracle, n_spins, count):
    """Maps of 2-4.6*10^4..6*10^4 terms (several sort tiles, every key width)
    under all-pairs couplings: the device generator equals the oracle's."""
    rng = np.random.default_rng(n_spins)
    k, v = random_map(rng, n_spins, count)
    terms = H.ring_all_pairs(n_spins, cutoff=4)
    st_o, ok, ov = oracle.liouvillian(k, v, n_spins, terms, sorted_sums=True)
    assert st_o == 0
    src = engine.map(n_spins, k, v)
    st, out, msg = src.liouvillian(terms)
    assert st == 0, msg
    k2, v2 = out.download()
    assert np.array_equal(k2, ok) and np.array_equal(bits(v2), bits(ov))
    # in place: the map becomes its own generator
    st, same, msg = src.liouvillian(terms, src)
    assert st == 0 and same is src, msg
    k3, v3 = src.download()
    assert np.array_equal(k3, ok) and np.array_equal(bits(v3), bits(ov))
    out.close()
    src.close()
