"""The oracle's -i[H, A] against the reference engine's tpgp_liouvillian
(tests/golden/liouvillian.npz, made by tests/golden/make_liouvillian.py)."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "liouvillian.npz")


def golden_cases():
    z = dict(np.load(GOLDEN))
    for name in z["names"]:
        p = str(name) + "__"
        terms = [(int(a), int(b), int(c), int(d), float(h))
                 for (a, b, c, d), h in zip(z[p + "terms"], z[p + "h"])]
        yield (str(name), int(z[p + "n"]), z[p + "in_keys"], z[p + "in_values"], terms,
               int(z[p + "status"]), z[p + "out_keys"], z[p + "out_values"])


@pytest.mark.parametrize("sorted_sums", [False, True])
@pytest.mark.parametrize("case", list(golden_cases()), ids=lambda c: c[0])
def test_oracle_generator_matches_reference(oracle, case, sorted_sums):
    """Both restatements (sorted insertion; sort then sequential sums)."""
    name, n, k, v, terms, st, ok, ov = case
    got = oracle.liouvillian(k, v, n, terms, sorted_sums=sorted_sums)
    assert got[0] == st, name
    if st == 0:
        assert np.array_equal(got[1], ok), name
        assert np.array_equal(got[2].view(np.uint64), ov.view(np.uint64)), name
