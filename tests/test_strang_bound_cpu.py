"""The library's host Strang bound (tpgp_gb_strang_bound) against the
reference engine's tpgp_strang_bound on the golden term lists
(tests/golden/exact.npz, made by tests/golden/make_exact.py).  Host code
only: no GPU is needed."""
import ctypes as C
import math
import os

import numpy as np

from ddevol_gb300 import native
from ddevol_gb300.engine import terms_array

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "exact.npz")


def test_library_strang_bound_matches_reference():
    lib = native.load()
    lib.tpgp_gb_strang_bound.restype = C.c_double
    lib.tpgp_gb_strang_bound.argtypes = [C.POINTER(native.GbTerm), C.c_size_t, C.c_double]
    z = dict(np.load(GOLDEN))
    checked = 0
    for name in z["strang_names"]:
        p = "strang_" + str(name) + "_"
        terms = [(int(a), int(b), int(c), int(d), float(h))
                 for (a, b, c, d), h in zip(z[p + "terms"].reshape(-1, 4), z[p + "h"])]
        arr, count = terms_array(terms)
        got = lib.tpgp_gb_strang_bound(arr, count, float(z[p + "dt"]))
        want = float(z[p + "bound"])
        if math.isnan(want):
            assert math.isnan(got), name
        else:
            assert np.float64(got).view(np.uint64) == np.float64(want).view(np.uint64), name
        checked += 1
    assert checked >= 20


def test_oracle_strang_bound_matches_reference(oracle):
    """The oracle's restatement (orc_strang_bound, orc_strang_bound_taylor),
    which the GPU enclosure test uses, bitwise the reference's on the same lists."""
    z = dict(np.load(GOLDEN))
    for name in z["strang_names"]:
        p = "strang_" + str(name) + "_"
        terms = [(int(a), int(b), int(c), int(d), float(h))
                 for (a, b, c, d), h in zip(z[p + "terms"].reshape(-1, 4), z[p + "h"])]
        for taylor, key in ((False, "bound"), (True, "taylor")):
            got = oracle.strang_bound(terms, float(z[p + "dt"]), taylor_only=taylor)
            want = float(z[p + key])
            if math.isnan(want):
                assert math.isnan(got), (name, key)
            else:
                assert np.float64(got).view(np.uint64) == np.float64(want).view(np.uint64), \
                    (name, key)
