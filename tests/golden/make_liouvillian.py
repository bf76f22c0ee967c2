"""Golden vectors of the exact generator -i[H, A] from the reference engine.

Runs DDevol's own tpgp_liouvillian (engine/src/tpgp_rev.c:810-857, compiled
from the reference sources by `make -C oracle ref`) on seeded maps and term
lists and stores inputs and outputs in liouvillian.npz next to this script:

* maps reached by the reference's own Strang steps from X_0 (the 16-spin
  J1-J2 ring, the 64-spin all-pairs ring) and random maps of 24/60/90/120
  spins (one to four key words) under ring couplings;
* edge cases: every contribution cancelling (each term followed by its
  negative), a contribution and a sum that overflow (ENUMERIC), an invalid
  term reached before and after an overflowing one (EINVAL / ENUMERIC), an
  empty input map, an empty term list.

    DDEVOL_REFERENCE=<checkout> make -C oracle ref
    python tests/golden/make_liouvillian.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from ddevol_gb300 import hamiltonians as H  # noqa: E402
from gpu_helpers import random_map  # noqa: E402
from oracle.oracle import Reference  # noqa: E402

OUT = os.path.join(HERE, "liouvillian.npz")


def cases(ref):
    rng = np.random.default_rng(20261204)
    out = []
    k0, v0 = H.single_site_operator(16)
    st, k, v, _ = ref.strang_step(k0, v0, 16, H.ring_j1j2(16), 0.01, threshold=1e-6, steps=30)
    assert st == 0
    out.append(("ring16_step30", 16, k, v, H.ring_j1j2(16)))
    k0, v0 = H.single_site_operator(64)
    st, k, v, _ = ref.strang_step(k0, v0, 64, H.ring_all_pairs(64), 0.005, threshold=1e-5, steps=4)
    assert st == 0
    out.append(("ring64_step4", 64, k, v, H.ring_all_pairs(64)))
    for n in (24, 60, 90, 120):
        k, v = random_map(rng, n, 2000)
        out.append((f"random{n}", n, k, v, H.ring_j1j2(n, 1.0, 0.3)))
    k, v = random_map(rng, 20, 500)
    terms = H.ring_j1j2(20)
    cancel = []
    for (i, j, qi, qj, h) in terms:
        cancel += [(i, j, qi, qj, h), (i, j, qi, qj, -h)]
    out.append(("cancelling", 20, k, v, cancel))
    k = np.array([1 << 2 * 3], np.uint64)  # X on site 3
    v = np.array([10.0])
    out.append(("overflow_contribution", 8, k, v, [(3, 4, 3, 3, 1e308)]))
    out.append(("overflow_sum", 8, k, np.array([1.0]), [(3, 4, 3, 3, 6e307), (3, 4, 3, 3, 6e307)]))
    out.append(("invalid_then_overflow", 8, k, v, [(3, 4, 3, 3, 0.5), (3, 3, 3, 3, 1.0),
                                                   (3, 4, 3, 3, 1e308)]))
    out.append(("overflow_then_invalid", 8, k, v, [(3, 4, 3, 3, 1e308), (9, 1, 3, 3, 1.0)]))
    out.append(("empty_map", 12, np.zeros(0, np.uint64), np.zeros(0), H.ring_j1j2(12)))
    k, v = random_map(rng, 12, 100)
    out.append(("no_terms", 12, k, v, []))
    return out


def main():
    ref = Reference()
    z = {}
    names = []
    for name, n, k, v, terms in cases(ref):
        st, ok, ov = ref.liouvillian(k, v, n, terms)
        names.append(name)
        p = name + "__"
        z[p + "n"] = np.array(n)
        z[p + "in_keys"] = np.asarray(k, np.uint64)
        z[p + "in_values"] = np.asarray(v, np.float64)
        z[p + "terms"] = np.array([t[:4] for t in terms], np.int64).reshape(-1, 4)
        z[p + "h"] = np.array([t[4] for t in terms], np.float64)
        z[p + "status"] = np.array(st)
        z[p + "out_keys"] = ok
        z[p + "out_values"] = ov
        print(f"{name}: n={n} in={len(v)} terms={len(terms)} status={st} out={len(ov)}")
    z["names"] = np.array(names)
    np.savez_compressed(OUT, **z)


if __name__ == "__main__":
    main()
