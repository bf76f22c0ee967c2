"""Generate the fixtures that pin the exact-FID and Strang-bound references.

Writes ``exact.npz`` next to this script:

* ``ref_sector_n10`` / ``ref_sector_n14`` -- the reference's own S^z-sector
  program (DDevol engine/tests/sector_reference_rev.cpp, built by
  ``make -C oracle sector``; J1 = 1, J2 = 0.3 hard-coded there) at N = 10
  (104 steps of 1/32) and N = 14 (200 steps of 0.02).  They pin the
  parametrised restatements in ``oracle/exact.py``.
* ``ring16_exact`` -- the exact FID of the 16-spin J1-J2 benchmark ring
  (d(nn) = 1, d(nnn) = 1/8 in the /2 convention, i.e. 2 and 1/4 in the
  reference's /4 edge convention), F(k * 0.01) for k = 0..400, from the
  momentum-resolved sector restatement.
* ``ring16_lanczos_*`` -- the stochastic Krylov estimate of the same FID at
  t = 0.04 k, k = 0..100 (8 random-phase vectors, Krylov dimension 120): the
  mean, standard error, Student-t 95% half-width and the residual bound.
* ``strang_*`` -- the reference engine's tpgp_strang_bound and
  tpgp_strang_bound_taylor (engine/src/tpgp_rev.c:875-961, compiled by
  ``make -C oracle ref``) on the benchmark term lists and seeded random ones.

Needs the reference checkout (DDEVOL_REFERENCE) for the two reference
programs; runs in a few minutes:

    DDEVOL_REFERENCE=<checkout> make -C oracle ref sector
    python tests/golden/make_exact.py
"""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import exact as X  # noqa: E402
from oracle.oracle import Reference  # noqa: E402
from ddevol_gb300 import hamiltonians as H  # noqa: E402

SECTOR_BIN = os.path.join(ROOT, "oracle", "_ref", "sector_reference")
RING16_DISTANCE = {1: 2.0, 2: 0.25}  # /4 convention: 2 d with d = 1, 1/8


def reference_sector(n, *args):
    out = subprocess.run([SECTOR_BIN, str(n), *map(str, args)], capture_output=True, text=True,
                         check=True).stdout.strip().split("\n")
    assert out[0] == "time,F"
    return np.array([float(line.split(",")[1]) for line in out[1:]])


def strang_cases(rng):
    cases = [("ring16", H.ring_j1j2(16), 0.01), ("ring64", H.ring_all_pairs(64), 0.005),
             ("cubic", H.cubic_111(4), 0.005), ("chain20_cut3", H.chain_all_pairs(20, cutoff=3),
                                                -0.02)]
    for t in range(24):
        n = int(rng.integers(2, 9))
        terms = []
        for _ in range(int(rng.integers(0, 30))):
            i, j = rng.choice(n, 2, replace=False)
            h = 0.0 if rng.random() < 0.1 else float(rng.standard_normal())
            terms.append((int(i), int(j), int(rng.integers(0, 4)), int(rng.integers(0, 4)), h))
        cases.append((f"random{t:02d}", terms, float(10 ** rng.uniform(-3, 0))))
    cases.append(("nonfinite_dt", H.ring_j1j2(6), float("inf")))
    cases.append(("same_site_term", [(0, 0, 1, 1, 1.0)], 0.1))
    return cases


def main():
    out = {}
    out["ref_sector_n10"] = reference_sector(10)
    out["ref_sector_n14"] = reference_sector(14, 200, 0.02)
    out["ring16_exact"] = X.momentum_sector_fid(16, RING16_DISTANCE, 400, 0.01)
    times = np.arange(101) * 0.04
    mean, se, ci, res, _ = X.lanczos_fid(16, X.ring_couplings(16, RING16_DISTANCE), times,
                                         samples=8, dimension=120)
    out.update(ring16_lanczos_times=times, ring16_lanczos_mean=mean, ring16_lanczos_se=se,
               ring16_lanczos_ci95=ci, ring16_lanczos_residual=np.array(res))
    ref = Reference()
    names = []
    for name, terms, dt in strang_cases(np.random.default_rng(20261204)):
        names.append(name)
        arr = np.array([(i, j, qi, qj) for i, j, qi, qj, _ in terms], np.int64).reshape(-1, 4)
        out[f"strang_{name}_terms"] = arr
        out[f"strang_{name}_h"] = np.array([h for *_, h in terms], np.float64)
        out[f"strang_{name}_dt"] = np.array(dt)
        out[f"strang_{name}_bound"] = np.array(ref.strang_bound(terms, dt))
        out[f"strang_{name}_taylor"] = np.array(ref.strang_bound(terms, dt, taylor_only=True))
    out["strang_names"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "exact.npz"), **out)
    print(f"exact.npz: {len(names)} Strang cases, ring16 F(4) = {out['ring16_exact'][-1]:.17g}")


if __name__ == "__main__":
    main()
