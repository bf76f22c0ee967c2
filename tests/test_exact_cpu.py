"""The exact-FID references (oracle/exact.py) pinned to the reference's own program.

tests/golden/exact.npz holds the output of the reference's S^z-sector program
(engine/tests/sector_reference_rev.cpp, compiled by ``make -C oracle
sector``; J1 = 1, J2 = 0.3 hard-coded there) at N = 10 (104 steps of 1/32)
and N = 14 (200 steps of 0.02).  The restatements reproduce it to rounding
(the reference accumulates in long double), the momentum-resolved and
dense forms agree with the sector form, and the committed 16-spin benchmark
curve and Krylov estimate (the GPU enclosure test's references) are
consistent with each other.
"""
import os

import numpy as np
import pytest

from oracle import exact as X

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "exact.npz")
REFERENCE_RING = {1: 1.0, 2: 0.3}   # sector_reference_rev.cpp:17, the /4 edge convention
BENCH_RING = {1: 2.0, 2: 0.25}      # d(nn) = 1, d(nnn) = 1/8 in the /2 convention


@pytest.fixture(scope="module")
def golden():
    return dict(np.load(GOLDEN))


def test_sector_form_reproduces_the_reference_program_n10(golden):
    f = X.sector_fid(10, X.ring_couplings(10, REFERENCE_RING), 104, 1 / 32)
    ref = golden["ref_sector_n10"]
    assert len(ref) == 105 and ref[0] == pytest.approx(1.0, abs=1e-12)
    assert np.max(np.abs(f - ref)) < 1e-13


def test_momentum_form_reproduces_the_reference_program_n14(golden):
    f = X.momentum_sector_fid(14, REFERENCE_RING, 200, 0.02)
    assert np.max(np.abs(f - golden["ref_sector_n14"])) < 1e-13


def test_momentum_form_equals_sector_form_on_the_benchmark_couplings():
    f_m = X.momentum_sector_fid(12, BENCH_RING, 60, 0.01)
    f_s = X.sector_fid(12, X.ring_couplings(12, BENCH_RING), 60, 0.01)
    assert np.max(np.abs(f_m - f_s)) < 1e-13


def test_dense_density_matrix_equals_sector_form_on_irregular_couplings():
    """The plain 2^n density-matrix reference agrees with the block form for
    couplings with no symmetry beyond magnetisation (random edges, 8 spins)."""
    rng = np.random.default_rng(3)
    edges = [(i, j, float(rng.standard_normal())) for i in range(8) for j in range(i + 1, 8)
             if rng.random() < 0.5]
    times = np.arange(30) * 0.05
    assert np.max(np.abs(X.dense_fid(8, edges, times) - X.sector_fid(8, edges, 29, 0.05))) < 1e-13


def test_benchmark_curve_and_krylov_estimate_agree(golden):
    exact = golden["ring16_exact"]
    assert len(exact) == 401 and exact[0] == pytest.approx(1.0, abs=1e-12)
    t = golden["ring16_lanczos_times"]
    idx = np.rint(t / 0.01).astype(int)
    gap = np.abs(golden["ring16_lanczos_mean"] - exact[idx])
    assert np.all(gap <= golden["ring16_lanczos_ci95"] + golden["ring16_lanczos_residual"] + 1e-12)
