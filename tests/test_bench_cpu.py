"""bench.py's host-side pieces on CPU: the roofline byte count and the
per-kernel traffic figures it reads from the committed ncu summaries."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_algorithmic_bytes_per_rotation():
    # (8W + 8) bytes per term, read once as input and written once as output
    assert bench.algorithmic_bytes(2, 100, 120) == 24 * 220
    assert bench.algorithmic_bytes(1, 10, 0) == 16 * 10


def test_traffic_profiles_parse():
    # every dominant kernel the bench can report has a committed summary
    for kernel in ("k_hash_rotate", "k_merge", "k_flip_sort"):
        v = bench.read_traffic_profile(kernel, "ring64")
        assert v is not None and v > 0, kernel
    assert bench.read_traffic_profile("k_hash_rotate", "ring64", "l2_bytes_per_input_term") > 100
    assert bench.read_traffic_profile("k_unknown", "ring64") is None


def test_configs_match_the_benchmark_geometries():
    from ddevol_gb300 import hamiltonians as H
    assert len(bench.CONFIGS["ring64"]["terms"]()) == 6048   # 2016 edges x 3 terms
    assert len(bench.CONFIGS["ring16"]["terms"]()) == 96     # 32 edges x 3 terms
    assert len(bench.CONFIGS["cubic"]["terms"]()) == 1920    # 640 nonzero edges x 3 terms
    assert bench.POWDER["items"] == 512 and bench.POWDER["steps_total"] == 300
    assert H.serving_request.__defaults__[1] == 3  # documented pair cutoff
