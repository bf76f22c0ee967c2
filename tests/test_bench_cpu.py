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


def test_reference_arm_runs_on_the_window_state_without_the_gpu_library():
    """The reference arm starts from the committed window state, samples
    rotations across the whole step and maps no library of the GPU build."""
    import json
    import subprocess
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "3", "--cpu-budget", "1"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert not any("libtpgp_gb300" in lib for lib in line["libraries"]), line["libraries"]
    cfg = bench.CONFIGS["ring64"]
    assert line["config"]["window_state"] == "tests/golden/ring64_window.npz"
    assert line["config"]["window_state_terms"] == 100947
    assert line["config"]["rotations_per_step"] == 2 * len(cfg["terms"]())
    assert "every" in line["cpu_baseline"]["sample"] and line["value"] > 0
    # the serial backend beside the threaded one
    assert line["backends"]["serial"]["threads"] == 1 and line["backends"]["serial"]["value"] > 0
    assert line["backends"]["threads"]["value"] == line["value"]


def test_strided_sample_spreads_over_the_step():
    """cpu_sample visits every stride-th rotation of the forward and reverse
    lists (here with a fake engine that only records the calls)."""
    import numpy as np

    class Fake:
        def __init__(self):
            self.calls = []

        def rotate_timed(self, keys, vals, n, i, j, qi, qj, h, dur, thr, threads):
            self.calls.append((i, j, qi, qj))
            return 0, len(vals), 0.01

    terms = [(k, k + 1, 3, 3, 1.0) for k in range(50)]
    f = Fake()
    t, secs, rots, stride = bench.cpu_sample(f, np.zeros(1, np.uint64), np.ones(1), 64, terms, 0.01,
                                             1e-5, 0.1, 1, offset=3, per_rot_s=0.01)
    assert stride == 10 and rots == 10
    order = terms + terms[::-1]
    assert f.calls == [order[r][:4] for r in range(3, 100, 10)]
