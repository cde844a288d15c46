"""bench.py's host-side arithmetic (no GPU): the build roofline's algorithmic bytes and rate against
the measured HBM copy rate, and the DRAM traffic read from the committed walk profile."""

import json
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_build_roofline_arithmetic():
    import bench_configs as B

    n, nodes, ms = 1_000_000, 480_978, 1.0
    r = B.build_roofline(n, nodes, ms)
    alg = B.BUILD_BYTES_PER_PARTICLE * n + B.BUILD_BYTES_PER_NODE * nodes
    assert r["algorithmic_bytes"] == alg == 1_104_067_682
    assert r["achieved_gbs"] == pytest.approx(alg / 1e-3 / 1e9, abs=0.1)
    peaks = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks):
        hbm = json.load(open(peaks)).get("hbm_gbs")
        assert r["hbm_peak_gbs"] == hbm
        assert r["frac_of_hbm"] == pytest.approx(alg / 1e-3 / 1e9 / hbm, abs=1e-4)
    assert r["nodes"] == nodes and r["ms"] == ms


def test_walk_traffic_comes_from_the_committed_profile():
    import bench

    t = bench.read_traffic()
    assert isinstance(t, int) and 1e8 < t < 1e9  # bytes per walk launch at 1e6 (the arena fits the L2)
