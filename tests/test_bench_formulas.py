"""CPU tests of the bench's roofline arithmetic: the per-stage byte
formulas that `roofline.achieved` divides by the measured stage time."""
import importlib.util
import os

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _stats(n, w=1920, h=1080, points=1_447_463, pairs=270, cpoints=124_372, corners=5_000, peakc=120):
    st = np.zeros(n, dtype=[("width", "u4"), ("height", "u4"), ("n_points", "u4"), ("n_pairs", "u4"),
                            ("n_cluster_points", "u4"), ("n_corners", "u4"), ("n_peak_clusters", "u4")])
    st["width"], st["height"], st["n_points"], st["n_pairs"] = w, h, points, pairs
    st["n_cluster_points"], st["n_corners"], st["n_peak_clusters"] = cpoints, corners, peakc
    return st


def test_boundary_bytes_follow_the_two_formulas():
    b = _bench()
    st = _stats(64)
    N, P, Pf = 64 * 1920 * 1080, 64 * 1_447_463, 64 * 124_372
    assert b.survey_bytes(st)["boundaries_pairs"] == 4 * N + 4 * N + 12 * P
    assert b.stage_bytes(st, N)["boundaries_pairs"] == 4 * N + 8 * Pf


def test_formulas_scale_with_the_batch():
    b = _bench()
    one, many = _stats(1), _stats(64)
    for f in (lambda s: b.survey_bytes(s), lambda s: b.stage_bytes(s, int(s["width"][0]) * int(s["height"][0]) * len(s))):
        a, m = f(one), f(many)
        assert set(a) == set(m)
        for k in a:
            assert m[k] == 64 * a[k], k


def test_pixel_stage_bytes_are_per_pixel():
    b = _bench()
    st = _stats(2, w=640, h=480)
    N = 2 * 640 * 480
    s = b.stage_bytes(st, N)
    assert s["threshold"] == 2 * N and s["ccl_local"] == 5 * N and s["ccl_final"] == 9 * N and s["ccl_border"] == 0
