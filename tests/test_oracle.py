"""CPU checks of the oracle's own restatements: the per-cluster cyclic
fit_lines equals the reference's windowed work-group formulation, the
integer weight equals the reference's truncated hypotf, and the pipeline's
invariants hold."""
import ctypes
import ctypes.util
import math

import numpy as np
import pytest

import oracle
from conftest import small_frames


@pytest.fixture(scope="module")
def results(ref_images):
    frames = dict(ref_images)
    frames.update(small_frames())
    return {k: oracle.detect(v) for k, v in frames.items()}


def test_cyclic_fit_lines_equals_windowed(results):
    for name, r in results.items():
        if len(r["line_fit"]) == 0:
            continue
        a = oracle.fit_lines(r["line_fit"], r["cluster_indices"], r["extents"], windowed=True)
        b = oracle.fit_lines(r["line_fit"], r["cluster_indices"], r["extents"], windowed=False)
        assert a.tobytes() == b.tobytes(), name


def test_integer_weight_equals_truncated_hypotf():
    libm = ctypes.CDLL(ctypes.util.find_library("m"))
    libm.hypotf.restype = ctypes.c_float
    libm.hypotf.argtypes = [ctypes.c_float, ctypes.c_float]
    for gx in range(0, 256):
        for gy in range(0, 256, 3):
            want = int(libm.hypotf(gx, gy))
            assert want == math.isqrt(gx * gx + gy * gy), (gx, gy)
            assert int(oracle.hypotf(gx, gy)) == want


def test_pipeline_invariants(results):
    for name, r in results.items():
        keys = r["keys"]
        assert np.all(keys[1:] >= keys[:-1]), name
        ext = r["extents"]
        if len(ext):
            assert ext["start"][0] == 0
            assert np.array_equal(ext["start"][1:], np.cumsum(ext["count"])[:-1])
            assert np.all(ext["count"] >= 24)
        ci = r["cluster_indices"]
        assert np.all(ci[1:] >= ci[:-1]), name
        c = r["corners"]
        assert np.all(c["error"] != 0)
        # every quad's corners are finite and inside a frame-sized box
        q = r["quads"]
        if len(q):
            assert np.all(np.isfinite(q["corners"]))


def test_compat_and_aligned_agree_when_every_cluster_has_peaks(results):
    for name in ("decimate", "decimate4"):
        r = results[name]
        assert len(r["peak_extents"]) == len(r["filtered"])
        a = oracle.do_indexing(r["peak_extents"], r["corners"], r["line_fit"], r["extents"],
                               oracle.default_config(compat_peak_index=1))
        b = oracle.do_indexing(r["peak_extents"], r["corners"], r["line_fit"], r["extents"],
                               oracle.default_config(compat_peak_index=0))
        assert a.tobytes() == b.tobytes()


def test_compat_peak_index_uses_extent_of_rank(results):
    """Drop the peaks of one cluster: compat mode (fit_quad.cpp:405-408)
    reads cluster_extents by peak rank, so every later quad is fitted on the
    previous cluster's points, unlike aligned mode."""
    r = results["decimate"]
    pe, corners = r["peak_extents"], r["corners"]
    assert len(pe) >= 2
    keep = np.ones(len(corners), bool)
    s, n = pe[0]["start"], pe[0]["count"]
    keep[s:s + n] = False
    c2 = corners[keep]
    pe2 = pe[1:].copy()
    pe2["start"] -= n
    a = oracle.do_indexing(pe2, c2, r["line_fit"], r["extents"], oracle.default_config(compat_peak_index=1))
    b = oracle.do_indexing(pe2, c2, r["line_fit"], r["extents"], oracle.default_config(compat_peak_index=0))
    assert a.tobytes() != b.tobytes()
