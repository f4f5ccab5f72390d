"""The CPU oracle against golden vectors produced by the reference's own
sources (src/threshold.cpp, src/segmentation.cpp, src/find_boundaries.cpp,
src/fit_quad.cpp and include/*.h, built by oracle/refshim and run by
tests/golden/make_golden.py).  Every stage of every golden frame must have
the same element count and the same bytes."""
import json
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN

import sys
sys.path.insert(0, GOLDEN)
import golden_io  # noqa: E402


@pytest.fixture(scope="module")
def pipeline_golden():
    with open(os.path.join(GOLDEN, "pipeline.json")) as f:
        return json.load(f)


def golden_frames():
    out = {}
    with np.load(os.path.join(GOLDEN, "reference_images.npz")) as z:
        out.update({k: z[k] for k in z.files})
    with np.load(os.path.join(GOLDEN, "small_frames.npz")) as z:
        out.update({k: z[k] for k in z.files})
    return out


def oracle_stage_arrays(img):
    r = oracle.detect(img)
    thr, ext, flt = oracle.threshold(img)
    pts, keys = oracle.find_boundaries(r["labels"], r["sizes"])
    return {
        "thresholded": r["thresholded"].ravel(), "extrema": ext.ravel(), "filtered_extrema": flt.ravel(),
        "labels": r["labels"].ravel(), "sizes": r["sizes"], "dense_points": pts, "dense_keys": keys,
        "points": r["points"], "keys": r["keys"], "bounds": r["bounds"], "bound_keys": r["bound_keys"],
        "filtered_bounds": r["filtered"], "filtered_keys": r["filtered_keys"], "extents": r["extents"],
        "cluster_points": r["cluster_points"], "cluster_indices": r["cluster_indices"].astype(np.uint16),
        "line_fit": r["line_fit"], "found_corners": r["found_corners"], "corners": r["corners"],
        "peak_extents": r["peak_extents"], "fitted": r["fitted"], "quads": r["quads"],
    }


@pytest.mark.parametrize("name", sorted(golden_frames()))
def test_oracle_matches_reference_sources(pipeline_golden, name):
    img = golden_frames()[name]
    want = pipeline_golden[name]
    got = oracle_stage_arrays(img)
    assert set(got) == set(want)
    for stage in golden_io.PIPELINE_ARRAYS:
        assert len(got[stage]) == want[stage]["n"], (stage, len(got[stage]), want[stage]["n"])
        assert golden_io.digest(got[stage]) == want[stage]["sha256"], stage


@pytest.fixture(scope="module")
def records():
    with np.load(os.path.join(GOLDEN, "records.npz")) as z:
        return {k: z[k].view(golden_io.RECORD_ARRAYS[k]) if z[k].dtype == np.uint8 and
                golden_io.RECORD_ARRAYS[k] is not np.uint8 else z[k] for k in z.files}


def test_combinadics_decode(records):
    want = records["rec_combinadics"].reshape(210, 4)
    for n in range(210):
        assert list(oracle.combination_decode(n)) == list(want[n]), n


def test_bounds_theta_dot_filter(records):
    cx, cy, th, dot, valid = oracle.eval_bounds(records["rec_bounds"], records["rec_points"], 1920, 1080)
    for got, key in ((cx, "rec_cx"), (cy, "rec_cy"), (th, "rec_theta"), (dot, "rec_dot")):
        assert np.array_equal(got.view(np.uint32), records[key].view(np.uint32)), key
    assert np.array_equal(valid, records["rec_valid"])


def test_initial_linefit(records):
    img = records["rec_image"].reshape(192, 256)
    got = oracle.eval_linefit(records["rec_cluster_points"], 256, 192, img)
    assert golden_io.digest(got) == golden_io.digest(records["rec_linefit"])


def test_fit_line_including_wrapped_products(records):
    lp, err, mse = oracle.eval_fit_line(records["rec_moments"], records["rec_num_in_moment"])
    assert np.array_equal(lp.view(np.uint32), records["rec_line_params"].view(np.uint32))
    assert np.array_equal(err.view(np.uint32), records["rec_err"].view(np.uint32))
    assert np.array_equal(mse.view(np.uint32), records["rec_mse"].view(np.uint32))


def test_get_moment_cyclic_ranges(records):
    out, cnt = oracle.eval_get_moment(records["rec_prefix"], records["rec_moment_range"])
    assert golden_io.digest(out) == golden_io.digest(records["rec_moment"])
    assert np.array_equal(cnt, records["rec_moment_n"])


def test_colour_removal_matches_the_reference_loader():
    """oracle.to_grey against the reference's own colour removal: stb's
    STBI_grey decode of the same pixels (tests/golden/colour.npz); BGR
    orders are the RGB images with the channels reversed."""
    with np.load(os.path.join(GOLDEN, "colour.npz")) as z:
        cases = {k: z[k] for k in z.files}
    names = [k for k in cases if not k.endswith("_grey")]
    assert len(names) >= 5
    for name in names:
        img, want = cases[name], cases[name + "_grey"]
        assert np.array_equal(oracle.to_grey(img), want), name
        c = img.shape[2]
        if c in (3, 4):
            bgr = img.copy()
            bgr[..., [0, 2]] = img[..., [2, 0]]
            assert np.array_equal(oracle.to_grey(bgr, fmt=3 if c == 3 else 4), want), name
        # decimation samples the same pixels
        assert np.array_equal(oracle.to_grey(img, factor=2), want[::2, ::2][: img.shape[0] // 2, : img.shape[1] // 2])
