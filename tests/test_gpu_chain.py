"""The reference's whole main() sequence rebuilt from the stage entry points
alone, through the C ABI: threshold_image -> image_segmentation ->
find_boundaries -> atag_cluster (stages 4-11) -> fit_lines ->
atag_corner_peaks (stages 13-15) -> do_indexing -> process_fitted_quads.
Every intermediate must have the element count and the bytes of the golden
vectors made from the reference's own sources (tests/golden/pipeline.json);
counts travel to the host between stages, as src/main.cpp reads them."""
import json
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN

sys.path.insert(0, GOLDEN)
import golden_io  # noqa: E402

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _frames():
    out = {}
    for f in ("reference_images.npz", "small_frames.npz"):
        with np.load(os.path.join(GOLDEN, f)) as z:
            out.update({k: z[k] for k in z.files})
    return out


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(GOLDEN, "pipeline.json")) as f:
        return json.load(f)


def _check(entry, stage, arr):
    want = entry[stage]
    assert len(arr) == want["n"], (stage, len(arr), want["n"])
    assert golden_io.digest(arr) == want["sha256"], stage


def run_chain(img):
    """The stage-by-stage path; returns every intermediate as host records."""
    from atag import records as R
    from atag import stages
    h, w = img.shape
    grey = torch.from_numpy(img).cuda()
    out = {}
    thr, ext, flt = stages.threshold_image(grey, with_extrema=True)
    labels, sizes, _ = stages.image_segmentation(thr)
    pts, keys = stages.find_boundaries(labels, sizes)
    cl, counts = stages.cluster(pts, keys, grey)
    assert int(counts["status"]) == 0, hex(int(counts["status"]))
    C, Cf, Pf = int(counts["n_pairs"]), int(counts["n_clusters"]), int(counts["n_cluster_points"])
    found = stages.fit_lines(cl["line_fit"], cl["cluster_indices"], cl["cluster_extents"], Pf, on_device=True)
    corners, peak_ext, (K, Cp, st) = stages.corner_peaks(found, cl["cluster_extents"], Cf, max(Pf, 1))
    assert st == 0
    fitted = stages.do_indexing(peak_ext, corners, cl["line_fit"], cl["cluster_extents"], Cp, on_device=True)
    quads = stages.process_fitted_quads(fitted, w, h, n=Cp)
    host = stages.to_host
    out.update({
        "thresholded": thr.cpu().numpy().ravel(), "extrema": ext.cpu().numpy().ravel(),
        "filtered_extrema": flt.cpu().numpy().ravel(),
        "labels": labels.cpu().numpy().view(np.uint32).ravel(), "sizes": sizes.cpu().numpy().view(np.uint32),
        "dense_points": pts.cpu().numpy().view(golden_io.BOUNDARY_POINT),
        "dense_keys": keys.cpu().numpy().view(np.uint64),
        "bounds": host(cl["pair_bounds"], R.CLUSTER_BOUNDS)[:C],
        "bound_keys": host(cl["pair_keys"], np.uint64)[:C],
        "filtered_bounds": host(cl["filtered_bounds"], R.CLUSTER_BOUNDS)[:Cf],
        "filtered_keys": host(cl["filtered_keys"], np.uint64)[:Cf],
        "extents": host(cl["cluster_extents"], R.CLUSTER_EXTENTS)[:Cf],
        "cluster_points": host(cl["cluster_points"], R.CLUSTER_POINT)[:Pf],
        "cluster_indices": host(cl["cluster_indices"], np.uint16)[:Pf],
        "line_fit": host(cl["line_fit"], R.LINE_FIT_POINT)[:Pf],
        "found_corners": host(found, R.CORNER)[:Pf],
        "corners": host(corners, R.CORNER)[:K],
        "peak_extents": host(peak_ext, R.PEAK_EXTENTS)[:Cp],
        "fitted": host(fitted, R.FITTED_QUAD)[:Cp],
        "quads": quads,
        "n_points": int(counts["n_points"]),
    })
    return out


CHAIN_STAGES = ["thresholded", "extrema", "filtered_extrema", "labels", "sizes", "dense_points", "dense_keys",
                "bounds", "bound_keys", "filtered_bounds", "filtered_keys", "extents", "cluster_points",
                "cluster_indices", "line_fit", "found_corners", "corners", "peak_extents", "fitted", "quads"]


@pytest.mark.parametrize("name", sorted(_frames()))
def test_stage_chain_matches_reference_sources(golden, name):
    img = _frames()[name]
    g = golden[name]
    got = run_chain(img)
    for stage in CHAIN_STAGES:
        _check(g, stage, got[stage])
    # P: the compacted point count of stage 4
    assert got["n_points"] == g["points"]["n"]


def test_stage_chain_equals_fused_detector_on_1080p_and_4k():
    """On synthetic 1080p and 4K stress frames (the 4K one takes the radix
    path of clusters above 16384 points) the stage chain gives the fused
    detector's quads byte for byte, and the same clusters and sums."""
    from atag import synth
    from atag.detector import Detector
    for name, seed in (("1080p", 11), ("4k", 3)):
        img = synth.render(synth.CONFIGS[name], seed)
        h, w = img.shape
        det = Detector(w, h, keep_intermediates=True)
        quads, st = det.detect([torch.from_numpy(img).cuda()])
        v = det.views(0)
        got = run_chain(img)
        assert got["quads"].tobytes() == quads[0].tobytes(), name
        assert np.array_equal(got["filtered_keys"], v["cluster_keys"]), name
        assert got["line_fit"].tobytes() == v["line_fit"].tobytes(), name
        assert got["cluster_points"].tobytes() == v["cluster_points"].tobytes(), name
        assert got["n_points"] == int(st[0]["n_points"]), name


def test_cluster_reports_small_capacities_without_writing_past_them():
    """Capacities below the frame's needs set status bits, and what fits is
    what the call with room for everything writes."""
    from atag import records as R
    from atag import stages, synth
    img = synth.render(synth.CONFIGS["1080p"], 4)
    grey = torch.from_numpy(img).cuda()
    thr = stages.threshold_image(grey)
    labels, sizes, _ = stages.image_segmentation(thr)
    pts, keys = stages.find_boundaries(labels, sizes)
    full, c0 = stages.cluster(pts, keys, grey)
    Cf = int(c0["n_clusters"])
    assert Cf > 8
    small, c1 = stages.cluster(pts, keys, grey, cluster_capacity=8, pair_capacity=16)
    assert int(c1["status"]) & R.DEVFLAG_CLUSTER_OVERFLOW
    assert int(c1["status"]) & R.DEVFLAG_PAIR_OVERFLOW
    assert int(c1["n_clusters"]) == 8
    # the first 8 clusters are the same as with room for all of them
    a = stages.to_host(small["filtered_bounds"], R.CLUSTER_BOUNDS)[:8]
    b = stages.to_host(full["filtered_bounds"], R.CLUSTER_BOUNDS)[:8]
    assert a.tobytes() == b.tobytes()
    assert int(c1["n_pairs"]) == int(c0["n_pairs"]) > 16
    pa = stages.to_host(small["pair_bounds"], R.CLUSTER_BOUNDS)[:16]
    pb = stages.to_host(full["pair_bounds"], R.CLUSTER_BOUNDS)[:16]
    assert pa.tobytes() == pb.tobytes()
