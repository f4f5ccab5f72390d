"""The CUDA path against the golden vectors of the reference's own sources
(tests/golden/pipeline.json, made by tests/golden/make_golden.py from the
reference's src/*.cpp through oracle/refshim): same element counts, same
bytes, stage by stage, with no oracle in between."""
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


@pytest.fixture(scope="module")
def det():
    from atag.detector import Detector
    return Detector(1920, 1080, keep_intermediates=True)


def _check(golden_entry, stage, arr):
    want = golden_entry[stage]
    assert len(arr) == want["n"], (stage, len(arr), want["n"])
    assert golden_io.digest(arr) == want["sha256"], stage


@pytest.mark.parametrize("name", sorted(_frames()))
def test_cuda_path_matches_reference_sources(golden, det, name):
    from atag import stages
    img = _frames()[name]
    g = golden[name]
    t = torch.from_numpy(img).cuda()
    quads, st = det.detect([t])
    v = det.views(0)
    _check(g, "thresholded", v["thresholded"].ravel())
    _check(g, "labels", v["labels"].ravel())
    _check(g, "sizes", v["sizes"])
    _check(g, "filtered_keys", v["cluster_keys"])
    _check(g, "filtered_bounds", v["cluster_bounds"])
    _check(g, "extents", v["cluster_extents"])
    _check(g, "cluster_points", v["cluster_points"])
    _check(g, "line_fit", v["line_fit"])
    _check(g, "peak_extents", v["peak_extents"])
    _check(g, "fitted", v["fitted"])
    _check(g, "quads", quads[0])
    # stage entry points: tile extrema, dense boundary planes, fit_lines
    thr, ext, flt = stages.threshold_image(t, with_extrema=True)
    _check(g, "extrema", ext.cpu().numpy().ravel())
    _check(g, "filtered_extrema", flt.cpu().numpy().ravel())
    lab = torch.from_numpy(v["labels"].view(np.int32)).cuda()
    siz = torch.from_numpy(v["sizes"].view(np.int32)).cuda()
    pts, keys = stages.find_boundaries(lab, siz)
    _check(g, "dense_points", pts.cpu().numpy().view(golden_io.BOUNDARY_POINT))
    _check(g, "dense_keys", keys.cpu().numpy().view(np.uint64))
    ext_c = v["cluster_extents"]
    if len(ext_c):
        cidx = np.repeat(np.arange(len(ext_c), dtype=np.uint16), ext_c["count"])
        found = stages.fit_lines(v["line_fit"], cidx, ext_c)
        _check(g, "found_corners", found)
