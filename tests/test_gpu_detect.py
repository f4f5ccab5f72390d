"""Parity of the fused whole-path detector with the CPU oracle: every
intermediate (threshold, partition, sizes, boundary point sets, cluster
order and bounds, sorted cluster points, line-fit prefix sums, peaks,
fitted quads) bit-exact, quad corners within 1e-3 px."""
import numpy as np
import pytest

import oracle
from conftest import small_frames, synth_frame
from gpu_helpers import assert_detect_matches, assert_quads_match

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _run(det, img):
    g = torch.from_numpy(np.ascontiguousarray(img)).cuda()
    quads, st = det.detect([g])
    return quads[0], det.views(0)


@pytest.fixture(scope="module")
def det1080():
    from atag.detector import Detector
    return Detector(1920, 1080)


@pytest.mark.parametrize("name", ["decimate", "decimate4", "decimate2"])
def test_detect_reference_images(det1080, ref_images, name):
    img = ref_images[name]
    quads, views = _run(det1080, img)
    res = oracle.detect(img)
    assert_detect_matches(views, quads, res)
    assert len(quads) > 0


@pytest.mark.parametrize("seed", [1, 2])
def test_detect_synthetic_1080p(det1080, seed):
    img = synth_frame("1080p", seed)
    quads, views = _run(det1080, img)
    res = oracle.detect(img)
    assert_detect_matches(views, quads, res)


def test_detect_small_and_edge_frames(det1080):
    for name, img in small_frames().items():
        quads, views = _run(det1080, img)
        res = oracle.detect(img)
        assert_detect_matches(views, quads, res)


def test_detect_decimate2():
    from atag import lib
    from atag.detector import Detector
    cfg = lib.default_config(decimate=2)
    det = Detector(960, 540, config=cfg)
    img = synth_frame("1080p", 3)
    quads, views = _run(det, img)
    res = oracle.detect(img, oracle.default_config(decimate=2))
    assert np.array_equal(views["decimated"], res["decimated"])
    assert_detect_matches(views, quads, res)


def test_detect_aligned_peak_index_mode(ref_images):
    from atag import lib
    from atag.detector import Detector
    det = Detector(1920, 1080, config=lib.default_config(compat_peak_index=0))
    for name in ("decimate", "decimate2"):
        img = ref_images[name]
        quads, views = _run(det, img)
        res = oracle.detect(img, oracle.default_config(compat_peak_index=0))
        assert_detect_matches(views, quads, res)


def test_batch_equals_each_frame_alone(ref_images):
    from atag.detector import Detector
    imgs = [ref_images["decimate"], synth_frame("1080p", 1), ref_images["decimate4"], synth_frame("vga", 2),
            ref_images["decimate2"]]
    det = Detector(1920, 1080, max_frames=len(imgs), max_total_pixels=sum(i.size for i in imgs))
    batch = [torch.from_numpy(i).cuda() for i in imgs]
    quads_b, st_b = det.detect(batch)
    alone = Detector(1920, 1080)
    for i, img in enumerate(imgs):
        q, st = alone.detect([torch.from_numpy(img).cuda()])
        assert_quads_match(quads_b[i], q[0], tol=0.0)
        assert st_b[i].tobytes() == st[0].tobytes()
        res = oracle.detect(img)
        assert_quads_match(quads_b[i], res["quads"])


def test_repeat_runs_are_identical(det1080):
    img = synth_frame("1080p", 2)
    a, va = _run(det1080, img)
    b, vb = _run(det1080, img)
    assert a.tobytes() == b.tobytes()
    assert np.array_equal(va["cluster_points"], vb["cluster_points"])


def test_host_buffer_path_matches(det1080, ref_images):
    img = ref_images["decimate2"]
    q_host, st = det1080.detect_host(img)
    res = oracle.detect(img)
    assert_quads_match(q_host, res["quads"])
    assert int(st["n_quads"]) == len(res["quads"])


def test_detect_4k_stress():
    """3840x2160 with 3000 clutter shapes and salt-and-pepper noise: many
    pairs, clusters above the shared-memory sort capacity (global-memory
    radix path) and deep union-find merges."""
    from atag.detector import Detector
    img = synth_frame("4k", 1)
    det = Detector(3840, 2160)
    quads, views = _run(det, img)
    res = oracle.detect(img)
    assert_detect_matches(views, quads, res)
    assert int(res["extents"]["count"].max()) > 12288  # exercises the global-memory sort
