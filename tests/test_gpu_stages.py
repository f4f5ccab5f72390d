"""Parity of the drop-in stage entry points (threshold_image,
image_segmentation, find_boundaries, fit_lines, do_indexing,
process_fitted_quads) with the CPU oracle, through the C ABI."""
import numpy as np
import pytest

import oracle
from conftest import small_frames, synth_frame
from gpu_helpers import assert_quads_match

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _frames(ref_images):
    out = dict(ref_images)
    out.update(small_frames())
    out["vga_d2"] = oracle.decimate(synth_frame("vga", 3), 2)
    out["1080p"] = synth_frame("1080p", 1)
    return out


@pytest.fixture(scope="module")
def frames(ref_images):
    return _frames(ref_images)


def test_threshold_bit_exact(frames):
    from atag import stages
    for name, img in frames.items():
        g = torch.from_numpy(img).cuda()
        thr, ext, flt = stages.threshold_image(g, with_extrema=True)
        o_thr, o_ext, o_flt = oracle.threshold(img)
        assert np.array_equal(thr.cpu().numpy(), o_thr), name
        assert np.array_equal(ext.cpu().numpy(), o_ext), name
        assert np.array_equal(flt.cpu().numpy(), o_flt), name


def test_decimate_point_sampling(frames):
    from atag import stages
    img = frames["1080p"]
    for f in (2, 3, 4):
        h, w = img.shape[0] // f // 4 * 4 * f, img.shape[1] // f // 4 * 4 * f
        src = np.ascontiguousarray(img[:h, :w])
        out = stages.decimate(torch.from_numpy(src).cuda(), f).cpu().numpy()
        assert np.array_equal(out, oracle.decimate(src, f)), f


def test_segmentation_partition_and_sizes(frames):
    from atag import stages
    for name, img in frames.items():
        o_thr = oracle.threshold(img)[0]
        labels, sizes, _ = stages.image_segmentation(torch.from_numpy(o_thr).cuda())
        o_lab, o_sizes = oracle.segmentation(o_thr)
        assert np.array_equal(labels.cpu().numpy().view(np.uint32), o_lab), name
        assert np.array_equal(sizes.cpu().numpy().view(np.uint32), o_sizes), name


def test_segmentation_random_ternary_images():
    """Random {0,127,255} images exercise the two-forest links and the
    bridge through 2x2 blocks of the other colour."""
    from atag import stages
    rng = np.random.default_rng(11)
    for trial in range(6):
        h, w = [(4, 4), (8, 8), (36, 44), (100, 64), (256, 260), (1080, 1920)][trial]
        thr = rng.choice(np.array([0, 127, 255], np.uint8), size=(h, w), p=[0.45, 0.1, 0.45])
        labels, sizes, _ = stages.image_segmentation(torch.from_numpy(thr).cuda())
        o_lab, o_sizes = oracle.segmentation(thr)
        assert np.array_equal(labels.cpu().numpy().view(np.uint32), o_lab), (h, w)
        assert np.array_equal(sizes.cpu().numpy().view(np.uint32), o_sizes), (h, w)


def test_find_boundaries_dense_planes(frames):
    from atag import stages
    for name, img in frames.items():
        o_thr = oracle.threshold(img)[0]
        o_lab, o_sizes = oracle.segmentation(o_thr)
        pts, keys = stages.find_boundaries(torch.from_numpy(o_lab.view(np.int32)).cuda(),
                                           torch.from_numpy(o_sizes.view(np.int32)).cuda())
        o_pts, o_keys = oracle.find_boundaries(o_lab, o_sizes)
        assert np.array_equal(pts.cpu().numpy().view(np.uint32), o_pts.view(np.uint32)), name
        assert np.array_equal(keys.cpu().numpy().view(np.uint64), o_keys), name


@pytest.mark.parametrize("name", ["decimate", "decimate4", "decimate2", "1080p", "square"])
def test_fit_lines_do_indexing_process_quads(frames, name):
    from atag import stages
    res = oracle.detect(frames[name])
    if len(res["cluster_points"]) == 0:
        pytest.skip("no clusters")
    found = stages.fit_lines(res["line_fit"], res["cluster_indices"], res["extents"])
    assert np.array_equal(found, res["found_corners"])
    fitted = stages.do_indexing(res["peak_extents"], res["corners"], res["line_fit"], res["extents"])
    assert np.array_equal(fitted, res["fitted"])
    quads = stages.process_fitted_quads(res["fitted"], res["width"], res["height"])
    assert_quads_match(quads, res["quads"])


def test_invalid_dimensions_raise():
    from atag import stages, AtagError
    with pytest.raises(AtagError):
        stages.threshold_image(torch.zeros((10, 10), dtype=torch.uint8, device="cuda"))
    with pytest.raises(AtagError):
        stages.image_segmentation(torch.zeros((6, 8), dtype=torch.uint8, device="cuda"))
