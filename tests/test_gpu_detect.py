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
    return Detector(1920, 1080, keep_intermediates=True)


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


def test_default_detector_skips_only_unread_intermediates(det1080):
    """A detector that does not keep intermediates gives the same quads,
    labels, component sizes (at every label's root), surviving clusters and
    cluster points as one that writes the reference's full segmentation
    arrays."""
    from atag.detector import Detector
    lean = Detector(1920, 1080)
    for seed in (5, 6):
        img = synth_frame("1080p", seed)
        q_full, v_full = _run(det1080, img)
        q_lean, v_lean = _run(lean, img)
        assert len(q_full) > 0 and q_full.tobytes() == q_lean.tobytes()
        assert np.array_equal(v_full["labels"], v_lean["labels"])
        roots = np.unique(v_full["labels"].ravel() & 0x7FFFFFFF)
        assert np.array_equal(v_full["sizes"][roots], v_lean["sizes"][roots])
        assert np.array_equal(v_full["line_fit"], v_lean["line_fit"])
        assert np.array_equal(v_full["cluster_keys"], v_lean["cluster_keys"])
        assert np.array_equal(v_full["cluster_extents"], v_lean["cluster_extents"])
        fields = [f for f in v_full["cluster_bounds"].dtype.names if f != "start"]
        for f in fields:
            assert np.array_equal(v_full["cluster_bounds"][f], v_lean["cluster_bounds"][f]), f
        assert np.array_equal(v_full["cluster_points"], v_lean["cluster_points"])


def test_skipping_pairs_over_the_size_limit_changes_nothing():
    """In a lean batch the boundary tiles skip the points of pairs that
    earlier tiles already pushed over ValidBlobFilter's size limit (these
    frames have two to four such pairs, the largest of 1.1-1.2 M points; the
    frame's list holds two).  Quads and every per-frame count equal those of
    a detector that keeps the full per-pair sums."""
    from atag.detector import Detector
    imgs = [torch.from_numpy(synth_frame("1080p", 20 + i)).cuda() for i in range(12)]
    lean = Detector(1920, 1080, max_frames=len(imgs), max_total_pixels=len(imgs) * 1920 * 1080)
    full = Detector(1920, 1080, max_frames=len(imgs), max_total_pixels=len(imgs) * 1920 * 1080,
                    keep_intermediates=True)
    q_lean, st_lean = lean.detect(imgs)
    q_full, st_full = full.detect(imgs)
    fields = ("n_points", "n_pairs", "n_clusters", "n_cluster_points", "n_corners", "n_peak_clusters",
              "n_fitted", "n_quads", "status")
    for i in range(len(imgs)):
        assert int(st_lean[i]["status"]) == 0
        assert len(q_full[i]) > 0 and q_lean[i].tobytes() == q_full[i].tobytes()
        for f in fields:
            assert int(st_lean[i][f]) == int(st_full[i][f]), (i, f)


def test_detect_decimate2():
    from atag import lib
    from atag.detector import Detector
    cfg = lib.default_config(decimate=2)
    det = Detector(960, 540, config=cfg, keep_intermediates=True)
    img = synth_frame("1080p", 3)
    quads, views = _run(det, img)
    res = oracle.detect(img, oracle.default_config(decimate=2))
    assert np.array_equal(views["decimated"], res["decimated"])
    assert_detect_matches(views, quads, res)


def test_detect_aligned_peak_index_mode(ref_images):
    from atag import lib
    from atag.detector import Detector
    det = Detector(1920, 1080, config=lib.default_config(compat_peak_index=0), keep_intermediates=True)
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
    det = Detector(3840, 2160, keep_intermediates=True)
    quads, views = _run(det, img)
    res = oracle.detect(img)
    assert_detect_matches(views, quads, res)
    assert int(res["extents"]["count"].max()) > 12288  # exercises the global-memory sort


def test_mixed_resolution_batch_matches_oracle_and_singles():
    """A batch drawn like the 64-frame benchmark batch (sizes from 640x480 to
    2592x1944, 0-60 fiducials, 0-1000 clutter shapes each) gives every frame
    the same result as alone, and the oracle's."""
    from atag import synth
    from atag.detector import Detector
    specs = synth.batch_specs(10, seed=4)
    imgs = [synth.render(s, 500 + i) for i, s in enumerate(specs)]
    det = Detector(2592, 1944, max_frames=len(imgs), max_total_pixels=sum(i.size for i in imgs))
    quads, st = det.detect([torch.from_numpy(i).cuda() for i in imgs])
    alone = Detector(2592, 1944)
    for i, img in enumerate(imgs):
        assert int(st[i]["status"]) == 0
        q, s1 = alone.detect([torch.from_numpy(img).cuda()])
        assert_quads_match(quads[i], q[0], tol=0.0)
        if i < 3:
            assert_quads_match(quads[i], oracle.detect(img)["quads"])


def test_every_tuning_gives_identical_results_and_autotune_applies(tmp_path):
    from atag import autotune
    from atag.detector import Detector
    imgs = [synth_frame("1080p", 1), synth_frame("vga", 2)]
    frames = [torch.from_numpy(i).cuda() for i in imgs]
    det = Detector(1920, 1080, max_frames=2, max_total_pixels=sum(i.size for i in imgs))
    base, _ = det.detect(frames)
    for t in ({"ccl_tile_rows": 8, "boundary_tile_rows": 8, "small_cluster_max": 1024, "small_ctas_per_sm": 2,
               "large_ctas_divisor": 8, "index_ctas_per_sm": 4, "batch_lanes": 1},
              {"ccl_tile_rows": 16, "boundary_tile_rows": 8, "small_cluster_max": 2048, "small_ctas_per_sm": 6,
               "large_ctas_divisor": 2, "index_ctas_per_sm": 16, "batch_lanes": 2},
              {"ccl_tile_rows": 32, "boundary_tile_rows": 16, "small_cluster_max": 700, "small_ctas_per_sm": 8,
               "large_ctas_divisor": 1, "index_ctas_per_sm": 8, "batch_lanes": 4}):
        det.set_tuning(**t)
        q, st = det.detect(frames)
        for a, b in zip(q, base):
            assert a.tobytes() == b.tobytes()
    cache = str(tmp_path / "tune.json")
    out = autotune.autotune(det, frames, reps=2, passes=1, cache_path=cache)
    assert out["ms"] <= out["default_ms"] * 1.05
    det2 = Detector(1920, 1080, max_frames=2, max_total_pixels=sum(i.size for i in imgs))
    assert autotune.apply_cached(det2, frames, cache)
    assert det2.get_tuning() == out["tuning"]
