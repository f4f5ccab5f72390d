"""atag_image_segmentation_noalloc: image segmentation for callers that
cannot allocate device memory (a thread capturing a CUDA graph, an
allocation-free camera frame loop, a host that owns all device memory).

Its union-find forest lives in a fixed array inside the library, so its
labels and sizes must equal those of atag_image_segmentation (which takes a
caller-allocated scratch buffer) bit for bit, on consecutive calls that
reuse the array, and it must refuse frames larger than the array."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _noalloc(thr):
    from atag import lib
    L = lib.init()
    h, w = thr.shape
    labels = torch.empty((h, w), dtype=torch.int32, device="cuda")
    sizes = torch.empty(h * w, dtype=torch.int32, device="cuda")
    st = L.atag_image_segmentation_noalloc(ctypes.c_void_p(thr.data_ptr()), ctypes.c_void_p(labels.data_ptr()),
                                           ctypes.c_void_p(sizes.data_ptr()), w, h,
                                           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    lib.check(st, "atag_image_segmentation_noalloc")
    return labels, sizes


def test_noalloc_matches_allocating_entry_point_on_consecutive_calls(ref_images):
    from atag import stages
    # 1920x1080 (near the 2,097,152-pixel limit), then a smaller frame, then
    # the first again: each call must be independent of what the array held
    for name in ("decimate2", "decimate4", "decimate2"):
        thr = stages.threshold_image(torch.from_numpy(ref_images[name]).cuda())
        want_labels, want_sizes, _ = stages.image_segmentation(thr)
        got_labels, got_sizes = _noalloc(thr)
        torch.cuda.synchronize()
        assert torch.equal(got_labels, want_labels), name
        assert torch.equal(got_sizes, want_sizes), name


def test_noalloc_rejects_frames_larger_than_its_array():
    from atag import AtagError
    thr = torch.zeros((2160, 3840), dtype=torch.uint8, device="cuda")
    with pytest.raises(AtagError, match="2097152"):
        _noalloc(thr)
