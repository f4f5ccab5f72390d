"""Every device status flag fires on a real frame when its capacity or cap
is lowered (atag_detector_set_limits, a small quad capacity, a cluster
with more corners than the corner sort takes), the call returns, and the
memory right after each capped buffer keeps the pattern it was filled with.
The reference has none of this: its fixed 65536-entry buffers overflow
silently (src/main.cpp:286-297)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

POISON = 0xA5


def _frame(name="1080p", seed=21):
    from conftest import synth_frame
    return synth_frame(name, seed)


def _defaults(img):
    """Counts and capacities of the frame with the detector's own sizing."""
    from atag.detector import Detector
    h, w = img.shape
    det = Detector(w, h)
    quads, st = det.detect([torch.from_numpy(img).cuda()])
    assert int(st[0]["status"]) == 0
    return det.views(0)["capacities"], st[0], quads[0]


def _poisoned_detector(img, **limits):
    from atag.detector import Detector
    h, w = img.shape
    det = Detector(w, h)
    det.workspace.fill_(POISON)  # before the first call: nothing of it is in use yet
    det.set_limits(**limits)
    return det


def _ws_bytes(det, ptr, lo, hi):
    off = ptr - det.workspace.data_ptr()
    assert 0 <= off and off + hi <= det.workspace.numel()
    return det.workspace[off + lo: off + hi].cpu().numpy()


def _run(det, img):
    quads, st = det.detect([torch.from_numpy(img).cuda()])
    torch.cuda.synchronize()  # the call returned and the device is idle
    return quads[0], st[0], det.views(0)


def test_point_overflow():
    from atag import records as R
    img = _frame()
    caps, st0, _ = _defaults(img)
    det = _poisoned_detector(img, point_capacity=1000)
    q, st, v = _run(det, img)
    assert int(st["status"]) & R.DEVFLAG_POINT_OVERFLOW
    assert v["capacities"]["point"] == 1000
    guard = _ws_bytes(det, v["pointers"]["pair_points"], 8 * 1000, 8 * caps["point"])
    assert (guard == POISON).all()


def test_pair_overflow():
    from atag import records as R
    img = _frame()
    caps, st0, _ = _defaults(img)
    assert int(st0["n_pairs"]) > 64
    det = _poisoned_detector(img, pair_capacity=48)  # rounded down to 32 slots
    q, st, v = _run(det, img)
    assert int(st["status"]) & R.DEVFLAG_PAIR_OVERFLOW
    assert v["capacities"]["pair"] == 32
    assert int(st["n_pairs"]) <= 32
    for name, size in (("pair_keys", 8), ("pair_count", 4), ("pair_bbox", 16), ("pair_gsum", 8), ("pair_pxgx", 8)):
        guard = _ws_bytes(det, v["pointers"][name], size * 32, size * caps["pair"])
        assert (guard == POISON).all(), name


def test_cluster_overflow_by_count():
    from atag import records as R
    img = _frame()
    caps, st0, _ = _defaults(img)
    assert int(st0["n_clusters"]) > 4
    det = _poisoned_detector(img, cluster_capacity=4)
    q, st, v = _run(det, img)
    assert int(st["status"]) & R.DEVFLAG_CLUSTER_OVERFLOW
    assert int(st["n_clusters"]) == 4
    for name, size in (("cluster_bounds", 32), ("cluster_extents", 8), ("peak_count", 4), ("fitted", 272)):
        guard = _ws_bytes(det, v["pointers"][name], size * 4, size * caps["cluster"])
        assert (guard == POISON).all(), name


def test_cluster_overflow_by_points():
    from atag import records as R
    img = _frame()
    caps, st0, _ = _defaults(img)
    assert int(st0["n_cluster_points"]) > 2000
    det = _poisoned_detector(img, cluster_point_capacity=2000)
    q, st, v = _run(det, img)
    assert int(st["status"]) & R.DEVFLAG_CLUSTER_OVERFLOW
    assert int(st["n_cluster_points"]) <= 2000
    for name, size in (("cluster_points", 8), ("line_fit_points", 64)):
        guard = _ws_bytes(det, v["pointers"][name], size * 2000, size * caps["cluster_point"])
        assert (guard == POISON).all(), name


def test_quad_overflow_stays_in_its_frame():
    """Frame 0 finds more quads than the capacity: its status says so, its
    first quads are kept, and frame 1's slots (right after frame 0's) hold
    frame 1's own quads."""
    from atag import records as R
    from atag.detector import Detector
    from conftest import small_frames
    a, b = _frame(seed=21), small_frames()["square"]
    _, sa, qa = _defaults(a)
    _, sb, qb = _defaults(b)
    assert len(qa) > 3 and 0 < len(qb) <= 3
    det = Detector(1920, 1080, max_frames=2, quad_capacity=3)
    quads, st = det.detect([torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()])
    assert int(st[0]["status"]) & R.DEVFLAG_QUAD_OVERFLOW
    assert int(st[1]["status"]) == 0
    assert quads[0].tobytes() == qa[:3].tobytes()
    assert quads[1].tobytes() == qb.tobytes()


def test_sort_overflow_in_corner_peaks():
    """A cluster whose corner array holds more corners than a cluster of
    valid points can (more than the shared-memory corner sort takes) is
    flagged and skipped; the call returns and the other clusters' corners
    are sorted as usual."""
    from atag import records as R
    from atag import stages
    n_big = 40000
    found = np.zeros(n_big + 64, R.CORNER)
    found["error"][:n_big] = np.linspace(1.0, 2.0, n_big, dtype=np.float32)
    found["cluster_index"][:n_big] = 0
    found["line_fit_point_index"][:n_big] = np.arange(n_big)
    tail = found[n_big:]
    tail["cluster_index"] = 1
    tail["line_fit_point_index"] = np.arange(64)
    tail["error"][::4] = np.arange(16, dtype=np.float32)[::-1] + 0.5
    ext = np.array([(0, n_big), (n_big, 64)], R.CLUSTER_EXTENTS)
    d_found, d_ext = stages.to_device(found), stages.to_device(ext)
    corners, pe, (k, cp, status) = stages.corner_peaks(d_found, d_ext, 2, n_big + 64)
    assert status & R.DEVFLAG_SORT_OVERFLOW
    assert (k, cp) == (n_big + 16, 2)
    got = stages.to_host(corners, R.CORNER)[n_big: n_big + 16]
    assert np.array_equal(got["line_fit_point_index"], np.arange(0, 64, 4))
    assert np.all(np.diff(got["error"]) < 0)


def test_union_find_iteration_cap():
    """With the frame-wide union-find walks capped at one parent, a 4K stress
    frame (tens of thousands of components across tile borders) runs out of
    iterations: the flag is set and the call returns.  With the default
    bound the same frame is clean."""
    from atag import records as R
    from atag.detector import Detector
    img = _frame("4k", 3)
    det = Detector(3840, 2160)
    q, st, _ = _run(det, img)
    assert int(st["status"]) == 0
    det.set_limits(uf_iteration_cap=1)
    q, st, _ = _run(det, img)
    assert int(st["status"]) & R.DEVFLAG_UF_ITERATION_CAP
    det.set_limits()
    q2, st2, _ = _run(det, img)
    assert int(st2["status"]) == 0
