"""CUDA graphs captured from atag_detect_batch keep detecting the frames
they captured, however many eager calls with other frames run on the same
detector in between (the frame table of a captured call has a copy of its
own that eager calls never rewrite)."""
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _frames():
    from conftest import small_frames, synth_frame
    a = [synth_frame("1080p", 31), synth_frame("1080p", 32)]
    b = [synth_frame("vga", 33), small_frames()["square"], synth_frame("vga", 34)]
    return a, b


def test_replay_after_many_eager_calls_detects_the_captured_frames():
    from atag.detector import Detector
    a, b = _frames()
    det = Detector(1920, 1080, max_frames=4)
    A = [torch.from_numpy(x).cuda() for x in a]
    B = [torch.from_numpy(x).cuda() for x in b]
    want_q, want_st = det.detect(A)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        det.enqueue(A, stream=s)  # the eager call right before the capture has the same table
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        det.enqueue(A, stream=s)
    # more eager calls with other frames than the ring of eager tables holds
    for i in range(20):
        det.detect([B[i % len(B)]])
    with torch.cuda.stream(s):
        g.replay()
    s.synchronize()
    got_q, got_st = det.results(len(A))
    assert got_st.tobytes() == want_st.tobytes()
    for x, y in zip(got_q, want_q):
        assert x.tobytes() == y.tobytes()
    # eager calls still see their own frames afterwards
    q, st = det.detect([B[0]])
    q0, _ = Detector(640, 480).detect([B[0]])
    assert q[0].tobytes() == q0[0].tobytes()


def test_distinct_captured_tables_are_bounded_and_released():
    from atag import lib
    from atag.detector import Detector
    a, _ = _frames()
    det = Detector(1920, 1080)
    frames = [torch.from_numpy(a[0]).cuda() for _ in range(17)]  # 17 different device pointers
    s = torch.cuda.Stream()
    graphs = []
    for f in frames[:16]:
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            det.enqueue([f], stream=s)
        graphs.append(g)
    # the same table again shares its copy
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        det.enqueue([frames[0]], stream=s)
    graphs.append(g)
    with pytest.raises(lib.AtagError):
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            det.enqueue([frames[16]], stream=s)
    del graphs, g
    torch.cuda.synchronize()
    det.release_captures()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        det.enqueue([frames[16]], stream=s)
    with torch.cuda.stream(s):
        g.replay()
    s.synchronize()
    q, st = det.results(1)
    q0, st0 = Detector(1920, 1080).detect([frames[16]])
    assert q[0].tobytes() == q0[0].tobytes()
