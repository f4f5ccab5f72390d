"""The reference's host helpers exported by the library (atag_get_moment,
atag_fit_line, atag_compute_initial_linefit and their C++ names
get_moment, fit_line, compute_initial_linefit in include/atag.hpp) against
the record goldens evaluated by the reference's own headers and
src/fit_quad.cpp (tests/golden/records.npz).  Host code only: no device."""
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

sys.path.insert(0, GOLDEN)
import golden_io  # noqa: E402


@pytest.fixture(scope="module")
def records():
    with np.load(os.path.join(GOLDEN, "records.npz")) as z:
        return {k: z[k].view(golden_io.RECORD_ARRAYS[k]) if z[k].dtype == np.uint8 and
                golden_io.RECORD_ARRAYS[k] is not np.uint8 else z[k] for k in z.files}


def test_fit_line_matches_reference(records):
    from atag import stages
    m, nim = records["rec_moments"], records["rec_num_in_moment"]
    lp, err, mse = [], [], []
    for i in range(len(m)):
        a, e, s = stages.fit_line(m[i], int(nim[i]))
        lp.append(a)
        err.append(e)
        mse.append(s)
    assert np.array_equal(np.concatenate(lp).view(np.uint32), records["rec_line_params"].view(np.uint32))
    assert np.array_equal(np.array(err, np.float32).view(np.uint32), records["rec_err"].view(np.uint32))
    assert np.array_equal(np.array(mse, np.float32).view(np.uint32), records["rec_mse"].view(np.uint32))


def test_get_moment_matches_reference(records):
    from atag import lib, stages
    pre = records["rec_prefix"]
    ranges = records["rec_moment_range"].reshape(-1, 2)
    out, cnt = [], []
    for i0, i1 in ranges:
        o, n = stages.get_moment(pre, int(i0), int(i1))
        out.append(o)
        cnt.append(n)
    assert golden_io.digest(np.array(out, golden_io.LINE_FIT_POINT)) == golden_io.digest(records["rec_moment"])
    assert np.array_equal(np.array(cnt, np.uint64), records["rec_moment_n"])
    # ranges past the array are refused, not read
    with pytest.raises(lib.AtagError):
        stages.get_moment(pre, len(pre), 0)


def test_get_moment_keeps_the_leading_operand_a_b():
    """The reference copies the leading prefix entry (a and b included)."""
    from atag import records, stages
    pre = np.zeros(6, records.LINE_FIT_POINT)
    pre["W"] = np.arange(1, 7)
    pre["a"] = np.arange(10, 16)
    m, n = stages.get_moment(pre, 1, 3)
    assert (n, int(m["W"]), int(m["a"])) == (3, 4 - 1, 13)
    m, n = stages.get_moment(pre, 4, 1)
    assert (n, int(m["W"]), int(m["a"])) == (4, 6 - 4 + 2, 15)
    m, n = stages.get_moment(pre, 2, 2)
    assert (n, int(m["W"]), int(m["a"])) == (0, 0, 0)


def test_initial_linefit_matches_reference(records):
    from atag import stages
    img = records["rec_image"].reshape(192, 256)
    got = np.array([stages.compute_initial_linefit(p, 256, 192, img) for p in records["rec_cluster_points"]],
                   golden_io.LINE_FIT_POINT)
    assert golden_io.digest(got) == golden_io.digest(records["rec_linefit"])


def test_cpp_names_match_reference(records, tmp_path):
    """A C++ program written against include/atag.hpp calls get_moment,
    fit_line and compute_initial_linefit by the reference's names and
    argument order; its results are the reference's, bit for bit."""
    if not shutil.which("g++"):
        pytest.skip("no g++")
    from atag import lib
    lib.load()
    m = np.ascontiguousarray(records["rec_moments"])
    nim = np.ascontiguousarray(records["rec_num_in_moment"], np.uint64)
    pre = np.ascontiguousarray(records["rec_prefix"])
    rng = np.ascontiguousarray(records["rec_moment_range"], np.uint64)
    cps = np.ascontiguousarray(records["rec_cluster_points"])
    img = np.ascontiguousarray(records["rec_image"])
    for name, a in (("m", m), ("nim", nim), ("pre", pre), ("rng", rng), ("cps", cps), ("img", img)):
        a.tofile(tmp_path / f"{name}.bin")
    src = tmp_path / "helpers.cpp"
    src.write_text(r'''
#include <cstdio>
#include <vector>
#include "atag.hpp"
template <class T> std::vector<T> rd(const char* p) {
    std::vector<T> v; FILE* f = fopen(p, "rb"); T x;
    while (fread(&x, sizeof x, 1, f) == 1) v.push_back(x);
    fclose(f); return v;
}
template <class T> void wr(const char* p, const std::vector<T>& v) {
    FILE* f = fopen(p, "wb"); fwrite(v.data(), sizeof(T), v.size(), f); fclose(f);
}
int main() {
    auto m = rd<atag::LineFitPoint>("m.bin");
    auto nim = rd<uint64_t>("nim.bin");
    std::vector<float> lp(4 * m.size()), err(m.size()), mse(m.size());
    for (size_t i = 0; i < m.size(); i++) atag::fit_line(m[i], nim[i], &lp[4 * i], &err[i], &mse[i]);
    wr("lp.out", lp); wr("err.out", err); wr("mse.out", mse);
    auto pre = rd<atag::LineFitPoint>("pre.bin");
    auto rng = rd<uint64_t>("rng.bin");
    std::vector<atag::LineFitPoint> mo; std::vector<uint64_t> cnt;
    for (size_t i = 0; i + 1 < rng.size(); i += 2) {
        auto [moment, n] = atag::get_moment(pre.data(), pre.size(), rng[i], rng[i + 1]);
        mo.push_back(moment); cnt.push_back(n);
    }
    wr("mo.out", mo); wr("cnt.out", cnt);
    auto cps = rd<atag::ClusterPoint>("cps.bin");
    auto img = rd<uint8_t>("img.bin");
    std::vector<atag::LineFitPoint> lf;
    for (auto& p : cps) lf.push_back(atag::compute_initial_linefit(p, 256, 192, img.data()));
    wr("lf.out", lf);
    return 0;
}
''')
    libdir = os.path.dirname(lib.LIB_PATH)
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I",
                        "/usr/local/cuda/include", str(src), "-L", libdir, "-latag_gb300", f"-Wl,-rpath,{libdir}",
                        "-o", str(tmp_path / "helpers")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(tmp_path / "helpers")], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr

    def out(name, dtype):
        return np.fromfile(tmp_path / name, dtype=dtype)
    assert np.array_equal(out("lp.out", np.uint32), records["rec_line_params"].view(np.uint32))
    assert np.array_equal(out("err.out", np.uint32), records["rec_err"].view(np.uint32))
    assert np.array_equal(out("mse.out", np.uint32), records["rec_mse"].view(np.uint32))
    assert golden_io.digest(out("mo.out", golden_io.LINE_FIT_POINT)) == golden_io.digest(records["rec_moment"])
    assert np.array_equal(out("cnt.out", np.uint64), records["rec_moment_n"])
    assert golden_io.digest(out("lf.out", golden_io.LINE_FIT_POINT)) == golden_io.digest(records["rec_linefit"])
