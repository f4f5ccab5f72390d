"""CPU checks of the C ABI: the library builds/loads, exports every symbol
include/atag.h declares, records have the reference's sizes, defaults
match, and calls without a device fail with a status instead of crashing."""
import ctypes

import numpy as np
import pytest

from atag import lib, records


def test_library_exports_every_declared_symbol():
    L = lib.load()
    declared = lib.declared_symbols()
    assert len(declared) >= 20
    missing = [s for s in declared if not hasattr(L, s)]
    assert not missing, missing


def test_signature_table_covers_header():
    assert sorted(lib._SIGNATURES) == lib.declared_symbols()


def test_record_sizes_match_reference_layouts():
    # sizes of the reference's records (probed from its headers)
    assert records.BOUNDARY_POINT.itemsize == 4
    assert records.CLUSTER_POINT.itemsize == 8
    assert records.CLUSTER_BOUNDS.itemsize == 32
    assert records.LINE_FIT_POINT.itemsize == 64
    assert records.CORNER.itemsize == 12
    assert records.FITTED_QUAD.itemsize == 272
    assert records.QUAD_CORNERS.itemsize == 40
    assert ctypes.sizeof(records.Config) == 44


def test_config_defaults_match_reference_constants():
    c = lib.default_config()
    assert (c.decimate, c.min_white_black_diff, c.min_component_size, c.min_cluster_pixels) == (1, 5, 25, 5)
    assert (c.tag_width, c.normal_border, c.reversed_border) == (4, 1, 0)
    assert c.max_line_fit_mse == 10.0 and c.critical_angle_deg == 10.0
    assert c.min_tag_width == 8 and c.compat_peak_index == 1


def test_config_defaults_match_oracle():
    import oracle
    a, b = lib.default_config(), oracle.default_config()
    for name, _ in records.Config._fields_:
        assert getattr(a, name) == getattr(b, name), name


def test_status_strings():
    L = lib.load()
    for s in range(7):
        assert L.atag_status_string(s)
    assert L.atag_status_string(99) == b"unknown status"


def test_workspace_size_validates_arguments():
    L = lib.load()
    n = ctypes.c_size_t()
    c = lib.default_config()
    assert L.atag_workspace_size(ctypes.byref(c), 1920, 1080, 1, 0, ctypes.byref(n)) == 0
    assert n.value > 1920 * 1080 * 40
    # odd sizes are refused before anything is launched
    assert L.atag_workspace_size(ctypes.byref(c), 1922, 1080, 1, 0, ctypes.byref(n)) == 1
    assert L.atag_workspace_size(ctypes.byref(c), 8192, 1080, 1, 0, ctypes.byref(n)) == 1
    # batch bound grows with the pixel budget
    m = ctypes.c_size_t()
    assert L.atag_workspace_size(ctypes.byref(c), 2592, 1944, 64, 64 * 2592 * 1944, ctypes.byref(m)) == 0
    assert m.value > n.value


def test_stage_workspace_sizes_validate_arguments():
    L = lib.load()
    n = ctypes.c_size_t()
    assert L.atag_cluster_workspace_size(1920, 1080, 65535, 1 << 20, ctypes.byref(n)) == 0
    assert n.value > 16 * (1 << 20)
    assert L.atag_cluster_workspace_size(1922, 1080, 65535, 1 << 20, ctypes.byref(n)) == 1
    assert L.atag_cluster_workspace_size(1920, 1080, 0, 1 << 20, ctypes.byref(n)) == 1
    assert L.atag_corner_peaks_workspace_size(100, ctypes.byref(n)) == 0 and n.value >= 800


def test_calls_without_device_return_status(monkeypatch):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    L = lib.load()
    st = L.atag_init()
    assert st == 5  # ATAG_ERR_NO_DEVICE
    assert L.atag_last_error()
    st = L.atag_threshold_image(None, None, None, None, 64, 64, None)
    assert st == 5
    st = L.atag_estimate_pose(None, 32, 4, 1000.0, 1000.0, 960.0, 540.0, 0.16, 20, None, None)
    assert st == 5
    assert L.atag_refine_forward(None, 64, 64, None, 1, None, None, None, None) == 5
    assert L.atag_decode_quads(None, 64, 64, 64, None, 32, 1, None, None, None, None) == 5
    assert L.atag_cluster(None, None, None, 64, 64, None, 0, None, None) == 5
    assert L.atag_corner_peaks(None, None, 1, None, 0, None, 0, None, 0, None, None) == 5


def test_cpp_header_compiles_against_the_c_abi(tmp_path):
    """include/atag.hpp (reference-named C++ wrappers) compiles and links
    against the library (no device needed to link)."""
    import os
    import shutil
    import subprocess
    if not shutil.which("g++"):
        pytest.skip("no g++")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "use.cpp"
    src.write_text('#include "atag.hpp"\n'
                   "int main() {\n"
                   "  cudaStream_t q = nullptr;\n"
                   "  atag_status s = atag::threshold_image(q, nullptr, nullptr, nullptr, nullptr, 6, 6);\n"
                   "  return s == ATAG_ERR_INVALID_ARGUMENT || s == ATAG_ERR_NO_DEVICE ? 0 : 1;\n"
                   "}\n")
    lib.load()
    libdir = os.path.dirname(lib.LIB_PATH)
    cuda_inc = "/usr/local/cuda/include"
    r = subprocess.run(["g++", "-std=c++17", "-I", os.path.join(root, "include"), "-I", cuda_inc, str(src),
                        "-L", libdir, "-latag_gb300", f"-Wl,-rpath,{libdir}", "-o", str(tmp_path / "use")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(tmp_path / "use")], capture_output=True, text=True)
    assert r.returncode == 0
