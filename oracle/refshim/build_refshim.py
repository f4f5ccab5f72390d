"""Builds the reference's own kernel sources into a CPU golden-vector
generator (test infrastructure only).

Compiles, from the reference tree where they lie (read-only, never copied):
  src/threshold.cpp src/segmentation.cpp src/find_boundaries.cpp src/fit_quad.cpp
plus oracle/refshim/harness.cpp, against the host SYCL shim in
oracle/refshim/include, into oracle/_ref/refshim_harness; and the
reference's vendored include/stb_image.h + stb_image_write.h with
oracle/refshim/stb_grey.cpp into oracle/_ref/stb_grey (colour removal).  Needs only g++;
skipped when the reference tree is not mounted.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference tree: ATAG_REFERENCE_TREE, else a checkout named "reference"
# beside this repository
REF = os.environ.get("ATAG_REFERENCE_TREE") or os.path.normpath(
    os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "..", "..", "reference"))
OUT_DIR = os.path.join(HERE, "..", "_ref")
BIN = os.path.join(OUT_DIR, "refshim_harness")
REF_SOURCES = ["threshold.cpp", "segmentation.cpp", "find_boundaries.cpp", "fit_quad.cpp"]


STB_BIN = os.path.join(OUT_DIR, "stb_grey")


def build_stb_grey(force: bool = False):
    """The reference's vendored stb_image(.h/_write.h) colour removal, as a
    tool (oracle/refshim/stb_grey.cpp)."""
    if not os.path.isfile(os.path.join(REF, "include", "stb_image.h")):
        return None
    os.makedirs(OUT_DIR, exist_ok=True)
    src = os.path.join(HERE, "stb_grey.cpp")
    deps = [src, os.path.join(REF, "include", "stb_image.h"), os.path.join(REF, "include", "stb_image_write.h")]
    if not force and os.path.exists(STB_BIN) and all(os.path.getmtime(d) <= os.path.getmtime(STB_BIN) for d in deps):
        return STB_BIN
    cmd = ["g++", "-std=c++17", "-O2", "-w", "-I", os.path.join(REF, "include"), src, "-o", STB_BIN + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(STB_BIN + ".tmp", STB_BIN)
    return STB_BIN


def build(force: bool = False):
    if not os.path.isdir(os.path.join(REF, "src")):
        return None
    build_stb_grey(force)
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = [os.path.join(REF, "src", s) for s in REF_SOURCES] + [os.path.join(HERE, "harness.cpp")]
    deps = srcs + [os.path.join(HERE, "include", "sycl", "sycl.hpp")]
    if not force and os.path.exists(BIN) and all(os.path.getmtime(d) <= os.path.getmtime(BIN) for d in deps):
        return BIN
    cmd = ["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-fno-fast-math", "-w",
           "-I", os.path.join(HERE, "include"), "-I", os.path.join(REF, "include"), *srcs, "-o", BIN + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(BIN + ".tmp", BIN)
    return BIN


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
