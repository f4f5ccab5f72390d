"""Builds the reference's own kernel sources into a CPU golden-vector
generator (test infrastructure only).

Compiles, from the reference tree where they lie (read-only, never copied):
  src/threshold.cpp src/segmentation.cpp src/find_boundaries.cpp src/fit_quad.cpp
plus oracle/refshim/harness.cpp, against the host SYCL shim in
oracle/refshim/include, into oracle/_ref/refshim_harness.  Needs only g++;
skipped when the reference tree is not mounted.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("ATAG_REFERENCE_TREE", "/root/reference")
OUT_DIR = os.path.join(HERE, "..", "_ref")
BIN = os.path.join(OUT_DIR, "refshim_harness")
REF_SOURCES = ["threshold.cpp", "segmentation.cpp", "find_boundaries.cpp", "fit_quad.cpp"]


def build(force: bool = False):
    if not os.path.isdir(os.path.join(REF, "src")):
        return None
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
