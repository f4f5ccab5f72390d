"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/atag_oracle.c into oracle/lib/libatag_oracle.so with strict
IEEE float semantics (-ffp-contract=off, no fast-math) and OpenMP.  Run as
`python oracle/build_oracle.py` or through __graft_entry__.build().
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIB_DIR, "libatag_oracle.so")
SRC = os.path.join(HERE, "atag_oracle.c")

CFLAGS = ["-O2", "-std=c11", "-D_GNU_SOURCE", "-fPIC", "-shared", "-ffp-contract=off",
          "-fno-fast-math", "-fopenmp", "-Wall", "-Wextra", "-Wno-unused-parameter"]


def build(force: bool = False) -> str:
    os.makedirs(LIB_DIR, exist_ok=True)
    deps = [SRC, os.path.join(HERE, "atag_oracle.h"),
            os.path.join(HERE, "..", "include", "atag.h")]
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in deps):
            return LIB
    cmd = ["gcc", *CFLAGS, SRC, "-o", LIB + ".tmp", "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
