"""The integer emulations used on the device (FP64 and 64-bit conversions
are slow on this GPU) against the operations they replace, bit for bit:
hypotf's FP64 formula and C++'s int64 -> float conversion, compiled for the
host from the same header."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.skipif(shutil.which("nvcc") is None, reason="nvcc not installed")
def test_integer_emulations_are_bit_exact(tmp_path):
    exe = tmp_path / "arith_check"
    subprocess.run(["nvcc", "-O2", "-std=c++17", "-Xcompiler", "-ffp-contract=off", "-o", str(exe),
                    os.path.join(HERE, "native", "arith_check.cu")], check=True)
    out = subprocess.run([str(exe), "300000"], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout
    cases, bad = map(int, out.stdout.split()[-2:])
    assert cases > 5_000_000 and bad == 0
