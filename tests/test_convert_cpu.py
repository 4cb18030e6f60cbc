"""The mixed sweep's integer FP32 <-> FP64 conversions (fest_convert.cuh),
built for the host and compared bit for bit with the compiler's
conversions on 4 M random values each (FP32 subnormal results excluded:
the sweep flushes them to zero)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_integer_conversions_match_the_compiler(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "convert_check")
    subprocess.run([nvcc, "-x", "cu", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "fest-3d_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "convert_check.cu"), "-o", exe], check=True, timeout=300)
    out = subprocess.run([exe], capture_output=True, text=True, check=True, timeout=300).stdout.split()
    n, bad_f2d, bad_d2f = (int(x) for x in out)
    assert n >= 1 << 22
    assert bad_f2d == 0 and bad_d2f == 0, (bad_f2d, bad_d2f)
