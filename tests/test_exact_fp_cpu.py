"""The exact-rounding helpers the kernels use (aces4_gb300/csrc/exact_fp.h:
the integer-arithmetic FP64 division of the denominator and amplitude-update
passes, and the one-rounding integer -> FP64 conversions of the split-precision
recombine and direct epilogue), compiled for the host from the same source and
checked bit for bit against IEEE arithmetic on random and edge-case operands."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_exact_rounding_helpers_match_ieee(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not available")
    exe = tmp_path / "exact_check"
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-x", "cu", "-I", os.path.join(ROOT, "aces4_gb300", "csrc"),
                        "-o", str(exe), os.path.join(ROOT, "tests", "exact_fp", "check.cu")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), "400000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout
