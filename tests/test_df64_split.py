"""The integer float-float split used for FP64 vectors (df_split_bits in
thunderegg_gb300/csrc/te_df64.cuh) equals the FP64 formula hi = RN(d),
lo = RN(d - hi) bit for bit on random bit patterns, the solver's value
range, rounding ties and carries, and special values; and the integer widening
f2d_bits equals the float-to-double cast for every float class (host code, no GPU)."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT


def test_split_bits_matches_fp64_formula(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = tmp_path / "split_check"
    src = os.path.join(ROOT, "tests", "df64_split_check.cu")
    inc = os.path.join(ROOT, "thunderegg_gb300", "csrc")
    subprocess.run([nvcc, "-O2", "-std=c++17", "-I", inc, src, "-o", str(exe)], check=True, capture_output=True,
                   timeout=300)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
