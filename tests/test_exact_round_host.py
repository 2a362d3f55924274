"""The tensor-core update's epilogue rounds its exact integer level sums to FP64 with integer operations
(csrc/exact_round.cuh).  Built for the host, it must give bit for bit the FP64 expression it replaces,
fma((double)hi, 2^-35, (double)lo * 2^-56) * 2^(e + 56), on random sums, near-ties and exponent edges."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT


def test_exact_rounding_matches_the_fp64_expression(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "exact_round_check")
    subprocess.check_call([cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "slakonet_gb300", "csrc"),
                           os.path.join(ROOT, "tests", "exact_round_check.cpp"), "-o", exe])
    out = subprocess.run([exe, "2000000"], capture_output=True, text=True)
    print(out.stdout.strip())
    assert out.returncode == 0 and out.stdout.startswith("0 mismatches")
