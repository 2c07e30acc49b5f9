"""The DFT codelets of the FP32 PME transforms (csrc/nb_fft.cuh), checked on the host.

Radices 2, 3, 4, 5 and the composite 6, 8, 9, 10 (prime-factor and Cooley-Tukey compositions
that let the z columns of a grid of up to 100 points be transformed in two Stockham passes)
are compiled as host code with nvcc and compared with a direct DFT summed in long double on
seeded inputs in [-1/2, 1/2): within 1e-14 in FP64 and 2e-6 in FP32 (a few ulps of the
largest output, |X| <= R/2).
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "moil_fnrfd_gb300", "csrc")


def test_codelets_match_direct_dft(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "fft_codelets")
    subprocess.run([nvcc, "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "fft_codelets.cu"), "-o", exe],
                   check=True, capture_output=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n")
    rows = {int(r.split()[0]): (float(r.split()[1]), float(r.split()[2])) for r in out if r.strip()}
    assert sorted(rows) == [2, 3, 4, 5, 6, 8, 9, 10]
    for radix, (e64, e32) in rows.items():
        assert e64 < 1e-14, (radix, e64)
        assert e32 < 2e-6, (radix, e32)
