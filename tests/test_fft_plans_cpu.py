"""The FFT building blocks of the kernels (register DFTs, twiddles,
Stockham positions) for every per-size plan, emulated on the CPU in FP32
and compared with an FP64 DFT."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_every_plan_matches_fp64_dft(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "fftcheck")
    subprocess.run([nvcc, "-std=c++17", "-O1", "-diag-suppress", "177", "-I" + os.path.join(ROOT, "colore_gb300", "csrc"),
                    "-o", exe, os.path.join(HERE, "fft_host_check.cu")], check=True, capture_output=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n")
    rows = [l.split() for l in out if l.strip()]
    assert [int(r[0]) for r in rows] == [64, 96, 128, 192, 256, 384, 512, 1024, 2048]
    for n, ec, er in rows:
        assert float(ec) < 5e-7 and float(er) < 5e-7, (n, ec, er)
