"""The FFT's register DFTs and plan factorisation, checked on the host.

tests/host/fft_butterflies.cu includes the FFT source and runs its
host-callable parts (the radix 2, 3, 4, 5, 6, 8, 9 and 10 DFTs, the pass
constants of every supported length) against the direct DFT; needs nvcc,
no GPU.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_fft_butterflies_and_passes_on_host(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "fft_butterflies")
    build = subprocess.run([nvcc, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
                            "-I" + os.path.join(ROOT, "nexusmd_gb300", "csrc"), "-I" + os.path.join(ROOT, "include"),
                            os.path.join(HERE, "host", "fft_butterflies.cu"), "-o", exe],
                           capture_output=True, text=True)
    assert build.returncode == 0, build.stderr[-4000:]
    run = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    print(run.stdout)
    assert run.returncode == 0 and run.stdout.strip().endswith("OK"), run.stdout[-4000:]
