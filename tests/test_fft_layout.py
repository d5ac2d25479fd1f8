"""The line FFT layouts of the device code, emulated on the host (no GPU).

tests/fft_layout_check.cpp runs the device functions of cupss_gb300/csrc/fft.cuh for the
M threads of one line in turn: every supported length (1..1024) in the four-step form, and
512 and 1024 also in the split form; forward against a direct DFT and inverse back to the
input, and every register layout a permutation of the line's positions."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cuda_include():
    for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if d and os.path.isfile(os.path.join(d, "include", "cuda_runtime.h")):
            return os.path.join(d, "include")
    return None


def test_line_fft_layouts_on_host(tmp_path):
    cxx = shutil.which("g++")
    inc = _cuda_include()
    if cxx is None or inc is None:
        pytest.skip("needs g++ and the CUDA headers")
    exe = str(tmp_path / "fft_layout_check")
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "cupss_gb300", "csrc"), "-I", inc,
                    os.path.join(ROOT, "tests", "fft_layout_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("OK")
