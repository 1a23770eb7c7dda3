"""The mixed kernels' phase arithmetic in turns on the host, built with nvcc: the unit phase
factor e^{-2 pi i r} - 1 (unit_turn_minus_one) to 3e-7 over |r| <= 1/2 turn plus the
overshoot past a half-turn (where an earlier form took the sine's sign from r alone), and
the exact range reduction of double-float products (reduced_turn) to 1e-10 turns."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(os.path.dirname(HERE), "cudaprob3_gb300", "csrc")


def test_phase_factor_and_turn_reduction(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = tmp_path / "unit_phase_check"
    r = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2",
                        "-I", SRC,
                        os.path.join(HERE, "cpp", "unit_phase_check.cu"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout
