"""The host code under AddressSanitizer and UndefinedBehaviorSanitizer (CPU only): the
propagator library's host layer (cudaprob3_gb300/csrc/cp3_host.cpp) and the C oracle, built
with -fsanitize=address,undefined and no recovery, driven through every host entry point by
tests/cpp/host_sanitize.cpp.  The GPU side has no sanitizer here; this covers the code that
builds what the kernels read."""
import os
import shutil
import subprocess

import pytest

from tests.conftest import ROOT


def test_host_code_is_clean_under_asan_and_ubsan(tmp_path):
    if not shutil.which("g++") or not shutil.which("gcc"):
        pytest.skip("no host compiler")
    flags = ["-O1", "-g", "-fno-omit-frame-pointer", "-fsanitize=address,undefined",
             "-fno-sanitize-recover=all"]
    oracle_o = str(tmp_path / "oracle.o")
    r = subprocess.run(["gcc", "-std=gnu11", *flags, "-fopenmp", "-c",
                        os.path.join(ROOT, "oracle", "cp3_oracle.c"), "-o", oracle_o],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    exe = str(tmp_path / "host_sanitize")
    r = subprocess.run(["g++", "-std=c++17", *flags, "-fopenmp",
                        "-I", os.path.join(ROOT, "cudaprob3_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "cpp", "host_sanitize.cpp"),
                        os.path.join(ROOT, "cudaprob3_gb300", "csrc", "cp3_host.cpp"),
                        oracle_o, "-o", exe, "-lm"],
                       capture_output=True, text=True)
    if r.returncode != 0 and "asan" in r.stderr.lower():
        pytest.skip("sanitizer runtime not available: " + r.stderr[-200:])
    assert r.returncode == 0, r.stderr
    env = dict(os.environ, SANITIZE_TMP=str(tmp_path), ASAN_OPTIONS="detect_leaks=1",
               OMP_NUM_THREADS="2")
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert r.stdout.strip().endswith("ok")
    assert "runtime error" not in r.stderr and "AddressSanitizer" not in r.stderr
