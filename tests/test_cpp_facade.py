"""The C++ facade (include/cudaprob3_gb300.hpp): compiles against the header with the
reference's call order (CPU), and on the GPU reproduces the oracle through it."""
import os
import subprocess

import numpy as np
import pytest

from tests.conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cpp", "drop_in.cpp")


def build_program(tmp_path):
    from cudaprob3_gb300 import build
    lib = build.build()
    exe = str(tmp_path / "drop_in")
    cmd = ["g++", "-std=c++14", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           lib, "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_facade_compiles_and_links(tmp_path):
    exe = build_program(tmp_path)
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_facade_matches_oracle(tmp_path, oracle):
    from cudaprob3_gb300 import earth
    from oracle.oracle import Mixing as OMix
    exe = build_program(tmp_path)
    model = tmp_path / "prem4.dat"
    r, rho, ye = earth.PREM_4LAYER
    model.write_text("".join(f"{a} {b} {c}\n" for a, b, c in zip(r, rho, ye)))
    for args in ([exe], [exe, str(model)]):
        out = subprocess.run(args, capture_output=True, text=True, timeout=120)
        assert out.returncode == 0, out.stdout + out.stderr
        assert "caught: CudaPropagatorSingle::getProbability. Invalid indices" in out.stdout
        assert "boundaries 5" in out.stdout  # PREM 4-layer: 5 rows, from the file or setDensity
        nc, ne = 20, 16
        cz = -1.0 + 2.0 * np.arange(nc) / (nc - 1)
        en = 10 ** (-1.0 + 3.0 * np.arange(ne) / (ne - 1))
        m = OMix(0.5843, 0.1496, 0.7365, -1.601, 7.53e-5, 2.49e-3, 1)
        ref = oracle.atmos(m, False, cz, en, r, rho, ye, 22.0)
        eb = 0.1 + 9.9 * np.arange(1000) / 999.0
        refb = oracle.beam(m, False, eb, 2.6, 1300.0)
        n = 0
        for line in out.stdout.splitlines():
            f = line.split()
            if f[0] == "atmos":
                ic, ie, t, v = int(f[1]), int(f[2]), int(f[3]), float(f[4])
                assert abs(v - ref[ic, ie, t]) <= 1e-12
                n += 1
            elif f[0] == "beam":
                ie, t, v = int(f[1]), int(f[2]), float(f[3])
                assert abs(v - refb[ie, t]) <= 1e-12
                n += 1
        assert n > 100


def test_cmake_package_and_compat_headers(tmp_path):
    """find_package(CUDAProb3) gives the reference's target names; its header names resolve."""
    import shutil
    if not shutil.which("cmake"):
        pytest.skip("cmake not installed")
    from cudaprob3_gb300 import build
    build.build()
    src = os.path.join(ROOT, "tests", "cpp", "cmake_consumer")
    bld = str(tmp_path / "b")
    r = subprocess.run(["cmake", "-S", src, "-B", bld, f"-DCP3_ROOT={ROOT}"], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    r = subprocess.run(["cmake", "--build", bld], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = subprocess.run([os.path.join(bld, "consumer")], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0
    assert "REarth 6371" in out.stdout
    assert ("created" in out.stdout) or ("No GPU found" in out.stdout)


def build_batch_program(tmp_path):
    from cudaprob3_gb300 import build
    lib = build.build()
    exe = str(tmp_path / "batch_server")
    cmd = ["g++", "-std=c++14", "-O2", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "batch_server.cpp"), "-o", exe, lib,
           "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_batch_and_server_wrappers_compile(tmp_path):
    assert os.path.exists(build_batch_program(tmp_path))


@pytest.mark.gpu
def test_batch_and_server_wrappers_match_oracle(tmp_path, oracle):
    from cudaprob3_gb300 import earth
    from oracle.oracle import Mixing as OMix
    exe = build_batch_program(tmp_path)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "caught: no such problem" in out.stdout
    r, rho, ye = earth.PREM_4LAYER
    nc, ne = 20, 16
    cz = -1.0 + 2.0 * np.arange(nc) / (nc - 1)
    en = 10 ** (-1.0 + 3.0 * np.arange(ne) / (ne - 1))
    ref = {
        "nu": oracle.atmos(OMix(0.5843, 0.1496, 0.7365, -1.601, 7.53e-5, 2.49e-3, 1), False,
                           cz, en, r, rho, ye, 22.0),
        "nubar": oracle.atmos(OMix(0.5843, 0.1496, 0.7365, -1.601, 7.53e-5, 2.49e-3, -1), True,
                              cz, en, r, rho, ye, 22.0),
    }
    eb = 0.1 + 9.9 * np.arange(1000) / 999.0
    refb = oracle.beam(OMix(0.5843, 0.1496, 0.7365, -1.601, 7.53e-5, 2.49e-3, 1), False, eb, 2.6,
                       1300.0)
    counts = {"batch_nu": 0, "batch_nubar": 0, "batch_beam": 0, "served": 0}
    for line in out.stdout.splitlines():
        f = line.split()
        if f[0] in ("batch_nu", "batch_nubar", "served"):
            ic, ie, t, v = int(f[1]), int(f[2]), int(f[3]), float(f[4])
            want = ref["nubar" if f[0] == "batch_nubar" else "nu"][ic, ie, t]
            assert abs(v - want) <= 1e-5, line
            counts[f[0]] += 1
        elif f[0] == "batch_beam":
            ie, t, v = int(f[1]), int(f[2]), float(f[3])
            assert abs(v - refb[ie, t]) <= 1e-5, line
            counts[f[0]] += 1
    assert min(counts.values()) > 50, counts
