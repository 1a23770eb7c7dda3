"""The reference's own example programs (example/mainatmos.cpp, example/mainbeam.cpp), compiled
unchanged against include/compat/ and this library: the drop-in claim at its plainest.

The examples are the reference's files, read where a reference tree is found
($CP3_REFERENCE_DIR, or the untracked copy in baseline/_ref); without one these tests skip.
Nothing from the reference is kept in this repository."""
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

from tests.conftest import ROOT


def reference_tree():
    from oracle.oracle import reference_dir
    d = reference_dir()
    if d is None or not os.path.isfile(os.path.join(d, "example", "mainatmos.cpp")):
        pytest.skip("no reference tree with its examples (CP3_REFERENCE_DIR or baseline/_ref)")
    return d


def compile_example(name, out_dir):
    from cudaprob3_gb300 import build
    lib = build.build()
    exe = os.path.join(out_dir, name)
    src = os.path.join(reference_tree(), "example", name + ".cpp")
    cmd = ["g++", "-std=c++14", "-O2", "-I", os.path.join(ROOT, "include", "compat"),
           "-I", os.path.join(ROOT, "include"), src, "-o", exe, lib,
           "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, " ".join(cmd) + "\n" + r.stderr
    return exe


@pytest.mark.parametrize("name", ["mainatmos", "mainbeam"])
def test_reference_examples_compile_unchanged(tmp_path, name):
    assert os.path.exists(compile_example(name, str(tmp_path)))


def example_linspace(lo, hi, n):
    """example/mainatmos.cpp's linspace: the point is accumulated step by step."""
    out = [0.0] * n
    step = (hi - lo) / float(n - 1)
    e = lo
    for i in range(n - 1):
        out[i] = e
        e += step
    out[n - 1] = hi
    return np.array(out)


def example_logspace(lo, hi, n):
    """example/mainatmos.cpp's logspace: exp of an accumulated logarithm."""
    out = [0.0] * n
    a, b = math.log(lo), math.log(hi)
    step = (b - a) / float(n - 1)
    out[0] = lo
    e = a + step
    for i in range(1, n - 1):
        out[i] = math.exp(e)
        e += step
    out[n - 1] = hi
    return np.array(out)


@pytest.mark.gpu
def test_mainatmos_output_matches_the_oracle(tmp_path, oracle):
    """mainatmos as shipped: 200 x 200 bins, the reference's own PREM 4-layer model file read
    from ../models, FP64 AtmosCudaPropagatorSingle; its three output files (P(mu->e),
    P(mu->mu), P(mu->tau) printed to 20 digits) against the CPU oracle at 1e-12."""
    from oracle.oracle import Mixing as OMix
    ref_dir = reference_tree()
    exe = compile_example("mainatmos", str(tmp_path))
    run = tmp_path / "run"
    run.mkdir()
    (tmp_path / "models").mkdir()
    shutil.copy(os.path.join(ref_dir, "models", "PREM_4layer.dat"), tmp_path / "models")
    r = subprocess.run([exe], cwd=run, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    nc = ne = 200
    cz = example_linspace(-0.995, 0.0, nc)
    en = example_logspace(1.0, 100.0, ne)
    # the example's parameters (mainatmos.cpp:91-99): nu_flav = 2 is a neutrino
    m = OMix(0.5695951908800630486710466089860865317151404697548723,
             0.1608752771983210967007023071793306595103776477788280,
             0.7853981633974483096156608458198757210492923498437764, 0.0, 7.9e-5, 2.5e-3, 2)
    model = np.loadtxt(os.path.join(ref_dir, "models", "PREM_4layer.dat"))
    ref = oracle.atmos(m, False, cz, en, model[:, 0], model[:, 1], model[:, 2], 22.0,
                       nthreads=os.cpu_count() or 1)
    for fname, ch in (("out_m_e.txt", 3), ("out_m_m.txt", 4), ("out_m_t.txt", 5)):
        text = (run / fname).read_text().split()
        assert (int(text[0]), int(text[1])) == (nc, ne)
        got = np.array([float(x) for x in text[2:]]).reshape(nc, ne)
        assert np.abs(got - ref[:, :, ch]).max() <= 1e-12, fname


@pytest.mark.gpu
def test_mainbeam_fails_as_the_references_own_build_does(tmp_path):
    """mainbeam constructs BeamCudaPropagatorSingle(0, n_energies): in the reference that is
    the (n_energies, n_threads) constructor (beamcudapropagator.cuh:57), a propagator of zero
    energies, so the program ends on an uncaught std::runtime_error before it computes
    anything.  Compiled against this library it ends the same way, with no output file."""
    exe = compile_example("mainbeam", str(tmp_path))
    r = subprocess.run([exe], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert r.returncode != 0
    assert "std::runtime_error" in r.stderr
    assert not (tmp_path / "out_cudaboth_me.txt").exists()
