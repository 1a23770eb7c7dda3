"""The debug build (`build(device_checks=True)`: every arena access of a persistent-kernel
tile checked against the arena's size first, a failing tile skipped and reported) runs the
same batch and serving work as the product build with no check firing and bit-identical
results: the arena offsets the host computes keep every access in bounds."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_device_bounds_checks_pass_and_change_nothing(tmp_path):
    from cudaprob3_gb300 import build
    checked = build.build(device_checks=True)
    runs = {}
    for name, lib in (("product", build.LIB), ("checked", checked)):
        env = dict(os.environ, CP3GB300_LIB=lib)
        dst = tmp_path / f"{name}.npz"
        r = subprocess.run([sys.executable, os.path.join(ROOT, "tests", "device_checks_run.py"),
                            str(dst)], env=env, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stdout + r.stderr
        runs[name] = np.load(dst)
    a, b = runs["product"], runs["checked"]
    assert sorted(a.files) == sorted(b.files) and len(a.files) > 20
    for k in a.files:
        assert np.array_equal(a[k], b[k]), k
