"""The FP64 kernels' division by the energy (Markstein's correction from a correctly rounded
reciprocal, `div_by` in csrc/cp3_atmos.cu) gives the same double as IEEE division: checked
on the host, whose double arithmetic and fma round as the GPU's do."""
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_markstein_division_matches_ieee(tmp_path):
    exe = tmp_path / "div_by_check"
    src = os.path.join(HERE, "cpp", "div_by_check.c")
    r = subprocess.run(["gcc", "-O2", "-std=gnu11", "-ffp-contract=off", src, "-o", str(exe), "-lm"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("no C compiler: " + r.stderr[-200:])
    out = subprocess.run([str(exe), "20000000"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout
    assert out.stdout.strip().endswith("0 mismatches"), out.stdout
