"""Runs a fixed mix of batch and serving work with whichever library CP3GB300_LIB (or the
in-tree default) selects and saves every result to an .npz.  test_gpu_device_checks.py
runs it once per library and compares the debug build (device bounds checks) with the
product build.  Usage: python tests/device_checks_run.py OUT.npz"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from cudaprob3_gb300 import earth  # noqa: E402
from cudaprob3_gb300.batch import Batch  # noqa: E402
from cudaprob3_gb300.serve import Server  # noqa: E402


def main(path):
    out = {}
    rng = np.random.default_rng(21)
    sets = earth.gaussian_sets(4, seed=5)
    # a batch of both kinds, uneven grids, every tile shape the tests use
    b = Batch(0)
    b.set_earth(*earth.PREM_12LAYER, 22.0)
    ids = []
    for m in sets:
        nc, ne = int(rng.integers(3, 90)), int(rng.integers(1, 200))
        for anti in (False, True):
            pid = b.add_atmos(earth.cosine_grid(nc), earth.log_energy_grid(ne))
            b.set_params(pid, m, anti)
            ids.append(pid)
    for m in sets[:2]:
        for anti in (False, True):
            pid = b.add_beam(earth.lin_energy_grid(int(rng.integers(1, 3000))), 2.6, [295.0, 1300.0])
            b.set_params(pid, m, anti)
            ids.append(pid)
    b.commit()
    for shape in ((1, 0, 1), (4, 0, 4), (16, 0, 64)):
        b.set_shape(*shape)
        b.run()
        b.synchronize()  # raises on any kernel status, the bounds checks' included
        for pid in ids:
            out[f"batch_{shape[0]}_{shape[2]}_{pid}"] = b.result(pid)
    # the serving loop: the same kernel over its memory pool
    s = Server(0, pool_bytes=1 << 28, max_batch=32)
    s.set_earth(*earth.PREM_4LAYER, 22.0)
    ga = s.add_atmos_grid(earth.cosine_grid(37), earth.log_energy_grid(53))
    gb = s.add_beam_grid(earth.lin_energy_grid(777), 2.6, [810.0])
    s.start()
    reqs = []
    for i, m in enumerate(sets):
        for g in (ga, gb):
            reqs.append((s.submit(g, m, bool(i & 1)), g, i))
    for rid, g, i in reqs:
        assert s.wait(rid), "request timed out"
        out[f"serve_{g}_{i}"] = s.result(rid, g)
        s.release(rid)
    np.savez(path, **out)


if __name__ == "__main__":
    main(sys.argv[1])
