"""The batched workloads at their full sizes, checked through properties that do not need the
oracle to run over every bin: probability conservation of every initial flavour and of
every final flavour (the nine channels of a bin form a doubly stochastic matrix, since the
amplitude is unitary), for every bin of every problem; plus a few problems spread over each
batch against the oracle.

- batched atmospheric: 256 Gaussian parameter sets x nu/nubar (512 problems) on their own
  uneven grids (cosines U[100, 1000], energies U[100, 2000]), PREM 12-layer, 22 km;
- batched beam: 4096 parameter sets x nu/nubar (8192 problems), 1e5 energies, 2.6 g/cm^3,
  295 and 1300 km (59 GB of results, checked on the device).
"""
import os

import numpy as np
import pytest

from cudaprob3_gb300 import earth
from cudaprob3_gb300.batch import Batch

pytestmark = pytest.mark.gpu
MIXED_TOL = 1e-5


def conservation_error(b, shapes, chunk_floats=1 << 28):
    """Max |sum over b of P(a->b) - 1| and |sum over a - 1| over every bin of every problem,
    computed on the device: the result arena is copied in pieces (cp3_batch_copy_results)
    into a device buffer and reduced there."""
    import torch
    worst = 0.0
    buf = torch.empty(chunk_floats, dtype=torch.float32, device="cuda")
    pid = 0
    while pid < len(shapes):
        first = b.result_offset(pid)
        # as many whole problems as fit the buffer
        last, end = pid, first
        while last < len(shapes):
            off = b.result_offset(last)
            size = int(np.prod(shapes[last]))
            assert size <= chunk_floats
            if off + size - first > chunk_floats and last > pid:
                break
            end = off + size
            last += 1
        b.copy_results_async(first, end - first, buf.data_ptr())
        b.synchronize_stream()
        for q in range(pid, last):
            off = b.result_offset(q) - first
            shape = shapes[q]
            # atmospheric [9][nc][ne] or beam [nL][9][ne] -> [..][3][3][..]
            x = buf[off:off + int(np.prod(shape))].view(*shape)
            if len(shape) == 3 and shape[0] == 9:
                P = x.view(3, 3, shape[1], shape[2]).double()
            else:
                P = x.view(shape[0], 3, 3, shape[2]).permute(1, 2, 0, 3).double()
            worst = max(worst, float((P.sum(dim=1) - 1).abs().max()),
                        float((P.sum(dim=0) - 1).abs().max()))
        pid = last
    return worst


def test_batched_atmospheric_full_size():
    from oracle.oracle import Mixing as OMix, Oracle
    sets = earth.gaussian_sets(256, seed=2024)
    grids = earth.uneven_grids(256, seed=2025)
    b = Batch(0)
    b.set_earth(*earth.PREM_12LAYER, 22.0)
    shapes, probs = [], []
    for m, (nc, ne) in zip(sets, grids):
        cz, en = earth.cosine_grid(nc), earth.log_energy_grid(ne)
        for anti in (False, True):
            pid = b.add_atmos(cz, en)
            b.set_params(pid, m, anti)
            shapes.append((9, nc, ne))
            probs.append((pid, m, anti, cz, en))
    b.commit()
    b.set_shape(16, 0, 4)
    b.run()
    b.synchronize()
    assert conservation_error(b, shapes) <= MIXED_TOL
    orc = Oracle()
    for k in (0, 77, 255, 300, 511):
        pid, m, anti, cz, en = probs[k]
        om = OMix(m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq, -1 if anti else 1)
        rows = np.arange(0, len(cz), 7)
        ref = orc.atmos(om, anti, cz[rows], en, *earth.PREM_12LAYER, 22.0,
                        nthreads=os.cpu_count() or 1)
        got = np.transpose(b.result(pid), (1, 2, 0))[rows]
        assert np.abs(got - ref).max() <= MIXED_TOL


def test_batched_beam_full_size():
    from oracle.oracle import Mixing as OMix, Oracle
    sets = earth.gaussian_sets(4096, seed=2026)
    en = earth.lin_energy_grid(100000)
    b = Batch(0)
    shapes, probs = [], []
    for m in sets:
        for anti in (False, True):
            pid = b.add_beam(en, 2.6, [295.0, 1300.0])
            b.set_params(pid, m, anti)
            shapes.append((2, 9, len(en)))
            probs.append((pid, m, anti))
    b.commit()
    b.set_shape(2, 0, 16)
    b.run()
    b.synchronize()
    assert conservation_error(b, shapes) <= MIXED_TOL
    orc = Oracle()
    for k in (0, 1, 4097, 8191):
        pid, m, anti = probs[k]
        om = OMix(m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq, -1 if anti else 1)
        got = b.result(pid)
        for j, L in enumerate((295.0, 1300.0)):
            ref = orc.beam(om, anti, en, 2.6, L, nthreads=os.cpu_count() or 1)
            assert np.abs(got[j].T - ref).max() <= MIXED_TOL
