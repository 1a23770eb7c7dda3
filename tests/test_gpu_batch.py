"""Batches (one persistent launch over many problems) against single propagators, the
oracle, and themselves under every tile shape."""
import numpy as np
import pytest

from cudaprob3_gb300 import AtmosCudaPropagatorSingle, BeamCudaPropagatorSingle, earth
from cudaprob3_gb300._abi import CP3Error
from cudaprob3_gb300.batch import Batch
from tests.gpu_helpers import run_atmos

pytestmark = pytest.mark.gpu
MIXED_TOL = 1e-5


def single_atmos(m, anti, cz, en, model, h):
    p = AtmosCudaPropagatorSingle(0, len(cz), len(en), precision="mixed")
    p.setEnergyList(en)
    p.setCosineList(cz)
    p.setMNSMatrix(m.theta12, m.theta13, m.theta23, m.dcp, -1 if anti else 1)
    p.setNeutrinoMasses(m.dm12sq, m.dm23sq)
    p.setDensity(*model)
    p.setProductionHeight(h)
    p.calculateProbabilities(1 if anti else 0)
    return p.result()


def single_beam(m, anti, en, rho, L):
    b = BeamCudaPropagatorSingle(0, len(en), 1, precision="mixed")
    b.setEnergyList(en)
    b.setMNSMatrix(m.theta12, m.theta13, m.theta23, m.dcp, -1 if anti else 1)
    b.setNeutrinoMasses(m.dm12sq, m.dm23sq)
    b.setDensity(rho)
    b.setPathLength(L)
    b.calculateProbabilities(1 if anti else 0)
    return b.result()


def build_batch(sets, rng):
    b = Batch(0)
    model = earth.PREM_12LAYER
    b.set_earth(*model, 22.0)
    probs = []
    for i, m in enumerate(sets):
        nc, ne = int(rng.integers(20, 150)), int(rng.integers(30, 300))
        cz, en = earth.cosine_grid(nc), earth.log_energy_grid(ne)
        for anti in (False, True):
            pid = b.add_atmos(cz, en)
            b.set_params(pid, m, anti)
            probs.append(("atmos", pid, m, anti, cz, en))
    for i, m in enumerate(sets[:3]):
        en = earth.lin_energy_grid(int(rng.integers(1000, 5000)))
        for anti in (False, True):
            pid = b.add_beam(en, 2.6, [295.0, 1300.0])
            b.set_params(pid, m, anti)
            probs.append(("beam", pid, m, anti, en, None))
    b.commit()
    return b, probs


def test_batch_matches_single_propagators_and_oracle(oracle):
    from oracle.oracle import Mixing as OMix
    rng = np.random.default_rng(3)
    sets = earth.gaussian_sets(5, seed=12)
    b, probs = build_batch(sets, rng)
    b.run()
    b.synchronize()
    for kind, pid, m, anti, x, en in probs:
        got = b.result(pid)
        om = OMix(m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq, -1 if anti else 1)
        if kind == "atmos":
            cz = x
            want = single_atmos(m, anti, cz, en, earth.PREM_12LAYER, 22.0)
            assert np.abs(got - want).max() <= MIXED_TOL
            ref = oracle.atmos(om, anti, cz, en, *earth.PREM_12LAYER, 22.0)
            assert np.abs(np.transpose(got, (1, 2, 0)) - ref).max() <= MIXED_TOL
        else:
            for j, L in enumerate((295.0, 1300.0)):
                want = single_beam(m, anti, x, 2.6, L)
                assert np.abs(got[j] - want).max() <= MIXED_TOL
                ref = oracle.beam(om, anti, x, 2.6, L)
                assert np.abs(got[j].T - ref).max() <= MIXED_TOL


def test_whole_arena_copy_holds_every_result():
    """cp3_batch_copy_results moves the result arena in pieces of any size; each problem's
    result sits at its cp3_batch_result_offset, bit-identical to its own copy.  A range past
    the arena is refused."""
    rng = np.random.default_rng(6)
    b, probs = build_batch(earth.gaussian_sets(4, seed=14), rng)
    b.run()
    b.synchronize()
    total = b.info()["result_bytes"] // 4
    arena = np.full(total, np.nan, dtype=np.float32)
    piece = 123457  # an odd piece size: copies need not follow problem boundaries
    for first in range(0, total, piece):
        n = min(piece, total - first)
        b.copy_results_async(first, n, arena.ctypes.data + 4 * first)
    b.synchronize_stream()
    for _, pid, *_ in probs:
        mine = b.result(pid).ravel()
        off = b.result_offset(pid)
        assert np.array_equal(arena[off:off + mine.size], mine)
    with pytest.raises(CP3Error, match="beyond the result arena"):
        b.copy_results_async(total - 10, 11, arena.ctypes.data)


def test_run_to_host_matches_run():
    """cp3_batch_run_to_host: the bins in windows of whole problems, each window's arena range
    downloaded while the next computes.  Every problem's result lands at its arena offset,
    bit-identical to cp3_batch_run's, for any number of pieces, with and without eigen tables
    (a mixed batch and a beam-only one)."""
    import torch
    rng = np.random.default_rng(7)
    mixed, probs = build_batch(earth.gaussian_sets(4, seed=16), rng)
    beam = Batch(0)
    beam_probs = []
    for m in earth.gaussian_sets(6, seed=17):
        for anti in (False, True):
            pid = beam.add_beam(earth.lin_energy_grid(int(rng.integers(1000, 5000))), 2.6, [295.0, 1300.0])
            beam.set_params(pid, m, anti)
            beam_probs.append(pid)
    beam.commit()
    for b, pids in ((mixed, [q[1] for q in probs]), (beam, beam_probs)):
        b.run()
        b.synchronize()
        want = {pid: b.result(pid).ravel() for pid in pids}
        total = b.info()["result_bytes"] // 4
        for n_pieces in (1, 3, 8, 0):
            host = torch.full((total,), float("nan"), dtype=torch.float32).pin_memory()
            b.run_to_host(host.data_ptr(), n_pieces)
            b.synchronize()
            arena = host.numpy()
            for pid in pids:
                off = b.result_offset(pid)
                assert np.array_equal(arena[off:off + want[pid].size], want[pid]), (n_pieces, pid)
        # a plain run afterwards is unchanged
        b.run()
        b.synchronize()
        for pid in pids:
            assert np.array_equal(b.result(pid).ravel(), want[pid])


def test_runs_on_other_streams_wait_for_the_last_run_and_download():
    """A run queued on another stream right after a run to host memory, with new parameters
    and no host wait in between, must neither change the parameters nor the arena under the
    first run's kernels and copies."""
    import torch
    rng = np.random.default_rng(9)
    b, probs = build_batch(earth.gaussian_sets(4, seed=19), rng)
    pids = [q[1] for q in probs]
    sets_a = {pid: (m, anti) for _, pid, m, anti, *_ in probs}
    sets_b = {pid: (earth.gaussian_sets(8, seed=20)[k % 8], anti)
              for k, (_, pid, m, anti, *_) in enumerate(probs)}
    want = {}
    for name, sets in (("a", sets_a), ("b", sets_b)):
        for pid, (m, anti) in sets.items():
            b.set_params(pid, m, anti)
        b.run()
        b.synchronize()
        want[name] = {pid: b.result(pid).ravel() for pid in pids}
    assert any(not np.array_equal(want["a"][p], want["b"][p]) for p in pids)
    total = b.info()["result_bytes"] // 4
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    for rep in range(3):
        host = torch.full((total,), float("nan"), dtype=torch.float32).pin_memory()
        for pid, (m, anti) in sets_a.items():
            b.set_params(pid, m, anti)
        b.run_to_host(host.data_ptr(), 8, streams[0].cuda_stream)
        for pid, (m, anti) in sets_b.items():
            b.set_params(pid, m, anti)
        b.run(streams[1].cuda_stream)
        for st in streams:
            st.synchronize()
        b.synchronize()
        arena = host.numpy()
        for pid in pids:
            off = b.result_offset(pid)
            assert np.array_equal(arena[off:off + want["a"][pid].size], want["a"][pid]), (rep, pid)
            assert np.array_equal(b.result(pid).ravel(), want["b"][pid]), (rep, pid)


def test_run_to_host_errors():
    rng = np.random.default_rng(8)
    b, _ = build_batch(earth.gaussian_sets(2, seed=18), rng)
    host = np.zeros(b.info()["result_bytes"] // 4, dtype=np.float32)
    with pytest.raises(CP3Error, match="at most 8 pieces"):
        b.run_to_host(host.ctypes.data, 9)
    with pytest.raises(CP3Error, match="null destination"):
        b.run_to_host(0)
    b.debug_withhold_tables(True)
    with pytest.raises(CP3Error, match="withheld-tables"):
        b.run_to_host(host.ctypes.data)
    b.debug_withhold_tables(False)
    b.run_to_host(host.ctypes.data)
    b.synchronize()


def test_batch_results_do_not_depend_on_tile_shape():
    """Tile shapes and the launch split (one launch with waits, or a table launch then a bin
    launch) leave every result bit-identical."""
    rng = np.random.default_rng(4)
    b, probs = build_batch(earth.gaussian_sets(3, seed=13), rng)
    ref = None
    for split in (False, True):
        b.set_split_tables(split)
        assert b.split_tables() == split
        for shape in [(1, 0, 4), (2, 0, 1), (1, 2, 16), (4, 1, 4), (8, 0, 2), (16, 0, 64)]:
            b.set_shape(*shape)
            b.run()
            b.synchronize()
            res = [b.result(pid) for _, pid, *_ in probs]
            if ref is None:
                ref = res
            else:
                for a, c in zip(ref, res):
                    assert np.array_equal(a, c), (split, shape)


def test_batch_parameter_update_between_runs():
    rng = np.random.default_rng(5)
    sets = earth.gaussian_sets(2, seed=14)
    b, probs = build_batch(sets, rng)
    b.run()
    b.synchronize()
    new = earth.gaussian_sets(3, seed=99)[2]
    kind, pid, m, anti, cz, en = probs[0]
    b.set_params(pid, new, anti)
    b.run()
    b.synchronize()
    want = single_atmos(new, anti, cz, en, earth.PREM_12LAYER, 22.0)
    assert np.abs(b.result(pid) - want).max() <= MIXED_TOL


def test_batch_tuner_keeps_results():
    rng = np.random.default_rng(6)
    b, probs = build_batch(earth.gaussian_sets(2, seed=15), rng)
    b.run()
    b.synchronize()
    before = [b.result(pid) for _, pid, *_ in probs]
    b.tune(use_cache=False)
    b.run()
    b.synchronize()
    for (_, pid, *_), a in zip(probs, before):
        assert np.array_equal(b.result(pid), a)


def test_batch_errors():
    from cudaprob3_gb300._abi import CP3Error
    b = Batch(0)
    with pytest.raises(CP3Error, match="set_earth"):
        b.add_atmos([-1.0, 0.5], [1.0, 2.0])
    with pytest.raises(CP3Error, match="commit"):
        b.run()
    pid = b.add_beam([1.0, 2.0], 2.6, [810.0])
    with pytest.raises(CP3Error, match="no parameters"):
        b.commit()
    b.set_params(pid, earth.NOMINAL, False)
    b.commit()
    with pytest.raises(CP3Error, match="committed"):
        b.add_beam([1.0], 2.6, [810.0])
    with pytest.raises(CP3Error, match="no such problem"):
        b.result_ptr(7)
    for bad in [(0, 0, 4), (17, 0, 4), (1, -1, 4), (1, 0, 0), (1, 0, 65)]:
        with pytest.raises(CP3Error, match="shape"):
            b.set_shape(*bad)
