"""The continuous-batching server: results against the CPU oracle; a request gives the same
result alone and in a mix of requests of other sizes and parameters; admission waits for
device memory; the completion queue; a launch that fails (injected on the host, nothing on
the GPU) fails exactly its own requests; error paths."""
import os

import numpy as np
import pytest

from cudaprob3_gb300 import AtmosCudaPropagatorSingle, earth
from cudaprob3_gb300._abi import CP3Error
from cudaprob3_gb300.serve import Server

pytestmark = pytest.mark.gpu
MIXED_TOL = 1e-5


def make_server(pool_bytes=2 << 30, **kw):
    s = Server(0, pool_bytes=pool_bytes, **kw)
    s.set_earth(*earth.PREM_4LAYER, 22.0)
    grids = dict(
        a200=s.add_atmos_grid(earth.cosine_grid(200), earth.log_energy_grid(200)),
        a500=s.add_atmos_grid(earth.cosine_grid(500), earth.log_energy_grid(500)),
        b1e4=s.add_beam_grid(earth.lin_energy_grid(10000), 2.6, [1300.0]),
    )
    s.start()
    return s, grids


def test_same_result_alone_and_in_the_mix():
    s, g = make_server()
    m = earth.NOMINAL
    rid = s.submit(g["a500"], m, False)
    assert s.wait(rid)
    alone = s.result(rid, g["a500"])
    s.release(rid)
    rng = np.random.default_rng(1)
    sets = earth.gaussian_sets(60, seed=8)
    ids = []
    for i, mm in enumerate(sets):
        k = ["a200", "a500", "b1e4"][i % 3]
        ids.append((s.submit(g[k], mm, bool(rng.integers(2))), k))
        if i == 30:
            target = s.submit(g["a500"], m, False)
    for rid2, k in ids + [(target, "a500")]:
        assert s.wait(rid2)
    mixed = s.result(target, g["a500"])
    assert np.array_equal(alone, mixed)
    # and the same as the single-problem mixed propagator
    p = AtmosCudaPropagatorSingle(0, 500, 500, precision="mixed")
    p.setEnergyList(earth.log_energy_grid(500))
    p.setCosineList(earth.cosine_grid(500))
    p.setMNSMatrix(m.theta12, m.theta13, m.theta23, m.dcp, 1)
    p.setNeutrinoMasses(m.dm12sq, m.dm23sq)
    p.setDensity(*earth.PREM_4LAYER)
    p.setProductionHeight(22.0)
    p.calculateProbabilities(0)
    assert np.abs(mixed - p.result()).max() <= MIXED_TOL
    assert s.stats()["launches"] >= 2
    for rid2, _ in ids + [(target, "a500")]:
        s.release(rid2)


def test_admission_waits_for_device_memory():
    # room for about two 500x500 results at a time (9 MB each)
    s, g = make_server(pool_bytes=24 << 20, max_batch=64)
    ids = [s.submit(g["a500"], mm, False) for mm in earth.gaussian_sets(8, seed=3)]
    lat = []
    for rid in ids:
        assert s.wait(rid, 30.0)
        lat.append(s.latency_ms(rid))
        s.release(rid)  # frees the pool for the queued ones
    assert s.stats()["launches"] >= 3  # could not all run at once
    assert all(x > 0 for x in lat)


def test_server_errors():
    s = Server(0, pool_bytes=64 << 20)
    with pytest.raises(CP3Error, match="set_earth"):
        s.add_atmos_grid([-1.0, 0.5], [1.0, 2.0])
    with pytest.raises(CP3Error, match="start"):
        s.submit(0, earth.NOMINAL, False)
    s.set_earth(*earth.PREM_4LAYER, 22.0)
    s.add_atmos_grid(earth.cosine_grid(2000), earth.log_energy_grid(2000))  # 144 MB > pool
    with pytest.raises(CP3Error, match="does not fit"):
        s.start()


def oracle_mixing(m, anti):
    from oracle.oracle import Mixing as OMix
    return OMix(m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq, -1 if anti else 1)


def check_against_oracle(s, g, rid, key, m, anti):
    """One finished request against the CPU oracle (all channels, <= 1e-5)."""
    from oracle.oracle import Oracle
    orc = Oracle()
    got = s.result(rid, g[key])
    nt = os.cpu_count() or 1
    if key.startswith("a"):
        n = int(key[1:])
        ref = orc.atmos(oracle_mixing(m, anti), anti, earth.cosine_grid(n), earth.log_energy_grid(n),
                        *earth.PREM_4LAYER, 22.0, nthreads=nt)
        err = np.abs(np.transpose(got, (1, 2, 0)) - ref).max()
    else:
        ref = orc.beam(oracle_mixing(m, anti), anti, earth.lin_energy_grid(10000), 2.6, 1300.0,
                       nthreads=nt)
        err = np.abs(got[0].T - ref).max()
    assert err <= MIXED_TOL, (key, anti, err)
    return err


def test_results_match_the_oracle():
    """Requests of every registered size, nu and nubar, both orderings, submitted together so
    that they share launches, each against the CPU oracle."""
    s, g = make_server()
    sets = earth.gaussian_sets(12, seed=21)  # the second half has inverted ordering
    reqs = []
    for i, m in enumerate(sets):
        key = ["a200", "a500", "b1e4"][i % 3]
        anti = bool(i % 2)
        reqs.append((s.submit(g[key], m, anti), key, m, anti))
    for rid, key, m, anti in reqs:
        assert s.wait(rid, 30.0)
    for rid, key, m, anti in reqs:
        check_against_oracle(s, g, rid, key, m, anti)
        s.release(rid)


def test_poll_reports_every_request_once():
    s, g = make_server()
    s.poll(0)  # start recording
    sets = earth.gaussian_sets(40, seed=5)
    ids = {s.submit(g[["a200", "b1e4"][i % 2]], m, bool(i % 3 == 0)) for i, m in enumerate(sets)}
    seen = []
    for _ in range(200):
        seen += s.poll(16, 0.5)
        if len(seen) >= len(ids):
            break
    assert sorted(seen) == sorted(ids)  # each exactly once
    assert s.poll(16, 0.0) == []
    for rid in ids:
        assert s.wait(rid, 0.0)
        s.release(rid)


def test_failed_launch_fails_exactly_its_requests():
    """A launch made to fail on the host (cp3_server_debug_fail_launches; no GPU work is
    queued for it) finishes its requests with an error; the server keeps serving, and the
    requests of later launches are correct."""
    s, g = make_server()
    m = earth.NOMINAL
    s.debug_fail_launches(1)
    bad = s.submit(g["a200"], m, False)
    with pytest.raises(CP3Error, match="injected launch failure"):
        s.wait(bad, 30.0)
    with pytest.raises(CP3Error, match="no result"):
        s.result(bad, g["a200"])
    s.release(bad)  # a failed request's pool memory is released as any other's
    good = s.submit(g["a200"], m, False)
    assert s.wait(good, 30.0)
    check_against_oracle(s, g, good, "a200", m, False)
    s.release(good)

    # requests queued together: the failing launch takes the first of them (same size, so
    # in arrival order); every request either fails with the injected error or is correct
    s.poll(0)
    s.debug_fail_launches(1)
    sets = earth.gaussian_sets(6, seed=9)
    ids = [s.submit(g["a200"], mm, False) for mm in sets]
    failed = []
    for rid, mm in zip(ids, sets):
        try:
            assert s.wait(rid, 30.0)
        except CP3Error as e:
            assert "injected launch failure" in str(e)
            failed.append(rid)
            continue
        check_against_oracle(s, g, rid, "a200", mm, False)
    assert 1 <= len(failed) <= len(ids)
    assert failed == ids[:len(failed)]
    launches = s.stats()["launches"]
    for rid in ids:
        s.release(rid)
    # later requests run normally
    rid = s.submit(g["b1e4"], m, True)
    assert s.wait(rid, 30.0)
    check_against_oracle(s, g, rid, "b1e4", m, True)
    s.release(rid)
    assert s.stats()["launches"] > launches
