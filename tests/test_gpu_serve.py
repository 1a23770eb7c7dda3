"""The continuous-batching server: a request gives the same result alone and in a mix of
requests of other sizes and parameters; admission waits for device memory; error paths."""
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
