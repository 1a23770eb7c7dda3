"""Drop-in behaviour of the propagator classes on the GPU: setter checks and messages,
result access paths, handle independence."""
import numpy as np
import pytest

from cudaprob3_gb300 import (AtmosCudaPropagatorSingle, BeamCudaPropagatorSingle,
                             CudaPropagatorSingle, NeutrinoType, ProbType, earth)

pytestmark = pytest.mark.gpu

NOM = earth.NOMINAL


def configured(nc=6, ne=5, prec="fp64"):
    p = AtmosCudaPropagatorSingle(0, nc, ne, precision=prec)
    p.setEnergyList(earth.log_energy_grid(ne))
    p.setCosineList(earth.cosine_grid(nc))
    p.setMNSMatrix(NOM.theta12, NOM.theta13, NOM.theta23, NOM.dcp, 1)
    p.setNeutrinoMasses(NOM.dm12sq, NOM.dm23sq)
    p.setDensity(*earth.PREM_4LAYER)
    p.setProductionHeight(22.0)
    return p


def test_size_checks():
    p = AtmosCudaPropagatorSingle(0, 6, 5)
    with pytest.raises(RuntimeError, match="number of energy nodes"):
        p.setEnergyList(np.ones(4))
    with pytest.raises(RuntimeError, match="number of cosine nodes"):
        p.setCosineList(np.ones(7))
    with pytest.raises(RuntimeError, match="rhos.size"):
        p.setDensity([0, 1000, 6371], [1, 2], [0.5, 0.5, 0.5])
    with pytest.raises(RuntimeError, match="radii order"):
        p.setDensity([0, 3000, 2000, 6371], [1, 2, 3, 4], [0.5] * 4)


def test_production_height_order_and_required():
    p = AtmosCudaPropagatorSingle(0, 6, 5)
    with pytest.raises(RuntimeError, match="must set cosine list before production height"):
        p.setProductionHeight(22.0)
    p.setEnergyList(earth.log_energy_grid(5))
    p.setCosineList(earth.cosine_grid(6))
    p.setMNSMatrix(0.5, 0.1, 0.7, 0.0, 1)
    p.setNeutrinoMasses(7.5e-5, 2.5e-3)
    p.setDensity(*earth.PREM_4LAYER)
    with pytest.raises(RuntimeError, match="production height was not set"):
        p.calculateProbabilities(NeutrinoType.Neutrino)


def test_layer_limit():
    r = np.linspace(0, 6371, 140)
    p = AtmosCudaPropagatorSingle(0, 3, 2)
    p.setCosineList([-1.0, -0.5, 0.5])
    with pytest.raises(RuntimeError, match="invalid number of maxLayer"):
        p.setDensity(r, np.full(140, 5.0), np.full(140, 0.5))


def test_get_probability_paths_agree():
    p = configured()
    p.calculateProbabilities(NeutrinoType.Neutrino)
    res = p.result()
    arr = p.getProbabilityArr(ProbType.m_e)
    for ic in range(6):
        for ie in range(5):
            v = p.getProbability(ic, ie, ProbType.m_e)
            assert v == res[ProbType.m_e, ic, ie]
            assert arr[ie * 6 + ic] == v
    with pytest.raises(RuntimeError, match="Invalid indices"):
        p.getProbability(6, 0, ProbType.e_e)


def test_second_compute_overwrites():
    p = configured()
    p.calculateProbabilities(NeutrinoType.Neutrino)
    a = p.getProbability(0, 0, ProbType.m_m)
    p.setMNSMatrix(NOM.theta12, NOM.theta13, NOM.theta23, NOM.dcp, -1)
    p.calculateProbabilities(NeutrinoType.Antineutrino)
    b = p.getProbability(0, 0, ProbType.m_m)
    assert a != b


def test_handles_are_independent():
    a = configured(prec="mixed")
    b = configured(prec="mixed")
    b.setNeutrinoMasses(NOM.dm12sq, -2.5e-3)
    a.calculate_async(NeutrinoType.Neutrino)
    b.calculate_async(NeutrinoType.Neutrino)
    a.synchronize()
    b.synchronize()
    ra, rb = a.result(), b.result()
    a.calculateProbabilities(NeutrinoType.Neutrino)
    assert np.array_equal(a.result(), ra)
    assert not np.array_equal(ra, rb)


def test_density_file_formats(tmp_path, oracle):
    r, rho, ye = earth.PREM_4LAYER
    f3 = tmp_path / "prem3.dat"
    f3.write_text("# radius rho ye\n" + "".join(f"{a} {b} {c}\n" for a, b, c in zip(r, rho, ye)))
    f2 = tmp_path / "prem2.dat"
    f2.write_text("".join(f"{a}\t{b}\n" for a, b in zip(r, rho)))
    outs = []
    for f in (f3, f2):
        p = configured()
        p.setDensityFromFile(str(f))
        p.calculateProbabilities(NeutrinoType.Neutrino)
        outs.append(p.result())
    ref = configured()
    ref.calculateProbabilities(NeutrinoType.Neutrino)
    assert np.array_equal(outs[0], ref.result())
    assert np.array_equal(outs[1], ref.result())  # Ye rule reproduces PREM_4layer's column
    bad = tmp_path / "bad.dat"
    bad.write_text("0 1 2 3\n")
    with pytest.raises(RuntimeError, match="Unsupported"):
        configured().setDensityFromFile(str(bad))


def test_layer_boundaries(tmp_path):
    """getNlayerBoundaries: the model's rows (layers + 1) after setDensityFromFile, as the
    reference counts them, and after every other density setter too."""
    r, rho, ye = earth.PREM_4LAYER
    f = tmp_path / "prem.dat"
    f.write_text("".join(f"{a} {b} {c}\n" for a, b, c in zip(r, rho, ye)))
    p = configured()
    assert p.getNlayerBoundaries() == len(r)
    p.setDensityFromFile(str(f))
    assert p.getNlayerBoundaries() == len(r) == 5
    p.setDensity(*earth.PREM_12LAYER)
    assert p.getNlayerBoundaries() == len(earth.PREM_12LAYER[0])
    p.setDensity(*earth.PREM_4LAYER_QUAD_V2)
    assert p.getNlayerBoundaries() == len(earth.PREM_4LAYER_QUAD_V2[0])
    with pytest.raises(RuntimeError, match="density model was not set"):
        AtmosCudaPropagatorSingle(0, 6, 5).getNlayerBoundaries()


def test_beam_api_and_legacy_template_name():
    b = BeamCudaPropagatorSingle(0, 100, 1)
    b.setEnergyList(earth.lin_energy_grid(100))
    b.setMNSMatrix(NOM.theta12, NOM.theta13, NOM.theta23, NOM.dcp, 1)
    b.setNeutrinoMasses(NOM.dm12sq, NOM.dm23sq)
    with pytest.raises(RuntimeError, match="density was not set"):
        b.calculateProbabilities(NeutrinoType.Neutrino)
    b.setDensity(2.6)
    b.setPathLength(1300.0)
    b.calculateProbabilities(NeutrinoType.Neutrino)
    assert abs(b.getProbabilityArr(ProbType.m_m)[50] - b.getProbability(50, ProbType.m_m)) == 0
    t = CudaPropagatorSingle(0, 4, 4, float_type=np.float32)
    assert t.precision == 1


def test_unitarity_mixed_large():
    p = configured(nc=300, ne=200, prec="mixed")
    p.calculateProbabilities(NeutrinoType.Neutrino)
    P = p.result().astype(np.float64).reshape(3, 3, 300, 200)  # [a][b][ic][ie]
    assert np.abs(P.sum(axis=1) - 1).max() < 1e-5
    assert np.abs(P.sum(axis=0) - 1).max() < 1e-5


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("model", ["shells", "quadratic"])
def test_calculate_to_host_matches_device_result(prec, model):
    import torch
    nc, ne = 37, 29
    p = configured(nc=nc, ne=ne, prec=prec)
    if model == "quadratic":
        p.setDensity(*earth.PREM_4LAYER_QUAD_V2)
    for t in (NeutrinoType.Neutrino, NeutrinoType.Antineutrino):
        p.calculateProbabilities(t)
        want = p.result().copy()
        dtype = torch.float64 if prec == "fp64" else torch.float32
        for chunks in (0, 1, 3, 7, nc, nc + 5):
            host = torch.full((9 * nc * ne,), -1.0, dtype=dtype, pin_memory=True)
            p.calculate_to_host_async(t, host.data_ptr(), chunks)
            p.synchronize()
            assert np.array_equal(host.numpy().reshape(want.shape), want), chunks


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_energy_uploads_and_computes_ordered_across_streams(prec):
    """setEnergyList uploads asynchronously; computes on other streams wait for the upload,
    and an upload or compute that follows a compute on another stream waits for it."""
    import torch
    nc, ne = 48, 160
    en_a = earth.log_energy_grid(ne)
    en_b = en_a[::-1] * 0.7
    want = []
    for en in (en_a, en_b):
        q = configured(nc=nc, ne=ne, prec=prec)
        q.setEnergyList(en)
        q.calculateProbabilities(NeutrinoType.Neutrino)
        want.append(q.result().copy())
    assert not np.array_equal(want[0], want[1])
    dtype = torch.float64 if prec == "fp64" else torch.float32
    p = configured(nc=nc, ne=ne, prec=prec)
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    for rep in range(3):
        hosts = [torch.full((9 * nc * ne,), -1.0, dtype=dtype, pin_memory=True) for _ in range(2)]
        for k, en in enumerate((en_a, en_b)):
            p.setEnergyList(en)
            p.calculate_to_host_async(NeutrinoType.Neutrino, hosts[k].data_ptr(), 3,
                                      streams[k].cuda_stream)
        for st in streams:
            st.synchronize()
        for k in range(2):
            assert np.array_equal(hosts[k].numpy().reshape(want[k].shape), want[k]), (rep, k)


def test_pipelined_downloads_never_see_a_later_step():
    """Back-to-back calculate_to_host_async steps on two streams in turn: a step's row pieces
    are recomputed while the previous step's download is still on the link, each piece only
    after its own copy has left.  Every host buffer must hold its own step's result, and a
    plain compute queued behind the downloads must not reach them either."""
    import torch
    nc, ne = 1000, 1000
    grids = [earth.log_energy_grid(ne) * f for f in (1.0, 0.8, 1.3)]
    want = []
    for en in grids:
        q = configured(nc=nc, ne=ne, prec="mixed")
        q.setEnergyList(en)
        q.calculateProbabilities(NeutrinoType.Neutrino)
        want.append(q.result().copy())
    p = configured(nc=nc, ne=ne, prec="mixed")
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    steps = 6
    hosts = [torch.full((9 * nc * ne,), -1.0, dtype=torch.float32, pin_memory=True)
             for _ in range(steps)]
    for k in range(steps):
        p.setEnergyList(grids[k % 3])
        p.calculate_to_host_async(NeutrinoType.Neutrino, hosts[k].data_ptr(), 4,
                                  streams[k % 2].cuda_stream)
    # a plain compute of another grid, queued behind the last downloads
    p.setEnergyList(grids[1])
    p.calculateProbabilities(NeutrinoType.Neutrino)
    for st in streams:
        st.synchronize()
    for k in range(steps):
        assert np.array_equal(hosts[k].numpy().reshape(want[0].shape), want[k % 3]), k
    assert np.array_equal(p.result(), want[1])


def test_copies_on_another_stream_wait_for_the_compute():
    """cp3_copy_result_async on a stream other than the compute's, queued right behind it with
    no host wait, sees the finished result; so does a batch's arena copy on another stream."""
    import torch
    from cudaprob3_gb300.batch import Batch
    nc, ne = 1000, 1000
    p = configured(nc=nc, ne=ne, prec="mixed")
    p.calculateProbabilities(NeutrinoType.Neutrino)
    want = p.result().copy()
    a, b = torch.cuda.Stream(), torch.cuda.Stream()
    for rep in range(3):
        host = torch.full((9 * nc * ne,), -1.0, dtype=torch.float32, pin_memory=True)
        p.setMNSMatrix(NOM.theta12, NOM.theta13, NOM.theta23, NOM.dcp, -1)
        p.calculate_async(NeutrinoType.Antineutrino, a.cuda_stream)  # a different result first
        p.setMNSMatrix(NOM.theta12, NOM.theta13, NOM.theta23, NOM.dcp, 1)
        p.calculate_async(NeutrinoType.Neutrino, a.cuda_stream)
        p.copy_result_async(host.data_ptr(), b.cuda_stream)
        b.synchronize()
        assert np.array_equal(host.numpy().reshape(want.shape), want), rep
    bt = Batch(0)
    bt.set_earth(*earth.PREM_12LAYER, 22.0)
    pid = bt.add_atmos(earth.cosine_grid(800), earth.log_energy_grid(900))
    bt.set_params(pid, NOM, False)
    bt.commit()
    bt.run()
    bt.synchronize()
    want_b = bt.result(pid).ravel()
    total = bt.info()["result_bytes"] // 4
    for rep in range(3):
        host = torch.full((total,), -1.0, dtype=torch.float32, pin_memory=True)
        bt.set_params(pid, earth.gaussian_sets(2, seed=3)[1], True)
        bt.run(a.cuda_stream)  # a different result first
        bt.set_params(pid, NOM, False)
        bt.run(a.cuda_stream)
        bt.copy_results_async(0, total, host.data_ptr(), b.cuda_stream)
        b.synchronize()
        off = bt.result_offset(pid)
        assert np.array_equal(host.numpy()[off:off + want_b.size], want_b), rep


def test_calculate_to_host_beam():
    import torch
    ne = 101
    b = BeamCudaPropagatorSingle(0, ne, 1, precision="mixed")
    b.setEnergyList(earth.lin_energy_grid(ne))
    b.setMNSMatrix(NOM.theta12, NOM.theta13, NOM.theta23, NOM.dcp, 1)
    b.setNeutrinoMasses(NOM.dm12sq, NOM.dm23sq)
    b.setDensity(2.6)
    b.setPathLength(1300.0)
    b.calculateProbabilities(NeutrinoType.Neutrino)
    want = b.result().copy()
    host = torch.full((9 * ne,), -1.0, dtype=torch.float32, pin_memory=True)
    b.calculate_to_host_async(NeutrinoType.Neutrino, host.data_ptr())
    b.synchronize()
    assert np.array_equal(host.numpy().reshape(want.shape), want)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_probability_arr_device_and_host_paths_agree(prec):
    nc, ne = 67, 45
    p = configured(nc=nc, ne=ne, prec=prec)
    p.calculateProbabilities(NeutrinoType.Antineutrino)
    res = p.result().astype(np.float64)
    for t in (ProbType.e_e, ProbType.m_e, ProbType.t_t):
        dev = p.getProbabilityArr(t)  # nothing on the host yet: the device transpose
        assert np.array_equal(dev, res[t].T.ravel())
    p.getProbability(0, 0, ProbType.e_e)  # downloads the whole result
    for t in (ProbType.m_m, ProbType.e_t):
        host = p.getProbabilityArr(t)
        assert np.array_equal(host, res[t].T.ravel())


def test_probability_arr_beam():
    ne = 333
    b = BeamCudaPropagatorSingle(0, ne, 1, precision="mixed")
    b.setEnergyList(earth.lin_energy_grid(ne))
    b.setMNSMatrix(NOM.theta12, NOM.theta13, NOM.theta23, NOM.dcp, 1)
    b.setNeutrinoMasses(NOM.dm12sq, NOM.dm23sq)
    b.setDensity(2.6)
    b.setPathLength(810.0)
    b.calculateProbabilities(NeutrinoType.Neutrino)
    res = b.result().astype(np.float64)
    assert np.array_equal(b.getProbabilityArr(ProbType.m_e), res[ProbType.m_e])
