"""cp3_atmos_mixed_noalloc: the atmospheric mixed-precision entry point for callers that
cannot allocate device memory while they propagate (a fitter whose pool owns the GPU, code
where cudaMalloc is not allowed).  It must give what a MIXED atmospheric handle gives, call
after call, while its working memory is the library's fixed device scratch.

Collected last on purpose (a stop-at-first-failure run has run everything else first); it
also passes alone in a fresh process.  The test allocates its own device buffers for the
inputs and outputs -- the entry point under test does not."""
import ctypes as C

import numpy as np
import pytest

from cudaprob3_gb300 import AtmosCudaPropagatorSingle, _abi, build, earth

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-5  # the tolerance of the mixed kernels throughout the test-suite


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _abi.lib()


def regular_result(mix, knu, anti, cz, en, model, h):
    p = AtmosCudaPropagatorSingle(0, len(cz), len(en), precision="mixed")
    p.setEnergyList(en)
    p.setCosineList(cz)
    p.setMNSMatrix(mix.theta12, mix.theta13, mix.theta23, mix.dcp, knu)
    p.setNeutrinoMasses(mix.dm12sq, mix.dm23sq)
    p.setDensity(*model)
    p.setProductionHeight(h)
    p.calculateProbabilities(1 if anti else 0)
    return p.result()


def no_alloc_result(lib, mix, knu, anti, cz, en, model, h, out_pad=0, edit=None):
    import torch
    t = _abi.trajectory_table(model[0], model[1], model[2], cz, h)
    if edit is not None:
        edit(t)
    d_en = torch.tensor(np.asarray(en, dtype=np.float64), device="cuda")
    n_out = 9 * len(cz) * len(en)
    d_out = torch.full((n_out + out_pad,), float("nan"), dtype=torch.float32, device="cuda")
    err = C.create_string_buffer(256)
    ip = lambda a: np.ascontiguousarray(a, dtype=np.int32).ctypes.data_as(C.POINTER(C.c_int))  # noqa: E731
    dp = lambda a: np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    keep = [np.ascontiguousarray(t[k]) for k in ("seg_offset", "seg_len_km", "seg_class", "class_rho_e")]
    rc = lib.cp3_atmos_mixed_noalloc(
        0, C.c_void_p(d_en.data_ptr()), len(en), ip(keep[0]), dp(keep[1]), ip(keep[2]), len(cz),
        dp(keep[3]), len(keep[3]), mix.theta12, mix.theta13, mix.theta23, mix.dcp, knu,
        mix.dm12sq, mix.dm23sq, 1 if anti else 0, C.c_void_p(d_out.data_ptr()),
        C.c_void_p(torch.cuda.current_stream().cuda_stream), err, 256)
    torch.cuda.synchronize()
    return rc, err.value.decode(), d_out[:n_out].cpu().numpy().reshape(9, len(cz), len(en))


def test_no_alloc_matches_regular_entry_point_twice_in_a_row(lib):
    m = earth.NOMINAL
    # two different grids and models back to back: the second call reuses (and partly
    # overwrites) the scratch the first one left behind
    calls = [
        (False, 1, earth.cosine_grid(150), earth.log_energy_grid(230), earth.PREM_4LAYER, 22.0),
        (True, -1, earth.cosine_grid(400), earth.log_energy_grid(700), earth.synthetic_shells(59), 15.0),
    ]
    for anti, knu, cz, en, model, h in calls:
        want = regular_result(m, knu, anti, cz, en, model, h)
        rc, msg, got = no_alloc_result(lib, m, knu, anti, cz, en, model, h)
        assert rc == 0, msg
        assert np.isfinite(got).all()
        assert np.abs(got.astype(np.float64) - want.astype(np.float64)).max() <= MIXED_TOL


def test_no_alloc_rejects_grids_beyond_its_scratch(lib):
    m = earth.NOMINAL
    cz, en = earth.cosine_grid(8), earth.log_energy_grid(40000)  # 60 classes x 40000 energies
    rc, msg, _ = no_alloc_result(lib, m, 1, False, cz, en, earth.synthetic_shells(59), 22.0)
    assert rc == 1  # CP3_ERR_BAD_SIZE
    assert "scratch" in msg and str(8 * 1024 * 1024) in msg


def test_no_alloc_refuses_a_class_numbering_other_than_the_segment_index(lib):
    """The kernels read class l for a row's segment l (cp3_trajectory_table's numbering); a
    class array that says otherwise is refused, not silently ignored."""
    m = earth.NOMINAL
    cz, en = earth.cosine_grid(12), earth.log_energy_grid(16)

    def swap(t):
        cls = np.array(t["seg_class"])
        off = np.array(t["seg_offset"])
        row = int(np.argmax(np.diff(off) >= 3))  # a row crossing two shells or more
        cls[off[row] + 1], cls[off[row] + 2] = cls[off[row] + 2], cls[off[row] + 1]
        t["seg_class"] = cls

    rc, msg, _ = no_alloc_result(lib, m, 1, False, cz, en, earth.PREM_4LAYER, 22.0, edit=swap)
    assert rc == 6  # CP3_ERR_BAD_ARGUMENT
    assert "class" in msg
