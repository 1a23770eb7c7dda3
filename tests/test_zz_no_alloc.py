"""cp3_atmos_mixed_noalloc: the atmospheric mixed-precision entry point for callers that
cannot allocate device memory while they propagate (a fitter whose pool owns the GPU, code
where cudaMalloc is not allowed).  It must give what a MIXED atmospheric handle gives, call
after call, while its working memory is the library's fixed device scratch.

Collected last on purpose (a stop-at-first-failure run has run everything else first); it
also passes alone in a fresh process.  The test allocates its own device buffers for the
inputs and outputs -- the entry point under test does not, which one test checks through the
device's free memory and torch's allocator statistics around calls after the first."""
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


class NoAllocCall:
    """One cp3_atmos_mixed_noalloc call with every input and output buffer allocated up front
    (by the test, through torch), so that run() itself touches no allocator."""

    def __init__(self, lib, mix, knu, anti, cz, en, model, h, edit=None):
        import torch
        t = _abi.trajectory_table(model[0], model[1], model[2], cz, h)
        if edit is not None:
            edit(t)
        self.lib, self.nc, self.ne = lib, len(cz), len(en)
        self.args = (mix, knu, anti)
        self.d_en = torch.tensor(np.asarray(en, dtype=np.float64), device="cuda")
        self.d_out = torch.full((9 * self.nc * self.ne,), float("nan"), dtype=torch.float32,
                                device="cuda")
        self.keep = [np.ascontiguousarray(t["seg_offset"], dtype=np.int32),
                     np.ascontiguousarray(t["seg_len_km"], dtype=np.float64),
                     np.ascontiguousarray(t["seg_class"], dtype=np.int32),
                     np.ascontiguousarray(t["class_rho_e"], dtype=np.float64)]
        self.err = C.create_string_buffer(256)
        self.stream = torch.cuda.current_stream().cuda_stream

    def run(self):
        """The call and a synchronize; returns (status, message)."""
        import torch
        mix, knu, anti = self.args
        ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))  # noqa: E731
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
        k = self.keep
        rc = self.lib.cp3_atmos_mixed_noalloc(
            0, C.c_void_p(self.d_en.data_ptr()), self.ne, ip(k[0]), dp(k[1]), ip(k[2]), self.nc,
            dp(k[3]), len(k[3]), mix.theta12, mix.theta13, mix.theta23, mix.dcp, knu,
            mix.dm12sq, mix.dm23sq, 1 if anti else 0, C.c_void_p(self.d_out.data_ptr()),
            C.c_void_p(self.stream), self.err, 256)
        torch.cuda.synchronize()
        return rc, self.err.value.decode()

    def result(self):
        return self.d_out.cpu().numpy().reshape(9, self.nc, self.ne)


def no_alloc_result(lib, mix, knu, anti, cz, en, model, h, edit=None):
    call = NoAllocCall(lib, mix, knu, anti, cz, en, model, h, edit)
    rc, msg = call.run()
    return rc, msg, call.result()


def test_no_alloc_matches_regular_entry_point_twice_in_a_row(lib):
    """Bit for bit: the entry point runs the regular mixed handle's two kernels on the same
    inputs (its float pairs are split by the same rounding), only its working memory is the
    fixed scratch."""
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
        assert np.array_equal(got, want)


def test_no_alloc_on_the_headline_grid(lib):
    """The grid the header names as fitting: 59 shells, 2000 x 2000, neutrino then
    antineutrino in two calls in a row; bit-identical to the regular handle, and every 40th
    cosine row against the CPU oracle (all channels, <= 1e-5)."""
    import os
    from oracle.oracle import Mixing as OMix, Oracle
    m = earth.NOMINAL
    model = earth.synthetic_shells(59)
    cz, en = earth.cosine_grid(2000), earth.log_energy_grid(2000)
    orc = Oracle()
    rows = np.arange(0, 2000, 40)
    for anti, knu in ((False, 1), (True, -1)):
        rc, msg, got = no_alloc_result(lib, m, knu, anti, cz, en, model, 22.0)
        assert rc == 0, msg
        want = regular_result(m, knu, anti, cz, en, model, 22.0)
        assert np.array_equal(got, want)
        ref = orc.atmos(OMix(m.theta12, m.theta13, m.theta23, m.dcp, m.dm12sq, m.dm23sq, knu),
                        anti, cz[rows], en, *model, 22.0, nthreads=os.cpu_count() or 1)
        err = np.abs(np.transpose(got, (1, 2, 0))[rows].astype(np.float64) - ref).max()
        assert err <= MIXED_TOL, err


def test_no_alloc_allocates_nothing_after_the_first_call(lib):
    """After the set-up call on a device, calls on other grids leave the device's free memory
    (cudaMemGetInfo) and torch's allocator statistics exactly as they were."""
    import torch
    m = earth.NOMINAL
    first = NoAllocCall(lib, m, 1, False, earth.cosine_grid(30), earth.log_energy_grid(40),
                        earth.PREM_4LAYER, 22.0)
    later = [NoAllocCall(lib, m, -1, True, earth.cosine_grid(700), earth.log_energy_grid(900),
                         earth.synthetic_shells(59), 22.0),
             NoAllocCall(lib, m, 1, False, earth.cosine_grid(1000), earth.log_energy_grid(333),
                         earth.PREM_12LAYER, 10.0)]
    assert first.run()[0] == 0  # the set-up call (the first on this device, in a fresh process)
    keys = ("allocated_bytes.all.current", "reserved_bytes.all.current",
            "allocation.all.allocated", "segment.all.allocated")

    def snapshot():
        torch.cuda.synchronize()
        st = torch.cuda.memory_stats()
        return torch.cuda.mem_get_info()[0], {k: st.get(k) for k in keys}

    before = snapshot()
    for call in later + later:
        rc, msg = call.run()
        assert rc == 0, msg
        assert snapshot() == before
    for call in later:
        assert np.isfinite(call.result()).all()


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
