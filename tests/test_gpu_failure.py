"""Failure detection without a GPU fault: a batch whose eigen-table tiles are withheld on the
host (cp3_batch_debug_withhold_tables) leaves every atmospheric bin tile waiting for tables
that never come.  Each wait is bounded (2 s): the kernel sets a status word, the launch ends,
synchronize reports the failure, and the context stays usable for the next, normal run."""
import time

import numpy as np
import pytest

from cudaprob3_gb300 import earth
from cudaprob3_gb300.batch import Batch

pytestmark = pytest.mark.gpu


def make_batch():
    b = Batch(0)
    b.set_earth(*earth.PREM_4LAYER, 22.0)
    pid = b.add_atmos(earth.cosine_grid(24), earth.log_energy_grid(40))
    b.set_params(pid, earth.NOMINAL, False)
    beam = b.add_beam(earth.lin_energy_grid(300), 2.6, [1300.0])
    b.set_params(beam, earth.NOMINAL, False)
    b.commit()
    return b, pid, beam


def test_withheld_tables_time_out_and_the_context_recovers():
    b, pid, beam = make_batch()
    b.run()
    b.synchronize()
    want, want_beam = b.result(pid).copy(), b.result(beam).copy()

    b.debug_withhold_tables(True)
    t0 = time.perf_counter()
    b.run()
    with pytest.raises(RuntimeError, match="wait limit"):
        b.synchronize()
    waited = time.perf_counter() - t0
    assert 1.5 < waited < 30.0, waited
    with pytest.raises(RuntimeError, match="wait limit"):
        b.result(pid)  # the failed run's results are not handed out

    b.debug_withhold_tables(False)
    b.run()
    b.synchronize()
    assert np.array_equal(b.result(pid), want)
    assert np.array_equal(b.result(beam), want_beam)
