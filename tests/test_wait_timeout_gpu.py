"""The multi-frame sweep kernel's bounded dependency waits, made to run out on purpose:
cs_debug_stall_group points one word group's neighbour links of the next multi-frame launch at a
completion value that nothing writes.  Its waits give up after about a second, the launch abandons
its frames and ends, the host reports CS_ERR_CUDA from cs_get_counts and cs_synchronize, diagnostic
7 counts the timeouts, and the device stays usable for the next handle.  Nothing faults or hangs:
every wait of the kernel is bounded and no task runs on data its dependencies did not finish."""
import numpy as np
import pytest

from cell_simulation_gb300 import CellsimError, RNG_PHILOX, tiling_kinds, tiling_launches, tiling_variants
from tests.helpers import multi_region_model

pytestmark = pytest.mark.gpu


def _persistent(K):
    return next(i for i, (v, k, n) in enumerate(zip(tiling_variants(), tiling_kinds(), tiling_launches()))
                if v[0] == K and k[0] == 2 and n == 1)


def _model():
    return multi_region_model(res=(10, 12, 30), K=16)


def test_stalled_group_times_out_and_is_reported():
    sim = _model()
    sim.prepare_for_gpu(RNG_PHILOX, 0)
    sim.set_tiling(_persistent(16))
    sim.step_philox(3, 5)
    assert sim.counts().sum() > 0
    assert sim.diagnostics()[7] == 0
    sim.debug_stall_group(0)
    sim.step_philox(3, 5)
    with pytest.raises(CellsimError) as e:
        sim.counts()
    assert "timed out" in str(e.value)
    assert sim.diagnostics()[7] > 0
    with pytest.raises(CellsimError):
        sim.synchronize()
    sim.close()
    # the device is still usable: the persistent form and the default step agree on a new handle
    a, b = _model(), _model()
    for s in (a, b):
        s.prepare_for_gpu(RNG_PHILOX, 0)
    b.set_tiling(_persistent(16))
    a.step_philox(6, 5)
    b.step_philox(6, 5)
    assert np.array_equal(a.get_lattice()[0], b.get_lattice()[0])
    assert np.array_equal(a.counts(), b.counts())
    assert b.diagnostics()[7] == 0
