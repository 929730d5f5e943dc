"""Zero-order reactions (no reactants) fire in every voxel, empty ones included: both forms of the
sweep stream (four launches, and the Y and Z sweeps fused) match the oracle on such a model."""
import numpy as np
import pytest

from cell_simulation_gb300 import tiling_launches
from tests.helpers import multi_region_model
from tests.test_prod_gpu import gpu_prod, oracle_prod, stream_tilings

pytestmark = pytest.mark.gpu


def _model():
    sim = multi_region_model(res=(9, 8, 40), K=16, counts=(30, 20, 10, 5))
    sim.add_reaction([], ["A"], 40.0)
    sim.add_reaction(["A"], ["B"], 20.0)
    return sim


def test_zero_order_reactions_match_oracle(orc):
    want_s, want_c, _ = oracle_prod(orc, _model(), 6, seed=99)
    assert want_c.sum() > 0
    launches = tiling_launches()
    streams = stream_tilings(16)
    for ti in ([i for i in streams if launches[i] == 4][-1], next(i for i in streams if launches[i] == 3)):
        s, c, _ = gpu_prod(_model(), 6, 99, tiling=ti)
        assert np.array_equal(s, want_s), ti
        assert np.array_equal(c, want_c), ti
