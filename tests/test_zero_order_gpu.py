"""Zero-order reactions (no reactants) fire in every voxel, empty ones included: every kind of
production step (both forms of the sweep stream, a sparse brick pass whose crowded bricks spill, a
dense brick pass, a tile pipeline, the resident form) matches the oracle on such a model, and
particles appear in voxels that were empty."""
import numpy as np
import pytest

from cell_simulation_gb300 import tiling_kinds, tiling_launches, tiling_variants
from tests.helpers import multi_region_model
from tests.test_prod_gpu import gpu_prod, oracle_prod, stream_tilings

pytestmark = pytest.mark.gpu


def _model():
    sim = multi_region_model(res=(9, 8, 40), K=16, counts=(30, 20, 10, 5))
    sim.add_reaction([], ["A"], 40.0)
    sim.add_reaction(["A"], ["B"], 20.0)
    return sim


def _tilings():
    launches, kinds, var = tiling_launches(), tiling_kinds(), tiling_variants()
    streams = stream_tilings(16)
    k16 = [i for i, t in enumerate(var) if t[0] == 16]
    return {"unfused": [i for i in streams if launches[i] == 3][-1],
            "fused": next(i for i in streams if launches[i] == 2),
            "frames": next(i for i in streams if launches[i] == 1),
            "brick_sparse": next(i for i in k16 if kinds[i][0] == 1 and launches[i] == 2),
            "brick_dense": next(i for i in k16 if kinds[i][0] == 1 and launches[i] == 1),
            "tile": next(i for i in k16 if kinds[i][0] == 0),
            "resident": next(i for i in k16 if kinds[i][0] == 3)}


def test_zero_order_reactions_match_oracle(orc):
    sim0 = _model()
    s0 = sim0.get_lattice()[0].reshape(-1, 16)
    n0 = int((s0 > 0).sum())
    empty0 = ~(s0 > 0).any(1)
    want_s, want_c, _ = oracle_prod(orc, _model(), 6, seed=99)
    assert want_c.sum() > n0 + 20  # the zero-order source added particles
    assert (want_s.reshape(-1, 16)[empty0] > 0).any()  # a voxel empty at the start now holds a particle
    for tag, ti in _tilings().items():
        s, c, _ = gpu_prod(_model(), 6, 99, tiling=ti)
        assert np.array_equal(s, want_s), tag
        assert np.array_equal(c, want_c), tag
