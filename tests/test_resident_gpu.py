"""The resident form of the production step (one block per replicate holds its lattice in shared
memory for every frame of a step call): bit-exact with the oracle on the 64 x 64 x 1 lattice of the
reference's own small case and on a multi-region lattice with reservoirs, in calls of one and of
many frames; through switches to and from the other forms with odd frame counts (which hand over
the other parity's lattice buffer and work counters); and refused for a lattice larger than one
block's shared memory, the handle keeping its own form."""
import numpy as np
import pytest

from cell_simulation_gb300 import CellsimError, RNG_PHILOX, configs, tiling_kinds, tiling_launches, tiling_variants
from tests.helpers import multi_region_model
from tests.test_prod_gpu import gpu_prod, oracle_prod, stream_tilings

pytestmark = pytest.mark.gpu


def resident(K):
    return next(i for i, (t, k) in enumerate(zip(tiling_variants(), tiling_kinds())) if t[0] == K and k[0] == 3)


@pytest.mark.parametrize("K", [8, 16])
def test_resident_matches_oracle_with_reservoirs(orc, K):
    mk = lambda: multi_region_model(res=(9, 8, 40), K=K, counts=(60, 50, 40, 30), reservoir=True)
    want_s, want_c, want_d = oracle_prod(orc, mk(), 25, seed=4242)
    got_s, got_c, got_d = gpu_prod(mk(), 25, 4242, tiling=resident(K), chunks=4)
    assert np.array_equal(got_s, want_s)
    assert np.array_equal(got_c, want_c)
    assert np.array_equal(got_d[:4], want_d[:4])
    assert want_d[0] > 0  # reactions fired


def test_resident_on_the_small_2d_case_matches_oracle(orc):
    """64 x 64 x 1, K = 8, A + B <-> C: one call of 150 frames and 150 calls of one frame."""
    want_s, want_c, want_d = oracle_prod(orc, configs.c1_plain_2d().sim, 150, seed=2026)
    for chunks in (1, 150):
        got_s, got_c, got_d = gpu_prod(configs.c1_plain_2d().sim, 150, 2026, tiling=resident(8), chunks=chunks)
        assert np.array_equal(got_s, want_s), chunks
        assert np.array_equal(got_c, want_c), chunks
        assert np.array_equal(got_d[:4], want_d[:4]), chunks
    assert want_d[0] > 0


def test_switching_to_and_from_the_resident_form_matches_oracle(orc):
    mk = lambda: multi_region_model(res=(9, 8, 40), K=16, counts=(70, 60, 50, 40))
    want_s, want_c, _ = oracle_prod(orc, mk(), 31, seed=909)
    sim = mk()
    sim.prepare_for_gpu(RNG_PHILOX, 0)
    kinds, launches = tiling_kinds(), tiling_launches()
    brick = next(i for i, (t, k) in enumerate(zip(tiling_variants(), kinds)) if t[0] == 16 and k == (1, 8))
    unfused = [i for i in stream_tilings(16) if launches[i] == 3][-1]
    fused = next(i for i in stream_tilings(16) if launches[i] == 2)
    frames = next(i for i in stream_tilings(16) if launches[i] == 1)
    res16 = resident(16)
    for ti, n in ((res16, 3), (unfused, 3), (res16, 1), (frames, 4), (res16, 5), (fused, 3), (res16, 2),
                  (brick, 3), (res16, 3), (fused, 4)):
        sim.set_tiling(ti)
        sim.step_philox(n, 909)
    assert np.array_equal(sim.get_lattice()[0].astype(np.uint8), want_s)
    assert np.array_equal(sim.counts(), want_c)
    assert sim.diagnostics()[7] == 0


def test_resident_refuses_a_lattice_too_large_for_shared_memory():
    sim = multi_region_model(res=(24, 24, 24), K=16)  # 13,824 voxels: 0.5 MB of slots alone
    sim.prepare_for_gpu(RNG_PHILOX, 0)
    before = sim.get_tiling()
    with pytest.raises(CellsimError):
        sim.set_tiling(resident(16))
    assert sim.get_tiling() == before
    sim.step_philox(3, 1)
    assert sim.counts().sum() > 0
