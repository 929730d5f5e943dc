"""Reference-RNG (bit-parity) CUDA path against the serial oracle: slots,
occupancy, concentrations, species counts and diagnostics must be identical
after N frames.  Integer state: bit-exact."""
import numpy as np
import pytest

from cell_simulation_gb300 import RNG_REFERENCE, configs
from tests.helpers import crowded_model, itime_schedule, multi_region_model, oracle_args, ref_state

pytestmark = pytest.mark.gpu


def run_pair(orc, sim, n_frames, seed=987654321, chunks=1):
    args = oracle_args(sim)
    s, o, c, st = ref_state(sim)
    it = itime_schedule(n_frames, seed)
    ref = orc.ref_run(*args, orc.RefState(s, o, c, st), it, mode=1, threads=8)
    sim.prepare_for_gpu(RNG_REFERENCE, 0)
    for part in np.array_split(it, chunks):
        sim.step(part)
    gs, go, gc = sim.get_lattice()
    return ref, (gs, go, gc, sim.counts(), sim.diagnostics())


def assert_same(ref, gpu):
    gs, go, gc, counts, diag = gpu
    assert np.array_equal(gs, ref.slots), np.flatnonzero(gs != ref.slots)[:10]
    assert np.array_equal(go, ref.occ)
    assert np.array_equal(gc, ref.conc)
    assert np.array_equal(counts, ref.stat.astype(np.int64))
    for k in (0, 1, 2, 3, 4):
        assert diag[k] == ref.diag[k], (k, diag, ref.diag)


def test_c1_plain_parity(orc):
    w = configs.c1_plain_2d()
    ref, gpu = run_pair(orc, w.sim, 1000)
    assert_same(ref, gpu)
    assert ref.diag[4] > 0


@pytest.mark.parametrize("reservoir,transition", [(False, False), (True, False), (False, True)])
def test_multi_region_parity(orc, reservoir, transition):
    sim = multi_region_model(reservoir=reservoir, transition=transition)
    ref, gpu = run_pair(orc, sim, 300, chunks=3)
    assert_same(ref, gpu)


@pytest.mark.parametrize("res,K", [((7, 5, 9), 8), ((3, 11, 2), 16), ((1, 1, 40), 8), ((13, 1, 1), 4)])
def test_odd_shapes_parity(orc, res, K):
    sim = multi_region_model(res=res, K=K, counts=(8, 6, 4, 2)) if min(res) >= 3 else crowded_model(res=res, K=K, counts=(6, 4, 2))
    ref, gpu = run_pair(orc, sim, 200)
    assert_same(ref, gpu)


def test_contention_serial_resolution(orc):
    sim = crowded_model()
    ref, gpu = run_pair(orc, sim, 150)
    assert_same(ref, gpu)
    assert gpu[4][2] > 0  # frames resolved by the serial kernel


def test_stats_samples_match(orc):
    w = configs.c1_plain_2d()
    sim = w.sim
    args = oracle_args(sim)
    s, o, c, st = ref_state(sim)
    it = itime_schedule(100)
    sim.prepare_for_gpu(RNG_REFERENCE, 0)
    sim.step(it, write_freq=25)
    got = [(x.name, x.value, x.iteration_count) for x in sim.stats]
    names = sim.particle_names
    want = []
    state = orc.RefState(s, o, c, st)
    done = 0
    for f in (25, 50, 75):
        orc.ref_run(*args, state, it[done:f], mode=0)
        done = f
        for sp in (1, 2, 3):
            want.append((names[sp], int(state.stat[sp]), f))
    assert got == want
