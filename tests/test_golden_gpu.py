"""The CUDA paths against the stored golden vectors, through the C ABI:
the reference-RNG path reproduces the reference-semantics outputs and the
production path the Philox outputs, bit for bit."""
import numpy as np
import pytest

from cell_simulation_gb300 import RNG_PHILOX, RNG_REFERENCE
from tests import golden_cases as G

pytestmark = pytest.mark.gpu
DATA = G.load()


@pytest.mark.parametrize("name", G.cases(DATA, "ref"))
def test_reference_rng_path_golden(name):
    c = G.case(DATA, name)
    sim = G.simulation(c)
    sim.prepare_for_gpu(RNG_REFERENCE, 0)
    sim.step(c.g["itimes"])
    s, o, conc = sim.get_lattice()
    assert np.array_equal(s.astype(np.uint8), c.g["out_slots"])
    assert np.array_equal(o.astype(np.uint8), c.g["out_occ"])
    assert np.array_equal(conc, c.g["out_conc"].astype(np.int32))
    assert np.array_equal(sim.counts(), c.g["out_stat"].astype(np.int64))


@pytest.mark.parametrize("name", G.cases(DATA, "prod"))
def test_production_path_golden(name):
    c = G.case(DATA, name)
    sim = G.simulation(c)
    sim.prepare_for_gpu(RNG_PHILOX, 0)
    seed, n = (int(x) for x in c.g["seed"])
    sim.step_philox(n, seed)
    s, _, _ = sim.get_lattice()
    assert np.array_equal(s.astype(np.uint8), c.g["out_slots"])
    assert np.array_equal(sim.counts(), c.g["out_counts"])
