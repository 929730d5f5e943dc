"""The oracle against its stored golden vectors (tests/golden/make_golden.py):
every case is replayed from its stored inputs and must give the stored
outputs exactly."""
import numpy as np
import pytest

from tests import golden_cases as G

DATA = G.load()


@pytest.mark.parametrize("name", G.cases(DATA, "ref"))
def test_reference_semantics_golden(orc, name):
    c = G.case(DATA, name)
    g = c.g
    st = orc.RefState(g["in_slots"], g["in_occ"], g["in_conc"], g["in_stat"])
    r = orc.ref_run(c.res, c.K, c.NR, c.S, c.R, np.float32(c.tau), np.float32(c.lam), c.tab, st, g["itimes"], mode=0)
    assert np.array_equal(r.slots, g["out_slots"])
    assert np.array_equal(r.occ, g["out_occ"])
    assert np.array_equal(r.conc, g["out_conc"])
    assert np.array_equal(r.stat, g["out_stat"])
    assert np.array_equal(r.diag, g["out_diag"])
    # the parallel gather formulation reproduces the same vectors
    st2 = orc.RefState(g["in_slots"], g["in_occ"], g["in_conc"], g["in_stat"])
    r2 = orc.ref_run(c.res, c.K, c.NR, c.S, c.R, np.float32(c.tau), np.float32(c.lam), c.tab, st2, g["itimes"],
                     mode=1, threads=4)
    assert np.array_equal(r2.slots, g["out_slots"]) and np.array_equal(r2.conc, g["out_conc"])


@pytest.mark.parametrize("name", G.cases(DATA, "prod"))
def test_production_semantics_golden(orc, name):
    c = G.case(DATA, name)
    g = c.g
    slots = g["in_slots"].copy()
    counts = np.bincount(slots, minlength=c.S + 1).astype(np.int64)
    counts[0] = 0
    seed, n = (int(x) for x in g["seed"])
    diag = orc.prod_run(c.res, c.K, c.NR, c.S, c.R, c.tau, c.lam, c.tab, slots, counts, seed, 0, n)
    assert np.array_equal(slots, g["out_slots"])
    assert np.array_equal(counts, g["out_counts"])
    assert np.array_equal(diag, g["out_diag"])


def test_golden_cases_present():
    assert {"c1", "multi", "crowd"} <= set(G.cases(DATA, "ref"))
    assert "prod" in G.cases(DATA, "prod")


def test_drop_in_rebuild_from_golden_tables():
    """The stored reference-layout tables load through the C ABI unchanged."""
    for name in G.cases(DATA, "ref") + G.cases(DATA, "prod"):
        c = G.case(DATA, name)
        sim = G.simulation(c)
        t = sim.tables()
        assert np.array_equal(t.regions, c.tab.regions) and np.array_equal(t.rates, c.tab.rates)
        s, _, _ = sim.get_lattice()
        assert np.array_equal(s.astype(np.uint8), c.g["in_slots"])
        sim.close()


def test_reference_saved_model_loads_to_the_stored_tables(lib):
    """The reference's own saved model (tests/golden/saved_models/easy.json, the file the reference
    ships as saved_models/easy.json) through cs_from_json_string: region mask, diffusion matrix,
    stoichiometry, reactants, rates and the seeded initial lattice equal the stored golden case."""
    from pathlib import Path

    from cell_simulation_gb300.simulation import Simulation
    text = (Path(G.PATH).parent / "saved_models" / "easy.json").read_text()
    sim = Simulation.from_json(text, placement_seed=7)
    c = G.case(DATA, "easy")
    t = sim.tables()
    i = sim.info()
    assert tuple(int(x) for x in i.res) == c.res and i.max_particles_site == c.K
    assert (i.n_regions, i.n_species, i.n_reactions) == (c.NR, c.S, c.R)
    assert np.array_equal(t.regions.astype(np.uint8), c.g["regions"])
    assert np.array_equal(t.diffusion, c.g["diffusion"])
    assert np.array_equal(t.stoich, c.g["stoich"])
    assert np.array_equal(t.reactants.astype(np.uint8), c.g["reactants"])
    assert np.array_equal(t.rates, c.g["rates"])
    assert np.array_equal(t.reservoir.astype(np.uint8), c.g["reservoir"])
    s, o, conc = sim.get_lattice()
    assert np.array_equal(s, c.g["in_slots"].astype(np.uint32))
    assert np.array_equal(o, c.g["in_occ"].astype(np.uint32))
    assert np.array_equal(conc, c.g["in_conc"].astype(np.int32))


def test_second_reference_saved_model_is_refused_like_the_reference(lib):
    """saved_models/easy_2.json declares a "sparse" region, which the reference's loader does not
    build (it panics, src/simulation.rs:275-276): cs_from_json_string refuses it with
    CS_ERR_PARSE and says why, instead of panicking."""
    from pathlib import Path

    import pytest

    from cell_simulation_gb300 import CellsimError
    from cell_simulation_gb300.simulation import Simulation
    text = (Path(G.PATH).parent / "saved_models" / "easy_2.json").read_text()
    with pytest.raises(CellsimError) as e:
        Simulation.from_json(text, placement_seed=3)
    assert e.value.status == 5 and "sparse" in str(e.value)
