"""The C-ABI library loads and exports every declared symbol; the host model
builder (regions, particles, reactions, JSON) behaves like the reference's.
No device call is made here."""
import ctypes as C
import json
import re
from pathlib import Path

import numpy as np
import pytest

from cell_simulation_gb300 import CellsimError, native
from cell_simulation_gb300.simulation import LatticeParams, RegionType, Simulation
from tests.helpers import LAM

HEADER = Path(__file__).resolve().parents[1] / "include" / "cellsim.h"


def declared_symbols():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(cs_[a-z_0-9]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(lib):
    syms = declared_symbols()
    assert len(syms) >= 40
    raw = C.CDLL(str(native.LIB_PATH))
    missing = [s for s in syms if not hasattr(raw, s)]
    assert not missing, missing
    # and the Python binding covers every declared symbol
    assert sorted(native.SIGNATURES) == syms


def test_variant_tables(lib):
    """The compiled step variants as the autotuner and bench.py see them (no device call): every
    slot count has three-launch sweep streams, fused ones (two launches per frame) and persistent
    ones (one launch per step call); bricks with bounded pools take two launches, the tile
    pipeline one, the resident form one per step call."""
    from cell_simulation_gb300 import tiling_kinds, tiling_launches, tiling_variants

    v, k, n = tiling_variants(), tiling_kinds(), tiling_launches()
    assert len(v) == len(k) == len(n) > 0
    for K in (8, 16):
        stream = [n[i] for i in range(len(v)) if v[i][0] == K and k[i][0] == 2]
        assert 1 in stream and 2 in stream and 3 in stream
        # the persistent multi-frame form is marked by TY = 1
        assert all((v[i][1] == 1) == (n[i] == 1) for i in range(len(v)) if v[i][0] == K and k[i][0] == 2)
    assert all(n[i] == 1 for i in range(len(v)) if k[i][0] == 0)
    assert all(n[i] in (1, 2) for i in range(len(v)) if k[i][0] == 1)
    # the resident form: one launch per step call, for both slot counts
    assert sorted(v[i][0] for i in range(len(v)) if k[i][0] == 3) == [8, 16]
    assert all(n[i] == 1 for i in range(len(v)) if k[i][0] == 3)
    with pytest.raises(CellsimError):
        out = C.c_int32()
        native.check(lib.cs_tiling_launches(len(v), C.byref(out)))


def test_version_and_errors(lib):
    assert b"sm_103a" in lib.cs_version()
    with pytest.raises(CellsimError) as e:
        Simulation(LatticeParams([1, 1, 1], [0, 4, 4], 1e-4, 1e-8))
    assert e.value.status == 1
    with pytest.raises(CellsimError) as e:
        Simulation(LatticeParams([1, 1, 1], [4, 4, 4], 1e-4, 1e-8, max_particles_site=17))
    assert e.value.status == 3


def _small(res=(16, 16, 16), K=8):
    dims = [r * LAM for r in res]
    return Simulation(LatticeParams(dims, list(res), 1e-4, LAM, K))


def test_sphere_and_shell_volumes(lib):
    sim = _small((20, 20, 20))
    c = [10 * LAM, 10 * LAM, 10 * LAM]
    sim.add_region(RegionType.SphericalShell("mem", "cyt", c, 5 * LAM, 6 * LAM), 1e-12)
    sim.prepare_regions()
    t = sim.tables()
    reg = t.regions.reshape(20, 20, 20)
    f = np.float32
    x, y, z = (a.astype(f) for a in np.meshgrid(np.arange(20), np.arange(20), np.arange(20), indexing="ij"))
    vs = f(f(20 * LAM) / f(20))
    ctr = f(f(10 * LAM) / vs)
    vss = f(vs * vs)

    def inside(r):
        # the binary32 expression of src/simulation.rs:680-683
        dx, dy, dz = f(1) * (x - ctr), f(1) * (y - ctr), f(1) * (z - ctr)
        d = (dx * dx) * vss + (dy * dy) * vss
        d = d + (dz * dz) * vss
        return d < f(f(r) * f(r))

    inside6, inside5 = inside(6 * LAM), inside(5 * LAM)
    assert 400 < inside5.sum() < 600  # about 4/3 pi 5^3
    assert np.array_equal(reg == 2, inside5)
    assert np.array_equal(reg == 1, inside6 & ~inside5)
    vol = sim.region_volumes()
    assert vol[2] == inside5.sum() and vol[1] == (inside6 & ~inside5).sum()
    assert sim.region_names == ["background", "mem", "cyt"]


def test_capsid_joins_caps(lib):
    sim = _small((16, 16, 32))
    sim.add_region(RegionType.Capsid("membrane", "interior", [8 * LAM, 8 * LAM, 16 * LAM], [0, 0, 1], 5 * LAM,
                                     6 * LAM, 30 * LAM), 1e-14)
    names = sim.region_names
    assert names == ["background", "membrane", "interior"]
    t = sim.tables()
    assert set(np.unique(t.regions)) <= {0, 1, 2}
    assert (t.regions == 2).sum() > 0 and (t.regions == 1).sum() > 0
    # the diffusion matrix has shrunk back to 3 regions
    assert t.diffusion.size == 3 * 3 * 1


def test_particles_reactions_tables(lib):
    sim = _small((8, 8, 8))
    sim.add_region(RegionType.Cube("box", [0, 0, 0], [4 * LAM, 8 * LAM, 8 * LAM]), 2e-12)
    sim.prepare_regions()
    sim.add_particle_count("A", "box", 100, True, False)
    sim.add_particle_count("B", "background", 50, False, False)
    sim.add_particle_concentration("X", "box", 0.25, False, True)
    sim.set_diffusion_rate_particle("A", "background", 3e-12)
    sim.set_transition_rate_particle("A", "box", "background", 1e-13)
    sim.add_reaction(["A", "B"], ["A", "A"], 5.0)
    sim.add_reaction([], ["B"], 0.5)
    i = sim.info()
    assert (i.n_species, i.n_reactions, i.n_regions) == (3, 2, 2)
    t = sim.tables()
    st = t.stoich.reshape(3, 4)
    assert st[1].tolist() == [0, 1, -1, 0] and st[2].tolist() == [0, 0, 1, 0]
    assert t.reactants.reshape(3, 3)[1].tolist() == [1, 2, 0]
    assert t.reactants.reshape(3, 3)[2].tolist() == [0, 0, 0]
    D = t.diffusion.reshape(2, 2, 4)
    assert D[0, 0, 1] == np.float32(3e-12) and D[1, 1, 1] == np.float32(2e-12) and D[1, 0, 1] == np.float32(1e-13)
    # background default 8.15e-14 / 6 (binary32 arithmetic, src/simulation.rs:73) copied to the new species
    assert D[0, 0, 2] == np.float32(np.float32(8.15e-14) / np.float32(6))
    s, o, c = sim.get_lattice()
    c = c.reshape(-1, 4)
    assert c[:, 1].sum() == 100 and c[:, 2].sum() == 50
    assert (t.reservoir == 3).sum() == int(np.float32(0.25) * np.float32(sim.region_volumes()[1]))
    assert np.array_equal(o, (s.reshape(-1, 8) > 0).sum(1))
    with pytest.raises(CellsimError) as e:
        sim.add_reaction(["Z"], ["A"], 1.0)
    assert e.value.status == 2


MODEL = {
    "parameters": {"lattice_resolution": [8, 8, 16], "dimensions": [0.4, 0.4, 0.8], "tau": 2e-3, "lambda": 5e-8},
    "regions": [{"type": "capsid", "shell_name": "wall", "interior_name": "lumen", "center": [0.2, 0.2, 0.4],
                 "dir": [0.0, 0.0, 1.0], "internal_radius": 0.15, "external_radius": 0.19, "total_length": 0.78,
                 "base_diffusion_rate": 2e-14}],
    "particles": [
        {"name": "P", "to_region": "lumen", "count": 30, "logging": True, "is_reservoir": False,
         "diffusion_rate": {"lumen": 3e-14, "wall": 1e-15}},
        {"name": "Q", "to_region": "lumen", "count": 12, "logging": False, "is_reservoir": False},
        {"name": "W", "to_region": "wall", "concentration": 0.05, "logging": False, "is_reservoir": True},
    ],
    "reactions": {"Q -> P": 0.5, "P + Q -> Q 2": 3.0},
}


def test_json_loader(lib):
    sim = Simulation.from_json(json.dumps(MODEL), placement_seed=5)
    i = sim.info()
    assert (i.n_species, i.n_reactions, i.n_regions) == (3, 2, 3)
    assert sim.particle_names == ["void", "P", "Q", "W"]
    t = sim.tables()
    # reactions sorted by key: "P + Q -> Q 2" before "Q -> P"; the numeric token multiplies k
    assert np.allclose(t.rates, [0.0, 6.0, 0.5])
    assert t.reactants.reshape(3, 3)[1].tolist() == [1, 2, 0]
    D = t.diffusion.reshape(3, 3, 4)
    assert D[2, 2, 1] == np.float32(3e-14) and D[1, 1, 1] == np.float32(1e-15)
    s, o, c = sim.get_lattice()
    assert (s == 1).sum() == 30 and (s == 2).sum() == 12
    # same seed, same placement; other seed, other placement
    s2 = Simulation.from_json(json.dumps(MODEL), placement_seed=5).get_lattice()[0]
    s3 = Simulation.from_json(json.dumps(MODEL), placement_seed=6).get_lattice()[0]
    assert np.array_equal(s, s2) and not np.array_equal(s, s3)


def test_json_errors(lib):
    with pytest.raises(CellsimError) as e:
        Simulation.from_json("{ not json")
    assert e.value.status == 5
    bad = dict(MODEL, regions=[{"type": "sparse", "base_diffusion_rate": 1.0}])
    with pytest.raises(CellsimError) as e:
        Simulation.from_json(json.dumps(bad))
    assert e.value.status == 5
    with pytest.raises(CellsimError) as e:
        Simulation.from_file("/nonexistent/model.json")
    assert e.value.status == 6


def test_set_tables_and_lattice_roundtrip(lib):
    sim = _small((4, 4, 4), K=8)
    V = 64
    regions = np.zeros(V, np.uint32)
    regions[32:] = 1
    diffusion = np.full(2 * 2 * 3, 1e-12, np.float32)
    stoich = np.array([0, 0, 0, 0, -1, 1], np.int32)
    reactants = np.array([0, 0, 0, 1, 0, 0], np.uint32)
    rates = np.array([0, 2.0], np.float32)
    sim.set_tables(2, 2, 1, regions, diffusion, stoich, reactants, rates)
    slots = np.zeros(V * 8, np.uint32)
    slots[0:3] = [1, 2, 1]
    slots[8 * 40] = 2
    sim.set_lattice(slots)
    s, o, c = sim.get_lattice()
    assert np.array_equal(s, slots)
    assert o[0] == 3 and o[40] == 1 and o.sum() == 4
    c = c.reshape(V, 3)
    assert c[0].tolist() == [0, 2, 1] and c[40].tolist() == [0, 0, 1]
    with pytest.raises(CellsimError):
        bad = slots.copy()
        bad[5] = 9
        sim.set_lattice(bad)
