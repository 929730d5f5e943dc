"""Shared fixtures: small models and state extraction for oracle/library comparisons."""
from __future__ import annotations

import numpy as np

from cell_simulation_gb300 import configs
from cell_simulation_gb300.simulation import LatticeParams, RegionType, Simulation

LAM = configs.LAMBDA


def itime_schedule(n, seed=987654321, stride=7919):
    """Per-frame itime values itime_f = seed + stride * f (u32 wrap)."""
    return ((np.uint64(seed) + np.uint64(stride) * np.arange(n, dtype=np.uint64)) & np.uint64(0xFFFFFFFF)).astype(np.uint32)


def compact_slots(slots_u32, K):
    """Reference-layout slots (u32, V*K) as the production path's compacted u8 voxels: each voxel's
    particles moved to its first slots in slot order."""
    s = np.asarray(slots_u32).reshape(-1, K).astype(np.uint8)
    order = np.argsort(s == 0, axis=1, kind="stable")
    return np.take_along_axis(s, order, axis=1).reshape(-1)


def ref_state(sim: Simulation):
    i = sim.info()
    s, o, c = sim.get_lattice()
    stat = c.reshape(-1, i.n_species + 1).sum(0).astype(np.int32)
    return s, o, c, stat


def oracle_args(sim: Simulation):
    i = sim.info()
    return (tuple(int(x) for x in i.res), i.max_particles_site, i.n_regions, i.n_species, i.n_reactions,
            float(np.float32(i.tau)), float(np.float32(i.lambda_)), sim.tables())


def multi_region_model(res=(12, 10, 14), K=8, seed=7, counts=(40, 30, 20, 10), reservoir=False, D_scale=1.0,
                       transition=False) -> Simulation:
    """Sphere shell + inner sphere, 4 species, mixed first/second-order reactions."""
    D = 1e-12 * D_scale
    dims = [r * LAM for r in res]
    sim = Simulation(LatticeParams(dims, list(res), configs.stable_tau(D), LAM, K))
    sim.seed_placement(seed)
    c = [res[0] / 2 * LAM, res[1] / 2 * LAM, res[2] / 2 * LAM]
    sim.add_region(RegionType.SphericalShell("membrane", "cytoplasm", c, 3.5 * LAM, 4.6 * LAM), D)
    sim.add_region(RegionType.Sphere("nucleus", c, 2.0 * LAM), D * 0.5)
    sim.prepare_regions()
    names = ["A", "B", "C", "R"]
    homes = ["cytoplasm", "background", "cytoplasm", "membrane"]
    for n, h, k in zip(names, homes, counts):
        sim.add_particle_count(n, h, k, True, False)
    if reservoir:
        sim.add_particle_concentration("X", "membrane", 0.3, False, True)
    if transition:
        sim.set_transition_rate("cytoplasm", "nucleus", D * 0.3)
        sim.set_transition_rate("nucleus", "cytoplasm", D * 0.3)
        sim.set_transition_rate_particle("B", "background", "membrane", D)
    sim.add_reaction(["A", "B"], ["C"], 800.0)
    sim.add_reaction(["C"], ["A", "B"], 40.0)
    sim.add_reaction(["A"], ["B"], 25.0)
    sim.add_reaction(["R", "A"], ["C"], 900.0)
    sim.add_reaction(["C"], ["R"], 15.0)
    if reservoir:
        sim.add_reaction(["X", "B"], ["A"], 500.0)
    return sim


def crowded_model(res=(6, 5, 4), K=4, counts=(30, 20, 10), seed=3, D=1e-12) -> Simulation:
    """Small, nearly full lattice: moves into full voxels are common."""
    dims = [r * LAM for r in res]
    sim = Simulation(LatticeParams(dims, list(res), configs.stable_tau(D), LAM, K))
    sim.seed_placement(seed)
    sim.set_diffusion_rate("background", D)
    sim.prepare_regions()
    for n, k in zip(("A", "B", "C"), counts):
        sim.add_particle_count(n, "background", k, True, False)
    sim.set_diffusion_rate("background", D)
    sim.add_reaction(["A", "B"], ["C"], 300.0)
    sim.add_reaction(["C"], ["A", "B"], 200.0)
    return sim


def patchy_model(res=(19, 21, 70), K=16, seed=11, dense=3200, sparse=150, D=1e-12) -> Simulation:
    """Mostly empty lattice with one crowded cube (about four fifths of its voxels
    occupied; the fullest box holds 841 occupied voxels for 8-plane bricks and 1203
    for 16-plane ones, above every bounded pool): the production brick pass keeps
    the sparse bricks and hands the crowded ones to the full-capacity second pass."""
    dims = [r * LAM for r in res]
    sim = Simulation(LatticeParams(dims, list(res), configs.stable_tau(D), LAM, K))
    sim.seed_placement(seed)
    sim.add_region(RegionType.Cube("dense", [2 * LAM, 3 * LAM, 5 * LAM], [12 * LAM, 11 * LAM, 30 * LAM]), D)
    sim.prepare_regions()
    sim.set_diffusion_rate("background", D)
    sim.set_transition_rate("dense", "background", D * 0.5)
    sim.set_transition_rate("background", "dense", D * 0.5)
    sim.add_particle_count("A", "dense", dense, True, False)
    sim.add_particle_count("B", "background", sparse, True, False)
    sim.add_particle_count("C", "background", 0, True, False)
    sim.add_reaction(["A", "B"], ["C"], 700.0)
    sim.add_reaction(["C"], ["A", "B"], 60.0)
    sim.add_reaction(["A"], ["B"], 20.0)
    return sim


def network_template(sim: Simulation, res=(24, 24, 24), K=16, D=1e-12) -> Simulation:
    """A one-region ensemble template carrying sim's species and reactions (read back from its
    reference-layout tables) with diffusion D for every species: the well-mixed form of a
    configuration's reaction network."""
    t, i = sim.tables(), sim.info()
    S1, R = i.n_species + 1, i.n_reactions
    names = sim.particle_names
    tmpl = Simulation(LatticeParams([r * LAM for r in res], list(res), configs.stable_tau(D), LAM, K))
    tmpl.set_diffusion_rate("background", D)
    tmpl.prepare_regions()
    for n in names[1:]:
        tmpl.add_particle_count(n, "background", 0, True, False)
    tmpl.set_diffusion_rate("background", D)
    re = t.reactants.reshape(R + 1, 3)
    st = t.stoich.reshape(R + 1, S1)
    for r in range(1, R + 1):
        rs = [int(s) for s in re[r] if s]
        change = st[r].astype(np.int64).copy()
        prod = []
        have = np.bincount(np.array(rs, np.int64), minlength=S1) if rs else np.zeros(S1, np.int64)
        for s in range(1, S1):
            prod += [s] * int(have[s] + change[s])
        tmpl.add_reaction([names[s] for s in rs], [names[s] for s in prod], float(t.rates[r]))
    return tmpl
