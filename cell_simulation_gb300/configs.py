"""Synthetic workloads with the shapes, sizes and value distributions of the
five named configurations (no public dataset exists for this path).

All randomness derives from a master seed through numpy's SeedSequence.
Units: lambda = 32 nm, dims = res * lambda, macroscopic second-order rates
(/M/s) converted to per-voxel stochastic rates k / (N_A * lambda^3 * 1e3),
because the reference uses rates raw per voxel (cme.wgsl:39).  tau follows
the reference's implicit stability rule: the cumulative move probability
6 * D_max * tau / lambda^2 of rdme.wgsl:135,190 must not exceed 1.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .simulation import LatticeParams, RegionType, Simulation

LAMBDA = 32e-9
N_AVOGADRO = 6.02214076e23
MASTER_SEED = 20261203


def per_voxel_rate(k_molar: float, lam: float = LAMBDA) -> float:
    """Second-order rate in /M/s -> per-voxel pair rate in /s."""
    v_litre = lam ** 3 * 1e3
    return k_molar / (N_AVOGADRO * v_litre)


def stable_tau(d_max: float, lam: float = LAMBDA) -> float:
    """Largest binary32 tau with 6 * D_max * tau / lambda^2 <= 1 in binary32."""
    tau = np.float32(lam * lam / (6.0 * d_max))
    l2 = np.float32(lam) * np.float32(lam)
    while np.float32(np.float32(6.0) * (np.float32(d_max) * tau / l2)) > np.float32(1.0):
        tau = np.nextafter(tau, np.float32(0))
    return float(tau)


@dataclass
class Workload:
    name: str
    sim: Simulation
    n_steps: int
    K: int
    res: tuple
    meta: dict = field(default_factory=dict)


def _lattice(res, K, d_max):
    dims = [r * LAMBDA for r in res]
    return LatticeParams(dims, list(res), stable_tau(d_max), LAMBDA, K)


def c1_plain_2d(seed: int = MASTER_SEED, n_A: int = 200, n_B: int = 200) -> Workload:
    """64x64x1, K=8, one cytoplasm region, A + B -> C (1e6 /M/s), C -> A + B (0.1 /s), D = 1e-12."""
    D = 1e-12
    res = (64, 64, 1)
    sim = Simulation(_lattice(res, 8, D))
    sim.seed_placement(seed)
    dims = [r * LAMBDA for r in res]
    sim.add_region(RegionType.Cube("cytoplasm", [0, 0, 0], dims), D)
    sim.prepare_regions()
    for name, n in (("A", n_A), ("B", n_B), ("C", 0)):
        sim.add_particle_count(name, "cytoplasm", n, True, False)
    sim.add_reaction(["A", "B"], ["C"], per_voxel_rate(1e6))
    sim.add_reaction(["C"], ["A", "B"], 0.1)
    return Workload("c1_plain_64x64x1_K8", sim, 10_000, 8, res)


def _random_network(rng, n_species, n_reactions, first_range, second_range_molar):
    """Mass-action network: about half first order (A -> B, A -> B + C), half
    second order (A + B -> C, A + B -> C + D); no homodimers."""
    rx = []
    for r in range(n_reactions):
        if r % 2 == 0:
            a = int(rng.integers(n_species))
            k = float(np.exp(rng.uniform(np.log(first_range[0]), np.log(first_range[1]))))
            prods = rng.choice([s for s in range(n_species) if s != a], size=int(rng.integers(1, 3)), replace=False)
            rx.append(([a], [int(p) for p in prods], k))
        else:
            a, b = rng.choice(n_species, size=2, replace=False)
            km = float(np.exp(rng.uniform(np.log(second_range_molar[0]), np.log(second_range_molar[1]))))
            prods = rng.choice([s for s in range(n_species) if s not in (a, b)], size=int(rng.integers(1, 3)),
                               replace=False)
            rx.append(([int(a), int(b)], [int(p) for p in prods], per_voxel_rate(km)))
    return rx


def c2_single_cell(seed: int = MASTER_SEED, res=(128, 128, 128), r_ext: float = 56.0) -> Workload:
    """128^3, K=16, sphere r=56 voxels: 1-voxel membrane shell, cytoplasm inside, extracellular outside;
    8 species, 10 reactions, per-region D log-uniform 1e-13..1e-11, counts U{500..5000}."""
    rng = np.random.default_rng(np.random.SeedSequence([seed, 2]))
    S, R = 8, 10
    D = np.exp(rng.uniform(np.log(1e-13), np.log(1e-11), size=(3, S)))
    sim = Simulation(_lattice(res, 16, float(D.max())))
    sim.seed_placement(seed + 2)
    c = [res[0] / 2 * LAMBDA, res[1] / 2 * LAMBDA, res[2] / 2 * LAMBDA]
    sim.add_region(RegionType.SphericalShell("membrane", "cytoplasm", c, (r_ext - 1) * LAMBDA, r_ext * LAMBDA), 1e-12)
    sim.prepare_regions()
    regions = ["background", "membrane", "cytoplasm"]
    names = [f"S{i}" for i in range(S)]
    home = rng.integers(0, 3, size=S)
    for i, n in enumerate(names):
        sim.add_particle_count(n, regions[home[i]], int(rng.integers(500, 5001)), True, False)
    for i, n in enumerate(names):
        for r in range(3):
            sim.set_diffusion_rate_particle(n, regions[r], float(D[r, i]))
    for re, pr, k in _random_network(rng, S, R, (1e-2, 1e2), (1e5, 1e7)):
        sim.add_reaction([names[a] for a in re], [names[p] for p in pr], k)
    return Workload(f"c2_single_cell_{res[0]}x{res[1]}x{res[2]}_K16", sim, 1000, 16, tuple(res))


def c3_multi_region(seed: int = MASTER_SEED, res=(256, 256, 256), r_nuc: float = 40.0, r_cyt: float = 110.0,
                    total_particles: int = 1_000_000) -> Workload:
    """256^3, K=16: nucleus r=40 inside cytoplasm r=110 inside a 1-voxel membrane shell, extracellular
    outside; 16 species, 30 reactions; receptor species confined to the membrane; 1e6 particles."""
    rng = np.random.default_rng(np.random.SeedSequence([seed, 3]))
    S, R = 16, 30
    regions = ["background", "membrane", "cytoplasm", "nucleus"]
    D = np.exp(rng.uniform(np.log(1e-13), np.log(1e-11), size=(4, S)))
    receptors = [0, 1]  # membrane-bound species
    sim = Simulation(_lattice(res, 16, float(D.max())))
    sim.seed_placement(seed + 3)
    c = [res[0] / 2 * LAMBDA, res[1] / 2 * LAMBDA, res[2] / 2 * LAMBDA]
    sim.add_region(RegionType.SphericalShell("membrane", "cytoplasm", c, r_cyt * LAMBDA, (r_cyt + 1) * LAMBDA), 1e-12)
    sim.add_region(RegionType.Sphere("nucleus", c, r_nuc * LAMBDA), 1e-12)
    sim.prepare_regions()
    vol = sim.region_volumes()
    names = [f"P{i}" for i in range(S)]
    home = np.array([1 if i in receptors else int(rng.choice([0, 2, 3], p=[0.5, 0.35, 0.15])) for i in range(S)])
    w = rng.uniform(0.5, 1.5, size=S)
    counts = np.floor(w / w.sum() * total_particles).astype(int)
    # membrane capacity: keep receptors well below the shell's capacity
    cap = int(vol[1]) * 2
    counts[receptors] = np.minimum(counts[receptors], cap // len(receptors))
    counts[-1] += total_particles - counts.sum()
    for i, n in enumerate(names):
        sim.add_particle_count(n, regions[home[i]], int(counts[i]), True, False)
    for i, n in enumerate(names):
        for r in range(4):
            sim.set_diffusion_rate_particle(n, regions[r], float(D[r, i]))
    # region-restricted membrane binding: ligand + receptor -> complex (receptor cannot leave the membrane)
    rx = _random_network(rng, S, R - 2, (1e-2, 1e2), (1e5, 1e7))
    rx.append(([2, 0], [3], per_voxel_rate(1e6)))
    rx.append(([3], [2, 0], 1.0))
    for re, pr, k in rx:
        sim.add_reaction([names[a] for a in re], [names[p] for p in pr], k)
    return Workload(f"c3_multi_region_{res[0]}x{res[1]}x{res[2]}_K16", sim, 100, 16, tuple(res))


def c4_ensemble_template(K: int = 8) -> Simulation:
    """The 3-species model of c1 in 3-D (one lattice is built per replicate by the ensemble)."""
    D = 1e-12
    res = (8, 8, 8)
    sim = Simulation(_lattice(res, K, D))
    sim.set_diffusion_rate("background", D)
    sim.prepare_regions()
    for n in ("A", "B", "C"):
        sim.add_particle_count(n, "background", 0, True, False)
    sim.set_diffusion_rate("background", D)
    sim.add_reaction(["A", "B"], ["C"], per_voxel_rate(1e6))
    sim.add_reaction(["C"], ["A", "B"], 0.1)
    return sim


def c4_ensemble_spec(seed: int = MASTER_SEED, n_rep: int = 512, lo: int = 32, hi: int = 96):
    """Edges U{32..96}, per-replicate seeds and rate multipliers log-U[0.5, 2]."""
    rng = np.random.default_rng(np.random.SeedSequence([seed, 4]))
    edges = rng.integers(lo, hi + 1, size=n_rep)
    res = np.stack([edges, edges, edges], axis=1).astype(np.uint32)
    seeds = rng.integers(1, 2 ** 63, size=n_rep, dtype=np.uint64)
    mult = np.exp(rng.uniform(np.log(0.5), np.log(2.0), size=n_rep)).astype(np.float32)
    init = np.array([0, 200, 200, 0], np.uint32)
    return res, seeds, mult, init


def c5_network(seed: int = MASTER_SEED):
    """The stiff network of c5: 12 species, 24 first/second-order reactions, rates 1e-3..1e4 /s
    (second order: the same range per voxel pair)."""
    rng = np.random.default_rng(np.random.SeedSequence([seed, 5]))
    return _random_network(rng, 12, 24, (1e-3, 1e4), (1e-3 * 19733.5, 1e4 * 19733.5))


def c5_ensemble_template(seed: int = MASTER_SEED, res=(48, 48, 48)) -> Simulation:
    """The c5 model without particles, as the template of an ensemble of sub-lattices."""
    D = 1e-12
    sim = Simulation(_lattice(res, 16, D))
    sim.set_diffusion_rate("background", D)
    sim.prepare_regions()
    names = [f"Q{i}" for i in range(12)]
    for n in names:
        sim.add_particle_count(n, "background", 0, True, False)
    sim.set_diffusion_rate("background", D)
    for re, pr, k in c5_network(seed):
        sim.add_reaction([names[a] for a in re], [names[p] for p in pr], k)
    return sim


def c5_stiff(seed: int = MASTER_SEED, res=(192, 192, 192), total_particles: int = 1_000_000) -> Workload:
    """192^3, K=16, 12 species, 24 first/second-order reactions with rates 1e-3..1e4 /s (stiff), D = 1e-12."""
    S, R, D = 12, 24, 1e-12
    sim = Simulation(_lattice(res, 16, D))
    sim.seed_placement(seed + 5)
    sim.set_diffusion_rate("background", D)
    sim.prepare_regions()
    names = [f"Q{i}" for i in range(S)]
    for n in names:
        sim.add_particle_count(n, "background", total_particles // S, True, False)
    sim.set_diffusion_rate("background", D)
    for re, pr, k in c5_network(seed):
        sim.add_reaction([names[a] for a in re], [names[p] for p in pr], k)
    return Workload(f"c5_stiff_{res[0]}x{res[1]}x{res[2]}_K16", sim, 100, 16, tuple(res))
