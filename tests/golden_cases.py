"""Access to the stored golden vectors (tests/golden/golden.npz)."""
from __future__ import annotations

from pathlib import Path
from types import SimpleNamespace

import numpy as np

from cell_simulation_gb300.simulation import LatticeParams, Simulation, Tables

PATH = Path(__file__).resolve().parent / "golden" / "golden.npz"


def load():
    return np.load(PATH)


def cases(data, kind):
    """Case names of one kind: 'ref' (reference RNG) or 'prod' (Philox)."""
    names = sorted({k.split("/")[0] for k in data.files})
    return [n for n in names if (f"{n}/itimes" in data.files) == (kind == "ref")]


def case(data, name):
    g = {k.split("/", 1)[1]: data[k] for k in data.files if k.startswith(name + "/")}
    X, Y, Z, K, NR, S, R = (int(x) for x in g["params"])
    tau, lam = (float(x) for x in g["tau_lambda"])
    tab = Tables(g["regions"].astype(np.uint32), g["diffusion"], g["stoich"], g["reactants"].astype(np.uint32),
                 g["rates"], g["reservoir"].astype(np.uint32))
    return SimpleNamespace(res=(X, Y, Z), K=K, NR=NR, S=S, R=R, tau=tau, lam=lam, tab=tab, g=g)


def simulation(c) -> Simulation:
    """A drop-in Simulation rebuilt from the stored reference-layout tables and lattice."""
    sim = Simulation(LatticeParams([r * c.lam for r in c.res], list(c.res), c.tau, c.lam, c.K))
    t = c.tab
    sim.set_tables(c.NR, c.S, c.R, t.regions, t.diffusion, t.stoich, t.reactants, t.rates, t.reservoir)
    if "in_occ" in c.g:
        sim.set_lattice(c.g["in_slots"].astype(np.uint32), c.g["in_occ"].astype(np.uint32),
                        c.g["in_conc"].astype(np.int32))
    else:
        sim.set_lattice(c.g["in_slots"].astype(np.uint32))
    return sim
