"""Generates tests/golden/golden.npz: inputs and outputs of the CPU oracle on
small fixed cases, so later changes to the oracle (or to anything checked
against it) are caught against stored vectors.

Cases
  c1     the 64x64x1 two-species cell (configs.c1_plain_2d), reference RNG, 200 frames
  multi  sphere shell + nucleus, reservoir and transitions, reference RNG, 100 frames
  crowd  nearly full 6x5x4 lattice (capacity contention), reference RNG, 100 frames
  prod   11x13x37 multi-region lattice, K = 16, production (Philox) step, 30 frames
  easy   the reference's own saved model saved_models/easy.json, loaded by the
         drop-in JSON loader with placement seed 7, reference RNG, 20 frames
         (only when the reference checkout is present where this runs)

Each case stores the lattice parameters, the reference-layout tables, the
initial state and the outputs.  itime of frame f is 987654321 + 7919 f.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from cell_simulation_gb300 import configs  # noqa: E402
from cell_simulation_gb300.simulation import Simulation  # noqa: E402
from tests.helpers import crowded_model, itime_schedule, multi_region_model, oracle_args, ref_state  # noqa: E402

# the reference's own saved model (saved_models/easy.json), kept beside the fixtures
REFERENCE_EASY_JSON = Path(__file__).resolve().parent / "saved_models" / "easy.json"


def tables_dict(prefix, sim):
    res, K, NR, S, R, tau, lam, tab = oracle_args(sim)
    return {f"{prefix}/params": np.array([*res, K, NR, S, R], np.int64),
            f"{prefix}/tau_lambda": np.array([tau, lam], np.float32),
            f"{prefix}/regions": tab.regions.astype(np.uint8),
            f"{prefix}/diffusion": tab.diffusion.astype(np.float32),
            f"{prefix}/stoich": tab.stoich.astype(np.int32),
            f"{prefix}/reactants": tab.reactants.astype(np.uint8),
            f"{prefix}/rates": tab.rates.astype(np.float32),
            f"{prefix}/reservoir": tab.reservoir.astype(np.uint8)}


def ref_case(prefix, sim, n_frames):
    out = tables_dict(prefix, sim)
    args = oracle_args(sim)
    s, o, c, st = ref_state(sim)
    out.update({f"{prefix}/in_slots": s.astype(np.uint8), f"{prefix}/in_occ": o.astype(np.uint8),
                f"{prefix}/in_conc": c.astype(np.int16), f"{prefix}/in_stat": st.astype(np.int32)})
    it = itime_schedule(n_frames)
    r = oracle.ref_run(*args, oracle.RefState(s, o, c, st), it, mode=0)
    out.update({f"{prefix}/itimes": it, f"{prefix}/out_slots": r.slots.astype(np.uint8),
                f"{prefix}/out_occ": r.occ.astype(np.uint8), f"{prefix}/out_conc": r.conc.astype(np.int16),
                f"{prefix}/out_stat": r.stat.astype(np.int32), f"{prefix}/out_diag": r.diag.copy()})
    return out


def prod_case(prefix, sim, n_frames, seed):
    out = tables_dict(prefix, sim)
    res, K, NR, S, R, tau, lam, tab = oracle_args(sim)
    s, _, _ = sim.get_lattice()
    s = s.reshape(-1, K)
    slots = np.zeros_like(s, dtype=np.uint8)
    for v in np.flatnonzero((s > 0).any(1)):
        nz = s[v][s[v] > 0]
        slots[v, :len(nz)] = nz
    slots = slots.reshape(-1)
    counts = np.bincount(s.reshape(-1), minlength=S + 1).astype(np.int64)
    counts[0] = 0
    out.update({f"{prefix}/in_slots": slots.copy(), f"{prefix}/seed": np.array([seed, n_frames], np.uint64)})
    diag = oracle.prod_run(res, K, NR, S, R, tau, lam, tab, slots, counts, seed, 0, n_frames)
    out.update({f"{prefix}/out_slots": slots, f"{prefix}/out_counts": counts, f"{prefix}/out_diag": diag.copy()})
    return out


def main():
    oracle.build()
    data = {}
    data.update(ref_case("c1", configs.c1_plain_2d().sim, 200))
    data.update(ref_case("multi", multi_region_model(reservoir=True, transition=True), 100))
    data.update(ref_case("crowd", crowded_model(), 100))
    data.update(prod_case("prod", multi_region_model(res=(11, 13, 37), K=16, counts=(60, 50, 40, 30)), 30, 1234))
    if REFERENCE_EASY_JSON.exists():
        data.update(ref_case("easy", Simulation.from_json(REFERENCE_EASY_JSON.read_text(), placement_seed=7), 20))
    path = Path(__file__).with_name("golden.npz")
    np.savez_compressed(path, **data)
    print(f"wrote {path} ({path.stat().st_size} bytes, {len(data)} arrays)")


if __name__ == "__main__":
    main()
