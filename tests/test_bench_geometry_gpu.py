"""Parity at the geometries the benchmark runs: the production step on the full 256^3 multi-region
cell (Z = 256: eight full bitmap words per row, four rows per word group, no partial word) and on
the 128^3 single cell, the 512-replicate ensemble's edge range (edges 32, 33, 63, 64, 95 and 96:
full words, a partial word, multi-word rows), and the reference-RNG path on both cells.  Each run
is compared bit for bit with the oracle (integer state: the tolerance is zero)."""
import numpy as np
import pytest

from cell_simulation_gb300 import (Ensemble, RNG_PHILOX, RNG_REFERENCE, configs, tiling_kinds, tiling_launches,
                                   tiling_variants)
from tests.helpers import compact_slots, itime_schedule, oracle_args, ref_state

pytestmark = pytest.mark.gpu


def _variants(K):
    """The default step (Y and Z sweeps fused, three blocks per SM), the fused step at four blocks
    per SM, the three-launch sweep stream (Y and Z sweeps apart), the persistent multi-frame stream
    (groups heaviest first, and in plane order) and the 16-plane brick pass of slot count K."""
    kinds, launches, var = tiling_kinds(), tiling_launches(), tiling_variants()
    stream = [i for i, (t, k) in enumerate(zip(var, kinds)) if t[0] == K and k[0] == 2]
    fused = [i for i in stream if launches[i] == 2]
    apart = [i for i in stream if launches[i] == 3]
    frames = [i for i in stream if launches[i] == 1]
    brick = [i for i, (t, k) in enumerate(zip(var, kinds)) if t[0] == K and k == (1, 16)]
    return {"fused3": fused[0], "fused4": fused[-1], "unfused": apart[-1], "frames": frames[0], "frames_plane": frames[-1],
            "brick16": brick[-1]}


def _oracle_frames(orc, sim, n, seed):
    res, K, NR, S, R, tau, lam, tab = oracle_args(sim)
    s = sim.get_lattice()[0]
    slots = compact_slots(s, K)
    counts = np.bincount(slots, minlength=S + 1).astype(np.int64)
    counts[0] = 0
    for q in tab.reservoir[tab.reservoir > 0]:
        counts[q] += 1
    diag = orc.prod_run(res, K, NR, S, R, tau, lam, tab, slots, counts, seed, 0, n)
    return slots, counts, diag


def _gpu_frames(sim, n, seed, tiling, chunks=2):
    sim.prepare_for_gpu(RNG_PHILOX, 0)
    sim.set_tiling(tiling)
    for part in np.array_split(np.arange(n), chunks):
        sim.step_philox(len(part), seed)
    out = sim.get_lattice()[0].astype(np.uint8), sim.counts(), sim.diagnostics()
    sim.close()
    return out


def _check(got, want, tag):
    gs, gc, gd = got
    ws, wc, wd = want
    bad = np.flatnonzero(gs != ws)
    assert bad.size == 0, (tag, bad.size, bad[:8])
    assert np.array_equal(gc, wc), tag
    assert np.array_equal(gd[:4], wd[:4]), (tag, gd, wd)
    assert gd[7] == 0, (tag, gd)  # no dependency wait of the multi-frame kernel timed out


def test_c3_256_cube_matches_oracle(orc):
    """The benchmark's 256^3, 16-slot, 16-species cell: four frames in two step calls."""
    want = _oracle_frames(orc, configs.c3_multi_region().sim, 4, seed=0xC0FFEE)
    assert want[2][0] > 0  # reactions fired
    for tag, ti in _variants(16).items():
        _check(_gpu_frames(configs.c3_multi_region().sim, 4, 0xC0FFEE, ti), want, tag)


def test_c5_192_cube_matches_oracle(orc):
    """The stiff 192^3 lattice (Z = 192: six words per row, five rows per group of 30 words; 12
    species, 24 reactions up to k tau = 1.7): four frames in two step calls."""
    want = _oracle_frames(orc, configs.c5_stiff().sim, 4, seed=4242)
    assert want[2][0] > 0
    for tag, ti in _variants(16).items():
        _check(_gpu_frames(configs.c5_stiff().sim, 4, 4242, ti), want, tag)


def test_c2_128_cube_matches_oracle(orc):
    """The 128^3 single cell (Z = 128: four words per row, eight rows per group): six frames."""
    want = _oracle_frames(orc, configs.c2_single_cell().sim, 6, seed=2024)
    for tag, ti in _variants(16).items():
        _check(_gpu_frames(configs.c2_single_cell().sim, 6, 2024, ti, chunks=3), want, tag)


@pytest.mark.parametrize("variant", ["fused3", "fused4", "unfused", "frames", "frames_plane"])
def test_c4_edge_range_matches_oracle(orc, variant):
    """Replicates with the ensemble's extreme and word-boundary edges (32, 33, 63, 64, 95, 96) and
    the ensemble's particle counts, rate multipliers and seeds, batched in one launch per pass."""
    tmpl = configs.c4_ensemble_template(K=8)
    _, seeds_all, mult_all, init = configs.c4_ensemble_spec()
    edges = [32, 33, 63, 64, 95, 96]
    res = np.array([[e, e, e] for e in edges], np.uint32)
    seeds, mult = seeds_all[:len(edges)].copy(), mult_all[:len(edges)].copy()
    ens = Ensemble(tmpl, res, seeds, mult, init)
    ens.set_tiling(_variants(8)[variant])
    s0 = ens.slots()
    n = 20
    ens.step(n, batched=True)
    got, counts = ens.slots(), ens.counts()
    ens.close()
    tab, info = tmpl.tables(), tmpl.info()
    off = 0
    fired = 0
    for r, e in enumerate(edges):
        V = e ** 3
        sl = s0[off * 8:(off + V) * 8].copy()
        c0 = np.bincount(sl, minlength=4).astype(np.int64)
        c0[0] = 0
        t = type(tab)(np.zeros(V, np.uint32), tab.diffusion, tab.stoich, tab.reactants, tab.rates,
                      np.zeros(V, np.uint32))
        d = orc.prod_run((e, e, e), 8, info.n_regions, info.n_species, info.n_reactions, float(np.float32(info.tau)),
                         float(np.float32(info.lambda_)), t, sl, c0, int(seeds[r]), 0, n, rate_mult=float(mult[r]))
        fired += int(d[0])
        assert np.array_equal(got[off * 8:(off + V) * 8], sl), (variant, e)
        assert np.array_equal(counts[r], c0), (variant, e)
        off += V
    assert fired > 0


@pytest.mark.parametrize("cell", ["c2", "c3"])
def test_reference_rng_path_on_benchmark_cells(orc, cell):
    """The bit-parity path on the 128^3 single cell (eight frames) and on the 256^3 cell (three
    frames, the shape of its benchmark leg) against the reference-semantics restatement."""
    mk = configs.c2_single_cell if cell == "c2" else configs.c3_multi_region
    n = 8 if cell == "c2" else 3
    sim = mk().sim
    args = oracle_args(sim)
    s, o, c, st = ref_state(sim)
    it = itime_schedule(n, seed=12345)
    ref = orc.ref_run(*args, orc.RefState(s, o, c, st), it, mode=1, threads=0)
    sim.prepare_for_gpu(RNG_REFERENCE, 0)
    sim.step(it[:1])
    sim.step(it[1:])
    gs, go, gc = sim.get_lattice()
    assert np.array_equal(gs, ref.slots), np.flatnonzero(gs != ref.slots)[:8]
    assert np.array_equal(go, ref.occ)
    assert np.array_equal(gc, ref.conc)
    assert np.array_equal(sim.counts(), ref.stat.astype(np.int64))
    diag = sim.diagnostics()
    for k in (0, 1, 2, 3, 4):
        assert diag[k] == ref.diag[k], (k, diag, ref.diag)
    sim.close()
