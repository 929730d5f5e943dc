"""Species statistics of the configurations' own reaction networks, 1000 replicates each, run as
batched ensembles of the production path.

  - The 3-species model of the 64x64x1 configuration and of the 512-replicate ensemble (A + B -> C
    at 1e6 /M/s converted to a per-voxel rate, C -> A + B at 0.1 /s, D = 1e-12, 200 A and 200 B),
    in 3-D on 16^3 lattices and in 2-D on the 64x64x1 lattice itself.  Both are well mixed (a
    particle hops about 5,900 times per second, the per-voxel binding rate is 51 /s), so each
    precision mode is compared with the FP64 well-mixed SSA (second-order rate divided by the
    voxel count): C at three times (KS, mean z-test, Levene on variances) and the first passage of
    C to half its stationary mean (KS).
  - The networks of the 128^3 and 256^3 configurations (8 species / 10 reactions and 16 / 30) on
    well-mixed 16^3 replicates: their second-order rates reach 500 /s per voxel, close enough to
    the hopping rate that lattice and well-mixed kinetics differ physically, so the FP32 and mixed
    modes are compared with FP64 selection on the same lattice (KS per species, Bonferroni).
Each case prints its distribution error (KS distance and p, mean z)."""
import math

import numpy as np
import pytest
from scipy import stats

import oracle
from cell_simulation_gb300 import Ensemble, PREC_FP32, PREC_FP64, PREC_MIXED, configs
from tests.helpers import network_template

pytestmark = pytest.mark.gpu

N_REP = 1000
P_MIN = 0.01
PREC_NAME = {PREC_MIXED: "mixed", PREC_FP32: "fp32", PREC_FP64: "fp64"}


def _ssa_tables(sim, n_vox):
    t, i = sim.tables(), sim.info()
    S1, R = i.n_species + 1, i.n_reactions
    re = t.reactants.reshape(R + 1, 3)[1:].astype(np.uint8)
    rates = t.rates[1:].astype(np.float64).copy()
    rates[(re > 0).sum(1) == 2] /= n_vox
    st = t.stoich.reshape(R + 1, S1)[1:]
    csp = np.zeros((R, 8), np.uint8)
    cd = np.zeros((R, 8), np.int8)
    for r in range(R):
        nz = np.flatnonzero(st[r])
        csp[r, :len(nz)] = nz
        cd[r, :len(nz)] = st[r, nz]
    return re, rates, csp, cd


def _ens(tmpl, res, init, seed0, precision):
    resv = np.tile(np.array(res, np.uint32), (N_REP, 1))
    ens = Ensemble(tmpl, resv, (seed0 + np.arange(N_REP)).astype(np.uint64), np.ones(N_REP, np.float32),
                   np.asarray(init, np.uint32))
    ens.set_precision(precision)
    return ens


def _cmp(tag, a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    ks = stats.ks_2samp(a, b)
    se = math.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b)) or 1.0
    z = (a.mean() - b.mean()) / se
    lev = stats.levene(a, b).pvalue if a.var() > 0 and b.var() > 0 else 1.0
    print(f"{tag}: mean {a.mean():.3f} vs {b.mean():.3f} (z={z:+.2f}), var {a.var(ddof=1):.3f} vs "
          f"{b.var(ddof=1):.3f} (Levene p={lev:.3f}), KS D={ks.statistic:.4f} p={ks.pvalue:.3f}")
    return ks.pvalue, z, lev


def _three_species_case(res, precision, seed0):
    tmpl = configs.c4_ensemble_template(K=8)
    tau = float(np.float32(tmpl.info().tau))
    n_vox = int(np.prod(res))
    init = [0, 200, 200, 0]
    every = 5
    # sample frames on the first-passage grid (multiples of `every`)
    frames = [every * int(round(t / tau / every)) for t in (0.25, 1.0, 3.0)]
    times = [round(f * tau, 4) for f in frames]
    # SSA: stationary mean of C, then the sample times and a first-passage grid
    re, rates, csp, cd = _ssa_tables(tmpl, n_vox)
    long, _ = oracle.ssa_batch(3, re, rates, csp, cd, init, 1, 400, [40.0])
    half = int(round(long[:, 0, 3].mean() / 2))
    grid_n = frames[1] // every
    grid = np.arange(1, grid_n + 1) * every * tau
    ssa_grid, _ = oracle.ssa_batch(3, re, rates, csp, cd, init, seed0 + 7, N_REP, grid)
    ssa_t, _ = oracle.ssa_batch(3, re, rates, csp, cd, init, seed0 + 9, N_REP, [f * tau for f in frames])
    # lattice: the first-passage grid, then the remaining frames to the sample times
    ens = _ens(tmpl, res, init, seed0, precision)
    traj = []
    got_t = []
    for k in range(grid_n):
        ens.step(every)
        c = ens.counts()
        traj.append(c[:, 3])
        if (k + 1) * every in frames:
            got_t.append(c)
    done = grid_n * every
    for f in frames[len(got_t):]:
        ens.step(f - done)
        done = f
        got_t.append(ens.counts())
    ens.close()
    tr = np.stack(traj, 1)
    fl = (tr >= half)
    fs = (ssa_grid[:, :, 3] >= half)
    assert fl.any(1).mean() > 0.95 and fs.any(1).mean() > 0.95
    fpt_l = (fl.argmax(1)[fl.any(1)] + 1) * every * tau
    fpt_s = (fs.argmax(1)[fs.any(1)] + 1) * every * tau
    label = f"{'x'.join(map(str, res))} {PREC_NAME[precision]}"
    worst = 1.0
    for j, t in enumerate(times):
        gl = got_t[j]
        assert np.all(gl[:, 1] + gl[:, 3] == 200) and np.all(gl[:, 2] + gl[:, 3] == 200)
        p, z, lev = _cmp(f"{label} C at {t} s vs ssa_fp64", gl[:, 3], ssa_t[:, j, 3])
        worst = min(worst, p, lev)
        assert abs(z) < 4
    p, z, _ = _cmp(f"{label} first passage of C to {half} vs ssa_fp64", fpt_l, fpt_s)
    worst = min(worst, p)
    return worst


@pytest.mark.parametrize("precision", [PREC_MIXED, PREC_FP32, PREC_FP64])
def test_three_species_model_3d_against_ssa(precision):
    """The 512-replicate ensemble's model on 16^3 lattices against the FP64 well-mixed SSA."""
    assert _three_species_case((16, 16, 16), precision, 10_000) > P_MIN / 4


@pytest.mark.parametrize("precision", [PREC_MIXED, PREC_FP32])
def test_three_species_model_2d_against_ssa(precision):
    """The 64x64x1 configuration's own lattice and model against the FP64 well-mixed SSA."""
    assert _three_species_case((64, 64, 1), precision, 20_000) > P_MIN / 4


@pytest.mark.parametrize("cfg", ["c2", "c3"])
def test_config_networks_fp32_and_mixed_against_fp64_selection(cfg):
    """FP32 propensities and selection, and the mixed rule, against FP64 selection on the same
    lattice, for the reaction networks of the 128^3 and 256^3 configurations (16^3 replicates,
    100 particles of each species, 600 frames)."""
    w = configs.c2_single_cell() if cfg == "c2" else configs.c3_multi_region()
    tmpl = network_template(w.sim, res=(16, 16, 16), K=16)
    S = tmpl.info().n_species
    init = [0] + [100] * S
    runs = {}
    for prec, seed0 in ((PREC_FP64, 30_000), (PREC_FP32, 40_000), (PREC_MIXED, 50_000)):
        ens = _ens(tmpl, (16, 16, 16), init, seed0, prec)
        ens.step(600)
        runs[prec] = ens.counts()
        ens.close()
    worst, dmax = 1.0, 0.0
    for prec in (PREC_FP32, PREC_MIXED):
        for s in range(1, S + 1):
            a, b = runs[prec][:, s], runs[PREC_FP64][:, s]
            if a.var() == 0 and b.var() == 0 and a.mean() == b.mean():
                continue
            p, _, _ = _cmp(f"{cfg} species {s} {PREC_NAME[prec]} vs fp64 selection", a, b)
            worst = min(worst, p)
            dmax = max(dmax, stats.ks_2samp(a, b).statistic)
    print(f"{cfg}: worst KS p {worst:.4f}, largest KS distance {dmax:.4f}")
    assert worst > P_MIN / (2 * S)
