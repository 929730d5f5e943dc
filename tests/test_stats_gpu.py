"""Statistical equivalence of the production (Philox, SSA within tau) path
with an FP64 well-mixed exact SSA over >= 1000 replicates: two-sample KS
(p > 0.01) on species counts, z-tests on means and variances, and KS on
first-passage times.  Replicates run as one batched ensemble."""
import math

import numpy as np
import pytest
from scipy import stats

from cell_simulation_gb300 import Ensemble, PREC_FP32, PREC_FP64, PREC_MIXED, configs
from cell_simulation_gb300.simulation import LatticeParams, Simulation

pytestmark = pytest.mark.gpu

N_REP = 1000
P_MIN = 0.01


def template(reactions, species=("A", "B", "C"), K=16, D=1e-12, res=(6, 6, 6)):
    lam = configs.LAMBDA
    sim = Simulation(LatticeParams([r * lam for r in res], list(res), configs.stable_tau(D), lam, K))
    sim.set_diffusion_rate("background", D)
    sim.prepare_regions()
    for n in species:
        sim.add_particle_count(n, "background", 0, True, False)
    sim.set_diffusion_rate("background", D)
    for re, pr, k in reactions:
        sim.add_reaction(re, pr, k)
    return sim


def ssa_tables(sim, n_vox):
    """Well-mixed rates: first order k, second order k_voxel / n_voxels."""
    t = sim.tables()
    i = sim.info()
    S1, R = i.n_species + 1, i.n_reactions
    re = t.reactants.reshape(R + 1, 3)[1:].astype(np.uint8)
    rates = t.rates[1:].astype(np.float64).copy()
    order = (re > 0).sum(1)
    rates[order == 2] /= n_vox
    st = t.stoich.reshape(R + 1, S1)[1:]
    csp = np.zeros((R, 8), np.uint8)
    cd = np.zeros((R, 8), np.int8)
    for r in range(R):
        nz = np.flatnonzero(st[r])
        csp[r, :len(nz)] = nz
        cd[r, :len(nz)] = st[r, nz]
    return re, rates, csp, cd


def run_ensemble(sim, init, n_steps, res=(6, 6, 6), seed0=1000, precision=PREC_MIXED, sample_every=None):
    n = N_REP
    resv = np.tile(np.array(res, np.uint32), (n, 1))
    seeds = (seed0 + np.arange(n)).astype(np.uint64)
    ens = Ensemble(sim, resv, seeds, np.ones(n, np.float32), np.asarray(init, np.uint32))
    ens.set_precision(precision)
    traj = []
    if sample_every:
        for _ in range(n_steps // sample_every):
            ens.step(sample_every)
            traj.append(ens.counts())
    else:
        ens.step(n_steps)
    out = ens.counts()
    ens.close()
    return out, traj


def compare(name, a, b):
    ks = stats.ks_2samp(a, b)
    ma, mb = a.mean(), b.mean()
    se = math.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b)) or 1.0
    z_mean = (ma - mb) / se
    va, vb = a.var(ddof=1), b.var(ddof=1)
    # variance comparison with Levene's test (robust to non-normal counts)
    lev = stats.levene(a, b)
    print(f"{name}: mean {ma:.3f} vs {mb:.3f} (z={z_mean:.2f}), var {va:.3f} vs {vb:.3f} (levene p={lev.pvalue:.3f}), "
          f"KS D={ks.statistic:.4f} p={ks.pvalue:.3f}")
    return ks.pvalue, z_mean, lev.pvalue


def test_first_order_exact():
    """A <-> B: per-voxel SSA within tau is exact for first-order kinetics."""
    sim = template([(["A"], ["B"], 40.0), (["B"], ["A"], 25.0)], species=("A", "B"))
    tau = sim.info().tau
    n_steps = 2000
    counts, _ = run_ensemble(sim, [0, 60, 0], n_steps)
    re, rates, csp, cd = ssa_tables(sim, 216)
    import oracle
    out, _ = oracle.ssa_batch(2, re, rates, csp, cd, [0, 60, 0], 777, N_REP, [n_steps * tau])
    p, z, pv = compare("first-order B", counts[:, 2].astype(float), out[:, 0, 2].astype(float))
    assert p > P_MIN and abs(z) < 4 and pv > P_MIN


@pytest.mark.parametrize("precision", [PREC_MIXED, PREC_FP32, PREC_FP64])
def test_bimolecular_well_mixed(precision):
    """A + B <-> C on a small, fast-mixing lattice against the well-mixed SSA."""
    k_vox = 20.0  # per co-located pair per second: k_vox * tau ~ 3e-3, so geminate rebinding is negligible
    sim = template([(["A", "B"], ["C"], k_vox), (["C"], ["A", "B"], 3.0)])
    tau = sim.info().tau
    n_steps = 3000
    counts, _ = run_ensemble(sim, [0, 40, 30, 0], n_steps, precision=precision)
    re, rates, csp, cd = ssa_tables(sim, 216)
    import oracle
    out, _ = oracle.ssa_batch(3, re, rates, csp, cd, [0, 40, 30, 0], 4242, N_REP, [n_steps * tau])
    p, z, pv = compare(f"bimolecular C (precision {precision})", counts[:, 3].astype(float), out[:, 0, 3].astype(float))
    # conservation A + C and B + C is exact
    assert np.all(counts[:, 1] + counts[:, 3] == 40) and np.all(counts[:, 2] + counts[:, 3] == 30)
    assert p > P_MIN and abs(z) < 4 and pv > P_MIN


def test_first_passage_time():
    """Time until C first reaches 10: lattice (sampled every 10 frames) vs SSA."""
    sim = template([(["A"], ["C"], 30.0)], species=("A", "C"))
    tau = sim.info().tau
    every, n_steps = 10, 3000
    counts, traj = run_ensemble(sim, [0, 20, 0], n_steps, sample_every=every)
    tr = np.stack([t[:, 2] for t in traj], 1)  # [rep][sample]
    hit = (tr >= 10).argmax(1)
    reached = (tr >= 10).any(1)
    fpt_lat = (hit[reached] + 1) * every * tau
    re, rates, csp, cd = ssa_tables(sim, 216)
    import oracle
    grid = (np.arange(1, n_steps // every + 1) * every * tau)
    out, _ = oracle.ssa_batch(2, re, rates, csp, cd, [0, 20, 0], 99, N_REP, grid)
    sr = out[:, :, 2]
    hit2 = (sr >= 10).argmax(1)
    r2 = (sr >= 10).any(1)
    fpt_ssa = (hit2[r2] + 1) * every * tau
    p, z, pv = compare("first passage C>=10", fpt_lat, fpt_ssa)
    assert reached.mean() > 0.95 and r2.mean() > 0.95
    assert p > P_MIN and abs(z) < 4


def test_c5_precision_stress_fp32_vs_fp64():
    """The stiff c5 network (rates 1e-3..1e4 /s, k tau up to 1.7) on 1000
    replicates of 48^3: species counts after 150 frames with FP32 propensities
    and selection, with FP64 selection always, and with the mixed rule (FP64
    selection when a voxel's propensities span more than 6 decades) are one
    distribution.  Two-sample KS per species, Bonferroni over the 12 species."""
    sim = configs.c5_ensemble_template(res=(48, 48, 48))
    init = [0] + [1302] * 12
    n_steps = 150
    runs = {}
    for prec, seed0 in ((PREC_FP32, 50_000), (PREC_FP64, 60_000), (PREC_MIXED, 70_000)):
        n = N_REP
        resv = np.tile(np.array([48, 48, 48], np.uint32), (n, 1))
        seeds = (seed0 + np.arange(n)).astype(np.uint64)
        ens = Ensemble(sim, resv, seeds, np.ones(n, np.float32), np.asarray(init, np.uint32))
        ens.set_precision(prec)
        ens.step(n_steps)
        runs[prec] = (ens.counts(), ens.diagnostics())
        ens.close()
    fp32, fp64, mixed = runs[PREC_FP32][0], runs[PREC_FP64][0], runs[PREC_MIXED][0]
    assert runs[PREC_FP64][1][3] > 0  # FP64 selections counted
    assert runs[PREC_MIXED][1][3] > 0  # the 6-decade rule engages on this network
    worst = 1.0
    for s in range(1, 13):
        p1, _, _ = compare(f"c5 Q{s - 1} fp32 vs fp64", fp32[:, s].astype(float), fp64[:, s].astype(float))
        p2, _, _ = compare(f"c5 Q{s - 1} mixed vs fp64", mixed[:, s].astype(float), fp64[:, s].astype(float))
        worst = min(worst, p1, p2)
    assert worst > P_MIN / 24
