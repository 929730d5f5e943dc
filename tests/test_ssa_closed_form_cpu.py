"""The FP64 well-mixed SSA oracle against closed-form results: every statistical verdict on the
lattice paths rests on it, so it is pinned here on its own.

  - A <-> B (first order): the stationary count of A is Binomial(N, k2 / (k1 + k2));
  - A -> B (decay of A): at time t the count of A is Binomial(N, exp(-k t)), and with one A the
    first passage of B to 1 is exponential with rate k;
  - A + B <-> C: the stationary count of C follows the detailed-balance distribution
    pi(n + 1) / pi(n) = kf (A0 - n) (B0 - n) / (kb (n + 1)).

Each test draws a few thousand replicates and compares means (z-test), variances (z-test on the
sample variance, with its sampling variance from the fourth central moment of the exact
distribution) and the whole distribution (chi-square on the histogram, or KS for continuous
times) at a significance level of 1e-3 per check."""
import math

import numpy as np
from scipy import stats

N_REP = 4000
ALPHA = 1e-3


def _tables(reactions, S):
    """(reactants, species, deltas) in the oracle's layout from [(reactants, products, k)]."""
    R = len(reactions)
    re = np.zeros((R, 3), np.uint8)
    rates = np.zeros(R, np.float64)
    csp = np.zeros((R, 8), np.uint8)
    cd = np.zeros((R, 8), np.int8)
    for r, (rs, ps, k) in enumerate(reactions):
        re[r, :len(rs)] = rs
        rates[r] = k
        d = np.zeros(S + 1, np.int64)
        for s in rs:
            d[s] -= 1
        for s in ps:
            d[s] += 1
        nz = np.flatnonzero(d)
        csp[r, :len(nz)] = nz
        cd[r, :len(nz)] = d[nz]
    return re, rates, csp, cd


def _check_discrete(sample, support, pmf, tag):
    pmf = np.asarray(pmf, np.float64)
    pmf = pmf / pmf.sum()
    mean = float((support * pmf).sum())
    var = float(((support - mean) ** 2 * pmf).sum())
    m4 = float(((support - mean) ** 4 * pmf).sum())
    n = len(sample)
    z_mean = (sample.mean() - mean) / math.sqrt(var / n)
    # sampling variance of the unbiased variance estimator: (m4 - (n-3)/(n-1) var^2) / n
    z_var = (sample.var(ddof=1) - var) / math.sqrt((m4 - (n - 3) / (n - 1) * var * var) / n)
    # chi-square over bins of expected count >= 5 (tails merged)
    counts = np.array([(sample == k).sum() for k in support], np.float64)
    exp = pmf * n
    keep = exp >= 5
    obs_b = list(counts[keep])
    exp_b = list(exp[keep])
    obs_b.append(counts[~keep].sum())
    exp_b.append(exp[~keep].sum())
    if exp_b[-1] < 5:
        obs_b[-2] += obs_b.pop()
        exp_b[-2] += exp_b.pop()
    chi = stats.chisquare(obs_b, exp_b)
    print(f"{tag}: mean {sample.mean():.4f} vs {mean:.4f} (z={z_mean:.2f}), var {sample.var(ddof=1):.4f} vs "
          f"{var:.4f} (z={z_var:.2f}), chi-square p={chi.pvalue:.3f}")
    zc = stats.norm.isf(ALPHA / 2)
    assert abs(z_mean) < zc, (tag, z_mean)
    assert abs(z_var) < zc, (tag, z_var)
    assert chi.pvalue > ALPHA, (tag, chi.pvalue)


def test_isomerisation_stationary_binomial(orc):
    k1, k2, N = 3.0, 2.0, 40
    re, rates, csp, cd = _tables([([1], [2], k1), ([2], [1], k2)], 2)
    x0 = np.array([0, N, 0], np.int64)
    out, _ = orc.ssa_batch(2, re, rates, csp, cd, x0, 1234, N_REP, np.array([8.0]))
    a = out[:, 0, 1]
    assert np.all(out[:, 0, 1] + out[:, 0, 2] == N)
    k = np.arange(N + 1)
    _check_discrete(a, k, stats.binom.pmf(k, N, k2 / (k1 + k2)), "A<->B stationary")


def test_decay_binomial_and_exponential_first_passage(orc):
    k, N, t = 0.7, 60, 1.3
    re, rates, csp, cd = _tables([([1], [2], k)], 2)
    out, _ = orc.ssa_batch(2, re, rates, csp, cd, np.array([0, N, 0], np.int64), 99, N_REP, np.array([t]))
    n = np.arange(N + 1)
    _check_discrete(out[:, 0, 1], n, stats.binom.pmf(n, N, math.exp(-k * t)), "A decay")
    # one A: the first time B reaches 1 is Exp(k); samples run long enough that nearly all arrive
    t_end = 40.0 / k
    _, fpt = orc.ssa_batch(2, re, rates, csp, cd, np.array([0, 1, 0], np.int64), 4321, N_REP, np.array([t_end]),
                           fpt_species=2, fpt_threshold=1)
    assert np.isfinite(fpt).all()
    ks = stats.kstest(fpt, stats.expon(scale=1.0 / k).cdf)
    print(f"first passage: mean {fpt.mean():.4f} vs {1 / k:.4f}, KS p={ks.pvalue:.3f}")
    assert ks.pvalue > ALPHA
    assert abs(fpt.mean() - 1 / k) / ((1 / k) / math.sqrt(N_REP)) < stats.norm.isf(ALPHA / 2)


def test_bimolecular_stationary_distribution(orc):
    kf, kb, A0, B0 = 0.05, 1.5, 30, 20
    re, rates, csp, cd = _tables([([1, 2], [3], kf), ([3], [1, 2], kb)], 3)
    out, _ = orc.ssa_batch(3, re, rates, csp, cd, np.array([0, A0, B0, 0], np.int64), 777, N_REP,
                           np.array([25.0]))
    c = out[:, 0, 3]
    assert np.all(out[:, 0, 1] + c == A0) and np.all(out[:, 0, 2] + c == B0)
    n = np.arange(min(A0, B0) + 1)
    logp = np.zeros(len(n))
    for i in range(1, len(n)):
        logp[i] = logp[i - 1] + math.log(kf * (A0 - (i - 1)) * (B0 - (i - 1)) / (kb * i))
    _check_discrete(c, n, np.exp(logp - logp.max()), "A+B<->C stationary")


def test_homodimer_uses_falling_factorial(orc):
    """A + A -> B fires with propensity k n (n - 1): from two A the waiting time is Exp(2k)."""
    k = 0.8
    re, rates, csp, cd = _tables([([1, 1], [2], k)], 2)
    _, fpt = orc.ssa_batch(2, re, rates, csp, cd, np.array([0, 2, 0], np.int64), 55, N_REP, np.array([60.0]),
                           fpt_species=2, fpt_threshold=1)
    ks = stats.kstest(fpt, stats.expon(scale=1.0 / (2 * k)).cdf)
    assert ks.pvalue > ALPHA, ks
