/*
 * ssa_fp64.c — well-mixed exact stochastic simulation (Gillespie direct
 * method) in FP64.  Test infrastructure only: the statistical reference the
 * lattice paths are compared against (species means, variances and
 * first-passage-time distributions).
 *
 * Propensity of reaction r: rates[r] * prod_j (x[s_j] - m_j), where s_j are
 * the non-void reactants and m_j counts earlier equal reactants (falling
 * factorial).  Uniforms come from xoshiro256** (Blackman and Vigna) seeded by
 * SplitMix64; one generator per replicate.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "oracle.h"

typedef struct { uint64_t s[4]; } xoshiro_t;

static uint64_t splitmix64(uint64_t* x) {
    uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static uint64_t xo_next(xoshiro_t* g) {
    uint64_t r = rotl(g->s[1] * 5, 7) * 9, t = g->s[1] << 17;
    g->s[2] ^= g->s[0]; g->s[3] ^= g->s[1]; g->s[1] ^= g->s[2]; g->s[0] ^= g->s[3];
    g->s[2] ^= t; g->s[3] = rotl(g->s[3], 45);
    return r;
}
/* uniform in (0, 1] */
static double xo_unit(xoshiro_t* g) { return (double)((xo_next(g) >> 11) + 1) * 0x1p-53; }

static double propensity(const uint8_t* re, double k, const int64_t* x) {
    double a = k;
    for (int j = 0; j < 3; j++) {
        uint8_t s = re[j];
        if (s == 0) continue;
        int m = 0;
        for (int i = 0; i < j; i++) m += re[i] == s;
        int64_t n = x[s] - m;
        if (n <= 0) return 0.0;
        a *= (double)n;
    }
    return a;
}

static int64_t ssa_one(uint32_t S, uint32_t R, const uint8_t* reactants, const double* rates,
                       const uint8_t* ch_species, const int8_t* ch_delta, const int64_t* x0,
                       uint64_t seed, uint32_t n_samples, const double* t_samples, int64_t* out,
                       int32_t fpt_species, int64_t fpt_threshold, double* fpt) {
    int64_t* x = (int64_t*)malloc(sizeof(int64_t) * (S + 1));
    double* a = (double*)malloc(sizeof(double) * (R ? R : 1));
    memcpy(x, x0, sizeof(int64_t) * (S + 1));
    xoshiro_t g;
    uint64_t sm = seed;
    for (int i = 0; i < 4; i++) g.s[i] = splitmix64(&sm);
    double t = 0.0;
    uint32_t si = 0;
    int64_t events = 0;
    if (fpt) *fpt = INFINITY;
    if (fpt && fpt_species > 0 && x[fpt_species] >= fpt_threshold) *fpt = 0.0;
    double t_end = n_samples ? t_samples[n_samples - 1] : 0.0;
    while (si < n_samples) {
        double a0 = 0.0;
        for (uint32_t r = 0; r < R; r++) { a[r] = propensity(reactants + 3 * r, rates[r], x); a0 += a[r]; }
        double t_next = (a0 > 0.0) ? t + (-log(xo_unit(&g)) / a0) : INFINITY;
        while (si < n_samples && t_samples[si] < t_next) {
            memcpy(out + (size_t)si * (S + 1), x, sizeof(int64_t) * (S + 1));
            si++;
        }
        if (si >= n_samples || !(a0 > 0.0)) break;
        double target = xo_unit(&g) * a0, cum = 0.0;
        uint32_t sel = R;
        for (uint32_t r = 0; r < R; r++) {
            cum += a[r];
            if (target <= cum && a[r] > 0.0) { sel = r; break; }
        }
        if (sel == R) { for (uint32_t r = R; r-- > 0;) if (a[r] > 0.0) { sel = r; break; } }
        for (int j = 0; j < 8; j++) {
            uint8_t s = ch_species[8 * sel + j];
            if (s) x[s] += ch_delta[8 * sel + j];
        }
        events++;
        t = t_next;
        if (fpt && fpt_species > 0 && *fpt == INFINITY && x[fpt_species] >= fpt_threshold && t <= t_end)
            *fpt = t;
    }
    while (si < n_samples) { memcpy(out + (size_t)si * (S + 1), x, sizeof(int64_t) * (S + 1)); si++; }
    free(x);
    free(a);
    return events;
}

int64_t orc_ssa_fp64(uint32_t S, uint32_t R, const uint8_t* reactants, const double* rates,
                     const uint8_t* ch_species, const int8_t* ch_delta, const int64_t* x0,
                     uint64_t seed, uint32_t n_samples, const double* t_samples, int64_t* out) {
    return ssa_one(S, R, reactants, rates, ch_species, ch_delta, x0, seed, n_samples, t_samples,
                   out, 0, 0, NULL);
}

/* n_rep independent replicates (seed = seed0 + rep), samples written to
 * out[rep][n_samples][S+1]; first-passage times of x[fpt_species] >=
 * fpt_threshold into fpt[rep] (INFINITY if not reached by the last sample). */
int64_t orc_ssa_fp64_batch(uint32_t S, uint32_t R, const uint8_t* reactants, const double* rates,
                           const uint8_t* ch_species, const int8_t* ch_delta, const int64_t* x0,
                           uint64_t seed0, uint32_t n_rep, uint32_t n_samples,
                           const double* t_samples, int64_t* out, int32_t fpt_species,
                           int64_t fpt_threshold, double* fpt) {
    int64_t total = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : total)
    for (int64_t rep = 0; rep < (int64_t)n_rep; rep++) {
        total += ssa_one(S, R, reactants, rates, ch_species, ch_delta, x0, seed0 + (uint64_t)rep,
                         n_samples, t_samples, out + (size_t)rep * n_samples * (S + 1),
                         fpt_species, fpt_threshold, fpt ? fpt + rep : NULL);
    }
    return total;
}
