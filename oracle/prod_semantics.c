/*
 * prod_semantics.c — plain CPU restatement of the production (Philox) step
 * of libcellsim (test infrastructure only).  It sweeps the whole lattice one
 * axis at a time with no tiling, so agreement with the fused tile kernel
 * checks the kernel's halo, ring-buffer and work-queue logic bit for bit.
 *
 * Algorithm (the kernel's contract):
 *  - region code c(v) = region + 1, 0 outside the lattice; move threshold
 *    T[a][b][q] = floor(min(D[a-1][b-1][q] * tau / lambda^2, 1) * 2^32) in
 *    FP64 (the probabilities of res/shader/rdme.wgsl:132-136), 0 if a or b
 *    is 0;
 *  - random words: B(v, s) = Philox4x32-10(ctr = {v, frame, s, 0}, key = seed)
 *    for slot s < K, E(v, e) = Philox4x32-10(ctr = {v, frame, 0x80000000 | e, 0});
 *  - sweep a in (x, y, z) = (0, 1, 2): the particle at slot s of voxel v draws
 *    u = B(v, s)[a]; it moves down if u < T[c(v)][c(v-a)][q], up if
 *    u < that + T[c(v)][c(v+a)][q];
 *  - room K - n(w) of a receiving voxel is split: lower neighbour gets
 *    (room + ((w + frame + a) & 1)) / 2, upper neighbour the rest; the first
 *    movers in slot order up to the share are accepted;
 *  - new content: own stayers (slot order), accepted arrivals from below,
 *    then from above;
 *  - reactions: SSA inside the voxel for one tau (see react below); event e
 *    draws its waiting-time word from B(v, 0)[3] when e = 0 and from
 *    E(v, e)[0] otherwise, and its selection word from E(v, e)[1].
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "oracle.h"

typedef struct {
    uint32_t X, Y, Z, K, S1, R, NC;
    uint64_t V;
    uint32_t* thr;
    uint8_t* code;
    uint8_t (*rre)[3];
    float* rate;
    uint8_t (*csp)[8];
    int8_t (*cd)[8];
} pctx;

static uint32_t thr_of(double D, double tau, double lambda) {
    double p = D * tau / (lambda * lambda);
    if (!(p > 0.0)) return 0u;
    if (p >= 1.0) return 0xFFFFFFFFu;
    double t = floor(p * 4294967296.0);
    return t >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)t;
}

static uint32_t nbytes(const uint8_t* c, uint32_t K) {
    uint32_t n = 0;
    for (uint32_t s = 0; s < K; s++) n += c[s] != 0;
    return n;
}

static uint32_t popc(uint32_t m) { uint32_t n = 0; while (m) { m &= m - 1; n++; } return n; }

static uint32_t lowest_bits(uint32_t m, uint32_t c) {
    while (popc(m) > c) {
        uint32_t hb = 31;
        while (!(m >> hb & 1u)) hb--;
        m &= ~(1u << hb);
    }
    return m;
}

static uint32_t decide(const pctx* c, const uint8_t* cont, uint32_t v, uint32_t frame, uint32_t sweep, uint32_t rs,
                       uint32_t rlo, uint32_t rhi, const uint32_t key[2]) {
    uint32_t n = nbytes(cont, c->K), mask = 0, ph[4];
    for (uint32_t s = 0; s < n; s++) {
        uint32_t q = cont[s];
        uint32_t tm = c->thr[((size_t)rs * c->NC + rlo) * c->S1 + q];
        uint32_t tp = c->thr[((size_t)rs * c->NC + rhi) * c->S1 + q];
        if ((tm | tp) == 0u) continue;
        uint32_t ctr[4] = {v, frame, s, 0u};
        orc_philox4x32_10(ctr, key, ph);
        uint32_t u = ph[sweep];
        if (u < tm) mask |= 1u << s;
        else if ((uint64_t)u < (uint64_t)tm + tp) mask |= 1u << (16 + s);
    }
    return mask;
}

static void combine(const pctx* c, const uint8_t* own, uint32_t down, const uint8_t* lo, uint32_t dlo,
                    const uint8_t* hi, uint32_t dhi, uint32_t v, uint32_t vlo, uint32_t vhi, uint32_t frame,
                    uint32_t sweep, uint8_t* out) {
    uint32_t K = c->K;
    memset(out, 0, K);
    uint32_t in_lo = dlo >> 16, in_hi = dhi & 0xFFFFu;
    if ((down | in_lo | in_hi) == 0u) { memcpy(out, own, K); return; }
    uint32_t n_self = nbytes(own, K), room = K - n_self;
    uint32_t sl = (room + ((v + frame + sweep) & 1u)) >> 1, sh = room - sl;
    uint32_t acc_lo = lowest_bits(in_lo, sl), acc_hi = lowest_bits(in_hi, sh);
    uint32_t out_m = down & 0xFFFFu, out_p = down >> 16;
    if (out_m) {
        uint32_t rl = K - nbytes(lo, K);
        out_m = lowest_bits(out_m, rl - ((rl + ((vlo + frame + sweep) & 1u)) >> 1));
    }
    if (out_p) {
        uint32_t rh = K - nbytes(hi, K);
        out_p = lowest_bits(out_p, (rh + ((vhi + frame + sweep) & 1u)) >> 1);
    }
    uint32_t keep = ((1u << n_self) - 1u) & ~(out_m | out_p), j = 0;
    for (uint32_t s = 0; s < 16; s++) if (keep >> s & 1u) out[j++] = own[s];
    for (uint32_t s = 0; s < 16; s++) if (acc_lo >> s & 1u) out[j++] = lo[s];
    for (uint32_t s = 0; s < 16; s++) if (acc_hi >> s & 1u) out[j++] = hi[s];
}

static float prop(const pctx* c, uint32_t r, const int32_t* cnt, float mult) {
    uint32_t ff = 1;
    for (int j = 0; j < 3; j++) {
        uint32_t s = c->rre[r][j];
        if (!s) continue;
        uint32_t m = 0;
        for (int i = 0; i < j; i++) m += c->rre[r][i] == s;
        uint32_t have = (uint32_t)cnt[s];
        if (have <= m) return 0.0f;
        ff *= have - m;
    }
    float k = c->rate[r] * mult;
    return k * (float)ff;
}

/* SSA within tau; counts c[] of the voxel (reservoir species forced to 1). */
static void react(const pctx* c, const orc_prod_params* p, uint8_t* cont, uint32_t resv, uint32_t v, uint32_t frame,
                  const uint32_t key[2], int64_t* counts, uint32_t* diag) {
    uint32_t K = c->K, S1 = c->S1;
    int32_t* cnt = (int32_t*)calloc(S1, sizeof(int32_t));
    uint32_t n = 0;
    for (uint32_t s = 0; s < K; s++) if (cont[s]) { cnt[cont[s]]++; n++; }
    if (resv) cnt[resv] = 1;
    double td = 0.0;
    float tf = 0.0f;
    int fired = 0;
    uint32_t ev = 0;
    for (; ev < p->max_events; ev++) {
        float a0 = 0.0f, amax = 0.0f, amin = INFINITY;
        for (uint32_t r = 0; r < c->R; r++) {
            float a = prop(c, r, cnt, p->rate_mult);
            a0 = a0 + a;
            if (a > 0.0f) { amax = fmaxf(amax, a); amin = fminf(amin, a); }
        }
        if (!(a0 > 0.0f)) break;
        uint32_t ctr[4] = {v, frame, 0x80000000u | ev, 0u}, ph[4], w1;
        orc_philox4x32_10(ctr, key, ph);
        if (ev == 0) {
            uint32_t c0[4] = {v, frame, 0u, 0u}, b0[4];
            orc_philox4x32_10(c0, key, b0);
            w1 = b0[3];
        } else {
            w1 = ph[0];
        }
        uint32_t w2 = ph[1];
        float u1 = (float)((w1 >> 8) + 1u) * 0x1p-24f;
        float dt = -orc_logf(u1) / a0;
        if (p->precision == 1) {
            tf = tf + dt;
            if (tf > p->tau) break;
        } else {
            td = td + (double)dt;
            if (td > (double)p->tau) break;
        }
        float u2 = (float)(w2 >> 8) * 0x1p-24f;
        int use64 = (p->precision == 2) || (p->precision == 0 && amax > 1e6f * amin);
        int sel = -1, last_pos = -1;
        if (!use64) {
            float target = u2 * a0, run = 0.0f;
            for (uint32_t r = 0; r < c->R; r++) {
                float a = prop(c, r, cnt, p->rate_mult);
                if (a > 0.0f) last_pos = (int)r;
                run = run + a;
                if (target < run) { sel = (int)r; break; }
            }
        } else {
            diag[ORC_PD_FP64_SEL]++;
            double a0d = 0.0;
            for (uint32_t r = 0; r < c->R; r++) a0d = a0d + (double)prop(c, r, cnt, p->rate_mult);
            double target = (double)u2 * a0d, run = 0.0;
            for (uint32_t r = 0; r < c->R; r++) {
                float a = prop(c, r, cnt, p->rate_mult);
                if (a > 0.0f) last_pos = (int)r;
                run = run + (double)a;
                if (target < run) { sel = (int)r; break; }
            }
        }
        if (sel < 0) sel = last_pos;
        if (sel < 0) break;
        int total = (int)n, ok = 1;
        for (int j = 0; j < 8; j++) {
            uint32_t s = c->csp[sel][j];
            if (!s) break;
            if (s == resv) continue;
            int d = c->cd[sel][j];
            if (cnt[s] + d < 0) ok = 0;
            total += d;
        }
        if (!ok || total > (int)K) { diag[ORC_PD_REJECT_CAP]++; continue; }
        for (int j = 0; j < 8; j++) {
            uint32_t s = c->csp[sel][j];
            if (!s) break;
            if (s == resv) continue;
            int d = c->cd[sel][j];
            cnt[s] += d;
            counts[s] += d;
        }
        n = (uint32_t)total;
        diag[ORC_PD_EVENTS]++;
        fired = 1;
    }
    if (ev == p->max_events) diag[ORC_PD_EVENT_CAP]++;
    if (fired) {
        uint32_t j = 0;
        memset(cont, 0, K);
        for (uint32_t s = 1; s < S1; s++) {
            if (s == resv) continue;
            for (int32_t k = 0; k < cnt[s]; k++) cont[j++] = (uint8_t)s;
        }
    }
    free(cnt);
}

int orc_prod_run(const orc_prod_params* p, const orc_tables* t, uint8_t* slots, int64_t* counts, uint32_t frame0,
                 uint32_t n_steps, uint32_t* diag) {
    pctx c;
    c.X = p->res[0]; c.Y = p->res[1]; c.Z = p->res[2];
    c.K = p->K; c.S1 = p->n_species + 1; c.R = p->n_reactions; c.NC = p->n_regions + 1;
    c.V = (uint64_t)c.X * c.Y * c.Z;
    if (c.K != 8 && c.K != 16) return -1;
    c.thr = (uint32_t*)calloc((size_t)c.NC * c.NC * c.S1, sizeof(uint32_t));
    c.code = (uint8_t*)malloc(c.V);
    c.rre = malloc(sizeof(*c.rre) * (c.R ? c.R : 1));
    c.rate = (float*)malloc(sizeof(float) * (c.R ? c.R : 1));
    c.csp = calloc(c.R ? c.R : 1, sizeof(*c.csp));
    c.cd = calloc(c.R ? c.R : 1, sizeof(*c.cd));
    for (uint32_t a = 1; a < c.NC; a++)
        for (uint32_t b = 1; b < c.NC; b++)
            for (uint32_t q = 0; q < c.S1; q++)
                c.thr[((size_t)a * c.NC + b) * c.S1 + q] =
                    thr_of((double)t->diffusion[((size_t)(a - 1) * p->n_regions + (b - 1)) * c.S1 + q], (double)p->tau,
                           (double)p->lambda);
    for (uint64_t v = 0; v < c.V; v++) c.code[v] = (uint8_t)(t->regions[v] + 1);
    for (uint32_t r = 0; r < c.R; r++) {
        for (int j = 0; j < 3; j++) c.rre[r][j] = (uint8_t)t->reactants[(r + 1) * 3 + j];
        c.rate[r] = t->rates[r + 1];
        int n = 0;
        for (uint32_t s = 1; s < c.S1; s++) {
            int32_t d = t->stoich[(size_t)(r + 1) * c.S1 + s];
            if (d && n < 8) { c.csp[r][n] = (uint8_t)s; c.cd[r][n] = (int8_t)d; n++; }
        }
    }
    uint32_t key[2] = {(uint32_t)p->seed, (uint32_t)(p->seed >> 32)};
    uint32_t K = c.K;
    uint8_t* nxt = (uint8_t*)malloc(c.V * K);
    uint32_t* dec = (uint32_t*)malloc(sizeof(uint32_t) * c.V);
    uint8_t zero[16] = {0};
    for (uint32_t st = 0; st < n_steps; st++) {
        uint32_t frame = frame0 + st;
        for (uint32_t sweep = 0; sweep < 3; sweep++) {
            uint64_t stride = sweep == 0 ? (uint64_t)c.Y * c.Z : sweep == 1 ? c.Z : 1;
            uint32_t dim = sweep == 0 ? c.X : sweep == 1 ? c.Y : c.Z;
            for (uint64_t v = 0; v < c.V; v++) {
                uint32_t coord = (uint32_t)((v / stride) % dim);
                uint32_t rlo = coord > 0 ? c.code[v - stride] : 0u;
                uint32_t rhi = coord + 1 < dim ? c.code[v + stride] : 0u;
                dec[v] = decide(&c, slots + v * K, (uint32_t)v, frame, sweep, c.code[v], rlo, rhi, key);
            }
            for (uint64_t v = 0; v < c.V; v++) {
                uint32_t coord = (uint32_t)((v / stride) % dim);
                const uint8_t* lo = coord > 0 ? slots + (v - stride) * K : zero;
                const uint8_t* hi = coord + 1 < dim ? slots + (v + stride) * K : zero;
                uint32_t dlo = coord > 0 ? dec[v - stride] : 0u;
                uint32_t dhi = coord + 1 < dim ? dec[v + stride] : 0u;
                combine(&c, slots + v * K, dec[v], lo, dlo, hi, dhi, (uint32_t)v, (uint32_t)(v - stride),
                        (uint32_t)(v + stride), frame, sweep, nxt + v * K);
            }
            memcpy(slots, nxt, c.V * K);
        }
        for (uint64_t v = 0; v < c.V; v++) {
            uint32_t resv = t->reservoir ? t->reservoir[v] : 0u;
            react(&c, p, slots + v * K, resv, (uint32_t)v, frame, key, counts, diag);
        }
    }
    free(nxt); free(dec); free(c.thr); free(c.code); free(c.rre); free(c.rate); free(c.csp); free(c.cd);
    return 0;
}

/* Number of draws m in [lo, hi] (u1 = m * 2^-24) whose first reaction event
 * falls inside tau, dt = -logf(u1) / a0 <= tau, for a voxel with total
 * propensity a0.  The production step skips the exact SSA for draws below a
 * tabulated threshold; this counts the draws that would contradict it. */
uint32_t orc_first_event_inside(float a0, float tau, uint32_t lo, uint32_t hi) {
    uint32_t n = 0;
    for (uint64_t m = lo; m <= hi; m++) {
        float u1 = (float)(uint32_t)m * 0x1p-24f;
        float dt = -orc_logf(u1) / a0;
        if (!((double)dt > (double)tau)) n++;
    }
    return n;
}
