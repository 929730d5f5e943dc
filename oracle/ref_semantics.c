/*
 * ref_semantics.c — CPU restatement of the reference RDME timestep
 * (test infrastructure only; see oracle.h for the parity status).
 *
 * One timestep = diffusion (res/shader/rdme.wgsl:194-230) -> reactions
 * (res/shader/cme.wgsl:26-120) -> stable slot compaction
 * (res/shader/final_stage.wgsl:25-33) -> destination becomes source
 * (src/simulation.rs:99-150).
 *
 * The reference runs one GPU invocation per voxel with spin locks and
 * atomics, so its slot placement is nondeterministic.  This file defines the
 * canonical serial order: voxels in linear index order (x-major, z fastest,
 * functions.wgsl:42-51), slots in index order.  Deterministic quirks of the
 * shaders are reproduced:
 *   - the diffusion seed itime + X % Y + Z + i_part uses the voxel coordinates
 *     and the global slot index (rdme.wgsl:220); X % 0 is taken as 0, the
 *     WGSL-specified result of integer remainder by zero;
 *   - a uniform of exactly 0 selects direction 0 even when its probability is
 *     0 (rdme.wgsl:223-226);
 *   - propensities are k * f32(c0*c1*c2) with no n(n-1) correction, and
 *     conc[v][0] is forced to 1 (cme.wgsl:31,42-44);
 *   - only cumulative entries 0..R-1 are normalised (cme.wgsl:50-52);
 *   - the second uniform is UniformFloat(state + 1) (cme.wgsl:68);
 *   - the reservoir test reads reservoirs[v*K], the slot index, not the voxel
 *     index (cme.wgsl:80); reads past the end of the array return 0;
 *   - the rewrite rolls back as soon as j reaches K, even exactly
 *     (cme.wgsl:95), and the rollback loop also reverts skipped species.
 * Canonical choices where the reference is nondeterministic or out of bounds:
 *   - a move into a voxel whose occupancy is already >= K, or that has no
 *     zero slot among its K slots, is rejected and counted in
 *     ORC_DIAG_SPILL (the shader's `old <= K` test at rdme.wgsl:62 and its
 *     CAS loop over K+1 slots at rdme.wgsl:30-40 would write into the next
 *     voxel's slot 0);
 *   - the diffusion scan visits min(occupancy, K) slots (ORC_DIAG_OCC_RANGE
 *     counts voxels whose occupancy exceeded K);
 *   - reaction invocations past res.x for odd res.x (cme.wgsl:25 dispatches
 *     ceil(X/2) workgroups of 2 with no bounds guard) do nothing.
 * Floating point: every operation is a single binary32 operation rounded to
 * nearest (no contraction); division is IEEE division; exp is orc_expf.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "oracle.h"
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
    uint32_t X, Y, Z, K, S1, NR, R;
    uint64_t V;
    float* P;  /* [NR][NR][S1] move probability, rdme.wgsl:132-136 */
} ctx_t;

static int ctx_init(ctx_t* c, const orc_params* p, const orc_tables* t) {
    c->X = p->res[0]; c->Y = p->res[1]; c->Z = p->res[2];
    c->K = p->K; c->S1 = p->n_species + 1; c->NR = p->n_regions; c->R = p->n_reactions;
    c->V = (uint64_t)c->X * c->Y * c->Z;
    if (c->K < 1 || c->K > 16 || c->R > 99 || c->NR < 1) return -1;
    c->P = (float*)malloc(sizeof(float) * (size_t)c->NR * c->NR * c->S1);
    if (!c->P) return -2;
    float l2 = p->lambda * p->lambda;
    for (uint32_t a = 0; a < c->NR; a++)
        for (uint32_t b = 0; b < c->NR; b++)
            for (uint32_t q = 0; q < c->S1; q++) {
                float val = t->diffusion[q + c->S1 * b + c->S1 * c->NR * a];
                float num = val * p->tau;
                c->P[((size_t)a * c->NR + b) * c->S1 + q] = num / l2;
            }
    return 0;
}

static inline float prob(const ctx_t* c, uint32_t a, uint32_t b, uint32_t q) {
    return c->P[((size_t)a * c->NR + b) * c->S1 + q];
}

/* Direction chosen by the particle at global slot index i_part of voxel v,
 * rdme.wgsl:138-191,212-226.  Returns 0..5 for a move that stays inside the
 * lattice, 6 otherwise. */
static int decide_direction(const ctx_t* c, const orc_tables* t, uint64_t v, uint32_t x,
                            uint32_t y, uint32_t z, uint32_t q, uint32_t i_part,
                            uint32_t itime) {
    const uint32_t* reg = t->regions;
    uint64_t YZ = (uint64_t)c->Y * c->Z;
    uint32_t sr = reg[v];
    float pv[7];
    pv[0] = (x > 0u) ? prob(c, sr, reg[v - YZ], q) : 0.0f;
    pv[1] = (x < c->X - 1u) ? pv[0] + prob(c, sr, reg[v + YZ], q) : pv[0];
    pv[2] = (y > 0u) ? pv[1] + prob(c, sr, reg[v - c->Z], q) : pv[1];
    pv[3] = (y < c->Y - 1u) ? pv[2] + prob(c, sr, reg[v + c->Z], q) : pv[2];
    pv[4] = (z > 0u) ? pv[3] + prob(c, sr, reg[v - 1], q) : pv[3];
    pv[5] = (z < c->Z - 1u) ? pv[4] + prob(c, sr, reg[v + 1], q) : pv[4];
    pv[6] = 1.0f;
    uint32_t xmody = (y == 0u) ? 0u : (x % y);
    uint32_t state = orc_pcg(itime + xmody + z + i_part);
    float r = orc_uniform_float(state);
    int d = 0;
    while (d < 6 && r > pv[d]) d++;
    switch (d) { /* move_particle, rdme.wgsl:91-130 */
        case 0: return (x == 0u) ? 6 : 0;
        case 1: return (x == c->X - 1u) ? 6 : 1;
        case 2: return (y == 0u) ? 6 : 2;
        case 3: return (y == c->Y - 1u) ? 6 : 3;
        case 4: return (z == 0u) ? 6 : 4;
        case 5: return (z == c->Z - 1u) ? 6 : 5;
        default: return 6;
    }
}

static inline int64_t nb_offset(const ctx_t* c, int d) {
    int64_t YZ = (int64_t)c->Y * c->Z;
    switch (d) {
        case 0: return -YZ;
        case 1: return YZ;
        case 2: return -(int64_t)c->Z;
        case 3: return (int64_t)c->Z;
        case 4: return -1;
        default: return 1;
    }
}

static inline int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
static inline int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }

/* ---------------- diffusion, canonical serial order ---------------- */
static void rdme_serial(const ctx_t* c, const orc_tables* t, const uint32_t* src,
                        const uint32_t* occS, uint32_t* dst, uint32_t* occD, int32_t* conc,
                        uint32_t itime, uint32_t* diag, int count_occ_range) {
    uint32_t K = c->K, S1 = c->S1;
    for (uint64_t v = 0; v < c->V; v++) {
        uint32_t z = (uint32_t)(v % c->Z);
        uint32_t y = (uint32_t)((v / c->Z) % c->Y);
        uint32_t x = (uint32_t)(v / ((uint64_t)c->Z * c->Y));
        uint32_t o = occS[v];
        if (o > K) { if (count_occ_range) diag[ORC_DIAG_OCC_RANGE]++; o = K; }
        for (uint32_t s = 0; s < o; s++) {
            uint32_t i_part = (uint32_t)(v * K + s);
            uint32_t q = src[i_part];
            if (q == 0u) continue;
            int d = decide_direction(c, t, v, x, y, z, q, i_part, itime);
            if (d == 6) continue;
            uint64_t w = (uint64_t)((int64_t)v + nb_offset(c, d));
            /* move_particle_site, rdme.wgsl:45-88 */
            if (occD[w] >= K) { diag[ORC_DIAG_SPILL]++; continue; }
            uint32_t j = 0;
            while (j < K && dst[w * K + j] != 0u) j++;
            if (j == K) { diag[ORC_DIAG_SPILL]++; continue; }
            dst[w * K + j] = q;
            occD[w] += 1u;
            conc[w * S1 + q] = wadd(conc[w * S1 + q], 1);
            occD[v] -= 1u;
            dst[i_part] = 0u;
            conc[v * S1 + q] = wsub(conc[v * S1 + q], 1);
        }
    }
}

/* ---------------- diffusion, gather formulation ----------------
 * Directions are a pure function of the source lattice, so every voxel can
 * assemble its destination slots independently: arrivals from the -x, -y, -z
 * neighbours (lower linear index, slot order), then its own departures, then
 * arrivals from the +z, +y, +x neighbours, each arrival taking the lowest
 * free slot.  This equals the serial order whenever no arrival can be
 * rejected, which holds if max(occ, nonzero slots) + arrivals <= K for every
 * voxel; otherwise the step is redone serially. */
static int rdme_gather(const ctx_t* c, const orc_tables* t, const uint32_t* src,
                       const uint32_t* occS, const int32_t* concS, uint32_t* dst,
                       uint32_t* occD, int32_t* concD, uint8_t* dirs, uint32_t itime,
                       uint32_t* diag) {
    uint32_t K = c->K, S1 = c->S1;
    int64_t V = (int64_t)c->V;
    uint64_t occ_range = 0;
#pragma omp parallel for schedule(static) reduction(+ : occ_range)
    for (int64_t v = 0; v < V; v++) {
        uint32_t z = (uint32_t)(v % c->Z);
        uint32_t y = (uint32_t)((v / c->Z) % c->Y);
        uint32_t x = (uint32_t)(v / ((int64_t)c->Z * c->Y));
        uint32_t o = occS[v];
        if (o > K) { occ_range++; o = K; }
        for (uint32_t s = 0; s < K; s++) {
            uint32_t i_part = (uint32_t)((uint64_t)v * K + s);
            uint32_t q = src[i_part];
            dirs[i_part] = 7;
            if (s < o && q != 0u) dirs[i_part] = (uint8_t)decide_direction(c, t, (uint64_t)v, x, y, z, q, i_part, itime);
        }
    }
    diag[ORC_DIAG_OCC_RANGE] += (uint32_t)occ_range;
    int bad = 0;
    static const int lower_dirs[3] = {1, 3, 5};  /* arrivals from -x, -y, -z: moved +x, +y, +z */
    static const int upper_dirs[3] = {4, 2, 0};  /* arrivals from +z, +y, +x: moved -z, -y, -x */
#pragma omp parallel for schedule(static) reduction(| : bad)
    for (int64_t w = 0; w < V; w++) {
        uint32_t z = (uint32_t)(w % c->Z);
        uint32_t y = (uint32_t)((w / c->Z) % c->Y);
        uint32_t x = (uint32_t)(w / ((int64_t)c->Z * c->Y));
        int has_nb[6] = {x > 0u, x < c->X - 1u, y > 0u, y < c->Y - 1u, z > 0u, z < c->Z - 1u};
        uint32_t slots[16];
        uint32_t nnz = 0, in = 0;
        for (uint32_t s = 0; s < K; s++) { slots[s] = src[w * K + s]; nnz += slots[s] != 0u; }
        uint32_t o = occS[w];
        int32_t* cw = concD + w * S1;
        memcpy(cw, concS + w * S1, sizeof(int32_t) * S1);
        /* count arrivals */
        for (int side = 0; side < 6; side++) {
            /* neighbour in direction `side` sends particles moving in the opposite direction */
            if (!has_nb[side]) continue;
            int64_t u = w + nb_offset(c, side);
            int want = side ^ 1;
            for (uint32_t s = 0; s < K; s++) in += dirs[u * K + s] == want;
        }
        uint32_t base = (o > nnz) ? o : nnz;
        if (base + in > K) { bad = 1; continue; }
        for (int k = 0; k < 3; k++) {
            int want = lower_dirs[k];
            int side = want ^ 1;
            if (!has_nb[side]) continue;
            int64_t u = w + nb_offset(c, side);
            for (uint32_t s = 0; s < K; s++) {
                if (dirs[u * K + s] != want) continue;
                uint32_t q = src[u * K + s], j = 0;
                while (slots[j] != 0u) j++;
                slots[j] = q; o++; cw[q] = wadd(cw[q], 1);
            }
        }
        for (uint32_t s = 0; s < K; s++) {
            if (dirs[w * K + s] < 6) {
                uint32_t q = slots[s];
                slots[s] = 0u; o--; cw[q] = wsub(cw[q], 1);
            }
        }
        for (int k = 0; k < 3; k++) {
            int want = upper_dirs[k];
            int side = want ^ 1;
            if (!has_nb[side]) continue;
            int64_t u = w + nb_offset(c, side);
            for (uint32_t s = 0; s < K; s++) {
                if (dirs[u * K + s] != want) continue;
                uint32_t q = src[u * K + s], j = 0;
                while (slots[j] != 0u) j++;
                slots[j] = q; o++; cw[q] = wadd(cw[q], 1);
            }
        }
        memcpy(dst + w * K, slots, sizeof(uint32_t) * K);
        occD[w] = o;
    }
    return bad;
}

/* ---------------- reactions + compaction, per voxel ---------------- */
static void cme_voxel(const ctx_t* c, const orc_params* p, const orc_tables* t, uint64_t v,
                      uint32_t* dst, uint32_t* occD, int32_t* conc, int32_t* stat_delta,
                      uint32_t itime, uint32_t* fired, uint32_t* rolled) {
    uint32_t K = c->K, S1 = c->S1, R = c->R, S = S1 - 1;
    uint32_t z = (uint32_t)(v % c->Z);
    uint32_t y = (uint32_t)((v / c->Z) % c->Y);
    uint32_t x = (uint32_t)(v / ((uint64_t)c->Z * c->Y));
    int32_t* cv = conc + v * S1;
    uint32_t* sl = dst + v * K;
    cv[0] = 1;
    float cum[100];
    cum[0] = 0.0f;
    float total = 0.0f;
    for (uint32_t r = 1; r <= R; r++) {
        float k = t->rates[r];
        uint32_t prod = (uint32_t)cv[t->reactants[r * 3]] * (uint32_t)cv[t->reactants[r * 3 + 1]] *
                        (uint32_t)cv[t->reactants[r * 3 + 2]];
        float a = k * (float)(int32_t)prod;
        total = total + a;
        cum[r] = cum[r - 1] + a;
    }
    for (uint32_t i = 0; i < R; i++) cum[i] = cum[i] / total;
    uint32_t snap[16];
    for (uint32_t s = 0; s < K; s++) snap[s] = sl[s];
    uint32_t state = orc_pcg(itime + x * y + z);
    float r1 = orc_uniform_float(state);
    float fire_p = 1.0f - orc_expf(-total * p->tau);
    if (r1 <= fire_p) {
        (*fired)++;
        float r2 = orc_uniform_float(state + 1u);
        uint32_t i = 0;
        while ((r2 > cum[i]) & (i < R)) i++;
        const int32_t* st = t->stoich + (uint64_t)i * S1;
        uint32_t j = 0;
        int32_t new_occ = (int32_t)occD[v];
        uint64_t ri = v * K; /* reservoirs[idx_lattice], cme.wgsl:80 */
        uint32_t resv = (ri < c->V) ? t->reservoir[ri] : 0u;
        int rolled_back = 0;
        for (uint32_t s = 1; s <= S && !rolled_back; s++) {
            if (resv == s) continue;
            cv[s] = wadd(cv[s], st[s]);
            new_occ = wadd(new_occ, st[s]);
            stat_delta[s] = wadd(stat_delta[s], st[s]);
            int32_t cc = cv[s];
            while (cc > 0) {
                sl[j] = s;
                cc--;
                j++;
                if (j >= K) {
                    for (uint32_t k = 0; k < K; k++) sl[k] = snap[k];
                    for (uint32_t s2 = 1; s2 <= s; s2++) {
                        cv[s2] = wsub(cv[s2], st[s2]);
                        stat_delta[s2] = wsub(stat_delta[s2], st[s2]);
                    }
                    (*rolled)++;
                    rolled_back = 1;
                    break;
                }
            }
        }
        if (!rolled_back) {
            occD[v] = (uint32_t)new_occ;
            while (j < K) sl[j++] = 0u;
        }
    }
    /* final_stage.wgsl:25-33: stable move of non-zero slots to the front */
    uint32_t jj = 0;
    for (uint32_t s = 0; s < K; s++) {
        if (sl[s] != 0u) {
            uint32_t tmp = sl[s];
            sl[s] = sl[jj];
            sl[jj] = tmp;
            jj++;
        }
    }
}

static void cme_all(const ctx_t* c, const orc_params* p, const orc_tables* t, uint32_t* dst,
                    uint32_t* occD, int32_t* conc, int32_t* stat, uint32_t itime, uint32_t* diag,
                    int parallel) {
    uint32_t S1 = c->S1;
    int64_t V = (int64_t)c->V;
    uint64_t fired = 0, rolled = 0;
    int32_t* delta = (int32_t*)calloc(S1, sizeof(int32_t));
    if (parallel) {
#pragma omp parallel
        {
            int32_t* ld = (int32_t*)calloc(S1, sizeof(int32_t));
            uint32_t f = 0, rb = 0;
#pragma omp for schedule(static)
            for (int64_t v = 0; v < V; v++) cme_voxel(c, p, t, (uint64_t)v, dst, occD, conc, ld, itime, &f, &rb);
#pragma omp critical
            {
                for (uint32_t s = 0; s < S1; s++) delta[s] = wadd(delta[s], ld[s]);
                fired += f;
                rolled += rb;
            }
            free(ld);
        }
    } else {
        uint32_t f = 0, rb = 0;
        for (int64_t v = 0; v < V; v++) cme_voxel(c, p, t, (uint64_t)v, dst, occD, conc, delta, itime, &f, &rb);
        fired = f;
        rolled = rb;
    }
    for (uint32_t s = 0; s < S1; s++) stat[s] = wadd(stat[s], delta[s]);
    diag[ORC_DIAG_FIRED] += (uint32_t)fired;
    diag[ORC_DIAG_ROLLBACKS] += (uint32_t)rolled;
    free(delta);
}

int orc_ref_run(const orc_params* p, const orc_tables* t, uint32_t* slots, uint32_t* occ,
                int32_t* conc, int32_t* stat, uint32_t n_steps, const uint32_t* itimes,
                uint32_t* diag, int mode, int threads) {
    ctx_t c;
    if (!p || !t || !slots || !occ || !conc || !stat || !diag) return -1;
    int rc = ctx_init(&c, p, t);
    if (rc) return rc;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    uint64_t VK = c.V * c.K, VS = c.V * c.S1;
    uint32_t* dst = (uint32_t*)malloc(sizeof(uint32_t) * VK);
    uint32_t* occD = (uint32_t*)malloc(sizeof(uint32_t) * c.V);
    int32_t* concD = (int32_t*)malloc(sizeof(int32_t) * VS);
    uint8_t* dirs = (uint8_t*)malloc(VK);
    if (!dst || !occD || !concD || !dirs) { free(dst); free(occD); free(concD); free(dirs); free(c.P); return -2; }
    for (uint32_t st = 0; st < n_steps; st++) {
        uint32_t itime = itimes[st];
        int serial = (mode == 0);
        if (!serial) {
            int bad = rdme_gather(&c, t, slots, occ, conc, dst, occD, concD, dirs, itime, diag);
            if (bad) {
                serial = 1;
                diag[ORC_DIAG_SLOW_STEPS]++;
            } else {
                memcpy(conc, concD, sizeof(int32_t) * VS);
            }
        }
        if (serial) {
            memcpy(dst, slots, sizeof(uint32_t) * VK);
            memcpy(occD, occ, sizeof(uint32_t) * c.V);
            /* the gather pass already counted out-of-range occupancies */
            rdme_serial(&c, t, slots, occ, dst, occD, conc, itime, diag, mode == 0);
        }
        cme_all(&c, p, t, dst, occD, conc, stat, itime, diag, mode != 0);
        memcpy(slots, dst, sizeof(uint32_t) * VK);
        memcpy(occ, occD, sizeof(uint32_t) * c.V);
    }
    free(dst); free(occD); free(concD); free(dirs); free(c.P);
    return 0;
}
