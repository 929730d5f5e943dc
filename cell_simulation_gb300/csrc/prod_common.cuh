// prod_common.cuh — per-voxel operations of the production (Philox) step,
// shared by the fused tile kernel.  The algorithm (restated on the CPU in
// oracle/prod_semantics.c) is:
//
//  Random words: B(v, s) = Philox4x32-10({v, frame, s, 0}, seed) for slot s,
//  E(v, e) = Philox4x32-10({v, frame, 0x80000000 | e, 0}, seed) for reaction
//  event e.  One block B(v, 0) serves slot 0 of voxel v in all three sweeps
//  and the first reaction event, so a voxel holding one particle needs one
//  Philox evaluation per frame.
//
//  Diffusion, three sweeps per frame (x, then y, then z).  In the sweep
//  along axis a = 0, 1, 2 every particle of voxel v (slot s of its compacted
//  content) draws u = B(v, s)[a] and moves to v-a when
//  u < T[r(v)][r(v-a)][q], to v+a when T[.][r(v-a)][q] <= u < that + T[r(v)][r(v+a)][q],
//  where T = floor(D*tau/lambda^2 * 2^32) for the region codes (id+1; code 0
//  = outside the lattice, all thresholds 0) -- the move probabilities of
//  rdme.wgsl:132-136.  Capacity: the free room K - n(w) of a receiving voxel
//  w is split between its lower neighbour (ceil or floor half, alternating
//  with the parity of w + frame + sweep) and its upper neighbour; the first
//  movers in slot order up to that share are accepted, the rest stay.  The
//  new content of w is its staying particles (slot order), then accepted
//  arrivals from the lower neighbour, then from the upper neighbour.  A
//  voxel's new content therefore depends only on itself and its two
//  neighbours along the axis, never on arrival order, so the result is
//  independent of tiling and thread scheduling.
//
//  Reactions: an exact SSA (Gillespie direct method) inside each voxel over
//  one tau, with FP32 propensities and FP32 exponential waiting times, an
//  FP64 clock, and FP64 cumulative selection when max/min non-zero
//  propensity exceeds 1e6 (or always, or never, by precision mode).  Event e
//  takes its waiting-time word from B(v, 0)[3] (e = 0) or E(v, e)[0], and its
//  selection word from E(v, e)[1].  A reaction that would exceed K particles
//  is rejected.  If anything fired, the voxel's slots are rewritten
//  species-major (cme.wgsl:90-97).
#pragma once
#include <cstdint>

#include "devmath.cuh"

namespace cellsim {

// Diagnostic counters: events fired, events rejected for capacity, voxels that hit the event cap,
// FP64 selections, bricks spilled to the second pass, bricks lost (never), voxels that ran the SSA,
// dependency waits of the multi-frame sweep kernel that timed out (never).
enum {
    PD_EVENTS = 0, PD_REJECT_CAP = 1, PD_EVENT_CAP = 2, PD_FP64_SEL = 3, PD_DENSE_BRICKS = 4, PD_LOST_BRICKS = 5,
    PD_SSA_VOXELS = 6, PD_WAIT_TIMEOUTS = 7, PD_N = 8
};

struct RepDesc {
    uint64_t base;   // first voxel of this replicate in the packed slot/reservoir arrays
    uint64_t rbase;  // first byte of this replicate's padded region-code array
    uint32_t X, Y, Z;
    uint32_t Zr;     // padded row length of the region-code array (z stored at column z + 2)
    uint32_t seed_lo, seed_hi;
    float rate_mult;
    uint32_t counts_index;  // replicate index into the counts array
    uint32_t flags;         // bit 0: the whole lattice is region 0 (no region-code array)
    uint32_t Wz;            // occupancy-bitmap words per (x, y) row: ceil(Z / 32)
    uint64_t obase;         // first word of this replicate in the occupancy bitmaps
};
static_assert(sizeof(RepDesc) == 64, "RepDesc is 64 bytes");

// pad[0] of a brick item: the region code (id + 1) of every lattice voxel of
// the brick's region window (planes x0-2..x0+BX+1, rows y0-2..y0+BY+1,
// columns z0-2..z0+45) when they all share one, else 0.
struct WorkItem {
    uint32_t rep, y0, z0, x0, x1, pad[3];
};

struct ProdTables {
    uint32_t S1, R, NC, K;
    float tau;
    int32_t precision;  // cs_precision
    uint32_t max_events;
    uint32_t n_zero_order;  // reactions without reactants (fire in empty voxels)
    double tau_d;
    const uint32_t* thr;          // [NC][NC][S1]
    const uint8_t* rx_reactants;  // [R][3]
    const float* rx_rate;         // [R]
    const uint8_t* rx_ch_sp;      // [R][8]
    const int8_t* rx_ch_d;        // [R][8]
    const unsigned long long* rmask;  // [S1][2] bit r set when species s is a reactant of reaction r (R <= 128)
    unsigned long long zmask[2];      // reactions without reactants
    const float* one;                 // [n_rep][S1][3]: a0, max a, min non-zero a for a voxel holding
                                      // exactly one particle of species q (q = 0: an empty voxel)
    const uint32_t* quiet;            // [n_rep][S1][QS]: a voxel without reservoir holding one particle of
                                      // species p (q = 0), or one of p and one of q, has no reaction event
                                      // in the frame when (B(v,0)[3] >> 8) + 1 <= quiet[p][q]
    uint32_t QS;                      // S1 when two-particle entries are tabulated, else 1
    const float* g23;                 // [n_rep][2]: summed second- and third-order rates (times the
                                      // replicate's multiplier), for the propensity bound of fuller voxels
    const float* a2;                  // [n_rep][S1][S1] when QS == S1, else null: second-order propensity of
                                      // one particle pair (p, q), rounded up (the pair terms of that bound)
};


// K slot bytes held in 64-bit words, byte s = slot s.
template <int K>
struct alignas(K) Vox {
    uint64_t w[K / 8];
};

template <int K>
__device__ __forceinline__ Vox<K> vox_zero() {
    Vox<K> c;
#pragma unroll
    for (int i = 0; i < K / 8; i++) c.w[i] = 0;
    return c;
}

// Particles in a voxel.  Contents on this path are always compacted (no empty
// slot before an occupied one), so the count is the index of the highest
// non-zero byte plus one.
template <int K>
__device__ __forceinline__ uint32_t vox_n(const Vox<K>& c) {
    if (K == 16 && c.w[K / 8 - 1]) return 8u + ((71u - (uint32_t)__clzll((long long)c.w[K / 8 - 1])) >> 3);
    return c.w[0] ? (71u - (uint32_t)__clzll((long long)c.w[0])) >> 3 : 0u;
}

template <int K>
__device__ __forceinline__ bool vox_empty(const Vox<K>& c) {
    uint64_t o = 0;
#pragma unroll
    for (int i = 0; i < K / 8; i++) o |= c.w[i];
    return o == 0;
}

template <int K>
__device__ __forceinline__ uint32_t vox_get(const Vox<K>& c, uint32_t i) {
    if (K == 8) return (uint32_t)(c.w[0] >> (8 * i)) & 0xFFu;
    uint64_t w = (i < 8) ? c.w[0] : c.w[K / 8 - 1];
    return (uint32_t)(w >> (8 * (i & 7))) & 0xFFu;
}

template <int K>
__device__ __forceinline__ void vox_or(Vox<K>& c, uint32_t i, uint32_t q) {
    if (K == 8 || i < 8) c.w[0] |= (uint64_t)q << (8 * (i & 7));
    else c.w[K / 8 - 1] |= (uint64_t)q << (8 * (i & 7));
}

template <int K>
__device__ __forceinline__ void vox_set(Vox<K>& c, uint32_t i, uint32_t q) {
    uint64_t m = ~(0xFFull << (8 * (i & 7)));
    if (K == 8 || i < 8) c.w[0] = (c.w[0] & m) | ((uint64_t)q << (8 * (i & 7)));
    else c.w[K / 8 - 1] = (c.w[K / 8 - 1] & m) | ((uint64_t)q << (8 * (i & 7)));
}

template <int K>
__device__ __forceinline__ uint32_t vox_count(const Vox<K>& c, uint32_t q) {
    uint32_t rep = q * 0x01010101u, n = 0;
#pragma unroll
    for (int i = 0; i < K / 8; i++)
        n += __popc(__vcmpeq4((uint32_t)c.w[i], rep)) + __popc(__vcmpeq4((uint32_t)(c.w[i] >> 32), rep));
    return n >> 3;
}

// True when the first reaction event of a voxel with content c (no
// reservoir, no zero-order reaction) certainly falls beyond tau.  One or two
// particles: the tabulated bound of the exact a0.  More: a0 is at most
// sum_s a1(q_s) + sum_{i<j} a2(q_i, q_j) + n(n-1)(n-2) G3: the first-order
// propensities of the particles, the second-order propensity of every pair of
// particles (a2, tabulated per species pair and rounded up: the falling
// factorials of second-order reactions split exactly into pairs), and every
// third-order rate times the largest possible falling factorial.  Without the
// pair table (very many replicates and species) n(n-1) G2 bounds the pairs.
// A draw m <= exp(-bound tau (1 + 2^-10)) 2^24 (1 - 2^-20) gives dt > tau; the
// margins cover the binary32 sums and the portable expf.
template <int K>
__device__ __forceinline__ bool calm_voxel(const Vox<K>& c, uint32_t w3, const uint32_t* quiet_rep, uint32_t QS,
                                           const float* one_rep, const float* g23, const float* a2_rep, float tau) {
    const uint32_t n = vox_n<K>(c);
    if (n == 0u) return false;
    const uint32_t m = (w3 >> 8) + 1u;
    if (n == 1u || (n == 2u && QS != 1u)) {
        const uint32_t p = vox_get<K>(c, 0), q = n == 2u ? vox_get<K>(c, 1) : 0u;
        return m <= quiet_rep[p * QS + q];
    }
    float a = 0.0f;
    for (uint32_t s = 0; s < n; s++) a = __fadd_rn(a, one_rep[vox_get<K>(c, s) * 3]);
    const float nnn = (float)(n * (n - 1u) * (n - 2u));
    if (a2_rep) {
        for (uint32_t i = 0; i + 1u < n; i++) {
            const float* row = a2_rep + vox_get<K>(c, i) * QS;
            for (uint32_t j = i + 1u; j < n; j++) a = __fadd_rn(a, row[vox_get<K>(c, j)]);
        }
        a = __fadd_rn(a, __fmul_rn(nnn, g23[1]));
    } else {
        const float nn = (float)(n * (n - 1u));
        a = __fadd_rn(a, __fadd_rn(__fmul_rn(nn, g23[0]), __fmul_rn(nnn, g23[1])));
    }
    const float x = __fmul_rn(__fmul_rn(a, tau), 1.0009765625f);  // 1 + 2^-10
    if (!(x >= 0.0f)) return false;
    if (x > 20.0f) return false;
    const float lim = __fmul_rn(__fmul_rn(d_expf(-x), 16777216.0f), 0.99999904632568359375f);  // 1 - 2^-20
    return (float)m <= lim;
}

// Keep the c lowest set bits of m.
__device__ __forceinline__ uint32_t lowest_bits(uint32_t m, uint32_t c) {
    while ((uint32_t)__popc(m) > c) m &= ~(0x80000000u >> __clz(m));
    return m;
}

__device__ __forceinline__ uint32_t sweep_word(const U4& b, uint32_t sweep) {
    return sweep == 0u ? b.x : sweep == 1u ? b.y : b.z;
}

// Move decisions of one voxel for one sweep: bit s = slot s moves to the
// lower neighbour, bit 16+s = to the upper neighbour.  tlo / thi are the
// threshold rows T[r(v)][r(lower)][.] and T[r(v)][r(upper)][.]; w0 is slot
// 0's word B(v, 0)[sweep], evaluated by the caller.
template <int K>
__device__ __forceinline__ uint32_t decide_moves(const Vox<K>& c, uint32_t v, uint32_t frame, uint32_t sweep,
                                                 const uint32_t* tlo, const uint32_t* thi, uint32_t k0, uint32_t k1,
                                                 uint32_t w0) {
    const uint32_t n = vox_n<K>(c);
    uint32_t mask = 0;
    for (uint32_t s = 0; s < n; s++) {
        const uint32_t q = vox_get<K>(c, s);
        const uint32_t tm = tlo[q], tp = thi[q];
        if ((tm | tp) == 0u) continue;
        const uint32_t u = s == 0u ? w0 : sweep_word(d_philox(v, frame, s, 0u, k0, k1), sweep);
        if (u < tm) mask |= 1u << s;
        else if (u - tm < tp) mask |= 1u << (16 + s);  // tm <= u < tm + tp, without the 33-bit sum
    }
    return mask;
}

// New content of a voxel after one sweep.
template <int K>
__device__ __forceinline__ Vox<K> combine(const Vox<K>& own, uint32_t down, const Vox<K>& lo, uint32_t dlo, const Vox<K>& hi,
                                          uint32_t dhi, uint32_t v_self, uint32_t v_lo, uint32_t v_hi, uint32_t frame,
                                          uint32_t sweep) {
    uint32_t in_lo = dlo >> 16, in_hi = dhi & 0xFFFFu;
    if ((down | in_lo | in_hi) == 0u) return own;
    uint32_t n_self = vox_n<K>(own);
    uint32_t room = K - n_self;
    uint32_t share_lo = (room + ((v_self + frame + sweep) & 1u)) >> 1, share_hi = room - share_lo;
    uint32_t acc_lo = lowest_bits(in_lo, share_lo), acc_hi = lowest_bits(in_hi, share_hi);
    uint32_t out_m = down & 0xFFFFu, out_p = down >> 16;
    if (out_m) {
        uint32_t room_l = K - vox_n<K>(lo);
        uint32_t sh = room_l - ((room_l + ((v_lo + frame + sweep) & 1u)) >> 1);
        out_m = lowest_bits(out_m, sh);
    }
    if (out_p) {
        uint32_t room_h = K - vox_n<K>(hi);
        uint32_t sl = (room_h + ((v_hi + frame + sweep) & 1u)) >> 1;
        out_p = lowest_bits(out_p, sl);
    }
    uint32_t keep = ((1u << n_self) - 1u) & ~(out_m | out_p);
    Vox<K> r = vox_zero<K>();
    uint32_t j = 0;
    while (keep) {
        uint32_t s = __ffs(keep) - 1;
        keep &= keep - 1;
        vox_or<K>(r, j++, vox_get<K>(own, s));
    }
    while (acc_lo) {
        uint32_t s = __ffs(acc_lo) - 1;
        acc_lo &= acc_lo - 1;
        vox_or<K>(r, j++, vox_get<K>(lo, s));
    }
    while (acc_hi) {
        uint32_t s = __ffs(acc_hi) - 1;
        acc_hi &= acc_hi - 1;
        vox_or<K>(r, j++, vox_get<K>(hi, s));
    }
    return r;
}

// Reads of the reaction tables.  Plain (generic) loads, because a kernel may
// hand react_voxel tables staged in shared memory as well as global ones.
template <typename T>
__device__ __forceinline__ T tab_ld(const T* p) {
    return *p;
}

// Propensity of reaction r (0-based) for the voxel content c.
template <int K>
__device__ __forceinline__ float propensity(const ProdTables& T, uint32_t r, const Vox<K>& c, uint32_t resv, float mult) {
    const uint8_t* re = T.rx_reactants + 3 * r;
    uint32_t s0 = tab_ld(re), s1 = tab_ld(re + 1), s2 = tab_ld(re + 2);
    uint32_t ff = 1;
    uint32_t sp[3] = {s0, s1, s2};
#pragma unroll
    for (int j = 0; j < 3; j++) {
        uint32_t s = sp[j];
        if (s == 0) continue;
        uint32_t m = 0;
#pragma unroll
        for (int i = 0; i < j; i++) m += sp[i] == s;
        uint32_t cnt = (s == resv) ? 1u : vox_count<K>(c, s);
        if (cnt <= m) return 0.0f;
        ff *= cnt - m;
    }
    return __fmul_rn(__fmul_rn(tab_ld(T.rx_rate + r), mult), (float)ff);
}

// Reactions whose propensity can be non-zero in the voxel: those with a
// reactant present, and those without reactants.  Every other reaction has
// propensity exactly +0, so summing only these in index order gives the
// same binary32 and binary64 sums as summing all of them.
template <int K>
__device__ __forceinline__ void candidates(const ProdTables& T, const Vox<K>& c, uint32_t n, uint32_t resv,
                                           unsigned long long& m0, unsigned long long& m1) {
    m0 = T.zmask[0];
    m1 = T.zmask[1];
    for (uint32_t i = 0; i < n; i++) {
        uint32_t q = vox_get<K>(c, i);
        m0 |= tab_ld(T.rmask + 2 * q);
        m1 |= tab_ld(T.rmask + 2 * q + 1);
    }
    if (resv) {
        m0 |= tab_ld(T.rmask + 2 * resv);
        m1 |= tab_ld(T.rmask + 2 * resv + 1);
    }
}

__device__ __forceinline__ int next_bit(unsigned long long& m0, unsigned long long& m1) {
    if (m0) {
        int b = __ffsll((long long)m0) - 1;
        m0 &= m0 - 1;
        return b;
    }
    if (m1) {
        int b = __ffsll((long long)m1) - 1;
        m1 &= m1 - 1;
        return 64 + b;
    }
    return -1;
}

// SSA within tau for one voxel.  Returns true when any reaction fired (the
// content is then rewritten species-major).  s_delta[S1] and s_diag[PD_N]
// are block-shared accumulators.
// w3 is B(v, 0)[3], evaluated by the caller.  react_voxel_inline is the body,
// for kernels that run the SSA in a loop of their own; react_voxel is the
// out-of-line call for kernels whose register budget must not grow for it.
template <int K>
__device__ __forceinline__ bool react_voxel_inline(Vox<K>& c, uint32_t resv, uint32_t v, uint32_t frame, uint32_t k0,
                                                   uint32_t k1, float mult, uint32_t rep, const ProdTables& T,
                                                   int32_t* s_delta, uint32_t* s_diag, uint32_t w3) {
    if (T.R == 0) return false;
    atomicAdd(s_diag + PD_SSA_VOXELS, 1u);
    uint32_t n = vox_n<K>(c);
    double td = 0.0;
    float tf = 0.0f;
    bool fired = false;
    uint32_t ev = 0;
    for (; ev < T.max_events; ev++) {
        unsigned long long c0, c1;
        candidates<K>(T, c, n, resv, c0, c1);
        float a0 = 0.0f, amax = 0.0f, amin = __int_as_float(0x7f800000);
        if (resv == 0u && n <= 1u) {
            // one particle or none: the candidate sum is tabulated (same binary32 sum)
            const float* o = T.one + ((size_t)rep * T.S1 + (n ? vox_get<K>(c, 0) : 0u)) * 3;
            a0 = tab_ld(o);
            amax = tab_ld(o + 1);
            amin = tab_ld(o + 2);
        } else {
            unsigned long long m0 = c0, m1 = c1;
            for (int r = next_bit(m0, m1); r >= 0; r = next_bit(m0, m1)) {
                float a = propensity<K>(T, (uint32_t)r, c, resv, mult);
                a0 = __fadd_rn(a0, a);
                if (a > 0.0f) { amax = fmaxf(amax, a); amin = fminf(amin, a); }
            }
        }
        if (!(a0 > 0.0f)) break;
        U4 ph{0u, 0u, 0u, 0u};
        uint32_t w1 = w3;
        if (ev != 0u) {
            ph = d_philox(v, frame, 0x80000000u | ev, 0u, k0, k1);
            w1 = ph.x;
        }
        float u1 = __fmul_rn((float)((w1 >> 8) + 1u), 0x1p-24f);
        float dt = __fdiv_rn(-d_logf(u1), a0);
        if (T.precision == 1) {
            tf = __fadd_rn(tf, dt);
            if (tf > T.tau) break;
        } else {
            td = __dadd_rn(td, (double)dt);
            if (td > T.tau_d) break;
        }
        if (ev == 0u) ph = d_philox(v, frame, 0x80000000u, 0u, k0, k1);
        const uint32_t w2 = ph.y;
        float u2 = __fmul_rn((float)(w2 >> 8), 0x1p-24f);
        bool use64 = (T.precision == 2) || (T.precision == 0 && amax > __fmul_rn(1e6f, amin));
        int sel = -1;
        int last_pos = -1;
        if (!use64) {
            float target = __fmul_rn(u2, a0), run = 0.0f;
            unsigned long long m0 = c0, m1 = c1;
            for (int r = next_bit(m0, m1); r >= 0; r = next_bit(m0, m1)) {
                float a = propensity<K>(T, (uint32_t)r, c, resv, mult);
                if (a > 0.0f) last_pos = r;
                run = __fadd_rn(run, a);
                if (target < run) { sel = r; break; }
            }
        } else {
            atomicAdd(s_diag + PD_FP64_SEL, 1u);
            double a0d = 0.0;
            {
                unsigned long long m0 = c0, m1 = c1;
                for (int r = next_bit(m0, m1); r >= 0; r = next_bit(m0, m1))
                    a0d = __dadd_rn(a0d, (double)propensity<K>(T, (uint32_t)r, c, resv, mult));
            }
            double target = __dmul_rn((double)u2, a0d), run = 0.0;
            unsigned long long m0 = c0, m1 = c1;
            for (int r = next_bit(m0, m1); r >= 0; r = next_bit(m0, m1)) {
                float a = propensity<K>(T, (uint32_t)r, c, resv, mult);
                if (a > 0.0f) last_pos = r;
                run = __dadd_rn(run, (double)a);
                if (target < run) { sel = r; break; }
            }
        }
        if (sel < 0) sel = last_pos;
        if (sel < 0) break;
        // apply the change list, skipping the voxel's reservoir species
        const uint8_t* csp = T.rx_ch_sp + 8 * sel;
        const int8_t* cd = T.rx_ch_d + 8 * sel;
        int total = (int)n;
        bool ok = true;
        for (int j = 0; j < 8; j++) {
            uint32_t s = tab_ld(csp + j);
            if (s == 0) break;
            if (s == resv) continue;
            int d = tab_ld(cd + j);
            int have = (int)vox_count<K>(c, s);
            if (have + d < 0) ok = false;
            total += d;
        }
        if (!ok || total > (int)K) {
            atomicAdd(s_diag + PD_REJECT_CAP, 1u);
            continue;
        }
        // removals first, so that the content never exceeds K slots in between
        for (int pass = 0; pass < 2; pass++) {
            for (int j = 0; j < 8; j++) {
                uint32_t s = tab_ld(csp + j);
                if (s == 0) break;
                if (s == resv) continue;
                int d = tab_ld(cd + j);
                if (pass == 0) {
                    for (; d < 0; d++) {  // remove one occurrence: move the last particle into its slot
                        uint32_t idx = 0;
                        for (uint32_t i = 0; i < n; i++)
                            if (vox_get<K>(c, i) == s) idx = i;
                        vox_set<K>(c, idx, vox_get<K>(c, n - 1));
                        vox_set<K>(c, n - 1, 0u);
                        n--;
                    }
                } else {
                    for (; d > 0; d--) vox_set<K>(c, n++, s);
                    atomicAdd(s_delta + s, tab_ld(cd + j));
                }
            }
        }
        atomicAdd(s_diag + PD_EVENTS, 1u);
        fired = true;
    }
    if (ev == T.max_events) atomicAdd(s_diag + PD_EVENT_CAP, 1u);
    if (fired) {
        // species-major rewrite, ascending species id
        Vox<K> out = vox_zero<K>();
        uint32_t j = 0, prev = 0;
        for (;;) {
            uint32_t best = 256;
            for (uint32_t i = 0; i < n; i++) {
                uint32_t b = vox_get<K>(c, i);
                if (b > prev && b < best) best = b;
            }
            if (best == 256) break;
            uint32_t cnt = vox_count<K>(c, best);
            for (uint32_t k = 0; k < cnt; k++) vox_or<K>(out, j++, best);
            prev = best;
        }
        c = out;
    }
    return fired;
}

// Index of set bit k (0-based) of the 128-bit mask (m0, m1); k < popcount.
__device__ __forceinline__ int nth_bit(unsigned long long m0, unsigned long long m1, uint32_t k) {
    uint32_t off = 0u;
    uint32_t p0 = (uint32_t)__popcll(m0);
    unsigned long long m = m0;
    if (k >= p0) {
        k -= p0;
        m = m1;
        off = 64u;
    }
    uint32_t w = (uint32_t)m, pl = (uint32_t)__popc(w);
    if (k >= pl) {
        k -= pl;
        w = (uint32_t)(m >> 32);
        off += 32u;
    }
#pragma unroll
    for (uint32_t sh = 16u; sh; sh >>= 1) {
        const uint32_t c = (uint32_t)__popc(w & ((1u << sh) - 1u));
        if (k >= c) {
            k -= c;
            w >>= sh;
            off += sh;
        }
    }
    return (int)off;
}

// Byte positions [a, b) of a 64-bit word (0 <= a, b <= 8) as a bit mask.
__device__ __forceinline__ uint64_t byte_run_mask(int a, int b) {
    a = min(max(a, 0), 8);
    b = min(max(b, 0), 8);
    if (b <= a) return 0ull;
    const uint64_t hi = b == 8 ? ~0ull : (1ull << (8 * b)) - 1ull;
    return hi & ~((1ull << (8 * a)) - 1ull);  // a < 8 here
}

// Words of the per-warp shared scratch react_voxel_warp uses (1408 bytes).
constexpr int SSA_WARP_SCRATCH = 352;

// The SSA of react_voxel_inline run by a whole warp: every lane calls it with
// the same voxel and gets the same result.  The warp works on the voxel's
// species histogram (in its shared scratch `ws`) instead of its slots: every
// quantity of the SSA depends on the counts alone, and the content it returns
// is rewritten species-major as react_voxel_inline's is.  Lane l owns
// reactions l, l + 32, ...: the candidates' propensities go to their rank in
// index order, lane 0 forms the running sums in that order (binary32 and, when
// the selection needs it, binary64) exactly as react_voxel_inline does, and
// the selected candidate is the first whose running sum exceeds the target (a
// ballot over the stored binary32 sums; lane 0 scans the binary64 ones).  An
// event's change list is applied one entry per lane, its species deltas added
// to s_delta (shared) or, when that is null, to the global counts row
// g_counts.  So every result, and so the lattice, equals react_voxel_inline's.
template <int K>
__device__ __forceinline__ bool react_voxel_warp(Vox<K>& c, uint32_t resv, uint32_t v, uint32_t frame, uint32_t k0,
                                                 uint32_t k1, float mult, uint32_t rep, const ProdTables& T,
                                                 int32_t* s_delta, unsigned long long* g_counts, uint32_t* s_diag,
                                                 uint32_t w3, float* ws) {
    const uint32_t lane = threadIdx.x & 31u;
    if (T.R == 0) return false;
    if (lane == 0u) atomicAdd(s_diag + PD_SSA_VOXELS, 1u);
    float* const a_s = ws;                                      // [128] propensities by candidate rank
    float* const p_s = ws + 128;                                // [128] their binary32 running sums
    uint8_t* const hist = reinterpret_cast<uint8_t*>(ws + 256);  // [256] particles per species
    uint8_t* const r_s = reinterpret_cast<uint8_t*>(ws + 320);   // [128] reaction of each rank
    const uint32_t S1 = T.S1, R = T.R;
    uint32_t n = vox_n<K>(c);
    for (uint32_t s = lane; s < S1; s += 32u) hist[s] = s ? (uint8_t)vox_count<K>(c, s) : (uint8_t)0;
    __syncwarp();
    double td = 0.0;
    float tf = 0.0f;
    bool fired = false;
    uint32_t ev = 0;
    for (; ev < T.max_events; ev++) {
        // candidates: reactions with a reactant present (or none at all)
        unsigned long long c0 = 0ull, c1 = 0ull;
        for (uint32_t s = 1u + lane; s < S1; s += 32u)
            if (hist[s] > 0) {
                c0 |= tab_ld(T.rmask + 2 * s);
                c1 |= tab_ld(T.rmask + 2 * s + 1);
            }
        c0 = ((unsigned long long)__reduce_or_sync(0xffffffffu, (uint32_t)(c0 >> 32)) << 32) |
             __reduce_or_sync(0xffffffffu, (uint32_t)c0);
        c1 = ((unsigned long long)__reduce_or_sync(0xffffffffu, (uint32_t)(c1 >> 32)) << 32) |
             __reduce_or_sync(0xffffffffu, (uint32_t)c1);
        c0 |= T.zmask[0];
        c1 |= T.zmask[1];
        if (resv) {
            c0 |= tab_ld(T.rmask + 2 * resv);
            c1 |= tab_ld(T.rmask + 2 * resv + 1);
        }
        const uint32_t p0 = (uint32_t)__popcll(c0);
        const uint32_t nc = p0 + (uint32_t)__popcll(c1);
        uint32_t bmax = 0u, bmin = 0x7f800000u;  // bit patterns of positive binary32 order like the values
        for (uint32_t r = lane; r < R; r += 32u) {
            const bool cand = r < 64u ? ((c0 >> r) & 1ull) != 0ull : ((c1 >> (r - 64u)) & 1ull) != 0ull;
            if (!cand) continue;
            const uint32_t rank = r < 64u ? (uint32_t)__popcll(c0 & ((1ull << r) - 1ull))
                                          : p0 + (uint32_t)__popcll(c1 & ((1ull << (r - 64u)) - 1ull));
            // the propensity of react_voxel_inline, from the histogram
            const uint8_t* re = T.rx_reactants + 3 * r;
            const uint32_t sp[3] = {tab_ld(re), tab_ld(re + 1), tab_ld(re + 2)};
            uint32_t ff = 1u;
            bool zero = false;
#pragma unroll
            for (int j = 0; j < 3; j++) {
                const uint32_t q = sp[j];
                if (q == 0u) continue;
                uint32_t m = 0u;
#pragma unroll
                for (int i = 0; i < j; i++) m += sp[i] == q;
                const uint32_t cnt = q == resv ? 1u : (uint32_t)hist[q];
                if (cnt <= m) zero = true;
                else ff *= cnt - m;
            }
            const float a = zero ? 0.0f : __fmul_rn(__fmul_rn(tab_ld(T.rx_rate + r), mult), (float)ff);
            a_s[rank] = a;
            r_s[rank] = (uint8_t)r;
            if (a > 0.0f) {
                bmax = max(bmax, __float_as_uint(a));
                bmin = min(bmin, __float_as_uint(a));
            }
        }
        __syncwarp();
        if (lane == 0u) {
            float run = 0.0f;
            for (uint32_t k = 0; k < nc; k++) {
                run = __fadd_rn(run, a_s[k]);
                p_s[k] = run;
            }
        }
        __syncwarp();
        const uint32_t rounds = (nc + 31u) >> 5;
        float a0, amax, amin;
        if (resv == 0u && n <= 1u) {
            uint32_t sole = 0u;  // the species of the voxel's one particle
            if (n == 1u)
                for (uint32_t base = 0; base < S1; base += 32u) {
                    const uint32_t b = __ballot_sync(0xffffffffu, base + lane < S1 && hist[base + lane] > 0);
                    if (b) {
                        sole = base + (uint32_t)__ffs((int)b) - 1u;
                        break;
                    }
                }
            const float* o = T.one + ((size_t)rep * S1 + sole) * 3;
            a0 = tab_ld(o);
            amax = tab_ld(o + 1);
            amin = tab_ld(o + 2);
        } else {
            a0 = nc ? p_s[nc - 1u] : 0.0f;
            amax = __uint_as_float(__reduce_max_sync(0xffffffffu, bmax));
            amin = __uint_as_float(__reduce_min_sync(0xffffffffu, bmin));
        }
        if (!(a0 > 0.0f)) break;
        U4 ph{0u, 0u, 0u, 0u};
        uint32_t w1 = w3;
        if (ev != 0u) {
            ph = d_philox(v, frame, 0x80000000u | ev, 0u, k0, k1);
            w1 = ph.x;
        }
        float u1 = __fmul_rn((float)((w1 >> 8) + 1u), 0x1p-24f);
        float dt = __fdiv_rn(-d_logf(u1), a0);
        if (T.precision == 1) {
            tf = __fadd_rn(tf, dt);
            if (tf > T.tau) break;
        } else {
            td = __dadd_rn(td, (double)dt);
            if (td > T.tau_d) break;
        }
        if (ev == 0u) ph = d_philox(v, frame, 0x80000000u, 0u, k0, k1);
        const uint32_t w2 = ph.y;
        float u2 = __fmul_rn((float)(w2 >> 8), 0x1p-24f);
        bool use64 = (T.precision == 2) || (T.precision == 0 && amax > __fmul_rn(1e6f, amin));
        // first candidate whose running sum exceeds the target; else the last one with a positive
        // propensity (the sequential scan's last_pos)
        int idx = -1;
        if (!use64) {
            const float target = __fmul_rn(u2, a0);
            for (uint32_t q = 0; q < rounds && idx < 0; q++) {
                const uint32_t k = q * 32u + lane;
                const uint32_t b = __ballot_sync(0xffffffffu, k < nc && target < p_s[k]);
                if (b) idx = (int)(q * 32u) + __ffs((int)b) - 1;
            }
        } else {
            if (lane == 0u) {
                atomicAdd(s_diag + PD_FP64_SEL, 1u);
                double a0d = 0.0;
                for (uint32_t k = 0; k < nc; k++) a0d = __dadd_rn(a0d, (double)a_s[k]);
                const double target = __dmul_rn((double)u2, a0d);
                double run = 0.0;
                for (uint32_t k = 0; k < nc; k++) {
                    run = __dadd_rn(run, (double)a_s[k]);
                    if (target < run) {
                        idx = (int)k;
                        break;
                    }
                }
            }
            idx = __shfl_sync(0xffffffffu, idx, 0);
        }
        if (idx < 0) {
            for (int q = (int)rounds - 1; q >= 0 && idx < 0; q--) {
                const uint32_t k = (uint32_t)q * 32u + lane;
                const uint32_t b = __ballot_sync(0xffffffffu, k < nc && a_s[k] > 0.0f);
                if (b) idx = q * 32 + 31 - __clz((int)b);
            }
        }
        const uint32_t sel = idx >= 0 ? (uint32_t)r_s[idx] : 0u;
        __syncwarp();  // the scratch is rewritten by the next event
        if (idx < 0) break;
        // the change list (distinct species, ending at the first zero), one entry per lane; the
        // voxel's reservoir species is skipped
        const uint32_t es = lane < 8u ? (uint32_t)tab_ld(T.rx_ch_sp + 8 * sel + lane) : 0u;
        const int ed = lane < 8u ? (int)tab_ld(T.rx_ch_d + 8 * sel + lane) : 0;
        const uint32_t zb = __ballot_sync(0xffffffffu, lane < 8u && es == 0u);
        const uint32_t n_ent = zb ? (uint32_t)__ffs((int)zb) - 1u : 8u;
        const bool act = lane < n_ent && es != resv;
        const int have = act ? hist[es] : 0;
        const int total = (int)n + __reduce_add_sync(0xffffffffu, (uint32_t)(act ? ed : 0));
        if (__any_sync(0xffffffffu, act && have + ed < 0) || total > (int)K) {
            if (lane == 0u) atomicAdd(s_diag + PD_REJECT_CAP, 1u);
            continue;
        }
        if (act) {
            hist[es] = (uint8_t)(have + ed);
            if (s_delta) atomicAdd(s_delta + es, ed);
            else atomicAdd(g_counts + es, (unsigned long long)(long long)ed);
        }
        __syncwarp();
        n = (uint32_t)total;
        if (lane == 0u) atomicAdd(s_diag + PD_EVENTS, 1u);
        fired = true;
    }
    if (ev == T.max_events && lane == 0u) atomicAdd(s_diag + PD_EVENT_CAP, 1u);
    if (fired) {
        // species-major rewrite, ascending species id: lane l writes the run of species
        // base + l at its exclusive prefix of the counts
        uint64_t w[K / 8];
#pragma unroll
        for (int i = 0; i < K / 8; i++) w[i] = 0ull;
        int off = 0;
        for (uint32_t base = 0; base < S1; base += 32u) {
            const uint32_t s = base + lane;
            const int cnt = (s > 0u && s < S1) ? hist[s] : 0;
            int incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_up_sync(0xffffffffu, incl, o);
                if ((int)lane >= o) incl += u;
            }
            const int a = off + incl - cnt;
            if (cnt > 0) {
                const uint64_t rep8 = (uint64_t)s * 0x0101010101010101ull;
#pragma unroll
                for (int i = 0; i < K / 8; i++) w[i] |= rep8 & byte_run_mask(a - 8 * i, a + cnt - 8 * i);
            }
            off += __shfl_sync(0xffffffffu, incl, 31);
        }
        Vox<K> out;
#pragma unroll
        for (int i = 0; i < K / 8; i++)
            out.w[i] = ((uint64_t)__reduce_or_sync(0xffffffffu, (uint32_t)(w[i] >> 32)) << 32) |
                       __reduce_or_sync(0xffffffffu, (uint32_t)w[i]);
        c = out;
    }
    return fired;
}

template <int K>
__device__ __noinline__ bool react_voxel(Vox<K>& c, uint32_t resv, uint32_t v, uint32_t frame, uint32_t k0, uint32_t k1,
                                         float mult, uint32_t rep, const ProdTables& T, int32_t* s_delta,
                                         uint32_t* s_diag, uint32_t w3) {
    return react_voxel_inline<K>(c, resv, v, frame, k0, k1, mult, rep, T, s_delta, s_diag, w3);
}

}  // namespace cellsim
