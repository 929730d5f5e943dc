// brick_kernel.cuh — the sparse brick pass of the production step.
//
// A work item is a brick of BX x BY x 32 voxels (x, y, z) of one replicate.
// The CTA loads the brick with a one-voxel halo (the "box", (BX+2) x (BY+2)
// x 34 voxels) and runs the whole frame on it in five phases separated by
// CTA barriers:
//
//   L  coalesced 16-byte loads of the box, row occupancy masks by warp
//      ballot, occupied contents appended to pool 0 (region codes of the box
//      plus one more voxel arrive by cp.async meanwhile)
//   A  x-move decisions of every occupied box voxel
//   B  X sweep of the interior planes (all box rows and columns), y-move
//      decisions of the results, into pool 1
//   C  Y sweep of the interior rows (all columns), z-move decisions, pool 2
//   D  Z sweep of the interior, reactions, store; voxels that nothing
//      reaches are stored as zeros with coalesced row stores
//
// Shared memory holds the box only in compacted form.  Per box row there is
// a 64-bit mask per quantity (occupied, moving down / up along an axis, has
// content after a sweep), and the contents of the voxels a phase produces
// are kept in a pool where every row's voxels are contiguous: the pool index
// of voxel (row, c) is rowbase[row] + popcount(mask[row] below c).  Warp w
// lists rows 32 w .. 32 w + 31 (one row per lane; warps past the last row
// sit the list out) and reserves the pool range of its rows with one
// shared-memory atomic, so no CTA-wide scan is needed.  A phase writes
// the positions of its voxels into a list indexed like its pool, and after a
// barrier the whole CTA runs the list with every lane busy.  The lattice is
// mostly empty, so a brick holds a few hundred entries per pool where the
// dense box has thousands of voxels, and the CTA footprint stays small
// enough for four CTAs per SM.
//
// The Philox block B(v, 0) of a voxel is evaluated once per frame, in the
// first phase that sees the voxel non-empty, and its words (x, y, z draw of
// slot 0, first reaction event) are kept beside that phase's pool entry.
//
// A brick whose occupancy overflows a pool is abandoned before it writes
// anything to global memory and appended to the spill list.  A second launch
// of this kernel with pools as large as the box (never overflows) finishes
// the spilled bricks in groups of a few planes, so crowded regions get the
// same result.
#pragma once
#include <cstdint>

#include "prod_common.cuh"
#include "prod_kernel.cuh"

namespace cellsim {

template <int K, int BX, int BY, int NT, int CAP0, int CAP1, int CAP2>
struct Brick {
    static constexpr int NW = NT / 32;
    // WP: one warp per interior plane; the X/Y/Z sweeps of a plane then depend only on that
    // warp, so they run without CTA barriers.  Otherwise each phase runs CTA-wide.
    static constexpr bool WP = NW == BX;
    static constexpr int PX = BX + 2, WY = BY + 2, WZ = 34;
    static constexpr int NROW0 = PX * WY;  // box rows (plane, row)
    static constexpr int NROW1 = BX * WY;  // X-sweep rows: interior planes, all rows
    static constexpr int NROW2 = BX * BY;  // Y/Z-sweep rows: interior planes, interior rows
    static constexpr int RPX = BX + 4, RWY = BY + 4, RWZB = 48, RPLANE = RWY * RWZB;
    static constexpr int NCH = RPX * RWY * (RWZB / 16);  // 16-byte region chunks
    static constexpr int MAXC = CAP0 > CAP1 ? (CAP0 > CAP2 ? CAP0 : CAP2) : (CAP1 > CAP2 ? CAP1 : CAP2);
    // CTA-wide path: pool 2 shares pool 0's storage (dead after the X sweep), one list array
    static constexpr int C02 = WP ? CAP0 : (CAP0 > CAP2 ? CAP0 : CAP2);
    // CTA-wide D list: each pool-2 voxel and at most its two z-move targets (3 CAP2 entries); with
    // reservoirs or zero-order reactions every interior voxel is stepped without a list.  The lists
    // sit in dead storage when it fits: the B and C lists in pool 0's position list (read only in
    // phase A), the D list in pool 1's contents (read last in phase C); else in one list array.
    static constexpr int DCAP = 3 * CAP2;
    static constexpr bool ALIAS = !WP && CAP1 <= CAP0 && CAP2 <= CAP0 && CAP1 * K / 2 >= DCAP;
    static constexpr int LCAP = WP ? 0 : ALIAS ? CAP1 * K / 2 : (MAXC > DCAP ? MAXC : DCAP);
    static constexpr int LDW = BY * 32;  // per-warp D list (warp-per-plane path)
    static constexpr bool DENSE = CAP0 >= NROW0 * WZ && CAP1 >= NROW1 * WZ && CAP2 >= NROW2 * WZ;  // never overflows
    static_assert(NT % 32 == 0 && WY <= 32 && BY <= 32, "one lane per row of a plane (warp-per-plane path)");
    // CTA-wide lists: warp w lists rows 32 w .. 32 w + 31 in one pass, so every row needs a thread
    static_assert(NW == BX || (NT >= NROW1 && NT >= NROW2), "one thread per row of the B, C and D lists");
    static_assert(NROW0 * 64 <= 65536 && MAXC < 65536, "positions and pool indices fit 16 bits");
    enum : int {
        M_OCC0 = 0, M_XM = NROW0, M_XP = 2 * NROW0,
        M_S1 = 3 * NROW0, M_YM = M_S1 + NROW1, M_YP = M_YM + NROW1, M_PB1 = M_YP + NROW1,
        M_S2 = M_PB1 + NROW1, M_ZM = M_S2 + NROW2, M_ZP = M_ZM + NROW2, M_PB2 = M_ZP + NROW2,
        M_N = M_PB2 + NROW2
    };
    static constexpr size_t a16(size_t x) { return (x + 15) / 16 * 16; }
    static constexpr size_t off_c0 = 0;                                   // Vox [C02] pool 0 (and pool 2 if shared)
    static constexpr size_t off_c1 = off_c0 + (size_t)C02 * K;            // Vox [CAP1] pool 1
    static constexpr size_t off_c2 = WP ? off_c1 + (size_t)CAP1 * K : off_c0;  // Vox [CAP2] pool 2
    static constexpr size_t end_c = WP ? off_c2 + (size_t)CAP2 * K : off_c1 + (size_t)CAP1 * K;
    // u32 arrays.  Warp-per-plane: DEC0 [CAP0], DEC1 [CAP1], DEC2 [CAP2].  CTA-wide: DEC0|DEC2,
    // W01|W23, W02, W03 [C02] and DEC1, W12, W13 [CAP1] (Philox words kept beside the pools).
    static constexpr size_t U_WORDS = WP ? (size_t)CAP0 + CAP1 + CAP2 : (size_t)4 * C02 + (size_t)3 * CAP1;
    static constexpr size_t off_u = end_c;
    static constexpr size_t off_m = a16(off_u + U_WORDS * 4);            // u64 [M_N] row masks
    static constexpr size_t off_rb = off_m + (size_t)M_N * 8;            // u16 rowbases [NROW0 + NROW1 + NROW2]
    static constexpr size_t off_pos = a16(off_rb + (size_t)(NROW0 + NROW1 + NROW2) * 2);  // u16 [CAP0]
    // u16 lists: warp-per-plane L1 [CAP1], L2 [CAP2], LD [NW][LDW]; CTA-wide L [LCAP]
    static constexpr size_t LIST_WORDS = WP ? (size_t)CAP1 + CAP2 + (size_t)NW * LDW : ALIAS ? 0 : (size_t)LCAP;
    static constexpr size_t off_list = a16(off_pos + (size_t)CAP0 * 2);
    static constexpr size_t off_reg = a16(off_list + LIST_WORDS * 2);    // u8 [RPX][RWY][RWZB]
    static constexpr size_t off_nocc = a16(off_reg + (size_t)RPX * RPLANE);  // u64 [NROW0] next item's OCC0
    // u32 tops[4], old and new occupancy words of the interior rows [2][NROW2], delta[S1],
    // diag[PD_N], this item's diag[PD_N], thr
    static constexpr size_t off_tail = off_nocc + (size_t)NROW0 * 8;
    static size_t smem(uint32_t S1, uint32_t thr_words) {
        return off_tail + (size_t)(4 + 2 * NROW2 + S1 + 2 * PD_N + thr_words) * 4;
    }
};

// P.sub != 0 (the pass over spilled bricks): item i is plane group i % sub of
// brick P.items[i / sub], BX planes each, and the item count is
// *P.n_items_dev * sub.
template <int K, int BX, int BY, int NT, int MINB, int CAP0, int CAP1, int CAP2>
__global__ void __launch_bounds__(NT, MINB) brick_step_kernel(ProdParams P) {
    using B = Brick<K, BX, BY, NT, CAP0, CAP1, CAP2>;
    constexpr bool WP = B::WP;
    constexpr int NW = B::NW, WY = B::WY, NROW0 = B::NROW0, NROW1 = B::NROW1, NROW2 = B::NROW2;
    constexpr int RWY = B::RWY, RWZB = B::RWZB, NCH = B::NCH, C02 = B::C02;
    constexpr int LCAP = B::LCAP, LDW = B::LDW;
    extern __shared__ __align__(16) uint8_t smem[];
    Vox<K>* cont0 = reinterpret_cast<Vox<K>*>(smem + B::off_c0);
    Vox<K>* cont1 = reinterpret_cast<Vox<K>*>(smem + B::off_c1);
    Vox<K>* cont2 = reinterpret_cast<Vox<K>*>(smem + B::off_c2);
    uint32_t* U = reinterpret_cast<uint32_t*>(smem + B::off_u);
    uint32_t* DEC0 = U;
    uint32_t* DEC1 = WP ? U + CAP0 : U + 4 * C02;
    uint32_t* DEC2 = WP ? U + CAP0 + CAP1 : U;
    uint32_t* W01 = U + C02;  // Philox words: CTA-wide path only
    uint32_t* W23 = U + C02;
    uint32_t* W02 = U + 2 * C02;
    uint32_t* W03 = U + 3 * C02;
    uint32_t* W12 = U + 4 * C02 + CAP1;
    uint32_t* W13 = U + 4 * C02 + 2 * CAP1;
    uint64_t* msk = reinterpret_cast<uint64_t*>(smem + B::off_m);
    uint64_t* OCC0 = msk + B::M_OCC0;  // occupied at the start of the frame (box rows)
    uint64_t* XM = msk + B::M_XM;      // has x-movers down / up (box rows)
    uint64_t* XP = msk + B::M_XP;
    uint64_t* S1m = msk + B::M_S1;     // X-sweep voxels (may end up empty)
    uint64_t* YM = msk + B::M_YM;
    uint64_t* YP = msk + B::M_YP;
    uint64_t* PB1 = msk + B::M_PB1;    // B(v, 0) evaluated in the X-sweep phase (CTA-wide path)
    uint64_t* S2m = msk + B::M_S2;     // Y-sweep voxels
    uint64_t* ZM = msk + B::M_ZM;
    uint64_t* ZP = msk + B::M_ZP;
    uint64_t* PB2 = msk + B::M_PB2;    // B(v, 0) evaluated in the Y-sweep phase (CTA-wide path)
    uint16_t* RB0 = reinterpret_cast<uint16_t*>(smem + B::off_rb);
    uint16_t* RB1 = RB0 + NROW0;
    uint16_t* RB2 = RB1 + NROW1;
    uint16_t* pos0 = reinterpret_cast<uint16_t*>(smem + B::off_pos);
    uint16_t* Lbase = reinterpret_cast<uint16_t*>(smem + B::off_list);
    uint16_t* L1 = WP ? Lbase : B::ALIAS ? pos0 : Lbase;   // positions of pool 1 entries
    uint16_t* L2 = WP ? Lbase + CAP1 : B::ALIAS ? pos0 : Lbase;  // positions of pool 2 entries
    uint16_t* LD = WP ? Lbase + CAP1 + CAP2 : B::ALIAS ? reinterpret_cast<uint16_t*>(cont1) : Lbase;  // D lists
    uint8_t* reg = smem + B::off_reg;
    uint64_t* nocc = reinterpret_cast<uint64_t*>(smem + B::off_nocc);  // box masks staged for item s_staged
    uint32_t* top = reinterpret_cast<uint32_t*>(smem + B::off_tail);  // [4] pool 0, pool 1, pool 2, D list
    uint32_t* OLDW = top + 4;       // destination occupancy word of each interior row before the frame
    uint32_t* NEWW = OLDW + NROW2;  // and after it
    int32_t* s_delta = reinterpret_cast<int32_t*>(NEWW + NROW2);
    uint32_t* s_diag = reinterpret_cast<uint32_t*>(s_delta + P.T.S1);
    uint32_t* s_bdiag = s_diag + PD_N;  // diagnostics of the current item, kept only if it completes
    uint32_t* s_thr = s_bdiag + PD_N;
    __shared__ uint32_t s_item, s_next, s_staged, s_over;
    __shared__ WorkItem s_nwi;  // item s_staged and its replicate, loaded during the previous item
    __shared__ RepDesc s_nrd;

    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const uint32_t frame = P.stepbuf[P.parity];
    if (blockIdx.x == 0 && tid == 0) {
        for (uint32_t i = 0; i < P.n_reset; i++) P.reset[i] = 0u;
        if (P.advance) P.stepbuf[P.parity ^ 1u] = frame + 1u;
    }
    const uint32_t S1 = P.T.S1, NC = P.T.NC;
    const uint32_t* thr = P.T.thr;
    if (P.thr_smem) {
        const uint32_t nt = NC * NC * S1;
        for (uint32_t i = tid; i < nt; i += NT) s_thr[i] = P.T.thr[i];
        thr = s_thr;
    }
    for (uint32_t s = tid; s < S1; s += NT) s_delta[s] = 0;
    for (int i = tid; i < 2 * PD_N; i += NT) s_diag[i] = 0u;
    const bool zero_order = P.T.n_zero_order != 0u;
    const uint32_t sub = P.sub;
    const uint32_t n_items = P.n_items_dev ? *P.n_items_dev * (sub ? sub : 1u) : P.n_items;

    // Staging of item nx (the next item of this CTA) while the current one
    // computes: its work item and replicate go to shared memory, its region
    // rows are prefetched into L2 (phase A), and its box occupancy masks are
    // read from the bitmap into shared memory (phase B), so that the next
    // item starts without waiting on global memory.
    auto stage_item = [&](uint32_t nx) {
        if (nx >= n_items) return;
        if (tid == NT - 32) {
            s_nwi = P.items[nx];
            s_nrd = P.reps[s_nwi.rep];
        }
        const WorkItem nw = P.items[nx];
        const RepDesc nr = P.reps[nw.rep];
        if ((nr.flags & 1u) || nw.pad[0]) return;
        const int nX = (int)nr.X, nY = (int)nr.Y;
        for (int k = tid; k < B::RPX * RWY; k += NT) {
            const int rp = k / RWY, ry = k - rp * RWY;
            const int x = (int)nw.x0 - 2 + rp, y = (int)nw.y0 - 2 + ry;
            if (x < 0 || x >= nX || y < 0 || y >= nY) continue;
            prefetch_l2(P.region_pad + nr.rbase + ((uint64_t)x * (uint64_t)nY + (uint64_t)y) * nr.Zr + nw.z0);
        }
    };
    // OCC0 row i of item (nw, nr) from the occupancy bitmap: columns c = 0..33 are
    // z = z0 - 1 + c: bit 31 of the word before, the word at z0 (z0 is a multiple
    // of 32), bit 0 of the word after
    auto box_mask = [&](const WorkItem& nw, const RepDesc& nr, int i) -> uint64_t {
        const int p = i / WY, r = i - p * WY, x = (int)nw.x0 - 1 + p, y = (int)nw.y0 - 1 + r;
        if (x < 0 || x >= (int)nr.X || y < 0 || y >= (int)nr.Y) return 0ull;
        const uint32_t* wr = P.osrc + nr.obase + ((uint64_t)x * (uint64_t)nr.Y + (uint64_t)y) * nr.Wz;
        const int wz = (int)(nw.z0 >> 5);
        const uint32_t cur = __ldg(wr + wz);
        const uint32_t prv = wz > 0 ? __ldg(wr + wz - 1) : 0u;
        const uint32_t nx = wz + 1 < (int)nr.Wz ? __ldg(wr + wz + 1) : 0u;
        return (uint64_t)(prv >> 31) | ((uint64_t)cur << 1) | ((uint64_t)(nx & 1u) << 33);
    };

    if (tid == 0) {
        s_item = atomicAdd(P.queue, 1u);
        s_staged = 0xFFFFFFFFu;
        s_over = 0xFFFFFFFFu;
        top[0] = 0u; top[1] = 0u; top[2] = 0u; top[3] = 0u;
    }
    for (;;) {
        __syncthreads();  // s_item and the pool tops are set, the previous item's shared state is dead
        const uint32_t it = s_item;
        if (it >= n_items) break;
        uint32_t nxt = 0u, cidx = 0u;
        bool done = false;  // the item ran to the end of its phases
        int dnp = 0, dny = 0;
        uint64_t orow0 = 0;  // bitmap word of interior row (pi, r) = orow0 + (pi - 1) * Y Wz + (r - 1) * Wz
        uint32_t oY = 0, oWz = 0;
        WorkItem wcur{};
        auto orow = [&](int pi, int r) -> uint64_t {
            return orow0 + ((uint64_t)(pi - 1) * oY + (uint64_t)(r - 1)) * oWz;
        };
        if (tid == 0) nxt = atomicAdd(P.queue, 1u);  // the next item, needed only at the end of this one
        do {
            const bool staged = s_staged == it;  // wi, rd and the box masks are in shared memory
            WorkItem wi = staged ? s_nwi : P.items[sub ? it / sub : it];
            if (sub) {
                const uint32_t xs = wi.x0 + (it % sub) * (uint32_t)BX;
                if (xs >= wi.x1) break;
                wi.x0 = xs;
                wi.x1 = min(wi.x1, xs + (uint32_t)BX);
            }
            wcur = wi;
            const RepDesc rd = staged ? s_nrd : P.reps[wi.rep];
            cidx = rd.counts_index;
            const int X = (int)rd.X, Y = (int)rd.Y, Z = (int)rd.Z, Zr = (int)rd.Zr;
            const int x0 = (int)wi.x0, y0 = (int)wi.y0, z0 = (int)wi.z0;
            const int np = (int)(wi.x1 - wi.x0);  // interior planes inside the lattice
            const int ny = min(BY, Y - y0);       // interior rows inside the lattice
            dnp = np;
            dny = ny;
            oY = (uint32_t)Y;
            oWz = rd.Wz;
            orow0 = rd.obase + ((uint64_t)x0 * (uint64_t)Y + (uint64_t)y0) * rd.Wz + (uint64_t)(z0 >> 5);
            const uint64_t colv = ((1ull << min(32, Z - z0)) - 1ull) << 1;  // interior columns inside
            const uint32_t k0 = rd.seed_lo, k1 = rd.seed_hi;
            // one region code over the whole region window (a one-region replicate, or a brick whose
            // window the host found to hold one region): no region rows are staged
            const uint32_t ucode = (rd.flags & 1u) ? 1u : wi.pad[0];
            const bool flat = ucode != 0u;
            const uint8_t* src = P.src + rd.base * K;
            uint8_t* dst = P.dst + rd.base * K;
            const uint8_t* rpad = P.region_pad + rd.rbase;
            const uint8_t* resv = P.reservoir ? P.reservoir + rd.base : nullptr;
            const bool all_react = zero_order || resv != nullptr;
            const uint32_t YZ = (uint32_t)Y * (uint32_t)Z;
            const uint32_t* quiet = P.T.quiet + (size_t)rd.counts_index * S1 * P.T.QS;
            const float* one_rep = P.T.one + (size_t)rd.counts_index * S1 * 3;
            auto lin = [&](int x, int y, int z) -> uint32_t {
                return ((uint32_t)x * (uint32_t)Y + (uint32_t)y) * (uint32_t)Z + (uint32_t)z;
            };
            // region code of box voxel (p, r, c); p, r, c may step one outside the box
            auto code = [&](int p, int r, int c) -> uint32_t {
                if (flat) {
                    const int x = x0 - 1 + p, y = y0 - 1 + r, z = z0 - 1 + c;
                    return (x >= 0 && x < X && y >= 0 && y < Y && z >= 0 && z < Z) ? ucode : 0u;
                }
                return reg[((p + 1) * RWY + (r + 1)) * RWZB + c + 1];
            };
            auto trow = [&](uint32_t a, uint32_t b) -> const uint32_t* { return thr + ((size_t)a * NC + b) * S1; };
            // pool index of column c of a row with mask m and rowbase rb (the bit must be set)
            auto rank = [](uint64_t m, uint32_t rb, int c) -> uint32_t {
                return rb + (uint32_t)__popcll(m & ((1ull << c) - 1ull));
            };
            // Appends the set bits of one row mask per lane (row index `row`, only when `valid`) to
            // list `out` of capacity `cap`.  With t >= 0 the warp reserves a contiguous range of
            // pool t with one shared atomic (top[t]); with t < 0 the range starts at 0 (a list of
            // this warp's own).  Sets base and total of the warp's range and returns the lane's row
            // base.  Nothing is written past `cap`.
            auto append_list = [&](uint64_t m, int row, bool valid, int t, uint32_t cap, uint16_t* out,
                                   uint32_t& base, uint32_t& total) -> uint32_t {
                const uint32_t c = valid ? (uint32_t)__popcll(m) : 0u;
                uint32_t incl = c;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += u;
                }
                total = __shfl_sync(0xffffffffu, incl, 31);
                base = 0u;
                if (t >= 0 && lane == 0 && total) base = atomicAdd(top + t, total);
                base = __shfl_sync(0xffffffffu, base, 0);
                const uint32_t rb = base + incl - c;
                uint64_t bits = valid ? m : 0ull;
                uint32_t o = rb;
                while (bits) {
                    const int col = __ffsll((long long)bits) - 1;
                    bits &= bits - 1ull;
                    if (o < cap) out[o] = (uint16_t)((row << 6) | col);
                    o++;
                }
                return rb;
            };
            auto spill = [&]() {
                if (tid == 0) {
                    if (P.spill) {
                        const uint32_t at = atomicAdd(P.n_spill, 1u);
                        P.spill[at] = wi;
                        s_diag[PD_DENSE_BRICKS] += 1u;
                    } else {
                        s_diag[PD_LOST_BRICKS] += 1u;  // cannot happen with full-capacity pools
                    }
                }
            };

            // the next item's box masks, by the highest threads, and an L2 prefetch of the slots of
            // its occupied voxels (called after a barrier that follows stage_item, which loads
            // s_nwi / s_nrd)
            auto stage_masks = [&]() {
                if (sub != 0u || s_next >= n_items) return;
                for (int i = NT - 1 - tid; i < NROW0; i += NT) {
                    const uint64_t m = box_mask(s_nwi, s_nrd, i);
                    nocc[i] = m;
                    if (m) {
                        const int p = i / WY, r = i - p * WY;
                        const uint64_t vrow = s_nrd.base + ((uint64_t)((int)s_nwi.x0 - 1 + p) * s_nrd.Y +
                                                            (uint64_t)((int)s_nwi.y0 - 1 + r)) * s_nrd.Z;
                        for (uint64_t b = m; b; b &= b - 1ull)
                            prefetch_l2(P.src + (vrow + (uint64_t)((int)s_nwi.z0 - 1 + __ffsll((long long)b) - 1)) * K);
                    }
                }
                if (tid == 0) s_staged = s_next;
            };

            // ---------------- L: box occupancy from the bitmap ----------------
            if (!flat) {
                for (int c = tid; c < NCH; c += NT) {
                    const int rp = c / (RWY * 3), rem = c - rp * (RWY * 3), ry = rem / 3, cz = rem - ry * 3;
                    const int x = x0 - 2 + rp, y = y0 - 2 + ry, zp = z0 + 16 * cz;  // zp: padded column (z + 2)
                    const bool ok = x >= 0 && x < X && y >= 0 && y < Y && zp + 16 <= Zr;
                    const uint8_t* g = ok ? rpad + ((uint64_t)x * (uint64_t)Y + (uint64_t)y) * (uint64_t)Zr + zp : rpad;
                    cp_async<16>(reg + (rp * RWY + ry) * RWZB + 16 * cz, g, ok);
                }
            }
            cp_async_commit();
            for (int i = tid; i < NROW0; i += NT) { XM[i] = 0ull; XP[i] = 0ull; }
            for (int i = tid; i < NROW1; i += NT) { YM[i] = 0ull; YP[i] = 0ull; PB1[i] = 0ull; }
            for (int i = tid; i < NROW2; i += NT) { ZM[i] = 0ull; ZP[i] = 0ull; PB2[i] = 0ull; }
            // box rows from the input occupancy bitmap: lane l of warp w takes row 32 w + l
            for (int ib = w * 32; ib < NROW0; ib += NT) {
                const int i = ib + lane;
                uint64_t m = 0ull;
                if (i < NROW0) m = staged ? nocc[i] : box_mask(wi, rd, i);
                // reserve this warp's pool range, then list the occupied voxels of each row
                uint32_t base, total;
                const uint32_t rb = append_list(m, i, i < NROW0, 0, (uint32_t)CAP0, pos0, base, total);
                if (i < NROW0) {
                    OCC0[i] = m;
                    RB0[i] = (uint16_t)min(rb, 65535u);
                }
            }
            if (tid == 0) s_next = nxt;
            cp_async_wait<0>();
            __syncthreads();
            if (top[0] > (uint32_t)CAP0) {
                spill();
                break;
            }
            if (top[0] == 0u && !all_react) {
                // Empty box: no particle can reach the interior and no reaction can fire, so the
                // interior ends the frame empty.  Only the destination's stale voxels need zeros.
                for (int j = w; j < NROW2; j += NW) {
                    const int pi = j / BY + 1, r = j - (pi - 1) * BY + 1;
                    uint32_t oldw = 0u;
                    if (pi <= np && r <= ny && lane == 0) oldw = P.odst[orow(pi, r)];
                    oldw = __shfl_sync(0xffffffffu, oldw, 0);
                    if ((oldw >> lane) & 1u)
                        st_vox_g<K>(dst + (uint64_t)lin(x0 - 1 + pi, y0 - 1 + r, z0 + lane) * K, vox_zero<K>());
                    if (lane == 0) NEWW[j] = 0u;
                }
                if (sub == 0u) stage_item(s_next);
                __syncthreads();
                stage_masks();
                done = true;
                break;
            }

            // ---------------- A: x-decisions of the occupied box voxels ----------------
            {
                const uint32_t n0 = top[0];
                for (uint32_t e = (uint32_t)tid; e < n0; e += NT) {
                    const uint32_t ps = pos0[e];
                    const int i = (int)(ps >> 6), c = (int)(ps & 63u), p = i / WY, r = i - p * WY;
                    const uint32_t v = lin(x0 - 1 + p, y0 - 1 + r, z0 - 1 + c);
                    const Vox<K> own = ld_vox_g<K>(src + (uint64_t)v * K);  // occupied: fetch its slots
                    const U4 b0 = d_philox(v, frame, 0u, 0u, k0, k1);
                    cont0[e] = own;
                    if (!WP) {
                        W01[e] = b0.y;
                        W02[e] = b0.z;
                        W03[e] = b0.w;
                    }
                    const uint32_t rs = code(p, r, c);
                    const uint32_t d = decide_moves<K>(own, v, frame, 0u, trow(rs, code(p - 1, r, c)),
                                                       trow(rs, code(p + 1, r, c)), k0, k1, b0.x);
                    DEC0[e] = d;
                    if (d & 0xFFFFu) atomicOr(reinterpret_cast<unsigned long long*>(XM + i), 1ull << c);
                    if (d >> 16) atomicOr(reinterpret_cast<unsigned long long*>(XP + i), 1ull << c);
                }
            }
            // the destination's occupancy words of the interior rows (read now, used in phase D)
            for (int j = NT - 1 - tid; j < NROW2; j += NT) {
                const int pi = j / BY + 1, r = j - (pi - 1) * BY + 1;
                OLDW[j] = (pi <= np && r <= ny) ? P.odst[orow(pi, r)] : 0u;
                NEWW[j] = 0u;
            }
            if (sub == 0u) stage_item(s_next);
            __syncthreads();

            // ---------------- the item bodies of the three sweeps ----------------
            // X sweep of voxel (interior plane pi, row r, column c) into pool 1 entry e1; y-decisions
            auto b_item = [&](uint32_t e1, uint32_t ps) {
                const int jj = (int)(ps >> 6), c = (int)(ps & 63u);
                const int pi = jj / WY + 1, r = jj - (pi - 1) * WY, i0 = pi * WY + r;
                const uint64_t bc = 1ull << c;
                Vox<K> own = vox_zero<K>(), lo = vox_zero<K>(), hi = vox_zero<K>();
                uint32_t dme = 0u, dlo = 0u, dhi = 0u;
                int e0 = -1;
                {
                    const uint64_t o = OCC0[i0];
                    if (o & bc) { e0 = (int)rank(o, RB0[i0], c); own = cont0[e0]; dme = DEC0[e0]; }
                }
                {
                    const uint64_t o = OCC0[i0 - WY];
                    if (o & bc) { const uint32_t e = rank(o, RB0[i0 - WY], c); lo = cont0[e]; dlo = DEC0[e]; }
                }
                {
                    const uint64_t o = OCC0[i0 + WY];
                    if (o & bc) { const uint32_t e = rank(o, RB0[i0 + WY], c); hi = cont0[e]; dhi = DEC0[e]; }
                }
                const uint32_t v = lin(x0 - 1 + pi, y0 - 1 + r, z0 - 1 + c);
                const Vox<K> r1 = combine<K>(own, dme, lo, dlo, hi, dhi, v, v - YZ, v + YZ, frame, 0u);
                cont1[e1] = r1;
                uint32_t d = 0u;
                if (!vox_empty<K>(r1)) {
                    uint32_t wy;
                    if (!WP && e0 >= 0) {
                        wy = W01[e0];
                    } else {
                        const U4 b0 = d_philox(v, frame, 0u, 0u, k0, k1);
                        wy = b0.y;
                        if (!WP) {
                            W12[e1] = b0.z;
                            W13[e1] = b0.w;
                            atomicOr(reinterpret_cast<unsigned long long*>(PB1 + jj), bc);
                        }
                    }
                    const uint32_t rs = code(pi, r, c);
                    d = decide_moves<K>(r1, v, frame, 1u, trow(rs, code(pi, r - 1, c)), trow(rs, code(pi, r + 1, c)), k0,
                                        k1, wy);
                    if (d & 0xFFFFu) atomicOr(reinterpret_cast<unsigned long long*>(YM + jj), bc);
                    if (d >> 16) atomicOr(reinterpret_cast<unsigned long long*>(YP + jj), bc);
                }
                DEC1[e1] = d;
            };
            // Y sweep of voxel (pi, interior row r, c) into pool 2 entry e2; z-decisions
            auto c_item = [&](uint32_t e2, uint32_t ps) {
                const int jj = (int)(ps >> 6), c = (int)(ps & 63u);
                const int pi = jj / BY + 1, r = jj - (pi - 1) * BY + 1, j1 = (pi - 1) * WY + r;
                const uint64_t bc = 1ull << c;
                Vox<K> own = vox_zero<K>(), lo = vox_zero<K>(), hi = vox_zero<K>();
                uint32_t dme = 0u, dlo = 0u, dhi = 0u;
                int e1 = -1;
                {
                    const uint64_t o = S1m[j1];
                    if (o & bc) { e1 = (int)rank(o, RB1[j1], c); own = cont1[e1]; dme = DEC1[e1]; }
                }
                {
                    const uint64_t o = S1m[j1 - 1];
                    if (o & bc) { const uint32_t e = rank(o, RB1[j1 - 1], c); lo = cont1[e]; dlo = DEC1[e]; }
                }
                {
                    const uint64_t o = S1m[j1 + 1];
                    if (o & bc) { const uint32_t e = rank(o, RB1[j1 + 1], c); hi = cont1[e]; dhi = DEC1[e]; }
                }
                const uint32_t v = lin(x0 - 1 + pi, y0 - 1 + r, z0 - 1 + c);
                const Vox<K> r2 = combine<K>(own, dme, lo, dlo, hi, dhi, v, v - (uint32_t)Z, v + (uint32_t)Z, frame, 1u);
                uint32_t d = 0u;
                if (!vox_empty<K>(r2)) {
                    uint32_t wz;
                    const int i0 = pi * WY + r;
                    const uint64_t o0 = OCC0[i0];
                    if (!WP && (o0 & bc)) {
                        wz = W02[rank(o0, RB0[i0], c)];
                    } else if (!WP && (PB1[j1] & bc)) {
                        wz = W12[e1];
                    } else {
                        const U4 b0 = d_philox(v, frame, 0u, 0u, k0, k1);
                        wz = b0.z;
                        if (!WP) {
                            W23[e2] = b0.w;
                            atomicOr(reinterpret_cast<unsigned long long*>(PB2 + jj), bc);
                        }
                    }
                    const uint32_t rs = code(pi, r, c);
                    d = decide_moves<K>(r2, v, frame, 2u, trow(rs, code(pi, r, c - 1)), trow(rs, code(pi, r, c + 1)), k0,
                                        k1, wz);
                    if (d & 0xFFFFu) atomicOr(reinterpret_cast<unsigned long long*>(ZM + jj), bc);
                    if (d >> 16) atomicOr(reinterpret_cast<unsigned long long*>(ZP + jj), bc);
                }
                cont2[e2] = r2;
                DEC2[e2] = d;
            };
            // Z sweep, reactions and store of interior voxel (pi, r, c)
            auto d_item = [&](uint32_t ps) {
                const int jj = (int)(ps >> 6), c = (int)(ps & 63u);
                const int pi = jj / BY + 1, r = jj - (pi - 1) * BY + 1, j1 = (pi - 1) * WY + r;
                const uint64_t o2 = S2m[jj];
                const uint32_t rb = RB2[jj];
                Vox<K> own = vox_zero<K>(), lo = vox_zero<K>(), hi = vox_zero<K>();
                uint32_t dme = 0u, dlo = 0u, dhi = 0u;
                int e2 = -1;
                if ((o2 >> c) & 1ull) { e2 = (int)rank(o2, rb, c); own = cont2[e2]; dme = DEC2[e2]; }
                if ((o2 >> (c - 1)) & 1ull) { const uint32_t e = rank(o2, rb, c - 1); lo = cont2[e]; dlo = DEC2[e]; }
                if ((o2 >> (c + 1)) & 1ull) { const uint32_t e = rank(o2, rb, c + 1); hi = cont2[e]; dhi = DEC2[e]; }
                const uint32_t v = lin(x0 - 1 + pi, y0 - 1 + r, z0 - 1 + c);
                Vox<K> r3 = combine<K>(own, dme, lo, dlo, hi, dhi, v, v - 1u, v + 1u, frame, 2u);
                const uint32_t rv = resv ? (uint32_t)resv[v] : 0u;
                if (rv != 0u || zero_order || !vox_empty<K>(r3)) {
                    uint32_t w3;
                    const uint64_t bc = 1ull << c;
                    const int i0 = pi * WY + r;
                    const uint64_t o0 = OCC0[i0];
                    if (!WP && (o0 & bc)) w3 = W03[rank(o0, RB0[i0], c)];
                    else if (!WP && (PB1[j1] & bc)) w3 = W13[rank(S1m[j1], RB1[j1], c)];
                    else if (!WP && (PB2[jj] & bc)) w3 = W23[e2];
                    else w3 = d_philox(v, frame, 0u, 0u, k0, k1).w;
                    const bool calm = rv == 0u && !zero_order &&
                                      calm_voxel<K>(r3, w3, quiet, P.T.QS, one_rep, P.T.g23 + 2 * rd.counts_index,
                                                P.T.a2 ? P.T.a2 + (size_t)rd.counts_index * S1 * S1 : nullptr, P.T.tau);
                    if (!calm)
                        react_voxel<K>(r3, rv, v, frame, k0, k1, rd.rate_mult, rd.counts_index, P.T, s_delta, s_bdiag,
                                       w3);
                }
                if (!vox_empty<K>(r3)) {
                    st_vox_g<K>(dst + (uint64_t)v * K, r3);
                    atomicOr(NEWW + jj, 1u << (c - 1));
                } else if ((OLDW[jj] >> (c - 1)) & 1u) {
                    st_vox_g<K>(dst + (uint64_t)v * K, vox_zero<K>());
                }
            };
            // D rows: stale voxels that end the frame empty get zero stores (coalesced per row);
            // returns the row's D mask (row_in: the row lies inside the lattice)
            auto d_row = [&](int j2, bool valid, bool& row_in) -> uint64_t {
                row_in = false;
                uint64_t s3 = 0ull;
                uint32_t oldw = 0u;
                if (valid) {
                    const int pi = j2 / BY + 1, r = j2 - (pi - 1) * BY + 1;
                    if (pi <= np && r <= ny) {
                        row_in = true;
                        // own voxel, +z movers of the column before, -z movers of the column after
                        s3 = all_react ? colv : ((S2m[j2] | (ZP[j2] << 1) | (ZM[j2] >> 1)) & colv);
                        oldw = OLDW[j2];
                    }
                }
                const uint32_t zb = oldw & ~(uint32_t)(s3 >> 1);  // bit b: column b + 1
                for (uint32_t act = __ballot_sync(0xffffffffu, zb != 0u); act; act &= act - 1u) {
                    const int k = __ffs(act) - 1;
                    const uint32_t zk = __shfl_sync(0xffffffffu, zb, k);
                    const int jk = __shfl_sync(0xffffffffu, j2, k);
                    const int pi = jk / BY + 1, r = jk - (pi - 1) * BY + 1;
                    if ((zk >> lane) & 1u)
                        st_vox_g<K>(dst + (uint64_t)lin(x0 - 1 + pi, y0 - 1 + r, z0 + lane) * K, vox_zero<K>());
                }
                return s3;
            };

            if constexpr (WP) {
                // ---------------- B, C, D per warp: warp w owns interior plane w + 1 ----------------
                const int pi = w + 1;
                const bool plane_in = pi <= np;
                bool ok = true;
                {
                    const int j = w * WY + lane;  // lanes < WY: the plane's rows
                    const bool valid = lane < WY;
                    uint64_t s1 = 0ull;
                    if (valid && plane_in) {
                        const int i0 = pi * WY + lane;
                        s1 = OCC0[i0] | XP[i0 - WY] | XM[i0 + WY];
                    }
                    uint32_t base, total;
                    const uint32_t rb = append_list(s1, j, valid, 1, (uint32_t)CAP1, L1, base, total);
                    if (valid) {
                        S1m[j] = s1;
                        RB1[j] = (uint16_t)min(rb, 65535u);
                    }
                    if (base + total > (uint32_t)CAP1) ok = false;
                    __syncwarp();
                    if (ok)
                        for (uint32_t e1 = base + lane; e1 < base + total; e1 += 32) b_item(e1, L1[e1]);
                }
                __syncwarp();
                if (ok) {
                    const int j2 = w * BY + lane;  // lanes < BY: the plane's interior rows
                    const bool valid = lane < BY;
                    uint64_t s2 = 0ull;
                    if (valid && plane_in && lane + 1 <= ny) {
                        const int j1 = w * WY + lane + 1;
                        s2 = S1m[j1] | YP[j1 - 1] | YM[j1 + 1];
                    }
                    uint32_t base, total;
                    const uint32_t rb = append_list(s2, j2, valid, 2, (uint32_t)CAP2, L2, base, total);
                    if (valid) {
                        S2m[j2] = s2;
                        RB2[j2] = (uint16_t)min(rb, 65535u);
                    }
                    if (base + total > (uint32_t)CAP2) ok = false;
                    __syncwarp();
                    if (ok)
                        for (uint32_t e2 = base + lane; e2 < base + total; e2 += 32) c_item(e2, L2[e2]);
                }
                __syncwarp();
                if (ok) {
                    const int j2 = w * BY + lane;
                    bool row_in;
                    const uint64_t s3 = d_row(j2, lane < BY, row_in);
                    uint16_t* Lw = LD + w * LDW;
                    uint32_t base, total;
                    append_list(s3, j2, lane < BY && row_in, -1, (uint32_t)LDW, Lw, base, total);
                    __syncwarp();
                    for (uint32_t t = lane; t < total; t += 32) d_item(Lw[t]);
                }
                if (!ok && lane == 0) s_over = it;
                stage_masks();
            } else {
                // ---------------- B, C, D CTA-wide, each list built before a barrier ----------------
                if (w * 32 < NROW1) {
                    const int j = w * 32 + lane;
                    const bool valid = j < NROW1;
                    uint64_t s1 = 0ull;
                    if (valid) {
                        const int pi = j / WY + 1, r = j - (pi - 1) * WY;
                        if (pi <= np) {
                            const int i0 = pi * WY + r;
                            // own voxel occupied, or +x movers of the plane below / -x movers of the plane above
                            s1 = OCC0[i0] | XP[i0 - WY] | XM[i0 + WY];
                        }
                    }
                    uint32_t base, total;
                    const uint32_t rb = append_list(s1, j, valid, 1, (uint32_t)CAP1, L1, base, total);
                    if (valid) {
                        S1m[j] = s1;
                        RB1[j] = (uint16_t)min(rb, 65535u);
                    }
                }
                __syncthreads();
                const uint32_t n1 = top[1];
                if (n1 > (uint32_t)CAP1) {
                    spill();
                    break;
                }
                for (uint32_t e1 = (uint32_t)tid; e1 < n1; e1 += NT) b_item(e1, L1[e1]);
                stage_masks();
                __syncthreads();
                if (w * 32 < NROW2) {
                    const int j2 = w * 32 + lane;
                    const bool valid = j2 < NROW2;
                    uint64_t s2 = 0ull;
                    if (valid) {
                        const int pi = j2 / BY + 1, r = j2 - (pi - 1) * BY + 1;
                        if (pi <= np && r <= ny) {
                            const int j1 = (pi - 1) * WY + r;
                            // own voxel, +y movers of the row below, -y movers of the row above
                            s2 = S1m[j1] | YP[j1 - 1] | YM[j1 + 1];
                        }
                    }
                    uint32_t base, total;
                    const uint32_t rb = append_list(s2, j2, valid, 2, (uint32_t)CAP2, L2, base, total);
                    if (valid) {
                        S2m[j2] = s2;
                        RB2[j2] = (uint16_t)min(rb, 65535u);
                    }
                }
                __syncthreads();
                const uint32_t n2 = top[2];
                if (n2 > (uint32_t)CAP2) {
                    spill();
                    break;
                }
                for (uint32_t e2 = (uint32_t)tid; e2 < n2; e2 += NT) c_item(e2, L2[e2]);
                __syncthreads();
                if (all_react) {
                    // every interior voxel inside the lattice is stepped (reservoir or zero-order
                    // reactions), so none is left stale and no list is needed
                    for (uint32_t t = (uint32_t)tid; t < (uint32_t)NROW2 * 32u; t += NT) {
                        const int j2 = (int)(t >> 5), c = (int)(t & 31u) + 1;
                        const int pi = j2 / BY + 1, r = j2 - (pi - 1) * BY + 1;
                        if (pi <= np && r <= ny && ((colv >> c) & 1ull)) d_item((uint32_t)((j2 << 6) | c));
                    }
                } else {
                    if (w * 32 < NROW2) {
                        const int j2 = w * 32 + lane;
                        const bool valid = j2 < NROW2;
                        bool row_in;
                        const uint64_t s3 = d_row(j2, valid, row_in);
                        uint32_t base, total;
                        append_list(s3, j2, valid && row_in, 3, (uint32_t)LCAP, LD, base, total);
                    }
                    __syncthreads();
                    const uint32_t nd = top[3];
                    for (uint32_t t = (uint32_t)tid; t < nd; t += NT) d_item(LD[t]);
                }
            }
            done = true;
        } while (0);
        __syncthreads();
        const bool kept = done && s_over != it;
        if (done && !kept) {
            // a warp's pool range overflowed after other warps stored their planes: the second pass
            // redoes the whole brick (the stores already made are the same values it writes)
            if (tid == 0) {
                const uint32_t at = atomicAdd(P.n_spill, 1u);
                P.spill[at] = wcur;
                s_diag[PD_DENSE_BRICKS] += 1u;
            }
        }
        if (kept) {
            // the interior rows' new occupancy words (each interior row is one word: z0 % 32 == 0)
            for (int j = tid; j < NROW2; j += NT) {
                const int pi = j / BY + 1, r = j - (pi - 1) * BY + 1;
                if (pi <= dnp && r <= dny) P.odst[orow(pi, r)] = NEWW[j];
            }
            for (int i = tid; i < PD_N; i += NT)
                if (s_bdiag[i]) s_diag[i] += s_bdiag[i];
        }
        for (uint32_t s = tid; s < S1; s += NT) {
            const int32_t dlt = s_delta[s];
            if (dlt) {
                if (kept) atomicAdd(P.counts + (size_t)cidx * S1 + s, (unsigned long long)(long long)dlt);
                s_delta[s] = 0;
            }
        }
        for (int i = tid; i < PD_N; i += NT) s_bdiag[i] = 0u;
        if (tid == 0) {
            s_item = nxt;
            top[0] = 0u; top[1] = 0u; top[2] = 0u; top[3] = 0u;
        }
    }
    __syncthreads();
    for (int i = tid; i < PD_N; i += NT)
        if (s_diag[i]) atomicAdd(P.diag + i, s_diag[i]);
}

}  // namespace cellsim
