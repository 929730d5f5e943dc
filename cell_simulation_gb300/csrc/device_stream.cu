// device_stream.cu — the passes of the sweep-stream step (three launches, or
// two with the Y and Z sweeps fused) and their launchers (see
// stream_kernel.cuh for the scheme).
#include <cuda_runtime.h>

#include <type_traits>

#include "cuda_check.h"
#include "stream_kernel.cuh"

namespace cellsim {

namespace {

// Per-lane words of a warp's current group, kept in shared memory so that
// the lane running an item can read the words of the item's lane.
enum : int {
    // fields are stored in pairs (even, odd) read together: lane i's pair p is the uint2 at p * 32 + i
    F_Y, F_KK,        // the lane's row and word
    F_VROW, F_CODE,   // first voxel of the lane's row, the word's uniform region code (or 0)
    F_OBS, F_OWK,     // this pass's base and work
    F_BS, F_WK,       // own word: base and work of the producing pass
    F_LBS, F_LWK,     // lower neighbour's word (previous word of the row in the Z sweep): base, work
    F_HBS, F_HWK,     // upper neighbour's word (next word of the row in the Z sweep): base, work
    F_LOCC, F_LP,     // lower neighbour: content, movers up
    F_HOCC, F_HM,     // upper neighbour: content, movers down
    F_M, F_P,         // own word: movers down / up
    F_OCC, F_OLD,     // own content, old destination word
    NF
};
// u32 index of field F of lane i
__device__ __forceinline__ int fi(int F, int i) { return (F >> 1) * 64 + 2 * i + (F & 1); }
constexpr int LIST = 1024;  // one group holds at most 32 words x 32 bits
// Voxels of a group's Z sweep whose SSA the warp runs itself, after the group's items: a count
// (padded to 16 bytes), then entries of two uint4 (content; Philox word, reservoir, record, item)
constexpr int PEND = 8;
constexpr int PEND_WORDS = 4 + 8 * PEND;

}  // namespace

// u32 words of one warp's shared-memory area: fields, three accumulators and
// the item list (u16)
__host__ __device__ constexpr size_t stream_warp_words() { return (size_t)NF * 32 + 96 + LIST / 2 + PEND_WORDS; }

// Records of a group's Y sweep (its z-decisions) that the fused pass keeps in the warp's shared
// memory for its Z sweep, instead of a round trip through L2: the first 96 of the group's records
// at three blocks per SM (C3: 0.1480 -> 0.1462 ms per frame in the multi-frame form, the two-launch
// form unchanged); none at four blocks per SM, where the smaller shared memory left per block cost
// the 512-replicate ensemble more (0.352 -> 0.357 ms with 32) than the staging saved; 0 for the
// other passes.
__host__ __device__ constexpr int stage_recs(int PASS, int MINB) { return PASS == PASS_YZ && MINB < 4 ? 96 : 0; }

size_t stream_smem(int NT, uint32_t S1, uint32_t thr_words, int recs) {
    (void)S1;
    return ((size_t)(NT / 32) * (stream_warp_words() + (size_t)recs * 8) + PD_N + thr_words) * 4;
}

// NC: the records were written by an earlier launch (read-only path); else
// by this launch (the fused Y and Z sweeps), read coherently through L2.
template <int K, bool NC = true>
__device__ __forceinline__ void rec_load(const uint4* rec, uint32_t i, Vox<K>& c, uint4& t) {
    // one 32-byte access per record (record buffers come from cudaMalloc, records are 32 bytes)
    const uint4* p = rec + 2 * (size_t)i;
    uint32_t a0, a1, a2, a3;
    if constexpr (NC)
        asm volatile("ld.global.nc.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                     : "=r"(a0), "=r"(a1), "=r"(a2), "=r"(a3), "=r"(t.x), "=r"(t.y), "=r"(t.z), "=r"(t.w)
                     : "l"(p));
    else
        asm volatile("ld.global.cg.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                     : "=r"(a0), "=r"(a1), "=r"(a2), "=r"(a3), "=r"(t.x), "=r"(t.y), "=r"(t.z), "=r"(t.w)
                     : "l"(p)
                     : "memory");
    c.w[0] = (uint64_t)a0 | ((uint64_t)a1 << 32);
    if constexpr (K == 16) c.w[1] = (uint64_t)a2 | ((uint64_t)a3 << 32);
}

template <int K>
__device__ __forceinline__ void rec_store(uint4* rec, uint32_t i, const Vox<K>& c, const uint4& t) {
    ulonglong4_32a v;
    v.x = c.w[0];
    v.y = K == 16 ? c.w[K / 8 - 1] : 0ull;
    v.z = (uint64_t)t.x | ((uint64_t)t.y << 32);
    v.w = (uint64_t)t.z | ((uint64_t)t.w << 32);
    *reinterpret_cast<ulonglong4_32a*>(rec + 2 * (size_t)i) = v;
}

__device__ __forceinline__ uint32_t below(uint32_t m, uint32_t bit) { return (uint32_t)__popc(m & (bit - 1u)); }

// Programmatic dependent launch: the passes are launched so that a launch's
// blocks may start while the previous launch drains.  Each kernel lets the
// next one launch at once, stages its constant tables, and waits for the
// previous launch to complete (and its memory to be visible) before it reads
// or writes anything the previous launches produced or read.  Without a
// programmatic dependency the wait returns at once.
__device__ __forceinline__ void allow_next_launch() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }
__device__ __forceinline__ void wait_previous_launch() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }

// The shared memory of one warp and what else a word group's passes need from its launch.
struct WarpArea {
    uint32_t* f;          // [NF][32] per-lane fields
    uint32_t* acc;        // [3][32]: content, movers down, movers up
    uint16_t* list;       // the group's items
    uint32_t* pend;       // [PEND_WORDS] voxels set aside for the warp's SSA
    uint32_t* s_diag;     // [PD_N] the block's diagnostic counters
    const uint32_t* thr;  // threshold table (shared memory or global)
    uint32_t gw;          // the warp's index in the launch
    int lane;
    uint4* stage;         // [2 n_stage] the fused pass's staged z-decision records
    uint32_t n_stage;
};

// A word written earlier: by an earlier launch (plain load), or (COH) possibly earlier in this
// launch by another warp, read through L2.
template <bool COH>
__device__ __forceinline__ uint32_t ldw(const uint32_t* p) {
    if constexpr (COH) return __ldcg(p);
    else return *p;
}

// Pass PASS (0..3, or PASS_YZ) of word group g in frame `frame`.  COH: the persistent multi-frame
// form, where the words and records a pass reads may have been written earlier in the same
// launch, so they are read through L2; par = 1 selects the lattice buffers of frame parity 1
// (in_occ1, odst1, dst1) there.  The per-pass launches pass par = 0.
template <int K, int PASS, bool COH>
__device__ __forceinline__ void stream_group(const StreamParams& SP, const WarpArea& A, uint32_t g, uint32_t frame,
                                             uint32_t par) {
    const ProdParams& P = SP.P;
    uint32_t* const f = A.f;
    uint32_t* const acc = A.acc;
    uint16_t* const list = A.list;
    uint32_t* const pend = A.pend;
    uint32_t* const s_diag = A.s_diag;
    const uint32_t* const thr = A.thr;
    const uint32_t gw = A.gw;
    const int lane = A.lane;
    const uint32_t S1 = P.T.S1, NC = P.T.NC;
    // field pair (F, F + 1) of lane i, F even
    auto fpair = [&](int F, int i) -> uint2 { return reinterpret_cast<const uint2*>(f)[(F >> 1) * 32 + i]; };
    const bool zero_order = P.T.n_zero_order != 0u;
    const bool all_react = zero_order || P.reservoir != nullptr;
    auto trow = [&](uint32_t a, uint32_t b) -> const uint32_t* { return thr + (a * NC + b) * S1; };  // < 2^32 entries
    const uint32_t* const in_occ = par ? SP.in_occ1 : SP.in.occ;
    uint32_t* const odst = par ? SP.odst1 : P.odst;
    uint8_t* const dst = par ? SP.dst1 : P.dst;
    // the fused pass's z-decision records: the group's first A.n_stage in shared memory, the rest
    // in rec_mid (read through L2: this launch wrote them)
    auto mid_store = [&](uint32_t ri, uint32_t rb, const Vox<K>& c, const uint4& t) {
        const uint32_t rel = ri - rb;
        if (rel < A.n_stage) {
            uint4 a;
            a.x = (uint32_t)c.w[0];
            a.y = (uint32_t)(c.w[0] >> 32);
            a.z = K == 16 ? (uint32_t)c.w[K / 8 - 1] : 0u;
            a.w = K == 16 ? (uint32_t)(c.w[K / 8 - 1] >> 32) : 0u;
            A.stage[2 * rel] = a;
            A.stage[2 * rel + 1] = t;
        } else {
            rec_store<K>(SP.rec_mid, ri, c, t);
        }
    };
    auto mid_load = [&](uint32_t ri, uint32_t rb, Vox<K>& c, uint4& t) {
        const uint32_t rel = ri - rb;
        if (rel < A.n_stage) {
            const uint4 a = A.stage[2 * rel];
            t = A.stage[2 * rel + 1];
            c.w[0] = (uint64_t)a.x | ((uint64_t)a.y << 32);
            if constexpr (K == 16) c.w[K / 8 - 1] = (uint64_t)a.z | ((uint64_t)a.w << 32);
        } else {
            rec_load<K, false>(SP.rec_mid, ri, c, t);
        }
    };
    const WordGroup G = SP.groups[g];
    const RepDesc rd = P.reps[G.rep];
    const int X = (int)rd.X, Y = (int)rd.Y, Z = (int)rd.Z;
    const uint32_t Wz = rd.Wz;
    const int nk = (int)G.nk;
    const bool valid = lane < (int)(G.nrows * G.nk);
    const int yl = valid ? lane / nk : 0;
    const int x = (int)G.x, y = (int)G.y0 + yl, kk = (int)G.k0 + (lane - yl * nk);
    const uint64_t wo = rd.obase + ((uint64_t)x * (uint64_t)Y + (uint64_t)y) * Wz + (uint64_t)kk;
    const int zb = 32 * kk;
    const uint32_t colm = !valid ? 0u : (Z - zb >= 32 ? 0xFFFFFFFFu : ((1u << (Z - zb)) - 1u));
    // One sweep PP of the group.  CH (PASS_YZ): the Y sweep leaves its output words in this
    // warp's shared memory and its records in rec_mid, and the Z sweep starts from them.
    auto sweep = [&](auto pass_c, auto chain_c) {
        constexpr int PP = decltype(pass_c)::value;
        constexpr bool CH = decltype(chain_c)::value;
        const uint4* const rin = (CH && PP == 3) ? SP.rec_mid : SP.rec_in;
        uint4* const rout = (CH && PP == 2) ? SP.rec_mid : SP.rec_out;
        uint32_t work = 0u, old = 0u, moving = 0u;  // moving: bits whose content changes along the axis
        uint32_t own_occ = 0u, own_m = 0u, own_p = 0u, own_wk = 0u, own_bs = 0u;
        uint32_t lo_occ = 0u, lo_p = 0u, lo_wk = 0u, lo_bs = 0u, hi_occ = 0u, hi_m = 0u, hi_wk = 0u, hi_bs = 0u;
        if constexpr (CH && PP == 3) {
            // the Y sweep's words of this lane; the row's previous and next words are the
            // neighbouring lanes' (a group holds whole rows)
            own_occ = acc[lane];
            own_m = acc[32 + lane];
            own_p = acc[64 + lane];
            own_wk = f[fi(F_OWK, lane)];
            own_bs = f[fi(F_OBS, lane)];
            const uint32_t u_occ = __shfl_up_sync(0xffffffffu, own_occ, 1), u_p = __shfl_up_sync(0xffffffffu, own_p, 1),
                           u_wk = __shfl_up_sync(0xffffffffu, own_wk, 1), u_bs = __shfl_up_sync(0xffffffffu, own_bs, 1);
            const uint32_t d_occ = __shfl_down_sync(0xffffffffu, own_occ, 1), d_m = __shfl_down_sync(0xffffffffu, own_m, 1),
                           d_wk = __shfl_down_sync(0xffffffffu, own_wk, 1), d_bs = __shfl_down_sync(0xffffffffu, own_bs, 1);
            if (valid) {
                if (kk > 0) {
                    lo_occ = u_occ;
                    lo_p = u_p;
                    lo_wk = u_wk;
                    lo_bs = u_bs;
                }
                if (kk + 1 < (int)Wz) {
                    hi_occ = d_occ;
                    hi_m = d_m;
                    hi_wk = d_wk;
                    hi_bs = d_bs;
                }
                old = ldw<COH>(odst + wo);
                const uint32_t from_lo = (own_p << 1) | (lo_p >> 31), from_hi = (own_m >> 1) | (hi_m << 31);
                work = (own_occ | from_lo | from_hi | (all_react ? colm : 0u)) & colm;
                moving = own_m | own_p | from_lo | from_hi;
            }
        } else if (valid) {
            if constexpr (PP == 0) {
                own_occ = P.osrc[wo];
                work = own_occ;
            } else {
                own_occ = ldw<COH>(in_occ + wo);
                own_m = ldw<COH>(SP.in.mv_m + wo);
                own_p = ldw<COH>(SP.in.mv_p + wo);
                own_wk = ldw<COH>(SP.in.work + wo);
                own_bs = ldw<COH>(SP.in.base + wo);
                // neighbour words: other rows for the X and Y sweeps, the row's adjacent words for Z
                const uint64_t st = PP == 1 ? (uint64_t)Y * Wz : PP == 2 ? (uint64_t)Wz : 1ull;
                const bool hl = PP == 1 ? x > 0 : PP == 2 ? y > 0 : kk > 0;
                const bool hh = PP == 1 ? x + 1 < X : PP == 2 ? y + 1 < Y : kk + 1 < (int)Wz;
                if (hl) {
                    lo_occ = ldw<COH>(in_occ + (wo - st));
                    lo_p = ldw<COH>(SP.in.mv_p + (wo - st));
                    lo_wk = ldw<COH>(SP.in.work + (wo - st));
                    lo_bs = ldw<COH>(SP.in.base + (wo - st));
                }
                if (hh) {
                    hi_occ = ldw<COH>(in_occ + (wo + st));
                    hi_m = ldw<COH>(SP.in.mv_m + (wo + st));
                    hi_wk = ldw<COH>(SP.in.work + (wo + st));
                    hi_bs = ldw<COH>(SP.in.base + (wo + st));
                }
                if constexpr (PP == 3) {
                    old = ldw<COH>(odst + wo);
                    const uint32_t from_lo = (own_p << 1) | (lo_p >> 31), from_hi = (own_m >> 1) | (hi_m << 31);
                    work = (own_occ | from_lo | from_hi | (all_react ? colm : 0u)) & colm;
                    moving = own_m | own_p | from_lo | from_hi;
                } else {
                    work = (own_occ | lo_p | hi_m) & colm;
                    moving = own_m | own_p | lo_p | hi_m;
                }
            }
        }
        // A group without work (most groups of sparse replicates) writes what the full path
        // would: empty words (base = the group's first record), and in the Z sweep zeros for
        // the voxels the destination held.  The fused Y sweep leaves its empty words in
        // shared memory.
        if (!__any_sync(0xffffffffu, work != 0u)) {
            if constexpr (CH && PP == 2) {
                acc[lane] = 0u;
                acc[32 + lane] = 0u;
                acc[64 + lane] = 0u;
                f[fi(F_OWK, lane)] = 0u;
                f[fi(F_OBS, lane)] = (uint32_t)G.rbase;
            } else if (valid) {
                if constexpr (PP == 3) {
                    odst[wo] = 0u;
                    const uint32_t vrow = ((uint32_t)x * (uint32_t)Y + (uint32_t)y) * (uint32_t)Z + (uint32_t)zb;
                    for (uint32_t bits = old; bits; bits &= bits - 1u)
                        st_vox_g<K>(dst + (rd.base + vrow + (uint32_t)(__ffs((int)bits) - 1)) * K, vox_zero<K>());
                    if (SP.fuse) {
                        SP.out.mv_m[wo] = 0u;
                        SP.out.mv_p[wo] = 0u;
                        SP.out.work[wo] = 0u;
                        SP.out.base[wo] = (uint32_t)G.rbase;
                    }
                } else {
                    if constexpr (PP != 0) SP.out.occ[wo] = 0u;
                    SP.out.mv_m[wo] = 0u;
                    SP.out.mv_p[wo] = 0u;
                    SP.out.work[wo] = 0u;
                    SP.out.base[wo] = (uint32_t)G.rbase;
                }
            }
            __syncwarp();
            return;
        }
        {
            // the word's uniform region code; bit 8: its whole window lies inside the lattice, so
            // every neighbour of its voxels has that code too
            const uint32_t uc = (rd.flags & 1u) ? 1u : (SP.wcode && valid) ? (uint32_t)SP.wcode[wo] : 0u;
            const bool inner = x > 0 && x + 1 < X && y > 0 && y + 1 < Y && kk > 0 && kk + 1 < (int)Wz;
            uint2* fp2 = reinterpret_cast<uint2*>(f) + lane;
            fp2[(F_OCC >> 1) * 32] = make_uint2(own_occ, old);
            fp2[(F_M >> 1) * 32] = make_uint2(own_m, own_p);
            fp2[(F_BS >> 1) * 32] = make_uint2(own_bs, own_wk);
            fp2[(F_LOCC >> 1) * 32] = make_uint2(lo_occ, lo_p);
            fp2[(F_LBS >> 1) * 32] = make_uint2(lo_bs, lo_wk);
            fp2[(F_HOCC >> 1) * 32] = make_uint2(hi_occ, hi_m);
            fp2[(F_HBS >> 1) * 32] = make_uint2(hi_bs, hi_wk);
            fp2[(F_Y >> 1) * 32] = make_uint2((uint32_t)y, (uint32_t)kk);
            fp2[(F_VROW >> 1) * 32] =
                make_uint2(((uint32_t)x * (uint32_t)Y + (uint32_t)y) * (uint32_t)Z, uc | (uc && inner ? 0x100u : 0u));
        }
        // List the work bits in three classes, so that the lanes of a warp mostly run the same
        // path: voxels with a record of the previous pass whose content does not change along
        // the axis, those whose content changes, and those without a record (arrivals), whose
        // Philox blocks are then evaluated by full warps.
        // Records are indexed by the work bits alone, whatever the list order.
        const uint32_t cls_a = PP == 0 ? work : (work & own_occ & ~moving);
        const uint32_t cls_b = PP == 0 ? 0u : (work & own_occ & moving);
        const uint32_t na = (uint32_t)__popc(cls_a), nb = (uint32_t)__popc(cls_b), nw = (uint32_t)__popc(work);
        uint32_t incl = na | (nb << 16), inw = nw;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o), uw = __shfl_up_sync(0xffffffffu, inw, o);
            if (lane >= o) {
                incl += u;
                inw += uw;
            }
        }
        const uint32_t tot = __shfl_sync(0xffffffffu, incl, 31), total = __shfl_sync(0xffffffffu, inw, 31);
        const uint32_t total_a = tot & 0xFFFFu, total_ab = total_a + (tot >> 16);
        const uint32_t ex = incl - (na | (nb << 16)), exa = ex & 0xFFFFu, exb = ex >> 16, exw = inw - nw;
        reinterpret_cast<uint2*>(f)[(F_OBS >> 1) * 32 + lane] = make_uint2((uint32_t)G.rbase + exw, work);
        acc[lane] = 0u;
        acc[32 + lane] = 0u;
        acc[64 + lane] = 0u;
        {
            auto put = [&](uint32_t bits, uint32_t o) {
                while (bits) {
                    const int b = __ffs((int)bits) - 1;
                    bits &= bits - 1u;
                    list[o++] = (uint16_t)((lane << 5) | b);
                }
            };
            put(cls_a, exa);
            put(cls_b, total_a + exb);
            put(work & ~(cls_a | cls_b), total_ab + (exw - exa - exb));
        }
        __syncwarp();

        const uint32_t k0 = rd.seed_lo, k1 = rd.seed_hi;
        const uint8_t* rpad = P.region_pad + rd.rbase;
        const uint64_t Zr = rd.Zr;
        // region code (id + 1) of voxel (xx, yy, zz) of the window of a word with uniform code uc
        // (0: look it up; bit 8: the whole window is inside the lattice); 0 outside the lattice
        auto code = [&](uint32_t uc, int xx, int yy, int zz) -> uint32_t {
            if (uc & 0x100u) return uc & 0xFFu;
            if ((unsigned)xx >= (unsigned)X || (unsigned)yy >= (unsigned)Y || (unsigned)zz >= (unsigned)Z) return 0u;
            if (uc) return uc;
            return __ldg(rpad + ((uint64_t)xx * (uint64_t)Y + (uint64_t)yy) * Zr + (uint64_t)zz + 2u);
        };
        const uint32_t YZ = (uint32_t)Y * (uint32_t)Z;
        for (uint32_t t = (uint32_t)lane; t < total; t += 32) {
            const uint32_t e = list[t];
            const int i = (int)(e >> 5), b = (int)(e & 31u);
            const uint32_t bit = 1u << b;
            const uint2 f_yk = fpair(F_Y, i), f_vc = fpair(F_VROW, i), f_ow = fpair(F_OBS, i);
            const int yy = (int)f_yk.x, zz = 32 * (int)f_yk.y + b;
            const uint32_t v = f_vc.x + (uint32_t)zz;
            const uint32_t uc = f_vc.y;
            const uint32_t ri = f_ow.x + below(f_ow.y, bit);  // this pass's record of the item
            if constexpr (PP == 0) {
                const Vox<K> own = ld_vox_g<K>(P.src + (rd.base + v) * K);
                const U4 b0 = d_philox(v, frame, 0u, 0u, k0, k1);
                const uint32_t rs = code(uc, x, yy, zz);
                const uint32_t d = decide_moves<K>(own, v, frame, 0u, trow(rs, code(uc, x - 1, yy, zz)),
                                                   trow(rs, code(uc, x + 1, yy, zz)), k0, k1, b0.x);
                rec_store<K>(rout, ri, own, make_uint4(d, b0.y, b0.z, b0.w));
                if (d & 0xFFFFu) atomicOr(acc + 32 + i, bit);
                if (d >> 16) atomicOr(acc + 64 + i, bit);
            } else {
                const uint32_t occ = f[fi(F_OCC, i)];
                const uint2 f_bw = fpair(F_BS, i), f_mp = fpair(F_M, i);
                Vox<K> own = vox_zero<K>(), lo = vox_zero<K>(), hi = vox_zero<K>();
                uint32_t dme = 0u, dlo = 0u, dhi = 0u;
                uint4 tw = make_uint4(0u, 0u, 0u, 0u);
                const bool own_in = (occ & bit) != 0u;
                if (own_in) {
                    if constexpr (CH && PP == 3) mid_load(f_bw.x + below(f_bw.y, bit), (uint32_t)G.rbase, own, tw);
                    else rec_load<K, !COH>(rin, f_bw.x + below(f_bw.y, bit), own, tw);
                    dme = tw.x;
                }
                // a neighbour's record is needed when it sends to this voxel or receives from it
                bool need_lo, need_hi;
                uint32_t ilo, ihi;
                if constexpr (PP == 3) {
                    const uint32_t m = f_mp.x, p = f_mp.y;
                    if (b > 0) {
                        const uint32_t lb = bit >> 1;
                        need_lo = (occ & lb) && ((m & bit) || (p & lb));
                        ilo = f_bw.x + below(f_bw.y, lb);
                    } else {
                        const uint2 f_lo = fpair(F_LOCC, i), f_lb = fpair(F_LBS, i);
                        need_lo = (f_lo.x >> 31) && ((m & bit) || (f_lo.y >> 31));
                        ilo = f_lb.x + below(f_lb.y, 0x80000000u);
                    }
                    if (b < 31) {
                        const uint32_t hb = bit << 1;
                        need_hi = (occ & hb) && ((p & bit) || (m & hb));
                        ihi = f_bw.x + below(f_bw.y, hb);
                    } else {
                        const uint2 f_hi = fpair(F_HOCC, i);
                        need_hi = (f_hi.x & 1u) && ((p & bit) || (f_hi.y & 1u));
                        ihi = f[fi(F_HBS, i)];
                    }
                } else {
                    const uint2 f_lo = fpair(F_LOCC, i), f_hi = fpair(F_HOCC, i);
                    const uint2 f_lb = fpair(F_LBS, i), f_hb = fpair(F_HBS, i);
                    need_lo = (f_lo.x & bit) && ((f_mp.x | f_lo.y) & bit);
                    need_hi = (f_hi.x & bit) && ((f_mp.y | f_hi.y) & bit);
                    ilo = f_lb.x + below(f_lb.y, bit);
                    ihi = f_hb.x + below(f_hb.y, bit);
                }
                if (need_lo) {
                    uint4 tl;
                    if constexpr (CH && PP == 3) mid_load(ilo, (uint32_t)G.rbase, lo, tl);
                    else rec_load<K, !COH>(rin, ilo, lo, tl);
                    dlo = tl.x;
                }
                if (need_hi) {
                    uint4 th;
                    if constexpr (CH && PP == 3) mid_load(ihi, (uint32_t)G.rbase, hi, th);
                    else rec_load<K, !COH>(rin, ihi, hi, th);
                    dhi = th.x;
                }
                const uint32_t vs = PP == 1 ? YZ : PP == 2 ? (uint32_t)Z : 1u;
                Vox<K> r = combine<K>(own, dme, lo, dlo, hi, dhi, v, v - vs, v + vs, frame, (uint32_t)(PP - 1));
                if constexpr (PP == 1 || PP == 2) {
                    if (!vox_empty<K>(r)) {
                        // this voxel's Philox words: carried in its record, or evaluated here
                        uint32_t wd, wn1, wn2;
                        if (own_in) {
                            wd = tw.y;
                            wn1 = tw.z;
                            wn2 = tw.w;
                        } else {
                            const U4 b0 = d_philox(v, frame, 0u, 0u, k0, k1);
                            wd = PP == 1 ? b0.y : b0.z;
                            wn1 = PP == 1 ? b0.z : b0.w;
                            wn2 = PP == 1 ? b0.w : 0u;
                        }
                        const uint32_t rs = code(uc, x, yy, zz);
                        const uint32_t clo = PP == 1 ? code(uc, x, yy - 1, zz) : code(uc, x, yy, zz - 1);
                        const uint32_t chi = PP == 1 ? code(uc, x, yy + 1, zz) : code(uc, x, yy, zz + 1);
                        const uint32_t d =
                            decide_moves<K>(r, v, frame, (uint32_t)PP, trow(rs, clo), trow(rs, chi), k0, k1, wd);
                        if constexpr (CH && PP == 2) mid_store(ri, (uint32_t)G.rbase, r, make_uint4(d, wn1, wn2, 0u));
                        else rec_store<K>(rout, ri, r, make_uint4(d, wn1, wn2, 0u));
                        atomicOr(acc + i, bit);
                        if (d & 0xFFFFu) atomicOr(acc + 32 + i, bit);
                        if (d >> 16) atomicOr(acc + 64 + i, bit);
                    }
                } else {
                    const uint32_t rv = P.reservoir ? (uint32_t)P.reservoir[rd.base + v] : 0u;
                    bool listed = false;
                    if (rv != 0u || zero_order || !vox_empty<K>(r)) {
                        const uint32_t w3 = own_in ? tw.y : d_philox(v, frame, 0u, 0u, k0, k1).w;
                        const bool calm =
                            rv == 0u && !zero_order &&
                            calm_voxel<K>(r, w3, P.T.quiet + (size_t)rd.counts_index * S1 * P.T.QS, P.T.QS,
                                          P.T.one + (size_t)rd.counts_index * S1 * 3, P.T.g23 + 2 * rd.counts_index,
                                          P.T.a2 ? P.T.a2 + (size_t)rd.counts_index * S1 * S1 : nullptr, P.T.tau);
                        if (!calm) {
                            // the warp runs this voxel's SSA after the group's items: the
                            // first PEND such voxels wait in shared memory, the others in their
                            // output record and the warp's overflow list
                            const uint32_t slot = atomicAdd(pend, 1u);
                            if (slot < (uint32_t)PEND) {
                                uint4* pe = reinterpret_cast<uint4*>(pend + 4) + 2 * slot;
                                pe[0] = make_uint4((uint32_t)r.w[0], (uint32_t)(r.w[0] >> 32),
                                                   K == 16 ? (uint32_t)r.w[K / 8 - 1] : 0u,
                                                   K == 16 ? (uint32_t)(r.w[K / 8 - 1] >> 32) : 0u);
                                pe[1] = make_uint4(w3, rv, ri, e);
                            } else {
                                rec_store<K>(rout, ri, r, make_uint4(v, w3, rv, G.rep));
                                SP.ssa_over[(size_t)gw * STREAM_SSA_OVER_PER_WARP + (slot - (uint32_t)PEND)] =
                                    make_uint2(ri, e);
                            }
                            listed = true;
                        }
                    }
                    if (!listed && !vox_empty<K>(r)) {
                        st_vox_g<K>(dst + (rd.base + v) * K, r);
                        atomicOr(acc + i, bit);
                        if (SP.fuse) {
                            // pass 0 of the next frame for this voxel
                            const uint32_t nf = frame + 1u;
                            const U4 b0 = d_philox(v, nf, 0u, 0u, k0, k1);
                            const uint32_t rs = code(uc, x, yy, zz);
                            const uint32_t d = decide_moves<K>(r, v, nf, 0u, trow(rs, code(uc, x - 1, yy, zz)),
                                                               trow(rs, code(uc, x + 1, yy, zz)), k0, k1, b0.x);
                            rec_store<K>(rout, ri, r, make_uint4(d, b0.y, b0.z, b0.w));
                            if (d & 0xFFFFu) atomicOr(acc + 32 + i, bit);
                            if (d >> 16) atomicOr(acc + 64 + i, bit);
                        }
                    }
                }
            }
        }
        __syncwarp();
        if constexpr (PP == 3) {
            // the SSA of the voxels this warp kept, by the whole warp (react_voxel_warp, its
            // scratch in the list's storage), then what pass 3 does for a quiet voxel: the store,
            // the occupancy bit and the next frame's x-decisions
            const uint32_t np = pend[0];
            if (np != 0u) {
                for (uint32_t q = 0; q < np; q++) {
                    Vox<K> r;
                    uint4 pt;  // Philox word, reservoir species, record, item
                    if (q < (uint32_t)PEND) {
                        const uint4* pe = reinterpret_cast<const uint4*>(pend + 4) + 2 * q;
                        const uint4 pc = pe[0];
                        pt = pe[1];
                        r.w[0] = (uint64_t)pc.x | ((uint64_t)pc.y << 32);
                        if constexpr (K == 16) r.w[K / 8 - 1] = (uint64_t)pc.z | ((uint64_t)pc.w << 32);
                    } else {
                        // written by this warp's lanes in this launch: read through L2
                        const uint2 oe = __ldcg(SP.ssa_over + (size_t)gw * STREAM_SSA_OVER_PER_WARP + (q - (uint32_t)PEND));
                        uint4 t;
                        rec_load<K, false>(rout, oe.x, r, t);
                        pt = make_uint4(t.y, t.z, oe.x, oe.y);
                    }
                    const uint32_t i = pt.w >> 5, bit = 1u << (pt.w & 31u);
                    const uint2 f_yk = fpair(F_Y, (int)i), f_vc = fpair(F_VROW, (int)i);
                    const int yy = (int)f_yk.x, zz = 32 * (int)f_yk.y + (int)(pt.w & 31u);
                    const uint32_t v = f_vc.x + (uint32_t)zz;
                    react_voxel_warp<K>(r, pt.y, v, frame, k0, k1, rd.rate_mult, rd.counts_index, P.T, nullptr,
                                        P.counts + (size_t)rd.counts_index * S1, s_diag, pt.x,
                                        reinterpret_cast<float*>(list));
                    if (lane == 0 && !vox_empty<K>(r)) {
                        st_vox_g<K>(dst + (rd.base + v) * K, r);
                        atomicOr(acc + i, bit);
                        if (SP.fuse) {
                            const uint32_t nf = frame + 1u;
                            const U4 b0 = d_philox(v, nf, 0u, 0u, k0, k1);
                            const uint32_t rs = code(f_vc.y, x, yy, zz);
                            const uint32_t d = decide_moves<K>(r, v, nf, 0u, trow(rs, code(f_vc.y, x - 1, yy, zz)),
                                                               trow(rs, code(f_vc.y, x + 1, yy, zz)), k0, k1, b0.x);
                            rec_store<K>(rout, pt.z, r, make_uint4(d, b0.y, b0.z, b0.w));
                            if (d & 0xFFFFu) atomicOr(acc + 32 + i, bit);
                            if (d >> 16) atomicOr(acc + 64 + i, bit);
                        }
                    }
                    __syncwarp();
                }
                if (lane == 0) pend[0] = 0u;
                __syncwarp();
            }
        }
        if (valid) {
            if constexpr (PP == 0) {
                SP.out.mv_m[wo] = acc[32 + lane];
                SP.out.mv_p[wo] = acc[64 + lane];
                SP.out.work[wo] = work;
                SP.out.base[wo] = f[fi(F_OBS, lane)];
            } else if constexpr (PP == 3) {
                odst[wo] = acc[lane];
                // voxels the destination held that end the frame empty get zeros
                for (uint32_t bits = old & ~acc[lane]; bits; bits &= bits - 1u)
                    st_vox_g<K>(dst + (rd.base + f[fi(F_VROW, lane)] + (uint32_t)zb + (uint32_t)(__ffs((int)bits) - 1)) * K,
                                vox_zero<K>());
                if (SP.fuse) {
                    SP.out.mv_m[wo] = acc[32 + lane];
                    SP.out.mv_p[wo] = acc[64 + lane];
                    SP.out.work[wo] = work;
                    SP.out.base[wo] = f[fi(F_OBS, lane)];
                }
            } else if constexpr (!CH) {
                SP.out.occ[wo] = acc[lane];
                SP.out.mv_m[wo] = acc[32 + lane];
                SP.out.mv_p[wo] = acc[64 + lane];
                SP.out.work[wo] = work;
                SP.out.base[wo] = f[fi(F_OBS, lane)];
            }
        }
        __syncwarp();
    };  // sweep
    if constexpr (PASS == PASS_YZ) {
        sweep(std::integral_constant<int, 2>{}, std::true_type{});
        sweep(std::integral_constant<int, 3>{}, std::true_type{});
    } else {
        sweep(std::integral_constant<int, PASS>{}, std::false_type{});
    }
}

// PASS 0: x-decisions; 1: X sweep + y-decisions; 2: Y sweep + z-decisions;
// 3: Z sweep + reactions + store; PASS_YZ: 2 and then 3 on each group.
template <int K, int PASS, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) sweep_pass_kernel(const StreamParams SP) {
    constexpr int NW = NT / 32;
    const ProdParams& P = SP.P;
    extern __shared__ __align__(16) uint32_t sm[];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const uint32_t S1 = P.T.S1, NC = P.T.NC;
    constexpr int STAGE = stage_recs(PASS, MINB);
    constexpr size_t WSTRIDE = stream_warp_words() + (size_t)STAGE * 8;  // u32 words of a warp's area
    uint32_t* f = sm + (size_t)w * WSTRIDE;  // [NF][32]
    uint32_t* acc = f + NF * 32;                            // [3][32]: content, movers down, movers up
    uint16_t* list = reinterpret_cast<uint16_t*>(acc + 96);
    uint32_t* pend = acc + 96 + LIST / 2;  // [PEND_WORDS]
    uint32_t* s_diag = sm + (size_t)NW * WSTRIDE;  // [PD_N]
    uint32_t* s_thr = s_diag + PD_N;
    allow_next_launch();
    const uint32_t* thr = P.T.thr;
    if (P.thr_smem) {
        const uint32_t nt = NC * NC * S1;
        for (uint32_t i = tid; i < nt; i += NT) s_thr[i] = P.T.thr[i];
        thr = s_thr;
    }
    for (int i = tid; i < PD_N; i += NT) s_diag[i] = 0u;
    if (lane == 0) pend[0] = 0u;
    wait_previous_launch();
    const uint32_t frame = P.stepbuf[P.parity];
    if (blockIdx.x == 0 && tid == 0) {
        for (uint32_t i = 0; i < P.n_reset; i++) P.reset[i] = 0u;
        if ((PASS == 3 || PASS == PASS_YZ) && P.advance) P.stepbuf[P.parity ^ 1u] = frame + 1u;
    }
    __syncthreads();
    const uint32_t TW = gridDim.x * NW;
    const WarpArea A{f, acc, list, pend, s_diag, thr, blockIdx.x * NW + (uint32_t)w, lane,
                     reinterpret_cast<uint4*>(f + stream_warp_words()), (uint32_t)STAGE};
    // groups from the pass's counter (one atomic per group, fetched a group ahead), else round-robin
    auto fetch = [&]() -> uint32_t {
        uint32_t q = 0u;
        if (lane == 0) q = atomicAdd(SP.queue, 1u);
        return __shfl_sync(0xffffffffu, q, 0);
    };
    // groups come from the pass's counter in batches of SP.batch consecutive groups (one atomic
    // per batch: same-address atomics serialise in L2), the next batch fetched while the last group
    // of the current one runs
    uint32_t g, g_end;
    if (SP.queue) {
        g = fetch() * SP.batch;
        g_end = g + SP.batch;
    } else {
        g = blockIdx.x * NW + (uint32_t)w;
        g_end = g + 1u;
    }
    while (g < SP.n_groups) {
        uint32_t g_next, g_next_end;
        if (g + 1u < g_end) {
            g_next = g + 1u;
            g_next_end = g_end;
        } else if (SP.queue) {
            g_next = fetch() * SP.batch;
            g_next_end = g_next + SP.batch;
        } else {
            g_next = g + TW;
            g_next_end = g_next + 1u;
        }
        stream_group<K, PASS, false>(SP, A, g, frame, 0u);
        g = g_next;
        g_end = g_next_end;
    }
    __syncthreads();
    for (int i = tid; i < PD_N; i += NT)
        if (s_diag[i]) atomicAdd(P.diag + i, s_diag[i]);
}

static void launch_pdl(void* fn, int grid, int threads, size_t smem, cudaStream_t s, const StreamParams& SP);

// Loads and stores that order a task's completion value with the words and records it wrote.
__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}

// Polls of a completion value before a task gives up (each poll is an L2 round trip plus a back-off
// of at most 1 us: one to two seconds in all, against microseconds for a real wait); then the task
// and the warp's remaining tasks are abandoned and PD_WAIT_TIMEOUTS counts it.
constexpr uint32_t kWaitPolls = 1u << 20;

// The persistent multi-frame form (FramesParams): pass 1 and the fused Y and Z sweeps of every
// group for every frame of the launch, as tasks of one counter.
template <int K, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) sweep_frames_kernel(const __grid_constant__ FramesParams FP) {
    constexpr int NW = NT / 32;
    const StreamParams& SX = FP.sp[0];
    const StreamParams& SYZ = FP.sp[1];
    const ProdParams& P = SYZ.P;
    extern __shared__ __align__(16) uint32_t sm[];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const uint32_t S1 = P.T.S1, NC = P.T.NC;
    constexpr int STAGE = stage_recs(PASS_YZ, MINB);
    constexpr size_t WSTRIDE = stream_warp_words() + (size_t)STAGE * 8;
    uint32_t* f = sm + (size_t)w * WSTRIDE;
    uint32_t* acc = f + NF * 32;
    uint16_t* list = reinterpret_cast<uint16_t*>(acc + 96);
    uint32_t* pend = acc + 96 + LIST / 2;
    uint32_t* s_diag = sm + (size_t)NW * WSTRIDE;
    uint32_t* s_thr = s_diag + PD_N;
    allow_next_launch();
    const uint32_t* thr = P.T.thr;
    if (P.thr_smem) {
        const uint32_t nt = NC * NC * S1;
        for (uint32_t i = tid; i < nt; i += NT) s_thr[i] = P.T.thr[i];
        thr = s_thr;
    }
    for (int i = tid; i < PD_N; i += NT) s_diag[i] = 0u;
    if (lane == 0) pend[0] = 0u;
    wait_previous_launch();
    const uint32_t frame0 = P.stepbuf[FP.cur0];
    if (blockIdx.x == 0 && tid == 0)
        for (uint32_t i = 0; i < FP.n_reset; i++) FP.reset[i] = 0u;
    __syncthreads();
    const WarpArea A{f, acc, list, pend, s_diag, thr, blockIdx.x * NW + (uint32_t)w, lane,
                     reinterpret_cast<uint4*>(f + stream_warp_words()), (uint32_t)STAGE};
    const uint32_t ng = FP.n_groups, per_frame = 2u * ng, total = FP.n_frames * per_frame;
    auto fetch = [&]() -> uint32_t {
        uint32_t q = 0u;
        if (lane == 0) q = atomicAdd(FP.tasks, 1u);
        return __shfl_sync(0xffffffffu, q, 0);
    };
    uint32_t t = fetch();
    while (t < total) {
        const uint32_t t_next = fetch();
        const uint32_t fi = t / per_frame, r = t - fi * per_frame;
        const bool yz = r >= ng;
        const uint32_t rank = yz ? r - ng : r;
        const uint32_t g = FP.order ? __ldg(FP.order + rank) : rank;
        if (yz || fi > 0u) {
            // lanes 0-4 wait for the group and its four neighbours
            const uint32_t* done = yz ? FP.done1 : FP.done2;
            const uint32_t want = FP.seq + fi + (yz ? 1u : 0u);
            bool late = false;
            if (lane < 5) {
                const uint32_t n = lane == 0 ? g : FP.nbr[4 * (size_t)g + (uint32_t)(lane - 1)];
                if (n != 0xFFFFFFFFu) {
                    // back-off doubling from 32 to 1024 ns, so that warps waiting far ahead (small
                    // lattices, where most warps hold tasks of later frames) poll L2 rarely
                    uint32_t polls = 0u, ns = 32u;
                    while ((int32_t)(ld_acquire_gpu(done + n) - want) < 0) {
                        if (++polls > kWaitPolls) {
                            late = true;
                            break;
                        }
                        __nanosleep(ns);
                        ns = min(ns * 2u, 1024u);
                    }
                }
            }
            __syncwarp();
            if (__any_sync(0xffffffffu, late)) {
                if (lane == 0) {
                    atomicAdd(P.diag + PD_WAIT_TIMEOUTS, 1u);
                    atomicAdd(FP.fault, 1ull);
                }
                break;
            }
        }
        const uint32_t frame = frame0 + fi, par = (FP.cur0 + fi) & 1u;
        if (yz) stream_group<K, PASS_YZ, true>(SYZ, A, g, frame, par);
        else stream_group<K, 1, true>(SX, A, g, frame, par);
        __syncwarp();
        if (lane == 0) st_release_gpu((yz ? FP.done2 : FP.done1) + g, FP.seq + fi + 1u);
        t = t_next;
    }
    __syncthreads();
    for (int i = tid; i < PD_N; i += NT)
        if (s_diag[i]) atomicAdd(P.diag + i, s_diag[i]);
    // the last warp to finish readies the counters for the next launch and leaves the next frame's
    // number for it (every warp has read this launch's first frame number by then)
    if (lane == 0 && atomicAdd(FP.exits, 1u) == gridDim.x * NW - 1u) {
        *FP.tasks = 0u;
        *FP.exits = 0u;
        P.stepbuf[(FP.cur0 + FP.n_frames) & 1u] = frame0 + FP.n_frames;
    }
}

// ------------------------------------------------------------------ launchers

namespace {
struct Variant {
    int NT, MINB, MINB3;  // threads per block, minimum resident blocks per SM of passes 0-2 and of pass 3
    bool fused;           // passes 2 and 3 as one launch (PASS_YZ at MINB3 blocks per SM)
    bool frames;          // the persistent multi-frame kernel at MINB3 blocks per SM (per-pass launches:
                          // the fused ones of the same shape); variant 6 takes a pass's groups
                          // heaviest first, variant 7 in plane order
};
// compiled launch shapes; pass 3 (reactions) needs more registers than the sweeps
constexpr Variant kVariants[] = {{256, 2, 2, false, false}, {256, 4, 4, false, false}, {256, 4, 3, false, false},
                                 {256, 4, 2, false, false}, {256, 4, 3, true, false},  {256, 4, 4, true, false},
                                 {256, 4, 3, true, true},   {256, 4, 3, true, true}};
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);

template <int K, int NT, int MINB, int MINB3>
void* pass_fn(int pass) {
    switch (pass) {
        case 0: return reinterpret_cast<void*>(&sweep_pass_kernel<K, 0, NT, MINB>);
        case 1: return reinterpret_cast<void*>(&sweep_pass_kernel<K, 1, NT, MINB>);
        case 2: return reinterpret_cast<void*>(&sweep_pass_kernel<K, 2, NT, MINB>);
        default: return reinterpret_cast<void*>(&sweep_pass_kernel<K, 3, NT, MINB3>);
    }
}

// fused variants: the Y and Z sweeps are launched as pass 2; there is no pass 3
template <int K, int NT, int MINB, int MINB3>
void* pass_fn_fused(int pass) {
    switch (pass) {
        case 0: return reinterpret_cast<void*>(&sweep_pass_kernel<K, 0, NT, MINB>);
        case 1: return reinterpret_cast<void*>(&sweep_pass_kernel<K, 1, NT, MINB>);
        case 2: return reinterpret_cast<void*>(&sweep_pass_kernel<K, PASS_YZ, NT, MINB3>);
        default: return nullptr;
    }
}

template <int K>
void* fn_of(int variant, int pass) {
    switch (variant) {
        case 0: return pass_fn<K, 256, 2, 2>(pass);
        case 1: return pass_fn<K, 256, 4, 4>(pass);
        case 2: return pass_fn<K, 256, 4, 3>(pass);
        case 3: return pass_fn<K, 256, 4, 2>(pass);
        case 4: case 6: case 7: return pass_fn_fused<K, 256, 4, 3>(pass);
        case 5: return pass_fn_fused<K, 256, 4, 4>(pass);
        default: return nullptr;
    }
}

template <int K>
void* frames_fn_of(int variant) {
    switch (variant) {
        case 6: case 7: return reinterpret_cast<void*>(&sweep_frames_kernel<K, 256, 3>);
        default: return nullptr;
    }
}

void* frames_kernel_of(int K, int variant) {
    return K == 16 ? frames_fn_of<16>(variant) : K == 8 ? frames_fn_of<8>(variant) : nullptr;
}

void* kernel_of(int K, int variant, int pass) {
    if (pass < 0 || pass > 3) return nullptr;
    return K == 16 ? fn_of<16>(variant, pass) : K == 8 ? fn_of<8>(variant, pass) : nullptr;
}
}  // namespace

int stream_variant_count() { return kNumVariants; }
bool stream_variant_fused(int variant) { return variant >= 0 && variant < kNumVariants && kVariants[variant].fused; }
bool stream_variant_frames(int variant) { return variant >= 0 && variant < kNumVariants && kVariants[variant].frames; }
bool stream_variant_plane_order(int variant) { return variant == 7; }
int stream_variant_threads(int variant) { return variant >= 0 && variant < kNumVariants ? kVariants[variant].NT : 0; }

// Launch with programmatic stream serialization (see wait_previous_launch).
static void launch_pdl(void* fn, int grid, int threads, size_t smem, cudaStream_t s, const StreamParams& SP) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void* args[] = {const_cast<StreamParams*>(&SP)};
    CS_CUDA(cudaLaunchKernelExC(&cfg, fn, args));
}

bool stream_launch(int K, int variant, int pass, int grid, size_t smem, cudaStream_t s, const StreamParams& SP) {
    void* fn = kernel_of(K, variant, pass);
    if (!fn) return false;
    launch_pdl(fn, grid, kVariants[variant].NT, smem, s, SP);
    return true;
}

size_t stream_pass_smem(int variant, int pass, uint32_t S1, uint32_t thr_words) {
    const Variant& v = kVariants[variant];
    // the fused pass (launched as pass 2) and the multi-frame kernel (pass 4 here) stage records
    const bool yz = v.fused && (pass == 2 || pass == 4);
    return stream_smem(v.NT, S1, thr_words, yz ? stage_recs(PASS_YZ, v.MINB3) : 0);
}

int stream_blocks_per_sm(int K, int variant, int pass, size_t smem) {
    void* fn = kernel_of(K, variant, pass);
    if (!fn) return 0;
    int n = 0;
    CS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, kVariants[variant].NT, smem));
    return n;
}

void stream_set_attrs(int K, int variant, uint32_t S1, uint32_t thr_words) {
    for (int pass = 0; pass < 5; pass++) {
        void* fn = pass < 4 ? kernel_of(K, variant, pass) : frames_kernel_of(K, variant);
        if (!fn) continue;
        const size_t smem = stream_pass_smem(variant, pass, S1, thr_words);
        CS_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        CS_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    }
}

int stream_frames_blocks_per_sm(int K, int variant, size_t smem) {
    void* fn = frames_kernel_of(K, variant);
    if (!fn) return 0;
    int n = 0;
    CS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, kVariants[variant].NT, smem));
    return n;
}

bool stream_frames_launch(int K, int variant, int grid, size_t smem, cudaStream_t s, const FramesParams& FP) {
    void* fn = frames_kernel_of(K, variant);
    if (!fn) return false;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)kVariants[variant].NT);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void* args[] = {const_cast<FramesParams*>(&FP)};
    CS_CUDA(cudaLaunchKernelExC(&cfg, fn, args));
    return true;
}

}  // namespace cellsim
