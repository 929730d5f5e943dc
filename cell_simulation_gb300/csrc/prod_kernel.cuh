// prod_kernel.cuh — the fused production step kernel (one launch per frame).
//
// Persistent CTAs take (replicate, TY x TZ tile, x-segment) items from an
// atomic work queue and roll along x.  The CTA holds rings of shared-memory
// planes (slot windows (TY+2) x (TZ+2) with a one-voxel halo, region-code
// windows with a two-voxel halo) filled by cp.async one plane ahead, and runs
// four stages as a software pipeline over planes; iteration j does
//
//   A  x-move decisions of plane j+2
//   B  X sweep of plane j from planes j-1, j, j+1, then y-move decisions
//   C  Y sweep of plane j-1 (interior rows), then z-move decisions
//   D  Z sweep of plane j-2 (interior), reactions, store
//
// The four stages of one iteration touch different planes, so they share two
// passes separated by barriers.  The dense pass touches every voxel with a
// few vector shared-memory accesses: it copies contents that nothing moves
// into or out of, and appends the voxels that need work (particles to draw
// for, movers to resolve, reactions to run) to per-stage shared work lists
// with one warp-aggregated atomic per warp.  The sparse pass then runs the
// Philox draws, the combines and the SSA of all four stages on the compacted
// lists with every lane busy.  The lattice is mostly empty, so this keeps the
// per-particle work from being replayed by whole warps and overlaps the long
// dependency chains of different stages.
#pragma once
#include <cstdint>

#include "prod_common.cuh"

namespace cellsim {

// Launch parameters shared by the brick pass and the tile pipeline.
struct ProdParams {
    ProdTables T;
    const RepDesc* reps;
    const WorkItem* items;
    uint32_t n_items;
    const uint32_t* n_items_dev;  // when set, the item count is read here at kernel start
    uint32_t* queue;              // work-queue counter of this launch (zero at launch)
    uint32_t* reset;              // n_reset counters that block 0 zeroes for the next frame
    uint32_t n_reset;
    uint32_t advance;             // nonzero: block 0 writes frame + 1 to stepbuf[parity ^ 1]
    uint32_t thr_smem;            // nonzero: the threshold table is staged in shared memory
    uint32_t parity;
    uint32_t* stepbuf;            // [2] frame numbers
    WorkItem* spill;              // brick pass: crowded bricks handed to the second pass
    uint32_t* n_spill;
    uint32_t sub;                 // brick pass over spilled bricks: plane groups per brick
    const uint8_t* src;
    uint8_t* dst;
    // occupancy bitmaps of src and dst (bit z % 32 of word obase + (x Y + y) Wz + z / 32 is set
    // exactly when the voxel holds a particle); maintained by the brick pass
    const uint32_t* osrc;
    uint32_t* odst;
    const uint8_t* region_pad;   // padded region codes, see RepDesc::rbase
    const uint8_t* reservoir;    // may be null
    unsigned long long* counts;  // [n_rep][S1]
    uint32_t* diag;
};

template <int K, int TY, int TZ>
struct Tile {
    static_assert(TZ % 16 == 0, "TZ must be a multiple of 16 (16-byte region rows)");
    static constexpr int WY = TY + 2, WZ = TZ + 2, WIN = WY * WZ;
    static constexpr int RWY = TY + 4, RWZB = TZ + 16, RPLANE = RWY * RWZB;  // region window rows, 16-byte padded
    static constexpr int NRAW = 5, NREG = 6, NLIST = 7;
    static constexpr size_t off_raw = 0;
    static constexpr size_t off_xp = off_raw + (size_t)NRAW * WIN * K;
    static constexpr size_t off_yp = off_xp + (size_t)2 * WIN * K;
    static constexpr size_t off_dx = off_yp + (size_t)2 * WIN * K;
    static constexpr size_t off_dy = off_dx + (size_t)4 * WIN * 4;
    static constexpr size_t off_dz = off_dy + (size_t)2 * WIN * 4;
    static constexpr size_t off_reg = off_dz + (size_t)2 * WIN * 4;
    static constexpr size_t off_wl = off_reg + (size_t)NREG * RPLANE;
    static constexpr size_t off_tail = off_wl + ((size_t)NLIST * WIN * 2 + 15) / 16 * 16;
    static size_t smem(uint32_t S1) { return off_tail + (size_t)(S1 + PD_N + 8) * 4; }
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// 8- or 16-byte asynchronous copy global -> shared; src_bytes 0 writes zeros.
template <int B>
__device__ __forceinline__ void cp_async(void* sdst, const void* gsrc, bool valid) {
    uint32_t n = valid ? (uint32_t)B : 0u;
    if (B == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_u32(sdst)), "l"(gsrc), "r"(n) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(smem_u32(sdst)), "l"(gsrc), "r"(n) : "memory");
}
// Prefetch of the L2 line holding p.
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];\n" ::"l"(p)); }
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// Appends `item` to a shared work list when `want`; called by all 32 lanes.
__device__ __forceinline__ void wl_push(bool want, uint32_t item, uint16_t* list, uint32_t* counter) {
    const unsigned m = __ballot_sync(0xffffffffu, want);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    uint32_t pos = 0;
    if (lane == leader) pos = atomicAdd(counter, (uint32_t)__popc(m));
    pos = __shfl_sync(0xffffffffu, pos, leader);
    if (want) list[pos + __popc(m & ((1u << lane) - 1u))] = (uint16_t)item;
}

template <int K>
__device__ __forceinline__ Vox<K> ld_vox_g(const uint8_t* p) {
    Vox<K> c;
    if (K == 16) {
        uint4 t = __ldg(reinterpret_cast<const uint4*>(p));
        c.w[0] = (uint64_t)t.x | ((uint64_t)t.y << 32);
        c.w[K / 8 - 1] = (uint64_t)t.z | ((uint64_t)t.w << 32);
    } else {
        uint2 t = __ldg(reinterpret_cast<const uint2*>(p));
        c.w[0] = (uint64_t)t.x | ((uint64_t)t.y << 32);
    }
    return c;
}

template <int K>
__device__ __forceinline__ void st_vox_g(uint8_t* p, const Vox<K>& c) {
    if (K == 16) {
        uint4 t;
        t.x = (uint32_t)c.w[0]; t.y = (uint32_t)(c.w[0] >> 32);
        t.z = (uint32_t)c.w[K / 8 - 1]; t.w = (uint32_t)(c.w[K / 8 - 1] >> 32);
        *reinterpret_cast<uint4*>(p) = t;
    } else {
        uint2 t;
        t.x = (uint32_t)c.w[0]; t.y = (uint32_t)(c.w[0] >> 32);
        *reinterpret_cast<uint2*>(p) = t;
    }
}

template <int K, int TY, int TZ, int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB) prod_step_kernel(ProdParams P) {
    using C = Tile<K, TY, TZ>;
    constexpr int WZ = C::WZ, WIN = C::WIN, RWZB = C::RWZB, RPLANE = C::RPLANE;
    constexpr int NCH = C::RWY * (RWZB / 16);  // 16-byte region chunks per plane
    constexpr int NCI = WIN - 2 * WZ;          // Y-sweep domain: interior rows, all columns
    constexpr int NDI = TY * TZ;               // Z-sweep domain: interior
    extern __shared__ __align__(16) uint8_t smem[];
    Vox<K>* raw = reinterpret_cast<Vox<K>*>(smem + C::off_raw);  // [5][WIN]
    Vox<K>* xpb = reinterpret_cast<Vox<K>*>(smem + C::off_xp);   // [2][WIN]
    Vox<K>* ypb = reinterpret_cast<Vox<K>*>(smem + C::off_yp);   // [2][WIN]
    uint32_t* dxb = reinterpret_cast<uint32_t*>(smem + C::off_dx);  // [4][WIN]
    uint32_t* dyb = reinterpret_cast<uint32_t*>(smem + C::off_dy);  // [2][WIN]
    uint32_t* dzb = reinterpret_cast<uint32_t*>(smem + C::off_dz);  // [2][WIN]
    uint8_t* reg = smem + C::off_reg;                               // [6][RWY][RWZB]
    uint16_t* wl = reinterpret_cast<uint16_t*>(smem + C::off_wl);   // [7][WIN]
    int32_t* s_delta = reinterpret_cast<int32_t*>(smem + C::off_tail);
    uint32_t* s_diag = reinterpret_cast<uint32_t*>(s_delta + P.T.S1);
    uint32_t* s_cnt = s_diag + PD_N;  // [8] work-list counters
    __shared__ uint32_t s_item;
    enum { LA = 0, LB1 = 1, LB2 = 2, LC1 = 3, LC2 = 4, LD1 = 5, LD2 = 6 };

    const int tid = threadIdx.x;
    const uint32_t frame = P.stepbuf[P.parity];
    if (blockIdx.x == 0 && tid == 0) {
        for (uint32_t i = 0; i < P.n_reset; i++) P.reset[i] = 0u;
        if (P.advance) P.stepbuf[P.parity ^ 1u] = frame + 1u;
    }
    for (int i = tid; i < PD_N; i += NT) s_diag[i] = 0u;
    const bool always_react = P.T.n_zero_order != 0u;
    const uint32_t n_items = P.n_items_dev ? *P.n_items_dev : P.n_items;

    for (;;) {
        __syncthreads();
        if (tid == 0) s_item = atomicAdd(P.queue, 1u);
        __syncthreads();
        const uint32_t it = s_item;
        if (it >= n_items) break;
        const WorkItem wi = P.items[it];
        const RepDesc rd = P.reps[wi.rep];
        const int X = (int)rd.X, Y = (int)rd.Y, Z = (int)rd.Z, Zr = (int)rd.Zr;
        const int y0 = (int)wi.y0, z0 = (int)wi.z0, x0 = (int)wi.x0, x1 = (int)wi.x1;
        const uint32_t k0 = rd.seed_lo, k1 = rd.seed_hi;
        const bool uniform = (rd.flags & 1u) != 0u;
        const uint8_t* src = P.src + rd.base * K;
        uint8_t* dst = P.dst + rd.base * K;
        const uint8_t* rpad = P.region_pad + rd.rbase;
        const uint8_t* resv = P.reservoir ? P.reservoir + rd.base : nullptr;
        const uint32_t YZ = (uint32_t)Y * (uint32_t)Z;
        const float mult = rd.rate_mult;
        for (uint32_t s = tid; s < P.T.S1; s += NT) s_delta[s] = 0;

        auto raw_plane = [&](int p) -> Vox<K>* { return raw + ((p + 10) % 5) * WIN; };
        auto reg_plane = [&](int p) -> uint8_t* { return reg + ((p + 12) % 6) * RPLANE; };
        auto dx_plane = [&](int p) -> uint32_t* { return dxb + ((p + 4) & 3) * WIN; };
        auto lin = [&](int p, int y, int z) -> uint32_t {
            return ((uint32_t)p * (uint32_t)Y + (uint32_t)y) * (uint32_t)Z + (uint32_t)z;
        };
        // move decisions of a non-empty voxel in sweep a between region codes rs (own), rlo, rhi
        auto decide = [&](const Vox<K>& c, uint32_t v, uint32_t a, uint32_t rs, uint32_t rlo, uint32_t rhi) -> uint32_t {
            const uint32_t* tlo = P.T.thr + ((size_t)rs * P.T.NC + rlo) * P.T.S1;
            const uint32_t* thi = P.T.thr + ((size_t)rs * P.T.NC + rhi) * P.T.S1;
            const U4 b0 = d_philox(v, frame, 0u, 0u, k0, k1);
            return decide_moves<K>(c, v, frame, a, tlo, thi, k0, k1, sweep_word(b0, a));
        };
        // region code at window position (wy, wz) of plane p (wy, wz may step one past the window)
        auto code_at = [&](int p, int wy, int wz) -> uint32_t {
            if (uniform) {
                int y = y0 - 1 + wy, z = z0 - 1 + wz;
                return (p >= 0 && p < X && y >= 0 && y < Y && z >= 0 && z < Z) ? 1u : 0u;
            }
            return reg_plane(p)[(wy + 1) * RWZB + wz + 1];
        };
        auto issue_raw = [&](int p) {
            Vox<K>* cp = raw_plane(p);
            for (int e = tid; e < WIN; e += NT) {
                int wy = e / WZ, wz = e - wy * WZ;
                int y = y0 - 1 + wy, z = z0 - 1 + wz;
                bool ok = p >= 0 && p < X && y >= 0 && y < Y && z >= 0 && z < Z;
                const uint8_t* g = ok ? src + (uint64_t)lin(p, y, z) * K : src;
                cp_async<K>(cp + e, g, ok);
            }
        };
        auto issue_reg = [&](int p) {
            if (uniform) return;
            uint8_t* rp = reg_plane(p);
            for (int c = tid; c < NCH; c += NT) {
                int ry = c / (RWZB / 16), cz = c - ry * (RWZB / 16);
                int y = y0 - 2 + ry, zp = z0 + 16 * cz;  // padded column index (z + 2)
                bool ok = p >= 0 && p < X && y >= 0 && y < Y && zp + 16 <= Zr;
                const uint8_t* g = ok ? rpad + ((uint64_t)p * (uint64_t)Y + (uint64_t)y) * (uint64_t)Zr + zp : rpad;
                cp_async<16>(rp + ry * RWZB + 16 * cz, g, ok);
            }
        };

        // prologue loads: raw x0-1 and regions x0-2..x0 for the x-decisions of plane x0-1
        issue_raw(x0 - 1);
        for (int p = x0 - 2; p <= x0; p++) issue_reg(p);
        cp_async_commit();

        // Iteration j: A = x-decisions of plane j+2, B = X sweep of plane j,
        // C = Y sweep of plane j-1, D = Z sweep + reactions + store of plane j-2.
        for (int j = x0 - 3; j <= x1 + 1; j++) {
            const int pA = j + 2, pB = j, pC = j - 1, pD = j - 2;
            const bool doA = pA >= x0 - 1 && pA <= x1;
            const bool doB = pB >= x0 && pB < x1;
            const bool doC = pC >= x0 && pC < x1;
            const bool doD = pD >= x0 && pD < x1;
            if (j + 3 <= x1) issue_raw(j + 3);
            if (j + 4 <= x1 + 1) issue_reg(j + 4);
            cp_async_commit();
            cp_async_wait<1>();
            if (tid < 8) s_cnt[tid] = 0u;
            __syncthreads();

            // ---------------- pass 1: dense classification ----------------
            if (doA) {
                const Vox<K>* cp = raw_plane(pA);
                uint32_t* dp = dx_plane(pA);
                for (int base = 0; base < WIN; base += NT) {
                    int e = base + tid;
                    bool want = false;
                    if (e < WIN) {
                        dp[e] = 0u;
                        want = !vox_empty<K>(cp[e]);
                    }
                    wl_push(want, (uint32_t)e, wl + LA * WIN, s_cnt + LA);
                }
            }
            if (doB) {
                const Vox<K>* rme = raw_plane(pB);
                const uint32_t* dlo = dx_plane(pB - 1);
                const uint32_t* dme = dx_plane(pB);
                const uint32_t* dhi = dx_plane(pB + 1);
                Vox<K>* xp = xpb + (pB & 1) * WIN;
                uint32_t* dy = dyb + (pB & 1) * WIN;
                for (int base = 0; base < WIN; base += NT) {
                    int e = base + tid;
                    bool mv = false, dec = false;
                    if (e < WIN) {
                        mv = (dme[e] | (dlo[e] >> 16) | (dhi[e] & 0xFFFFu)) != 0u;
                        if (!mv) {
                            Vox<K> own = rme[e];
                            xp[e] = own;
                            dy[e] = 0u;
                            dec = !vox_empty<K>(own);
                        }
                    }
                    wl_push(mv, (uint32_t)e, wl + LB1 * WIN, s_cnt + LB1);
                    wl_push(dec, (uint32_t)e, wl + LB2 * WIN, s_cnt + LB2);
                }
            }
            if (doC) {
                const Vox<K>* xp = xpb + (pC & 1) * WIN;
                const uint32_t* dy = dyb + (pC & 1) * WIN;
                Vox<K>* yp = ypb + (pC & 1) * WIN;
                uint32_t* dz = dzb + (pC & 1) * WIN;
                for (int base = 0; base < NCI; base += NT) {
                    int e = WZ + base + tid;
                    bool mv = false, dec = false;
                    if (base + tid < NCI) {
                        mv = (dy[e] | (dy[e - WZ] >> 16) | (dy[e + WZ] & 0xFFFFu)) != 0u;
                        if (!mv) {
                            Vox<K> own = xp[e];
                            yp[e] = own;
                            dz[e] = 0u;
                            dec = !vox_empty<K>(own);
                        }
                    }
                    wl_push(mv, (uint32_t)e, wl + LC1 * WIN, s_cnt + LC1);
                    wl_push(dec, (uint32_t)e, wl + LC2 * WIN, s_cnt + LC2);
                }
            }
            if (doD) {
                const Vox<K>* yp = ypb + (pD & 1) * WIN;
                const uint32_t* dz = dzb + (pD & 1) * WIN;
                for (int base = 0; base < NDI; base += NT) {
                    int t = base + tid;
                    bool mv = false, rx = false;
                    if (t < NDI) {
                        int ty = t / TZ, tz = t - ty * TZ;
                        int y = y0 + ty, z = z0 + tz;
                        if (y < Y && z < Z) {
                            int e = (ty + 1) * WZ + tz + 1;
                            mv = (dz[e] | (dz[e - 1] >> 16) | (dz[e + 1] & 0xFFFFu)) != 0u;
                            if (!mv) {
                                Vox<K> own = yp[e];
                                uint32_t v = lin(pD, y, z);
                                rx = always_react || !vox_empty<K>(own) || (resv && resv[v] != 0);
                                if (!rx) st_vox_g<K>(dst + (uint64_t)v * K, own);
                            }
                        }
                    }
                    wl_push(mv, (uint32_t)t, wl + LD1 * WIN, s_cnt + LD1);
                    wl_push(rx, (uint32_t)t, wl + LD2 * WIN, s_cnt + LD2);
                }
            }
            __syncthreads();

            // ---------------- pass 2: sparse work of all four stages ----------------
            {
                // each stage's items occupy a warp-aligned range, so a warp runs one kind of work
                const uint32_t nD1 = s_cnt[LD1], nD = nD1 + s_cnt[LD2];
                const uint32_t nB1 = s_cnt[LB1], nB = nB1 + s_cnt[LB2];
                const uint32_t nC1 = s_cnt[LC1], nC = nC1 + s_cnt[LC2];
                const uint32_t nA = s_cnt[LA];
                auto up = [](uint32_t x) { return (x + 31u) & ~31u; };
                const uint32_t bB = up(nD), bC = bB + up(nB), bA = bC + up(nC), e7 = bA + up(nA);
                for (uint32_t k = tid; k < e7; k += NT) {
                    if (k < bB) {  // D: Z sweep (movers) and/or reactions, then store
                        if (k >= nD) continue;
                        const Vox<K>* yp = ypb + (pD & 1) * WIN;
                        const uint32_t* dz = dzb + (pD & 1) * WIN;
                        const bool move = k < nD1;
                        int t = move ? wl[LD1 * WIN + k] : wl[LD2 * WIN + (k - nD1)];
                        int ty = t / TZ, tz = t - ty * TZ;
                        int y = y0 + ty, z = z0 + tz;
                        int e = (ty + 1) * WZ + tz + 1;
                        uint32_t v = lin(pD, y, z);
                        Vox<K> r = yp[e];
                        if (move)
                            r = combine<K>(r, dz[e], yp[e - 1], dz[e - 1], yp[e + 1], dz[e + 1], v, v - 1u, v + 1u, frame, 2u);
                        uint32_t rv = resv ? (uint32_t)resv[v] : 0u;
                        if (rv != 0u || always_react || !vox_empty<K>(r)) {
                            const uint32_t w3 = d_philox(v, frame, 0u, 0u, k0, k1).w;
                            const bool quiet =
                                rv == 0u && !always_react &&
                                calm_voxel<K>(r, w3, P.T.quiet + (size_t)rd.counts_index * P.T.S1 * P.T.QS, P.T.QS,
                                              P.T.one + (size_t)rd.counts_index * P.T.S1 * 3,
                                              P.T.g23 + 2 * rd.counts_index,
                                              P.T.a2 ? P.T.a2 + (size_t)rd.counts_index * P.T.S1 * P.T.S1 : nullptr,
                                              P.T.tau);
                            if (!quiet)
                                react_voxel<K>(r, rv, v, frame, k0, k1, mult, rd.counts_index, P.T, s_delta, s_diag, w3);
                        }
                        st_vox_g<K>(dst + (uint64_t)v * K, r);
                    } else if (k < bC) {  // B: X sweep (movers) and/or y-decisions
                        const uint32_t q = k - bB;
                        if (q >= nB) continue;
                        const bool move = q < nB1;
                        int e = move ? wl[LB1 * WIN + q] : wl[LB2 * WIN + (q - nB1)];
                        int wy = e / WZ, wz = e - wy * WZ;
                        uint32_t v = lin(pB, y0 - 1 + wy, z0 - 1 + wz);
                        Vox<K>* xp = xpb + (pB & 1) * WIN;
                        Vox<K> r;
                        if (move) {
                            const uint32_t* dlo = dx_plane(pB - 1);
                            const uint32_t* dme = dx_plane(pB);
                            const uint32_t* dhi = dx_plane(pB + 1);
                            r = combine<K>(raw_plane(pB)[e], dme[e], raw_plane(pB - 1)[e], dlo[e], raw_plane(pB + 1)[e],
                                           dhi[e], v, v - YZ, v + YZ, frame, 0u);
                            xp[e] = r;
                        } else {
                            r = xp[e];
                        }
                        uint32_t d = 0u;
                        if (!vox_empty<K>(r))
                            d = decide(r, v, 1u, code_at(pB, wy, wz), code_at(pB, wy - 1, wz), code_at(pB, wy + 1, wz));
                        dyb[(pB & 1) * WIN + e] = d;
                    } else if (k < bA) {  // C: Y sweep (movers) and/or z-decisions
                        const uint32_t q = k - bC;
                        if (q >= nC) continue;
                        const bool move = q < nC1;
                        int e = move ? wl[LC1 * WIN + q] : wl[LC2 * WIN + (q - nC1)];
                        int wy = e / WZ, wz = e - wy * WZ;
                        uint32_t v = lin(pC, y0 - 1 + wy, z0 - 1 + wz);
                        const Vox<K>* xp = xpb + (pC & 1) * WIN;
                        const uint32_t* dy = dyb + (pC & 1) * WIN;
                        Vox<K>* yp = ypb + (pC & 1) * WIN;
                        Vox<K> r;
                        if (move) {
                            r = combine<K>(xp[e], dy[e], xp[e - WZ], dy[e - WZ], xp[e + WZ], dy[e + WZ], v, v - (uint32_t)Z,
                                           v + (uint32_t)Z, frame, 1u);
                            yp[e] = r;
                        } else {
                            r = yp[e];
                        }
                        uint32_t d = 0u;
                        if (!vox_empty<K>(r))
                            d = decide(r, v, 2u, code_at(pC, wy, wz), code_at(pC, wy, wz - 1), code_at(pC, wy, wz + 1));
                        dzb[(pC & 1) * WIN + e] = d;
                    } else {  // A: x-decisions
                        const uint32_t q = k - bA;
                        if (q >= nA) continue;
                        int e = wl[LA * WIN + q];
                        int wy = e / WZ, wz = e - wy * WZ;
                        uint32_t v = lin(pA, y0 - 1 + wy, z0 - 1 + wz);
                        dx_plane(pA)[e] = decide(raw_plane(pA)[e], v, 0u, code_at(pA, wy, wz), code_at(pA - 1, wy, wz),
                                                 code_at(pA + 1, wy, wz));
                    }
                }
            }
            __syncthreads();
        }
        cp_async_wait<0>();
        // flush this work item's count deltas
        for (uint32_t s = tid; s < P.T.S1; s += NT) {
            int32_t d = s_delta[s];
            if (d) atomicAdd(P.counts + (size_t)rd.counts_index * P.T.S1 + s, (unsigned long long)(long long)d);
        }
    }
    __syncthreads();
    for (int i = tid; i < PD_N; i += NT)
        if (s_diag[i]) atomicAdd(P.diag + i, s_diag[i]);
}

}  // namespace cellsim
