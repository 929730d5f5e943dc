// device_ref.cu — reference-RNG (bit-parity) form of the RDME timestep.
//
// Reproduces the reference shaders' arithmetic exactly (res/shader/rdme.wgsl,
// cme.wgsl, final_stage.wgsl, random.wgsl) in a canonical serial order: voxels
// in linear index order, slots in index order (the reference's own GPU order
// is nondeterministic because of its spin locks and CAS slot insertion).
//
// Directions depend only on the source lattice, so each destination voxel can
// assemble its slots on its own, in serial order: arrivals from the -x, -y, -z
// neighbours, its own departures, arrivals from the +z, +y, +x neighbours,
// each arrival into the lowest free slot.  This equals the serial order when
// no arrival can be rejected; when max(occupancy, nonzero slots) + arrivals >
// K for some voxel (`contended`), a one-thread kernel redoes the frame's
// diffusion in serial order with the capacity rule.
//
// cs_step runs the sparse form on single (in-place) state buffers.  Each pass
// is a grid-stride loop over a voxel list compacted from a bitmap (one atomic
// per warp, word order kept within a warp), so every lane has a voxel however
// sparse the lattice.  Six launches per frame:
//   ref_sp_list_act     the act list: voxels holding a particle, a non-zero
//                       occupancy or a non-zero species count.
//   ref_sp_directions   over the act list: the direction of every particle
//                       from PCG(itime + x%y + z + slot index)
//                       (rdme.wgsl:138-226); voxels with a departure store
//                       their directions and a snapshot of their slots and set
//                       their `dep` bit; every departure counts one arrival at
//                       its destination, sets both voxels' `touch` bits and
//                       raises `contended` when the destination could overflow.
//   ref_sp_list_touch   the touch list and the union of act and touch.
//   ref_sp_gather       (not contended) over the touch list: the gather above,
//                       in place, with the species of arriving particles read
//                       from their sources' snapshots and the concentrations
//                       updated in place.
//   ref_sp_serial       (contended) one thread: the serial diffusion, in place.
//   ref_sp_cme          over the union list: one-event reaction test, rewrite
//                       with rollback, stable compaction (final_stage.wgsl:25-33),
//                       species-count deltas reduced per block; the next
//                       frame's act bitmap.
// A voxel on neither list holds no particle and no species count, its slots
// are compacted and its conc[v][0] is already 1, so the reaction pass leaves
// it unchanged unless its first uniform is 0: r1 = UniformFloat(PCG(itime +
// x*y + z)) is 0 exactly when the seed is 0 (PCG and the xorshift are
// bijections that fix 0), and r1 <= 1 - exp(-0 * tau) = 0 then fires the
// selection.  Pass 1 puts those voxels (x*y + z = -itime mod 2^32) on the
// touch list.  The first frame after an upload, and every frame of a model
// with a reaction without reactants (non-zero propensity in every voxel), run
// the reaction pass over every voxel.
//
// The allocation-free entry point (cs_ref_frame_noalloc) runs the dense form
// of the same frame on caller-owned ping-pong buffers: five launches of one
// thread per voxel (ref_directions, ref_gather, ref_serial_copy, ref_serial,
// ref_cme), the per-voxel operations shared with the sparse form.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "cuda_check.h"
#include "devmath.cuh"
#include "views.cuh"
#include "internal.h"

namespace cellsim {

enum { DIAG_SPILL = 0, DIAG_OCC_RANGE = 1, DIAG_SLOW_STEPS = 2, DIAG_ROLLBACKS = 3, DIAG_FIRED = 4, DIAG_N = 8 };

struct RefParams {
    uint32_t X, Y, Z, K, S1, R, NR;
    uint32_t YZ;
    uint64_t V;
    float tau;
    const float* P;            // [NR][NR][S1]
    const int32_t* stoich;     // [R+1][S1]
    const uint32_t* reactants; // [R+1][3]
    const float* rates;        // [R+1]
    const uint8_t* regions;    // [V]
    const uint8_t* reservoir;  // [V]
};

// State of a reference-RNG handle: one in-place copy of the lattice (slots,
// occupancy, concentrations) and the bitmaps and scratch of the sparse form.
struct DeviceRef {
    int device = 0;
    cudaStream_t stream = nullptr;
    RefParams p{};
    DevBuf<uint8_t> slots;
    DevBuf<uint32_t> occ;
    DevBuf<int32_t> conc;
    DevBuf<uint8_t> regions, reservoir, dirs, snap;
    DevBuf<float> P, rates;
    DevBuf<int32_t> stoich, stat;
    DevBuf<uint32_t> reactants, diag, flag, itimes;
    DevBuf<uint32_t> act_bm[2], touch_bm, dep_bm, act_list, touch_list, union_list, cnt, arrivals;
    DevBuf<int32_t> sample_ring;
    uint32_t par = 0;         // parity of the next frame's lists
    int grid = 1;             // blocks of the sparse passes (grid-stride loops)
    bool dense_next = true;   // the next reaction pass visits every voxel (first frame after an upload)
    bool dense_always = false;  // a reaction without reactants: every voxel may fire in every frame
    ~DeviceRef() {
        if (stream) cudaStreamDestroy(stream);
    }
};

// ------------------------------------------------------------------ kernels

__device__ __forceinline__ float ref_prob(const RefParams& p, uint32_t a, uint32_t b, uint32_t q) {
    return __ldg(p.P + ((size_t)a * p.NR + b) * p.S1 + q);
}

// rdme.wgsl:138-191 (probability vector), :212-226 (draw), :91-130 (edges).
__device__ int ref_decide(const RefParams& p, uint64_t v, uint32_t x, uint32_t y, uint32_t z, uint32_t q,
                          uint32_t i_part, uint32_t itime) {
    const uint8_t* reg = p.regions;
    uint32_t sr = reg[v];
    float pv[6];
    pv[0] = (x > 0u) ? ref_prob(p, sr, reg[v - p.YZ], q) : 0.0f;
    pv[1] = (x < p.X - 1u) ? __fadd_rn(pv[0], ref_prob(p, sr, reg[v + p.YZ], q)) : pv[0];
    pv[2] = (y > 0u) ? __fadd_rn(pv[1], ref_prob(p, sr, reg[v - p.Z], q)) : pv[1];
    pv[3] = (y < p.Y - 1u) ? __fadd_rn(pv[2], ref_prob(p, sr, reg[v + p.Z], q)) : pv[2];
    pv[4] = (z > 0u) ? __fadd_rn(pv[3], ref_prob(p, sr, reg[v - 1], q)) : pv[3];
    pv[5] = (z < p.Z - 1u) ? __fadd_rn(pv[4], ref_prob(p, sr, reg[v + 1], q)) : pv[4];
    uint32_t xmody = (y == 0u) ? 0u : (x % y);  // WGSL: e1 % 0 == 0
    float r = d_uniform_float(d_pcg(itime + xmody + z + i_part));
    int d = 0;
    while (d < 6 && r > pv[d]) d++;
    switch (d) {
        case 0: return (x == 0u) ? 6 : 0;
        case 1: return (x == p.X - 1u) ? 6 : 1;
        case 2: return (y == 0u) ? 6 : 2;
        case 3: return (y == p.Y - 1u) ? 6 : 3;
        case 4: return (z == 0u) ? 6 : 4;
        case 5: return (z == p.Z - 1u) ? 6 : 5;
        default: return 6;
    }
}

// ref_decide with the voxel's region codes loaded once for all its particles (rn: own, x-1, x+1,
// y-1, y+1, z-1, z+1; entries past the lattice edge are not read) and the probability table at Pt
// (shared memory when it fits): the same sums and the same draw.
__device__ __forceinline__ int ref_decide_rn(const RefParams& p, const float* Pt, const uint32_t (&rn)[7], uint32_t x,
                                             uint32_t y, uint32_t z, uint32_t q, uint32_t i_part, uint32_t itime) {
    const size_t row = (size_t)rn[0] * p.NR;
    auto prob = [&](uint32_t b) -> float { return Pt[(row + b) * p.S1 + q]; };
    float pv[6];
    pv[0] = (x > 0u) ? prob(rn[1]) : 0.0f;
    pv[1] = (x < p.X - 1u) ? __fadd_rn(pv[0], prob(rn[2])) : pv[0];
    pv[2] = (y > 0u) ? __fadd_rn(pv[1], prob(rn[3])) : pv[1];
    pv[3] = (y < p.Y - 1u) ? __fadd_rn(pv[2], prob(rn[4])) : pv[2];
    pv[4] = (z > 0u) ? __fadd_rn(pv[3], prob(rn[5])) : pv[3];
    pv[5] = (z < p.Z - 1u) ? __fadd_rn(pv[4], prob(rn[6])) : pv[4];
    uint32_t xmody = (y == 0u) ? 0u : (x % y);  // WGSL: e1 % 0 == 0
    float r = d_uniform_float(d_pcg(itime + xmody + z + i_part));
    int d = 0;
    while (d < 6 && r > pv[d]) d++;
    switch (d) {
        case 0: return (x == 0u) ? 6 : 0;
        case 1: return (x == p.X - 1u) ? 6 : 1;
        case 2: return (y == 0u) ? 6 : 2;
        case 3: return (y == p.Y - 1u) ? 6 : 3;
        case 4: return (z == 0u) ? 6 : 4;
        case 5: return (z == p.Z - 1u) ? 6 : 5;
        default: return 6;
    }
}

__global__ void ref_directions(RefParams p, const uint8_t* __restrict__ src, const uint32_t* __restrict__ occS,
                               const uint32_t* __restrict__ itimes, uint32_t step, uint8_t* __restrict__ dirs,
                               uint32_t* diag, uint32_t* contended) {
    uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v == 0) *contended = 0u;
    if (v >= p.V) return;
    uint32_t z = (uint32_t)(v % p.Z);
    uint32_t y = (uint32_t)((v / p.Z) % p.Y);
    uint32_t x = (uint32_t)(v / p.YZ);
    uint32_t o = occS[v];
    if (o > p.K) { atomicAdd(diag + DIAG_OCC_RANGE, 1u); o = p.K; }
    uint32_t itime = itimes[step];
    for (uint32_t s = 0; s < p.K; s++) {
        uint32_t i_part = (uint32_t)(v * p.K + s);
        uint32_t q = src[i_part];
        uint8_t d = 7;
        if (s < o && q != 0u) d = (uint8_t)ref_decide(p, v, x, y, z, q, i_part, itime);
        dirs[i_part] = d;
    }
}

__device__ __forceinline__ int64_t ref_nb_offset(const RefParams& p, int d) {
    switch (d) {
        case 0: return -(int64_t)p.YZ;
        case 1: return (int64_t)p.YZ;
        case 2: return -(int64_t)p.Z;
        case 3: return (int64_t)p.Z;
        case 4: return -1;
        default: return 1;
    }
}

__global__ void ref_gather(RefParams p, const uint8_t* __restrict__ src, const uint32_t* __restrict__ occS,
                           const int32_t* __restrict__ concS, const uint8_t* __restrict__ dirs,
                           uint8_t* __restrict__ dst, uint32_t* __restrict__ occD, int32_t* __restrict__ concD,
                           uint32_t* contended) {
    uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= p.V) return;
    const uint32_t K = p.K, S1 = p.S1;
    uint32_t z = (uint32_t)(w % p.Z);
    uint32_t y = (uint32_t)((w / p.Z) % p.Y);
    uint32_t x = (uint32_t)(w / p.YZ);
    bool has_nb[6] = {x > 0u, x < p.X - 1u, y > 0u, y < p.Y - 1u, z > 0u, z < p.Z - 1u};
    uint8_t sl[16];
    uint32_t nnz = 0, in = 0;
    for (uint32_t s = 0; s < K; s++) { sl[s] = src[w * K + s]; nnz += sl[s] != 0; }
    for (int side = 0; side < 6; side++) {
        if (!has_nb[side]) continue;
        uint64_t u = (uint64_t)((int64_t)w + ref_nb_offset(p, side));
        uint8_t want = (uint8_t)(side ^ 1);
        for (uint32_t s = 0; s < K; s++) in += dirs[u * K + s] == want;
    }
    uint32_t o = occS[w];
    uint32_t base = o > nnz ? o : nnz;
    if (base + in > K) {
        atomicOr(contended, 1u);
        return;
    }
    int32_t* cw = concD + w * S1;
    const int32_t* cs = concS + w * S1;
    for (uint32_t s = 0; s < S1; s++) cw[s] = cs[s];
    const int lower[3] = {1, 3, 5}, upper[3] = {4, 2, 0};
    for (int k = 0; k < 3; k++) {
        int want = lower[k], side = want ^ 1;
        if (!has_nb[side]) continue;
        uint64_t u = (uint64_t)((int64_t)w + ref_nb_offset(p, side));
        for (uint32_t s = 0; s < K; s++) {
            if (dirs[u * K + s] != want) continue;
            uint8_t q = src[u * K + s];
            uint32_t j = 0;
            while (sl[j] != 0) j++;
            sl[j] = q; o++; cw[q] += 1;
        }
    }
    for (uint32_t s = 0; s < K; s++) {
        if (dirs[w * K + s] < 6) {
            uint8_t q = sl[s];
            sl[s] = 0; o--; cw[q] -= 1;
        }
    }
    for (int k = 0; k < 3; k++) {
        int want = upper[k], side = want ^ 1;
        if (!has_nb[side]) continue;
        uint64_t u = (uint64_t)((int64_t)w + ref_nb_offset(p, side));
        for (uint32_t s = 0; s < K; s++) {
            if (dirs[u * K + s] != want) continue;
            uint8_t q = src[u * K + s];
            uint32_t j = 0;
            while (sl[j] != 0) j++;
            sl[j] = q; o++; cw[q] += 1;
        }
    }
    for (uint32_t s = 0; s < K; s++) dst[w * K + s] = sl[s];
    occD[w] = o;
}

__global__ void ref_serial_copy(RefParams p, const uint32_t* contended, const uint8_t* __restrict__ src,
                                const uint32_t* __restrict__ occS, const int32_t* __restrict__ concS,
                                uint8_t* __restrict__ dst, uint32_t* __restrict__ occD, int32_t* __restrict__ concD) {
    if (*contended == 0u) return;
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (uint64_t i = t; i < p.V * p.K; i += stride) dst[i] = src[i];
    for (uint64_t i = t; i < p.V; i += stride) occD[i] = occS[i];
    for (uint64_t i = t; i < p.V * p.S1; i += stride) concD[i] = concS[i];
}

// Serial diffusion with the capacity rule (rdme.wgsl:45-88): a move into a
// voxel whose occupancy is >= K, or that has no zero slot, is rejected.
__global__ void ref_serial(RefParams p, const uint32_t* contended, const uint8_t* __restrict__ src,
                           const uint32_t* __restrict__ occS, const uint8_t* __restrict__ dirs,
                           uint8_t* __restrict__ dst, uint32_t* __restrict__ occD, int32_t* __restrict__ concD,
                           uint32_t* diag) {
    if (*contended == 0u || threadIdx.x != 0 || blockIdx.x != 0) return;
    const uint32_t K = p.K, S1 = p.S1;
    uint32_t spills = 0;
    for (uint64_t v = 0; v < p.V; v++) {
        uint32_t o = occS[v];
        if (o > K) o = K;
        for (uint32_t s = 0; s < o; s++) {
            uint64_t i = v * K + s;
            int d = dirs[i];
            if (d >= 6) continue;
            uint64_t w = (uint64_t)((int64_t)v + ref_nb_offset(p, d));
            if (occD[w] >= K) { spills++; continue; }
            uint32_t j = 0;
            while (j < K && dst[w * K + j] != 0) j++;
            if (j == K) { spills++; continue; }
            uint8_t q = src[i];
            dst[w * K + j] = q;
            occD[w] += 1u;
            concD[w * S1 + q] += 1;
            occD[v] -= 1u;
            dst[i] = 0;
            concD[v * S1 + q] -= 1;
        }
    }
    diag[DIAG_SPILL] += spills;
    diag[DIAG_SLOW_STEPS] += 1u;
}

// Coordinates of voxel v (V * K < 2^32 on this path: the reference indexes
// slots with u32, functions.wgsl:42-51).
__device__ __forceinline__ void ref_coords(const RefParams& p, uint32_t v, uint32_t& x, uint32_t& y, uint32_t& z) {
    const uint32_t t = v / p.Z;
    z = v - t * p.Z;
    x = t / p.Y;
    y = t - x * p.Y;
}

// The K (<= 16) slot bytes of one voxel held in two 64-bit registers, byte i =
// slot i, so that the reaction pass touches the slot array with one load and
// at most one store per voxel.
struct RefSlots {
    uint64_t lo, hi;
};

__device__ __forceinline__ uint32_t rs_get(const RefSlots& a, uint32_t i) {
    return (uint32_t)((i < 8u ? a.lo >> (8u * i) : a.hi >> (8u * (i - 8u))) & 0xFFull);
}

__device__ __forceinline__ void rs_set(RefSlots& a, uint32_t i, uint32_t q) {
    if (i < 8u) a.lo = (a.lo & ~(0xFFull << (8u * i))) | ((uint64_t)q << (8u * i));
    else a.hi = (a.hi & ~(0xFFull << (8u * (i - 8u)))) | ((uint64_t)q << (8u * (i - 8u)));
}

// Vector access when K is 8 or 16 and the voxel's slots are aligned to it (the library's own
// buffers always are; a caller's buffer of the allocation-free entry point may not be).
__device__ __forceinline__ RefSlots rs_load(const uint8_t* sl, uint32_t K) {
    RefSlots a{0ull, 0ull};
    const uintptr_t al = (uintptr_t)sl;
    if (K == 16u && (al & 15u) == 0u) {
        const uint4 t = *reinterpret_cast<const uint4*>(sl);
        a.lo = (uint64_t)t.x | ((uint64_t)t.y << 32);
        a.hi = (uint64_t)t.z | ((uint64_t)t.w << 32);
    } else if (K == 8u && (al & 7u) == 0u) {
        const uint2 t = *reinterpret_cast<const uint2*>(sl);
        a.lo = (uint64_t)t.x | ((uint64_t)t.y << 32);
    } else {
        for (uint32_t i = 0; i < K; i++) rs_set(a, i, sl[i]);
    }
    return a;
}

__device__ __forceinline__ void rs_store(uint8_t* sl, uint32_t K, const RefSlots& a) {
    const uintptr_t al = (uintptr_t)sl;
    if (K == 16u && (al & 15u) == 0u) {
        *reinterpret_cast<uint4*>(sl) = make_uint4((uint32_t)a.lo, (uint32_t)(a.lo >> 32), (uint32_t)a.hi,
                                                   (uint32_t)(a.hi >> 32));
    } else if (K == 8u && (al & 7u) == 0u) {
        *reinterpret_cast<uint2*>(sl) = make_uint2((uint32_t)a.lo, (uint32_t)(a.lo >> 32));
    } else {
        for (uint32_t i = 0; i < K; i++) sl[i] = (uint8_t)rs_get(a, i);
    }
}

// cme.wgsl:26-120 and final_stage.wgsl:25-33 for voxel v, in place:
// conc[v][0] = 1, the one-event test, the species-major rewrite with rollback
// and the stable compaction.  s_delta[0..S1) collects species deltas,
// s_delta[S1] fired voxels and s_delta[S1 + 1] rollbacks (block-shared).
__device__ void ref_cme_voxel(const RefParams& p, uint64_t v, uint8_t* __restrict__ slots, uint32_t* __restrict__ occ,
                              int32_t* __restrict__ conc, uint32_t itime, int32_t* s_delta) {
    const uint32_t K = p.K, S1 = p.S1, R = p.R;
    const uint32_t S = S1 - 1;
    uint32_t x, y, z;
    ref_coords(p, (uint32_t)v, x, y, z);
    int32_t* c = conc + v * S1;
    uint8_t* slp = slots + v * K;
    if (c[0] != 1) c[0] = 1;  // stored only when it changes: an unchanged row is not written back
    float total = 0.0f;
    for (uint32_t r = 1; r <= R; r++) {
        uint32_t prod = (uint32_t)c[p.reactants[r * 3]] * (uint32_t)c[p.reactants[r * 3 + 1]] *
                        (uint32_t)c[p.reactants[r * 3 + 2]];
        total = __fadd_rn(total, __fmul_rn(p.rates[r], __int2float_rn((int32_t)prod)));
    }
    const RefSlots snap = rs_load(slp, K);
    RefSlots sl = snap;
    uint32_t state = d_pcg(itime + x * y + z);
    float r1 = d_uniform_float(state);
    float fire_p = __fsub_rn(1.0f, d_expf(__fmul_rn(-total, p.tau)));
    if (r1 <= fire_p) {
        atomicAdd(&s_delta[S1], 1);
        float r2 = d_uniform_float(state + 1u);
        // selection over cum[i] = cum[i-1] + a_i, normalised for i < R (cme.wgsl:50-52,70-73)
        uint32_t i = 0;
        float run = 0.0f;
        while (i < R) {
            if (!(r2 > __fdiv_rn(run, total))) break;
            i++;
            uint32_t prod = (uint32_t)c[p.reactants[i * 3]] * (uint32_t)c[p.reactants[i * 3 + 1]] *
                            (uint32_t)c[p.reactants[i * 3 + 2]];
            run = __fadd_rn(run, __fmul_rn(p.rates[i], __int2float_rn((int32_t)prod)));
        }
        const int32_t* st = p.stoich + (size_t)i * S1;
        uint32_t j = 0;
        int32_t new_occ = (int32_t)occ[v];
        uint64_t ri = v * K;  // reservoirs[idx_lattice], cme.wgsl:80
        uint32_t resv = (ri < p.V) ? p.reservoir[ri] : 0u;
        bool rolled = false;
        for (uint32_t s = 1; s <= S && !rolled; s++) {
            if (resv == s) continue;
            int32_t d = st[s];
            c[s] = (int32_t)((uint32_t)c[s] + (uint32_t)d);
            new_occ = (int32_t)((uint32_t)new_occ + (uint32_t)d);
            if (d) atomicAdd(&s_delta[s], d);
            int32_t cc = c[s];
            while (cc > 0) {
                rs_set(sl, j, s);
                cc--;
                j++;
                if (j >= K) {
                    sl = snap;
                    for (uint32_t s2 = 1; s2 <= s; s2++) {
                        int32_t d2 = st[s2];
                        c[s2] = (int32_t)((uint32_t)c[s2] - (uint32_t)d2);
                        if (d2) atomicAdd(&s_delta[s2], -d2);
                    }
                    atomicAdd(&s_delta[S1 + 1], 1);
                    rolled = true;
                    break;
                }
            }
        }
        if (!rolled) {
            occ[v] = (uint32_t)new_occ;
            while (j < K) rs_set(sl, j++, 0u);
        }
    }
    // stable move of the non-zero slots to the front
    RefSlots out{0ull, 0ull};
    uint32_t jj = 0;
    for (uint32_t s = 0; s < K; s++) {
        const uint32_t q = rs_get(sl, s);
        if (q != 0u) rs_set(out, jj++, q);
    }
    if (out.lo != snap.lo || out.hi != snap.hi) rs_store(slp, K, out);
}

// Adds a block's species deltas, fired voxels and rollbacks to the totals.
__device__ __forceinline__ void ref_flush_block(const RefParams& p, const int32_t* s_delta, int32_t* stat, uint32_t* diag) {
    for (uint32_t s = threadIdx.x; s < p.S1; s += blockDim.x)
        if (s_delta[s]) atomicAdd(stat + s, s_delta[s]);
    if (threadIdx.x == 0) {
        if (s_delta[p.S1]) atomicAdd(diag + DIAG_FIRED, (uint32_t)s_delta[p.S1]);
        if (s_delta[p.S1 + 1]) atomicAdd(diag + DIAG_ROLLBACKS, (uint32_t)s_delta[p.S1 + 1]);
    }
}

// Dense reaction pass: one thread per voxel.
__global__ void ref_cme(RefParams p, uint8_t* __restrict__ dst, uint32_t* __restrict__ occD, int32_t* __restrict__ concD,
                        const uint32_t* __restrict__ itimes, uint32_t step, int32_t* stat, uint32_t* diag) {
    extern __shared__ int32_t s_delta[];  // [S1] + 2 counters
    for (uint32_t s = threadIdx.x; s < p.S1 + 2; s += blockDim.x) s_delta[s] = 0;
    __syncthreads();
    uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v < p.V) ref_cme_voxel(p, v, dst, occD, concD, itimes[step], s_delta);
    __syncthreads();
    ref_flush_block(p, s_delta, stat, diag);
}

// ------------------------------------------------------------------ sparse form

// Bitmaps over the linear voxel index (word i holds voxels 32i .. 32i+31) and
// the voxel lists compacted from them, for a frame of parity c:
//   act bitmap c   voxels that hold a particle, a non-zero occupancy or a
//                  non-zero species count (s >= 1); the reaction pass sets
//                  act bitmap c ^ 1 for the next frame
//   touch bitmap   voxels that gain or lose particles this frame, or whose
//                  reaction seed is 0
//   dep bitmap     voxels with a departure this frame
//   act list       act bitmap c, compacted at the start of the frame
//   touch list     the touch bitmap, compacted after the directions pass
//   union list     act bitmap c | touch bitmap, compacted with it
// cnt[0..2]: entries of the act, touch and union lists.
struct RefSparse {
    uint32_t* act_bm[2];
    uint32_t* touch_bm;
    uint32_t* dep_bm;
    uint32_t* act_list;
    uint32_t* touch_list;
    uint32_t* union_list;
    uint32_t* cnt;       // [3]
    uint32_t* arrivals;  // [V] particles moving into the voxel this frame (zero between frames)
    uint8_t* dirs;       // [V*K] direction codes of a voxel with a departure (7 = stays)
    uint8_t* snap;       // [V*K] slots of a voxel with a departure, as the frame started
    uint32_t W;          // bitmap words
    uint32_t c;          // frame parity
};

// act bitmaps of this frame and the next, chosen by select (indexing the kernel parameter's
// array by a run-time value would copy the parameters to local memory)
__device__ __forceinline__ uint32_t* act_cur(const RefSparse& sp) { return sp.c ? sp.act_bm[1] : sp.act_bm[0]; }
__device__ __forceinline__ uint32_t* act_next(const RefSparse& sp) { return sp.c ? sp.act_bm[0] : sp.act_bm[1]; }

__device__ __forceinline__ bool bit_of(const uint32_t* bm, uint32_t v) { return (__ldcg(bm + (v >> 5)) >> (v & 31u)) & 1u; }
__device__ __forceinline__ void set_bit(uint32_t* bm, uint32_t v) { atomicOr(bm + (v >> 5), 1u << (v & 31u)); }

__device__ __forceinline__ uint32_t grid_threads() { return gridDim.x * blockDim.x; }
__device__ __forceinline__ uint32_t grid_tid() { return blockIdx.x * blockDim.x + threadIdx.x; }

// Appends the voxels of bitmap word `m` (word index i) to a list, every lane of
// the warp calling it with its own word: one atomic per warp reserves the
// warp's entries, which keep word order within the warp.
__device__ __forceinline__ void warp_compact(uint32_t m, uint32_t i, uint32_t* list, uint32_t* counter) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t n = (uint32_t)__popc(m);
    uint32_t incl = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += u;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    if (total == 0u) return;
    uint32_t base = 0;
    if (lane == 31u) base = atomicAdd(counter, total);
    base = __shfl_sync(0xffffffffu, base, 31) + incl - n;
    for (; m; m &= m - 1u) list[base++] = i * 32u + (uint32_t)(__ffs((int)m) - 1);
}

// Programmatic dependent launch between the passes of a frame: a pass lets the next one launch at
// once and waits for the previous one to complete (and its memory to be visible) before it touches
// anything; without a programmatic dependency the wait returns at once.
__device__ __forceinline__ void ref_pdl_start() {
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
}

// Each pass is a device body with grid-stride loops, run by its own launch (a thin kernel that
// waits for the previous pass first) or, on small lattices, by the one-block form
// ref_sp_frames_block.

// The act list of act bitmap c.
__device__ __forceinline__ void ref_sp_list_act_body(RefSparse sp) {
    for (uint32_t i0 = grid_tid() & ~31u; i0 < sp.W; i0 += grid_threads()) {
        const uint32_t i = i0 + (threadIdx.x & 31u);
        warp_compact(i < sp.W ? act_cur(sp)[i] : 0u, i, sp.act_list, sp.cnt + 0);
    }
}

__global__ void __launch_bounds__(256) ref_sp_list_act(RefSparse sp) {
    ref_pdl_start();
    ref_sp_list_act_body(sp);
}

// The touch list, and the union list of act bitmap c and the touch bitmap.
__device__ __forceinline__ void ref_sp_list_touch_body(RefSparse sp) {
    for (uint32_t i0 = grid_tid() & ~31u; i0 < sp.W; i0 += grid_threads()) {
        const uint32_t i = i0 + (threadIdx.x & 31u);
        const uint32_t t = i < sp.W ? __ldcg(sp.touch_bm + i) : 0u;
        const uint32_t a = i < sp.W ? act_cur(sp)[i] : 0u;
        warp_compact(t, i, sp.touch_list, sp.cnt + 1);
        warp_compact(a | t, i, sp.union_list, sp.cnt + 2);
    }
}

__global__ void __launch_bounds__(256) ref_sp_list_touch(RefSparse sp) {
    ref_pdl_start();
    ref_sp_list_touch_body(sp);
}

// Pass 1: directions of every particle of the act list; departures, arrival
// counts, touched voxels and the contention test.  Also marks the voxels whose
// reaction seed itime + x*y + z is 0 this frame, clears act bitmap c ^ 1 (the
// reaction pass fills it) and the touch and union list counters.
__device__ __forceinline__ void ref_sp_directions_body(RefParams p, RefSparse sp, const uint8_t* slots,
                                                       const uint32_t* occ, const uint32_t* itimes, uint32_t step,
                                                       uint32_t* diag, uint32_t* contended, uint32_t stage_P) {
    const uint32_t itime = __ldg(itimes + step);
    const uint32_t K = p.K;
    const uint32_t n = __ldcg(sp.cnt + 0);
    if (grid_tid() == 0) {
        sp.cnt[1] = 0u;
        sp.cnt[2] = 0u;
    }
    // the probability table in shared memory when the launch gave room for it
    extern __shared__ float s_P[];
    const float* Pt = p.P;
    if (stage_P) {
        for (uint32_t i = threadIdx.x; i < p.NR * p.NR * p.S1; i += blockDim.x) s_P[i] = p.P[i];
        __syncthreads();
        Pt = s_P;
    }
    for (uint32_t i = grid_tid(); i < sp.W; i += grid_threads()) act_next(sp)[i] = 0u;
    const uint32_t XY = p.X * p.Y;
    for (uint32_t g = grid_tid(); g < XY; g += grid_threads()) {
        const uint32_t x = g / p.Y, y = g - x * p.Y;
        const uint32_t z = 0u - itime - x * y;  // u32 wrap, as the shader's seed arithmetic
        if (z < p.Z) set_bit(sp.touch_bm, g * p.Z + z);
    }
    for (uint32_t e = grid_tid(); e < n; e += grid_threads()) {
        const uint32_t v = sp.act_list[e];
        uint32_t o = occ[v];
        if (o > K) {
            // the gather's contention test fails for this voxel whatever arrives
            atomicAdd(diag + DIAG_OCC_RANGE, 1u);
            atomicOr(contended, 1u);
            o = K;
        }
        const RefSlots sl = rs_load(slots + (size_t)v * K, K);
        uint32_t x, y, z;
        ref_coords(p, v, x, y, z);
        const uint8_t* reg = p.regions;
        uint32_t rn[7] = {reg[v], 0u, 0u, 0u, 0u, 0u, 0u};
        if (x > 0u) rn[1] = reg[v - p.YZ];
        if (x < p.X - 1u) rn[2] = reg[v + p.YZ];
        if (y > 0u) rn[3] = reg[v - p.Z];
        if (y < p.Y - 1u) rn[4] = reg[v + p.Z];
        if (z > 0u) rn[5] = reg[v - 1];
        if (z < p.Z - 1u) rn[6] = reg[v + 1];
        bool has_dep = false;
        RefSlots dr{0x0707070707070707ull, 0x0707070707070707ull};  // 7: stays
        for (uint32_t s = 0; s < K; s++) {
            const uint32_t q = rs_get(sl, s);
            if (s < o && q != 0u) {
                const int d = ref_decide_rn(p, Pt, rn, x, y, z, q, v * K + s, itime);
                rs_set(dr, s, (uint32_t)d);
                has_dep |= d < 6;
            }
        }
        if (!has_dep) continue;
        rs_store(sp.dirs + (size_t)v * K, K, dr);
        rs_store(sp.snap + (size_t)v * K, K, sl);
        set_bit(sp.dep_bm, v);
        set_bit(sp.touch_bm, v);
        for (uint32_t s = 0; s < K; s++) {
            const uint32_t ds = rs_get(dr, s);
            if (ds >= 6u) continue;
            const uint32_t w = (uint32_t)((int64_t)v + ref_nb_offset(p, (int)ds));
            const uint32_t before = atomicAdd(sp.arrivals + w, 1u);
            const RefSlots ws = rs_load(slots + (size_t)w * K, K);
            uint32_t nnz = 0;
            for (uint32_t t = 0; t < K; t++) nnz += rs_get(ws, t) != 0u;
            const uint32_t ow = occ[w];
            const uint32_t base = ow > nnz ? ow : nnz;
            if ((uint64_t)base + before + 1u > K) atomicOr(contended, 1u);
            set_bit(sp.touch_bm, w);
        }
    }
}

__global__ void __launch_bounds__(256) ref_sp_directions(RefParams p, RefSparse sp, const uint8_t* __restrict__ slots,
                                                         const uint32_t* __restrict__ occ,
                                                         const uint32_t* __restrict__ itimes, uint32_t step,
                                                         uint32_t* diag, uint32_t* contended, uint32_t stage_P) {
    ref_pdl_start();
    ref_sp_directions_body(p, sp, slots, occ, itimes, step, diag, contended, stage_P);
}

// Pass 2 (frames without contention): the gather of every touched voxel, in place.
__device__ __forceinline__ void ref_sp_gather_body(RefParams p, RefSparse sp, uint8_t* slots, uint32_t* occ,
                                                   int32_t* conc, const uint32_t* contended) {
    if (*contended) return;
    const uint32_t K = p.K, S1 = p.S1;
    const uint32_t n = __ldcg(sp.cnt + 1);
    for (uint32_t e = grid_tid(); e < n; e += grid_threads()) {
        const uint32_t w = sp.touch_list[e];
        sp.arrivals[w] = 0u;
        uint32_t x, y, z;
        ref_coords(p, w, x, y, z);
        const bool has_nb[6] = {x > 0u, x < p.X - 1u, y > 0u, y < p.Y - 1u, z > 0u, z < p.Z - 1u};
        RefSlots sl = rs_load(slots + (size_t)w * K, K);
        uint32_t o = occ[w];
        int32_t* cw = conc + (size_t)w * S1;
        // arrivals from the neighbour on `side`: the particles it moves in direction side ^ 1
        auto arrive = [&](int side) {
            if (!has_nb[side]) return;
            const uint32_t u = (uint32_t)((int64_t)w + ref_nb_offset(p, side));
            if (!bit_of(sp.dep_bm, u)) return;
            const uint32_t want = (uint32_t)(side ^ 1);
            const RefSlots nd = rs_load(sp.dirs + (size_t)u * K, K);
            const RefSlots ns = rs_load(sp.snap + (size_t)u * K, K);
            for (uint32_t s = 0; s < K; s++) {
                if (rs_get(nd, s) != want) continue;
                const uint32_t q = rs_get(ns, s);
                uint32_t j = 0;
                while (j < K && rs_get(sl, j) != 0u) j++;
                if (j == K) continue;  // unreachable without contention
                rs_set(sl, j, q);
                o++;
                cw[q] = (int32_t)((uint32_t)cw[q] + 1u);
            }
        };
        arrive(0);  // from -x
        arrive(2);  // from -y
        arrive(4);  // from -z
        if (bit_of(sp.dep_bm, w)) {
            const RefSlots nd = rs_load(sp.dirs + (size_t)w * K, K);
            for (uint32_t s = 0; s < K; s++) {
                if (rs_get(nd, s) >= 6u) continue;
                const uint32_t q = rs_get(sl, s);
                rs_set(sl, s, 0u);
                o--;
                cw[q] = (int32_t)((uint32_t)cw[q] - 1u);
            }
        }
        arrive(5);  // from +z
        arrive(3);  // from +y
        arrive(1);  // from +x
        rs_store(slots + (size_t)w * K, K, sl);
        occ[w] = o;
    }
}

__global__ void __launch_bounds__(256) ref_sp_gather(RefParams p, RefSparse sp, uint8_t* __restrict__ slots,
                                                     uint32_t* __restrict__ occ, int32_t* __restrict__ conc,
                                                     const uint32_t* __restrict__ contended) {
    ref_pdl_start();
    ref_sp_gather_body(p, sp, slots, occ, conc, contended);
}

// Pass 3 (contended frames): the serial diffusion of rdme.wgsl:45-88 in place,
// voxels in linear order.  A departing slot still holds its particle when its
// voxel's turn comes (arrivals only fill empty slots), and a slot that an
// arrival filled has direction 7.  One block scans the departure bitmap; its
// first thread makes the moves.
__device__ __forceinline__ void ref_sp_serial_body(RefParams p, RefSparse sp, uint8_t* slots, uint32_t* occ,
                                                   int32_t* conc, uint32_t* diag, const uint32_t* contended) {
    if (*contended == 0u) return;
    __shared__ uint32_t s_words[1024];
    const uint32_t K = p.K, S1 = p.S1;
    uint32_t spills = 0;
    for (uint32_t w0 = 0; w0 < sp.W; w0 += blockDim.x) {
        const uint32_t i = w0 + threadIdx.x;
        s_words[threadIdx.x] = i < sp.W ? sp.dep_bm[i] : 0u;
        __syncthreads();
        if (threadIdx.x == 0) {
            for (uint32_t k = 0; k < blockDim.x && w0 + k < sp.W; k++) {
                for (uint32_t m = s_words[k]; m; m &= m - 1u) {
                    const uint32_t v = (w0 + k) * 32u + (uint32_t)(__ffs((int)m) - 1);
                    for (uint32_t s = 0; s < K; s++) {
                        const int d = sp.dirs[(size_t)v * K + s];
                        if (d >= 6) continue;
                        const uint32_t w = (uint32_t)((int64_t)v + ref_nb_offset(p, d));
                        sp.arrivals[w] = 0u;
                        if (occ[w] >= K) { spills++; continue; }
                        uint32_t j = 0;
                        while (j < K && slots[(size_t)w * K + j] != 0) j++;
                        if (j == K) { spills++; continue; }
                        const uint8_t q = slots[(size_t)v * K + s];
                        slots[(size_t)w * K + j] = q;
                        occ[w] += 1u;
                        conc[(size_t)w * S1 + q] = (int32_t)((uint32_t)conc[(size_t)w * S1 + q] + 1u);
                        occ[v] -= 1u;
                        slots[(size_t)v * K + s] = 0;
                        conc[(size_t)v * S1 + q] = (int32_t)((uint32_t)conc[(size_t)v * S1 + q] - 1u);
                    }
                }
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        diag[DIAG_SPILL] += spills;
        diag[DIAG_SLOW_STEPS] += 1u;
    }
}

__global__ void ref_sp_serial(RefParams p, RefSparse sp, uint8_t* __restrict__ slots, uint32_t* __restrict__ occ,
                              int32_t* __restrict__ conc, uint32_t* diag, const uint32_t* __restrict__ contended) {
    ref_pdl_start();
    ref_sp_serial_body(p, sp, slots, occ, conc, diag, contended);
}

// The reaction pass on one voxel and its bit in act bitmap c ^ 1.
// The reaction tables of ref_cme_voxel staged in shared memory by the reaction pass.
struct RefTables {
    const uint32_t* reactants;  // [R+1][3]
    const float* rates;         // [R+1]
    const int32_t* stoich;      // [R+1][S1]
};

// ref_cme_voxel with the tables in shared memory (T) and the voxel's concentration row copied into
// the thread's shared-memory row `row` while it is evaluated (every change is written through to
// the global row): the same operations in the same order, so the same results, with the
// propensity and selection loops reading shared memory instead of about a hundred dependent
// global loads per voxel.
__device__ __forceinline__ void ref_cme_voxel_rows(const RefParams& p, const RefTables& T, uint64_t v,
                                                   uint8_t* __restrict__ slots, uint32_t* __restrict__ occ,
                                                   int32_t* __restrict__ conc, uint32_t itime, int32_t* s_delta,
                                                   int32_t* row) {
    const uint32_t K = p.K, S1 = p.S1, R = p.R;
    const uint32_t S = S1 - 1;
    uint32_t x, y, z;
    ref_coords(p, (uint32_t)v, x, y, z);
    int32_t* c = conc + v * S1;
    for (uint32_t s = 0; s < S1; s++) row[s] = c[s];
    if (row[0] != 1) {  // stored only when it changes: an unchanged row is not written back
        row[0] = 1;
        c[0] = 1;
    }
    auto prop_of = [&](uint32_t r) -> float {
        const uint32_t prod = (uint32_t)row[T.reactants[r * 3]] * (uint32_t)row[T.reactants[r * 3 + 1]] *
                              (uint32_t)row[T.reactants[r * 3 + 2]];
        return __fmul_rn(T.rates[r], __int2float_rn((int32_t)prod));
    };
    float total = 0.0f;
    for (uint32_t r = 1; r <= R; r++) total = __fadd_rn(total, prop_of(r));
    const RefSlots snap = rs_load(slots + v * K, K);
    RefSlots sl = snap;
    uint32_t state = d_pcg(itime + x * y + z);
    float r1 = d_uniform_float(state);
    float fire_p = __fsub_rn(1.0f, d_expf(__fmul_rn(-total, p.tau)));
    if (r1 <= fire_p) {
        atomicAdd(&s_delta[S1], 1);
        float r2 = d_uniform_float(state + 1u);
        // selection over cum[i] = cum[i-1] + a_i, normalised for i < R (cme.wgsl:50-52,70-73)
        uint32_t i = 0;
        float run = 0.0f;
        while (i < R) {
            if (!(r2 > __fdiv_rn(run, total))) break;
            i++;
            run = __fadd_rn(run, prop_of(i));
        }
        const int32_t* st = T.stoich + (size_t)i * S1;
        uint32_t j = 0;
        int32_t new_occ = (int32_t)occ[v];
        uint64_t ri = v * K;  // reservoirs[idx_lattice], cme.wgsl:80
        uint32_t resv = (ri < p.V) ? p.reservoir[ri] : 0u;
        bool rolled = false;
        for (uint32_t s = 1; s <= S && !rolled; s++) {
            if (resv == s) continue;
            int32_t d = st[s];
            row[s] = (int32_t)((uint32_t)row[s] + (uint32_t)d);
            if (d) c[s] = row[s];
            new_occ = (int32_t)((uint32_t)new_occ + (uint32_t)d);
            if (d) atomicAdd(&s_delta[s], d);
            int32_t cc = row[s];
            while (cc > 0) {
                rs_set(sl, j, s);
                cc--;
                j++;
                if (j >= K) {
                    sl = snap;
                    for (uint32_t s2 = 1; s2 <= s; s2++) {
                        int32_t d2 = st[s2];
                        row[s2] = (int32_t)((uint32_t)row[s2] - (uint32_t)d2);
                        if (d2) {
                            c[s2] = row[s2];
                            atomicAdd(&s_delta[s2], -d2);
                        }
                    }
                    atomicAdd(&s_delta[S1 + 1], 1);
                    rolled = true;
                    break;
                }
            }
        }
        if (!rolled) {
            occ[v] = (uint32_t)new_occ;
            while (j < K) rs_set(sl, j++, 0u);
        }
    }
    // stable move of the non-zero slots to the front
    RefSlots out{0ull, 0ull};
    uint32_t jj = 0;
    for (uint32_t s = 0; s < K; s++) {
        const uint32_t q = rs_get(sl, s);
        if (q != 0u) rs_set(out, jj++, q);
    }
    if (out.lo != snap.lo || out.hi != snap.hi) rs_store(slots + v * K, K, out);
}

// rows: the staged tables T and the thread's shared-memory concentration row `row` are used (else,
// when they do not fit, the global-memory form)
__device__ __forceinline__ void ref_sp_react(const RefParams& p, const RefSparse& sp, uint32_t v, uint8_t* slots,
                                             uint32_t* occ, int32_t* conc, uint32_t itime, int32_t* s_delta,
                                             bool rows, const RefTables& T, int32_t* row) {
    const uint32_t K = p.K, S1 = p.S1;
    const int32_t* c = conc + (size_t)v * S1;
    if (rows) {
        ref_cme_voxel_rows(p, T, v, slots, occ, conc, itime, s_delta, row);
        c = row;
    } else {
        ref_cme_voxel(p, v, slots, occ, conc, itime, s_delta);
    }
    const RefSlots sl = rs_load(slots + (size_t)v * K, K);
    bool keep = occ[v] != 0u || (sl.lo | sl.hi) != 0ull;
    for (uint32_t s = 1; s < S1 && !keep; s++) keep |= c[s] != 0;
    if (keep) set_bit(act_next(sp), v);
}

// Pass 4: the reaction pass over the union list (every voxel when `dense`),
// setting act bitmap c ^ 1; clears the contention flag, the touch and
// departure bitmaps and the act list counter for the next frame.
__device__ __forceinline__ void ref_sp_cme_body(RefParams p, RefSparse sp, uint8_t* slots, uint32_t* occ,
                                                int32_t* conc, const uint32_t* itimes, uint32_t step, uint32_t dense,
                                                int32_t* stat, uint32_t* diag, uint32_t* contended, uint32_t rows) {
    extern __shared__ int32_t s_delta[];  // [S1] + 2 counters, then (rows) the tables and the rows
    for (uint32_t s = threadIdx.x; s < p.S1 + 2; s += blockDim.x) s_delta[s] = 0;
    if (grid_tid() == 0) {
        *contended = 0u;  // every reader of this frame's flag has run
        sp.cnt[0] = 0u;
    }
    RefTables T{};
    int32_t* row = nullptr;
    if (rows) {
        uint32_t* s_re = reinterpret_cast<uint32_t*>(s_delta + p.S1 + 2);
        float* s_rate = reinterpret_cast<float*>(s_re + 3 * (p.R + 1));
        int32_t* s_st = reinterpret_cast<int32_t*>(s_rate + (p.R + 1));
        for (uint32_t i = threadIdx.x; i < 3 * (p.R + 1); i += blockDim.x) s_re[i] = p.reactants[i];
        for (uint32_t i = threadIdx.x; i < p.R + 1; i += blockDim.x) s_rate[i] = p.rates[i];
        for (uint32_t i = threadIdx.x; i < (p.R + 1) * p.S1; i += blockDim.x) s_st[i] = p.stoich[i];
        T = RefTables{s_re, s_rate, s_st};
        row = s_st + (p.R + 1) * p.S1 + threadIdx.x * p.S1;
    }
    __syncthreads();
    const uint32_t itime = __ldg(itimes + step);
    for (uint32_t i = grid_tid(); i < sp.W; i += grid_threads()) {
        sp.touch_bm[i] = 0u;
        sp.dep_bm[i] = 0u;
    }
    if (dense) {
        for (uint32_t v = grid_tid(); v < (uint32_t)p.V; v += grid_threads())
            ref_sp_react(p, sp, v, slots, occ, conc, itime, s_delta, rows != 0u, T, row);
    } else {
        const uint32_t n = __ldcg(sp.cnt + 2);
        for (uint32_t e = grid_tid(); e < n; e += grid_threads())
            ref_sp_react(p, sp, sp.union_list[e], slots, occ, conc, itime, s_delta, rows != 0u, T, row);
    }
    __syncthreads();
    ref_flush_block(p, s_delta, stat, diag);
}

__global__ void __launch_bounds__(256) ref_sp_cme(RefParams p, RefSparse sp, uint8_t* __restrict__ slots,
                                                  uint32_t* __restrict__ occ, int32_t* __restrict__ conc,
                                                  const uint32_t* __restrict__ itimes, uint32_t step, uint32_t dense,
                                                  int32_t* stat, uint32_t* diag, uint32_t* contended, uint32_t rows) {
    ref_pdl_start();
    ref_sp_cme_body(p, sp, slots, occ, conc, itimes, step, dense, stat, diag, contended, rows);
}

// Threads of the one-block form below.
constexpr int REF_BLOCK_THREADS = 512;
// Lattices of at most this many voxels run every frame of a call in the one-block form: one SM does
// such a frame's work sooner than six launches take to run back to back.  Measured on cubic
// lattices with one particle per 16 voxels: six launches take 31-36 us a frame at any size from
// 4,096 to 110,592 voxels, the one block 22.9 us at 4,096 and 69.8 us at 13,824 voxels (its time
// follows the particles).
constexpr uint64_t REF_BLOCK_MAX_VOXELS = 6144;

// Every frame of a step call in one block: the passes' own bodies in the same order, with block
// barriers where the launches were (the serial pass runs on the same block).  The bodies read
// nothing that the block writes through the non-coherent path (their pointers carry no
// __restrict__ here), so each pass sees the previous one's writes after the barrier.
__global__ void __launch_bounds__(REF_BLOCK_THREADS, 1)
    ref_sp_frames_block(RefParams p, RefSparse sp, uint8_t* slots, uint32_t* occ, int32_t* conc,
                        const uint32_t* itimes, uint32_t step0, uint32_t n, uint32_t dense_first,
                        uint32_t dense_always, int32_t* stat, uint32_t* diag, uint32_t* contended, uint32_t stage_P,
                        uint32_t rows) {
    for (uint32_t k = 0; k < n; k++) {
        ref_sp_list_act_body(sp);
        __syncthreads();
        ref_sp_directions_body(p, sp, slots, occ, itimes, step0 + k, diag, contended, stage_P);
        __syncthreads();
        ref_sp_list_touch_body(sp);
        __syncthreads();
        ref_sp_gather_body(p, sp, slots, occ, conc, contended);
        __syncthreads();
        ref_sp_serial_body(p, sp, slots, occ, conc, diag, contended);
        __syncthreads();
        const uint32_t dense = ((k == 0u && dense_first) || dense_always) ? 1u : 0u;
        ref_sp_cme_body(p, sp, slots, occ, conc, itimes, step0 + k, dense, stat, diag, contended, rows);
        __syncthreads();
        sp.c ^= 1u;
    }
}

// Act bitmap c of a freshly uploaded lattice.
__global__ void ref_sp_build_act(RefParams p, RefSparse sp, const uint8_t* __restrict__ slots,
                                 const uint32_t* __restrict__ occ, const int32_t* __restrict__ conc) {
    for (uint32_t v = grid_tid(); v < (uint32_t)p.V; v += grid_threads()) {
        bool keep = occ[v] != 0u;
        for (uint32_t s = 0; s < p.K && !keep; s++) keep |= slots[(size_t)v * p.K + s] != 0u;
        for (uint32_t s = 1; s < p.S1 && !keep; s++) keep |= conc[(size_t)v * p.S1 + s] != 0;
        if (keep) set_bit(act_cur(sp), v);
    }
}

// ------------------------------------------------------------------ host side

static RefSparse ref_sparse(DeviceRef* d) {
    RefSparse sp{};
    for (int b = 0; b < 2; b++) sp.act_bm[b] = d->act_bm[b].p;
    sp.touch_bm = d->touch_bm.p;
    sp.dep_bm = d->dep_bm.p;
    sp.act_list = d->act_list.p;
    sp.touch_list = d->touch_list.p;
    sp.union_list = d->union_list.p;
    sp.cnt = d->cnt.p;
    sp.arrivals = d->arrivals.p;
    sp.dirs = d->dirs.p;
    sp.snap = d->snap.p;
    sp.W = (uint32_t)d->touch_bm.n;
    sp.c = d->par;
    return sp;
}

static void ref_bind(DeviceRef* d) {
    d->p.P = d->P.p;
    d->p.stoich = d->stoich.p;
    d->p.reactants = d->reactants.p;
    d->p.rates = d->rates.p;
    d->p.regions = d->regions.p;
    d->p.reservoir = d->reservoir.p;
}

DeviceRef* ref_create(const Model& m, int device) {
    m.check_tables();
    if (m.n_reactions > 99) throw Error(CS_ERR_LIMIT, "at most 99 reactions");
    if (m.V * m.K >= (1ull << 32))
        throw Error(CS_ERR_LIMIT, "the reference-RNG path indexes slots with u32: V * K must be below 2^32");
    if (m.nr > 256) throw Error(CS_ERR_LIMIT, "at most 256 regions");
    if (m.n_species > 255) throw Error(CS_ERR_LIMIT, "at most 255 species");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        throw Error(CS_ERR_CUDA, "no CUDA device available (libcellsim has no CPU fallback)");
    if (device < 0 || device >= ndev) throw Error(CS_ERR_INVALID_ARG, "device index out of range");
    DeviceGuard g(device);
    std::unique_ptr<DeviceRef> d(new DeviceRef());
    d->device = device;
    CS_CUDA(cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking));
    RefParams& p = d->p;
    p.X = m.res[0]; p.Y = m.res[1]; p.Z = m.res[2];
    p.K = m.K; p.S1 = m.n_species + 1; p.R = m.n_reactions; p.NR = m.nr;
    p.YZ = p.Y * p.Z;
    p.V = m.V;
    p.tau = m.tau;
    uint64_t VK = m.V * m.K, VS = m.V * p.S1;
    d->slots.alloc(VK);
    d->occ.alloc(m.V);
    d->conc.alloc(VS);
    d->regions.alloc(m.V);
    d->reservoir.alloc(m.V);
    d->dirs.alloc(VK);
    d->snap.alloc(VK);
    const uint64_t W = (m.V + 31) / 32;
    for (int b = 0; b < 2; b++) d->act_bm[b].alloc(W);
    d->touch_bm.alloc(W);
    d->dep_bm.alloc(W);
    d->act_list.alloc(m.V);
    d->touch_list.alloc(m.V);
    d->union_list.alloc(m.V);
    d->cnt.alloc(3);
    d->arrivals.alloc(m.V);
    CS_CUDA(cudaMemset(d->arrivals.p, 0, m.V * 4));
    int sms = 1;
    CS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    d->grid = sms * 8;
    for (uint32_t r = 1; r <= m.n_reactions; r++)
        if (m.reactants[r * 3] == 0u && m.reactants[r * 3 + 1] == 0u && m.reactants[r * 3 + 2] == 0u)
            d->dense_always = true;
    std::vector<float> P;
    compute_ref_probabilities(m, P);
    d->P.alloc(P.size());
    d->rates.alloc(m.rates.size());
    d->stoich.alloc(m.stoich.size());
    d->reactants.alloc(m.reactants.size());
    d->stat.alloc(p.S1);
    d->diag.alloc(DIAG_N);
    d->flag.alloc(1);
    ref_bind(d.get());
    std::vector<uint8_t> r8(m.V), res8(m.V);
    for (uint64_t v = 0; v < m.V; v++) { r8[v] = (uint8_t)m.regions[v]; res8[v] = (uint8_t)m.reservoir[v]; }
    CS_CUDA(cudaMemcpy(d->regions.p, r8.data(), m.V, cudaMemcpyHostToDevice));
    CS_CUDA(cudaMemcpy(d->reservoir.p, res8.data(), m.V, cudaMemcpyHostToDevice));
    CS_CUDA(cudaMemcpy(d->P.p, P.data(), P.size() * sizeof(float), cudaMemcpyHostToDevice));
    CS_CUDA(cudaMemcpy(d->rates.p, m.rates.data(), m.rates.size() * sizeof(float), cudaMemcpyHostToDevice));
    CS_CUDA(cudaMemcpy(d->stoich.p, m.stoich.data(), m.stoich.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    CS_CUDA(cudaMemcpy(d->reactants.p, m.reactants.data(), m.reactants.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    CS_CUDA(cudaMemset(d->diag.p, 0, DIAG_N * sizeof(uint32_t)));
    CS_CUDA(cudaMemset(d->flag.p, 0, sizeof(uint32_t)));
    std::vector<int32_t> conc = m.concentrations();
    ref_set_lattice(d.get(), m.slots.data(), m.occupancy.data(), conc.data());
    return d.release();
}

void ref_destroy(DeviceRef* d) {
    if (!d) return;
    cudaSetDevice(d->device);
    if (d->stream) cudaStreamSynchronize(d->stream);
    delete d;
}

void ref_set_lattice(DeviceRef* d, const uint32_t* slots, const uint32_t* occ, const int32_t* conc) {
    DeviceGuard g(d->device);
    uint64_t VK = d->p.V * d->p.K, VS = d->p.V * d->p.S1;
    std::vector<uint8_t> s8(VK);
    for (uint64_t i = 0; i < VK; i++) {
        if (slots[i] > 255u) throw Error(CS_ERR_LIMIT, "slot value above 255");
        s8[i] = (uint8_t)slots[i];
    }
    CS_CUDA(cudaStreamSynchronize(d->stream));
    CS_CUDA(cudaMemcpy(d->slots.p, s8.data(), VK, cudaMemcpyHostToDevice));
    CS_CUDA(cudaMemcpy(d->occ.p, occ, d->p.V * sizeof(uint32_t), cudaMemcpyHostToDevice));
    CS_CUDA(cudaMemcpy(d->conc.p, conc, VS * sizeof(int32_t), cudaMemcpyHostToDevice));
    // the sparse passes start from the act list of the new lattice and empty
    // touch lists and bitmaps; its first reaction pass visits every voxel
    // (conc[v][0] = 1, compaction)
    const size_t wb = d->touch_bm.bytes();
    for (int b = 0; b < 2; b++) CS_CUDA(cudaMemset(d->act_bm[b].p, 0, wb));
    CS_CUDA(cudaMemset(d->touch_bm.p, 0, wb));
    CS_CUDA(cudaMemset(d->dep_bm.p, 0, wb));
    CS_CUDA(cudaMemset(d->cnt.p, 0, d->cnt.bytes()));
    CS_CUDA(cudaMemset(d->arrivals.p, 0, d->arrivals.bytes()));
    d->par = 0;
    ref_sp_build_act<<<d->grid, 256, 0, d->stream>>>(d->p, ref_sparse(d), d->slots.p, d->occ.p, d->conc.p);
    CS_LAUNCH_CHECK();
    CS_CUDA(cudaStreamSynchronize(d->stream));
    d->dense_next = true;
    // create_statistics, src/simulation.rs:361-388: the counts restart from the sum of the concentrations
    std::vector<int32_t> st(d->p.S1, 0);
    for (uint64_t v = 0; v < d->p.V; v++)
        for (uint32_t s = 0; s < d->p.S1; s++) st[s] = (int32_t)((uint32_t)st[s] + (uint32_t)conc[v * d->p.S1 + s]);
    CS_CUDA(cudaMemcpy(d->stat.p, st.data(), d->p.S1 * sizeof(int32_t), cudaMemcpyHostToDevice));
}

void ref_set_counts(DeviceRef* d, const int64_t* counts) {
    DeviceGuard g(d->device);
    std::vector<int32_t> st(d->p.S1);
    for (uint32_t s = 0; s < d->p.S1; s++) st[s] = (int32_t)counts[s];
    CS_CUDA(cudaStreamSynchronize(d->stream));
    CS_CUDA(cudaMemcpy(d->stat.p, st.data(), d->p.S1 * sizeof(int32_t), cudaMemcpyHostToDevice));
}

void ref_render_view(DeviceRef* d, int32_t view, int32_t slice_axis, uint32_t slice, float* out_host, void* out_device) {
    DeviceGuard g(d->device);
    DevBuf<float> tmp;
    float* out_dev = static_cast<float*>(out_device);
    if (!out_dev) {
        tmp.alloc(d->p.V);
        out_dev = tmp.p;
    }
    ViewParams v{};
    v.slots = d->slots.p;
    v.K = d->p.K;
    v.X = d->p.X; v.Y = d->p.Y; v.Z = d->p.Z;
    v.region_id = d->regions.p;
    v.reservoir = d->reservoir.p;
    v.view = view;
    v.slice_axis = slice_axis;
    v.slice = slice;
    v.out = out_dev;
    render_view_kernel<<<1024, 256, 0, d->stream>>>(v);
    CS_LAUNCH_CHECK();
    if (!out_device) CS_CUDA(cudaMemcpyAsync(out_host, out_dev, d->p.V * sizeof(float), cudaMemcpyDeviceToHost, d->stream));
    CS_CUDA(cudaStreamSynchronize(d->stream));
}

void ref_get_lattice(DeviceRef* d, uint32_t* slots, uint32_t* occ, int32_t* conc) {
    DeviceGuard g(d->device);
    CS_CUDA(cudaStreamSynchronize(d->stream));
    uint64_t VK = d->p.V * d->p.K, VS = d->p.V * d->p.S1;
    if (slots) {
        std::vector<uint8_t> s8(VK);
        CS_CUDA(cudaMemcpy(s8.data(), d->slots.p, VK, cudaMemcpyDeviceToHost));
        for (uint64_t i = 0; i < VK; i++) slots[i] = s8[i];
    }
    if (occ) CS_CUDA(cudaMemcpy(occ, d->occ.p, d->p.V * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (conc) CS_CUDA(cudaMemcpy(conc, d->conc.p, VS * sizeof(int32_t), cudaMemcpyDeviceToHost));
}

// Enqueues the sparse passes of one frame reading itimes[k].
// A launch with programmatic stream serialization (see ref_pdl_start).
template <typename... KArgs, typename... Args>
static void ref_launch(void (*kernel)(KArgs...), int grid, int block, size_t smem, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    CS_CUDA(cudaLaunchKernelEx(&cfg, kernel, args...));
}

// Shared memory of the reaction pass in blocks of tb threads: it stages the tables and one
// concentration row per thread when they fit in the default 48 KB (rows = 1).
static size_t ref_cme_smem(const RefParams& p, int tb, uint32_t& rows) {
    const size_t smem_rows =
        ((size_t)p.S1 + 2 + 4 * ((size_t)p.R + 1) + ((size_t)p.R + 1) * p.S1 + (size_t)tb * p.S1) * 4;
    rows = smem_rows <= 48u * 1024u ? 1u : 0u;
    return rows ? smem_rows : (p.S1 + 2) * sizeof(int32_t);
}

// The directions pass stages the probability table in shared memory when it takes at most 16 KB.
static size_t ref_dir_smem(const RefParams& p, uint32_t& stage_P) {
    const size_t smem_P = (size_t)p.NR * p.NR * p.S1 * sizeof(float);
    stage_P = smem_P <= 16u * 1024u ? 1u : 0u;
    return stage_P ? smem_P : 0u;
}

static bool ref_one_block(const DeviceRef* d) { return d->p.V <= REF_BLOCK_MAX_VOXELS; }

// Frames k0 .. k0 + n - 1 of the call (itimes[k]) in one launch of the one-block form.
static void ref_enqueue_block(DeviceRef* d, uint32_t k0, uint32_t n) {
    if (n == 0) return;
    const RefParams& p = d->p;
    const RefSparse sp = ref_sparse(d);
    uint32_t rows = 0, stage_P = 0;
    const size_t smem = std::max(ref_cme_smem(p, REF_BLOCK_THREADS, rows), ref_dir_smem(p, stage_P));
    ref_sp_frames_block<<<1, REF_BLOCK_THREADS, smem, d->stream>>>(
        p, sp, d->slots.p, d->occ.p, d->conc.p, (const uint32_t*)d->itimes.p, k0, n, d->dense_next ? 1u : 0u,
        d->dense_always ? 1u : 0u, d->stat.p, d->diag.p, d->flag.p, stage_P, rows);
    CS_LAUNCH_CHECK();
    d->dense_next = false;
    d->par ^= n & 1u;
}

static void ref_enqueue_frame(DeviceRef* d, uint32_t k) {
    const RefParams& p = d->p;
    const RefSparse sp = ref_sparse(d);
    const int TB = 256;
    uint32_t rows = 0, stage_P = 0;
    const size_t smem = ref_cme_smem(p, TB, rows);
    ref_launch(ref_sp_list_act, d->grid, TB, 0, d->stream, sp);
    const size_t smem_P = ref_dir_smem(p, stage_P);
    ref_launch(ref_sp_directions, d->grid, TB, smem_P, d->stream, p, sp, (const uint8_t*)d->slots.p,
               (const uint32_t*)d->occ.p, (const uint32_t*)d->itimes.p, k, d->diag.p, d->flag.p, stage_P);
    ref_launch(ref_sp_list_touch, d->grid, TB, 0, d->stream, sp);
    ref_launch(ref_sp_gather, d->grid, TB, 0, d->stream, p, sp, d->slots.p, d->occ.p, d->conc.p, d->flag.p);
    ref_launch(ref_sp_serial, 1, 1024, 0, d->stream, p, sp, d->slots.p, d->occ.p, d->conc.p, d->diag.p, d->flag.p);
    const uint32_t dense = (d->dense_next || d->dense_always) ? 1u : 0u;
    ref_launch(ref_sp_cme, d->grid, TB, smem, d->stream, p, sp, d->slots.p, d->occ.p, d->conc.p,
               (const uint32_t*)d->itimes.p, k, dense, d->stat.p, d->diag.p, d->flag.p, rows);
    CS_LAUNCH_CHECK();
    d->dense_next = false;
    d->par ^= 1u;
}

static void ref_enqueue(DeviceRef* d, uint32_t n) {
    if (ref_one_block(d)) {
        ref_enqueue_block(d, 0, n);
        return;
    }
    for (uint32_t k = 0; k < n; k++) ref_enqueue_frame(d, k);
}

void ref_step(DeviceRef* d, uint32_t n_steps, const uint32_t* itimes, uint64_t frame0, uint32_t write_freq,
              const std::vector<uint32_t>& logging, std::vector<cs_stat_sample>& samples) {
    DeviceGuard g(d->device);
    if (n_steps == 0) return;
    const RefParams& p = d->p;
    // frames f in [frame0, frame0+n) sample before executing when f > 0 and f % write_freq == 0
    std::vector<uint64_t> sample_frames;
    if (write_freq)
        for (uint64_t f = frame0; f < frame0 + n_steps; f++)
            if (f > 0 && f % write_freq == 0) sample_frames.push_back(f);
    if (d->itimes.n < n_steps) d->itimes.alloc(std::max<uint32_t>(n_steps, 64));
    CS_CUDA(cudaMemcpyAsync(d->itimes.p, itimes, n_steps * sizeof(uint32_t), cudaMemcpyHostToDevice, d->stream));
    if (!sample_frames.empty() && d->sample_ring.n < sample_frames.size() * p.S1)
        d->sample_ring.alloc(sample_frames.size() * p.S1);
    size_t si = 0;
    uint32_t k0 = 0;  // first frame not yet enqueued (the one-block form runs the frames between samples)
    for (uint32_t k = 0; k < n_steps; k++) {
        uint64_t f = frame0 + k;
        if (si < sample_frames.size() && sample_frames[si] == f) {
            if (ref_one_block(d)) ref_enqueue_block(d, k0, k - k0);
            k0 = k;
            CS_CUDA(cudaMemcpyAsync(d->sample_ring.p + si * p.S1, d->stat.p, p.S1 * sizeof(int32_t),
                                    cudaMemcpyDeviceToDevice, d->stream));
            si++;
        }
        if (!ref_one_block(d)) ref_enqueue_frame(d, k);
    }
    if (ref_one_block(d)) ref_enqueue_block(d, k0, n_steps - k0);
    if (!sample_frames.empty()) {
        std::vector<int32_t> h(sample_frames.size() * p.S1);
        CS_CUDA(cudaMemcpyAsync(h.data(), d->sample_ring.p, h.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, d->stream));
        CS_CUDA(cudaStreamSynchronize(d->stream));
        for (size_t i = 0; i < sample_frames.size(); i++)
            for (uint32_t sp : logging)
                samples.push_back(cs_stat_sample{sp, h[i * p.S1 + sp], (uint32_t)sample_frames[i]});
    }
}

void ref_get_counts(DeviceRef* d, int64_t* counts) {
    DeviceGuard g(d->device);
    std::vector<int32_t> h(d->p.S1);
    CS_CUDA(cudaMemcpyAsync(h.data(), d->stat.p, h.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, d->stream));
    CS_CUDA(cudaStreamSynchronize(d->stream));
    for (uint32_t s = 0; s < d->p.S1; s++) counts[s] = h[s];
}

void ref_get_diag(DeviceRef* d, uint32_t* diag, uint32_t n) {
    DeviceGuard g(d->device);
    uint32_t h[DIAG_N];
    CS_CUDA(cudaMemcpyAsync(h, d->diag.p, sizeof(h), cudaMemcpyDeviceToHost, d->stream));
    CS_CUDA(cudaStreamSynchronize(d->stream));
    for (uint32_t i = 0; i < n; i++) diag[i] = i < DIAG_N ? h[i] : 0u;
}

void ref_sync(DeviceRef* d) {
    DeviceGuard g(d->device);
    CS_CUDA(cudaStreamSynchronize(d->stream));
}

}  // namespace cellsim

namespace cellsim {
float ref_time_frames(DeviceRef* d, uint32_t n, const uint32_t* itimes, uint64_t frame0) {
    DeviceGuard g(d->device);
    if (d->itimes.n < n) d->itimes.alloc(std::max<uint32_t>(n, 64));
    CS_CUDA(cudaMemcpyAsync(d->itimes.p, itimes, n * sizeof(uint32_t), cudaMemcpyHostToDevice, d->stream));
    CS_CUDA(cudaStreamSynchronize(d->stream));
    cudaEvent_t a, b;
    CS_CUDA(cudaEventCreate(&a));
    CS_CUDA(cudaEventCreate(&b));
    std::vector<cs_stat_sample> none;
    float ms = 0.0f;
    try {
        CS_CUDA(cudaEventRecord(a, d->stream));
        ref_enqueue(d, n);
        CS_CUDA(cudaEventRecord(b, d->stream));
        CS_CUDA(cudaEventSynchronize(b));
        CS_CUDA(cudaEventElapsedTime(&ms, a, b));
    } catch (...) {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        throw;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    (void)frame0;
    return ms;
}
}  // namespace cellsim

// ------------------------------------------------------------------ allocation-free frame
//
// A reference-RNG frame on caller-owned device buffers that never allocates.
// It serves hosts that own all device memory themselves: an engine that
// reserves one arena at start-up and forbids further cudaMalloc (a cudaMalloc
// can synchronise the device and fragments that budget), or a real-time loop
// that cannot absorb an allocation's stall.  The only memory the frame needs
// beyond the caller's inputs and outputs (the per-slot direction bytes and the
// contention flag) lives in the fixed array below.  CUDA reserves that array
// on every GPU where this library's module is loaded, and it stays there until
// the process exits.
namespace cellsim {

constexpr size_t kNoAllocMaxSlots = (size_t)16 << 20;  // V * K <= 16 Mi slots (16 MiB of directions)
static __device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocMaxSlots + 256];

static std::mutex g_noalloc_mu;
static uint8_t* g_noalloc_addr[256];

// Device address of the scratch array on `device`, looked up once per device
// with that device current.
static uint8_t* noalloc_scratch(int device) {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (device < 0 || device >= 256) throw Error(CS_ERR_INVALID_ARG, "device ordinal out of range");
    if (!g_noalloc_addr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) throw Error(CS_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        g_noalloc_addr[device] = static_cast<uint8_t*>(p);
    }
    return g_noalloc_addr[device];
}

void ref_frame_noalloc(const cs_ref_frame_noalloc_args* a) {
    if (!a) throw Error(CS_ERR_INVALID_ARG, "args is NULL");
    const uint32_t K = a->max_particles_site;
    if (a->res[0] == 0 || a->res[1] == 0 || a->res[2] == 0) throw Error(CS_ERR_INVALID_ARG, "resolution must be positive");
    if (K < 1 || K > 16) throw Error(CS_ERR_LIMIT, "max_particles_site must be in 1..16");
    if (a->n_regions < 1 || a->n_regions > 256) throw Error(CS_ERR_LIMIT, "n_regions must be in 1..256");
    if (a->n_species > 255) throw Error(CS_ERR_LIMIT, "at most 255 species");
    if (a->n_reactions > 99) throw Error(CS_ERR_LIMIT, "at most 99 reactions");
    const uint64_t V = (uint64_t)a->res[0] * a->res[1] * a->res[2];
    if (V * K > kNoAllocMaxSlots)
        throw Error(CS_ERR_LIMIT, "cs_ref_frame_noalloc handles at most 16777216 slots (V*K); this lattice has " +
                                      std::to_string(V * K) + ": use cs_step, which allocates its own scratch");
    const void* ptrs[] = {a->slots_in, a->occupancy_in, a->conc_in, a->slots_out, a->occupancy_out, a->conc_out,
                          a->regions, a->reservoir, a->probabilities, a->stoich, a->reactants, a->rates, a->itime,
                          a->counts, a->diag};
    for (const void* q : ptrs)
        if (!q) throw Error(CS_ERR_INVALID_ARG, "every buffer pointer of cs_ref_frame_noalloc_args must be non-NULL");
    DeviceGuard g(a->device);
    uint8_t* scratch = noalloc_scratch(a->device);
    uint8_t* dirs = scratch;
    uint32_t* contended = reinterpret_cast<uint32_t*>(scratch + kNoAllocMaxSlots);
    RefParams p{};
    p.X = a->res[0]; p.Y = a->res[1]; p.Z = a->res[2];
    p.K = K; p.S1 = a->n_species + 1; p.R = a->n_reactions; p.NR = a->n_regions;
    p.YZ = p.Y * p.Z;
    p.V = V;
    p.tau = a->tau;
    p.P = a->probabilities;
    p.stoich = a->stoich;
    p.reactants = a->reactants;
    p.rates = a->rates;
    p.regions = a->regions;
    p.reservoir = a->reservoir;
    cudaStream_t st = static_cast<cudaStream_t>(a->stream);
    const int TB = 256;
    unsigned nb = (unsigned)((V + TB - 1) / TB);
    size_t smem = (p.S1 + 2) * sizeof(int32_t);
    // ref_directions rewrites every direction byte and clears the contention
    // flag before anything reads them, so stale scratch from an earlier call
    // never leaks into this frame.
    ref_directions<<<nb, TB, 0, st>>>(p, a->slots_in, a->occupancy_in, a->itime, 0u, dirs, a->diag, contended);
    ref_gather<<<nb, TB, 0, st>>>(p, a->slots_in, a->occupancy_in, a->conc_in, dirs, a->slots_out, a->occupancy_out,
                                  a->conc_out, contended);
    ref_serial_copy<<<std::min<unsigned>(nb, 4096u), TB, 0, st>>>(p, contended, a->slots_in, a->occupancy_in, a->conc_in,
                                                                  a->slots_out, a->occupancy_out, a->conc_out);
    ref_serial<<<1, 32, 0, st>>>(p, contended, a->slots_in, a->occupancy_in, dirs, a->slots_out, a->occupancy_out,
                                 a->conc_out, a->diag);
    ref_cme<<<nb, TB, smem, st>>>(p, a->slots_out, a->occupancy_out, a->conc_out, a->itime, 0u, a->counts, a->diag);
    CS_LAUNCH_CHECK();
}

}  // namespace cellsim
