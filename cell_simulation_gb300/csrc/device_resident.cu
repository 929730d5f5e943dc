// device_resident.cu — the resident form of the production step (see resident_kernel.cuh):
// one block per replicate holds its lattice in shared memory for every frame of a step call.
#include <cuda_runtime.h>

#include "cuda_check.h"
#include "resident_kernel.cuh"

namespace cellsim {

namespace {

constexpr int NT = RESIDENT_THREADS;
constexpr int NSSA = RESIDENT_SSA_WARPS;

// Byte offsets of a block's shared-memory areas, each 16-byte aligned.
struct ResidentLayout {
    size_t cnt;    // [16] list lengths and counts, then PD_N diagnostic counters
    size_t thr;    // [thr_words] threshold table
    size_t ws;     // [NSSA][SSA_WARP_SCRATCH] the SSA scratch of the warps that run the SSA
    size_t mark0, mark1;  // [vmax / 32] bitmaps: the voxel is on the current / the other work list
    size_t code;   // [vmax] region code (id + 1) of every voxel
    size_t dec;    // [vmax] move decisions of the current axis, valid for the voxels on the work
                   // list (a marked voxel); in the reaction step, the voxels set aside
    size_t list0, list1;  // [vmax] 16-bit voxel lists: the occupied voxels, then the sweep's work list
    size_t lat0, lat1;    // [vmax] slot contents: the current state and the one two sweeps back
    size_t total;
};

__host__ __device__ inline size_t take(size_t& o, size_t bytes) {
    const size_t at = o;
    o += (bytes + 15u) & ~(size_t)15u;
    return at;
}

__host__ __device__ inline ResidentLayout resident_layout(int K, uint64_t vmax, uint32_t thr_words) {
    ResidentLayout L;
    size_t o = 0;
    const size_t mark_words = (size_t)((vmax + 31) / 32);
    L.cnt = take(o, sizeof(uint32_t) * (16 + PD_N));
    L.thr = take(o, sizeof(uint32_t) * thr_words);
    L.ws = take(o, sizeof(float) * (size_t)SSA_WARP_SCRATCH * NSSA);
    L.mark0 = take(o, sizeof(uint32_t) * mark_words);
    L.mark1 = take(o, sizeof(uint32_t) * mark_words);
    L.code = take(o, (size_t)vmax);
    L.dec = take(o, sizeof(uint32_t) * (size_t)vmax);
    L.list0 = take(o, sizeof(uint16_t) * (size_t)vmax);
    L.list1 = take(o, sizeof(uint16_t) * (size_t)vmax);
    L.lat0 = take(o, (size_t)K * vmax);
    L.lat1 = take(o, (size_t)K * vmax);
    L.total = o;
    return L;
}

// Appends the lanes' voxels for which `want` holds to `list` (one shared atomic per warp); every
// lane of the warp calls it.
__device__ __forceinline__ void warp_append(bool want, uint32_t v, uint16_t* list, uint32_t* n, uint32_t lane) {
    const uint32_t m = __ballot_sync(0xffffffffu, want);
    uint32_t pos = 0u;
    if (lane == 0u && m) pos = atomicAdd(n, (uint32_t)__popc(m));
    pos = __shfl_sync(0xffffffffu, pos, 0);
    if (want) list[pos + (uint32_t)__popc(m & ((1u << lane) - 1u))] = (uint16_t)v;
}

__device__ __forceinline__ bool test_mark(const uint32_t* mark, uint32_t v) { return (mark[v >> 5] >> (v & 31u)) & 1u; }
__device__ __forceinline__ bool set_mark(uint32_t* mark, uint32_t v) {  // true when v was not marked yet
    const uint32_t bit = 1u << (v & 31u);
    return (atomicOr(&mark[v >> 5], bit) & bit) == 0u;
}

// A sweep is two block-wide steps.  With the lattice state of this sweep in `cur`, the state two
// sweeps back in `nx`, the occupied voxels in lists[b] (all marked in mark_cur) and the previous
// sweep's work list in lists[b ^ 1] (marked in mark_nx):
//   1. clear the previous work list's voxels in nx and mark_nx; move decisions of the occupied
//      voxels into dec, appending each receiving neighbour not marked yet (dec 0) to lists[b]:
//      the work list, every voxel once
//   2. new contents of the work list's voxels into nx (a neighbour's decision counts when the
//      neighbour is marked: every other voxel is empty), marking and listing in lists[b ^ 1] those
//      that end up occupied
// Voxels off the work list are empty before and after the sweep, and nx held nothing else, so nx
// is then the whole next state; the roles of the buffers swap.
template <int K>
__global__ void __launch_bounds__(NT, 1) resident_frames_kernel(const __grid_constant__ ResidentParams RP) {
    extern __shared__ __align__(16) unsigned char sm[];
    const ProdParams& P = RP.P;
    const ResidentLayout L = resident_layout(K, RP.vmax, RP.thr_words);
    // cnt[0], cnt[1]: lengths of list0 / list1; cnt[2 + a]: receiving voxels appended in sweeps of
    // parity a; cnt[4 + (f & 1)]: voxels set aside in frame f
    uint32_t* const cnt = reinterpret_cast<uint32_t*>(sm + L.cnt);
    uint32_t* const s_diag = cnt + 16;
    uint8_t* const code = sm + L.code;
    uint32_t* const dec = reinterpret_cast<uint32_t*>(sm + L.dec);
    uint16_t* const list0 = reinterpret_cast<uint16_t*>(sm + L.list0);
    uint16_t* const list1 = reinterpret_cast<uint16_t*>(sm + L.list1);
    auto lists = [&](uint32_t k) -> uint16_t* { return k ? list1 : list0; };
    uint32_t* mark_cur = reinterpret_cast<uint32_t*>(sm + L.mark0);
    uint32_t* mark_nx = reinterpret_cast<uint32_t*>(sm + L.mark1);
    Vox<K>* cur = reinterpret_cast<Vox<K>*>(sm + L.lat0);
    Vox<K>* nx = reinterpret_cast<Vox<K>*>(sm + L.lat1);
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t S1 = P.T.S1, NC = P.T.NC;
    const RepDesc rd = P.reps[RP.rep0 + blockIdx.x];
    const uint32_t X = rd.X, Y = rd.Y, Z = rd.Z, YZ = Y * Z, V = X * YZ;  // V <= vmax < 2^16
    const uint32_t mark_words = (V + 31) / 32;

    const uint32_t* thr = P.T.thr;
    if (RP.thr_words) {
        uint32_t* const s_thr = reinterpret_cast<uint32_t*>(sm + L.thr);
        for (uint32_t i = tid; i < RP.thr_words; i += NT) s_thr[i] = P.T.thr[i];
        thr = s_thr;
    }
    for (uint32_t i = tid; i < 16 + PD_N; i += NT) cnt[i] = 0u;
    for (uint32_t i = tid; i < mark_words; i += NT) {
        mark_cur[i] = 0u;
        mark_nx[i] = 0u;
    }
    // the other forms' work counters start the next frame at zero whatever parity it has
    if (blockIdx.x == 0 && tid == 0)
        for (uint32_t i = 0; i < P.n_reset; i++) P.reset[i] = 0u;
    const uint8_t* const rpad = (rd.flags & 1u) ? nullptr : P.region_pad + rd.rbase;
#pragma unroll 4
    for (uint32_t v = tid; v < V; v += NT) {  // unrolled: several global loads in flight per thread
        const uint32_t x = v / YZ, y = (v / Z) % Y, z = v % Z;
        code[v] = rpad ? rpad[((uint64_t)x * Y + y) * rd.Zr + z + 2u] : (uint8_t)1u;
        cur[v] = ld_vox_g<K>(P.src + (rd.base + v) * K);
        nx[v] = vox_zero<K>();
    }
    __syncthreads();
    // the occupied voxels, marked (loops that call warp_append run whole warps: base is warp-uniform)
    for (uint32_t base = warp * 32u; base < V; base += NT) {
        const uint32_t v = base + lane;
        const bool occupied = v < V && !vox_empty<K>(cur[v]);
        if (occupied) set_mark(mark_cur, v);
        warp_append(occupied, v, list0, &cnt[0], lane);
    }
    __syncthreads();

    const uint32_t k0 = rd.seed_lo, k1 = rd.seed_hi;
    const bool zero_order = P.T.n_zero_order != 0u;
    const bool all_react = zero_order || P.reservoir != nullptr;
    const uint32_t ci = rd.counts_index;
    const uint32_t* const quiet = P.T.quiet + (size_t)ci * S1 * P.T.QS;
    const float* const one = P.T.one + (size_t)ci * S1 * 3;
    const float* const g23 = P.T.g23 + 2 * ci;
    const float* const a2 = P.T.a2 ? P.T.a2 + (size_t)ci * S1 * S1 : nullptr;
    unsigned long long* const counts = P.counts + (size_t)ci * S1;
    auto trow = [&](uint32_t a, uint32_t b) -> const uint32_t* { return thr + (a * NC + b) * S1; };

    uint32_t b = 0;        // lists(b) holds the occupied voxels (and possibly voxels emptied since)
    uint32_t a = 0;        // parity of the sweeps run so far: cnt[2 + a] counts this sweep's appends
    uint32_t nw_prev = 0;  // length of the previous sweep's work list, lists(b ^ 1)
    for (uint32_t f = 0; f < RP.n_frames; f++) {
        const uint32_t fr = RP.frame0 + f;
        for (uint32_t sweep = 0; sweep < 3u; sweep++) {
            const uint32_t stride = sweep == 0u ? YZ : sweep == 1u ? Z : 1u;
            const uint32_t dim = sweep == 0u ? X : sweep == 1u ? Y : Z;
            // an axis of length 1 has no neighbour: every decision is 0 and every content stays
            if (dim == 1u) continue;
            uint16_t* const wl = lists(b);
            const uint16_t* const wprev = lists(b ^ 1u);
            const uint32_t na = cnt[b];
            uint32_t* const n_app = &cnt[2 + a];
            // 1.
            for (uint32_t i = tid; i < nw_prev; i += NT) {
                const uint32_t u = wprev[i];
                nx[u] = vox_zero<K>();
                atomicAnd(&mark_nx[u >> 5], ~(1u << (u & 31u)));
            }
            if (tid == 0) {
                cnt[2 + (a ^ 1u)] = 0u;
                cnt[b ^ 1u] = 0u;
            }
            for (uint32_t i = tid; i < na; i += NT) {
                const uint32_t v = wl[i];
                const Vox<K> c = cur[v];
                if (vox_empty<K>(c)) {
                    dec[v] = 0u;
                    continue;
                }
                const uint32_t coord = (v / stride) % dim;
                const uint32_t rs = code[v];
                const uint32_t rlo = coord > 0u ? code[v - stride] : 0u;
                const uint32_t rhi = coord + 1u < dim ? code[v + stride] : 0u;
                const U4 b0 = d_philox(v, fr, 0u, 0u, k0, k1);
                const uint32_t d =
                    decide_moves<K>(c, v, fr, sweep, trow(rs, rlo), trow(rs, rhi), k0, k1, sweep_word(b0, sweep));
                dec[v] = d;
                // a receiving voxel not marked yet is empty and on no list: nobody else writes its dec
                if ((d & 0xFFFFu) && set_mark(mark_cur, v - stride)) {
                    dec[v - stride] = 0u;
                    wl[na + atomicAdd(n_app, 1u)] = (uint16_t)(v - stride);
                }
                if ((d >> 16) && set_mark(mark_cur, v + stride)) {
                    dec[v + stride] = 0u;
                    wl[na + atomicAdd(n_app, 1u)] = (uint16_t)(v + stride);
                }
            }
            __syncthreads();
            // 2.
            const uint32_t nw = na + *n_app;
            for (uint32_t base = warp * 32u; base < nw; base += NT) {
                const uint32_t i = base + lane;
                bool occupied = false;
                uint32_t v = 0u;
                if (i < nw) {
                    v = wl[i];
                    const uint32_t coord = (v / stride) % dim;
                    const bool has_lo = coord > 0u, has_hi = coord + 1u < dim;
                    const uint32_t dme = dec[v];
                    const uint32_t dlo = has_lo && test_mark(mark_cur, v - stride) ? dec[v - stride] : 0u;
                    const uint32_t dhi = has_hi && test_mark(mark_cur, v + stride) ? dec[v + stride] : 0u;
                    Vox<K> r = cur[v];
                    if ((dme | (dlo >> 16) | (dhi & 0xFFFFu)) != 0u) {  // something leaves or arrives
                        const Vox<K> lo = has_lo ? cur[v - stride] : vox_zero<K>();
                        const Vox<K> hi = has_hi ? cur[v + stride] : vox_zero<K>();
                        r = combine<K>(r, dme, lo, dlo, hi, dhi, v, v - stride, v + stride, fr, sweep);
                    }
                    nx[v] = r;
                    occupied = !vox_empty<K>(r);
                    if (occupied) set_mark(mark_nx, v);
                }
                warp_append(occupied, v, lists(b ^ 1u), &cnt[b ^ 1u], lane);
            }
            __syncthreads();
            Vox<K>* const t = cur;
            cur = nx;
            nx = t;
            uint32_t* const tm = mark_cur;
            mark_cur = mark_nx;
            mark_nx = tm;
            b ^= 1u;
            a ^= 1u;
            nw_prev = nw;
        }
        // reactions: the voxels whose first event may fall inside the frame are set aside (their
        // indices in dec), then each runs its SSA on one warp
        uint32_t* const n_pend = &cnt[4 + (f & 1u)];
        const uint32_t na = all_react ? V : cnt[b];
        if (tid == 0) {
            cnt[4 + ((f + 1u) & 1u)] = 0u;
            cnt[b ^ 1u] = 0u;
        }
        for (uint32_t i = tid; i < na; i += NT) {
            const uint32_t v = all_react ? i : (uint32_t)lists(b)[i];
            const Vox<K> c = cur[v];
            const uint32_t rv = P.reservoir ? (uint32_t)P.reservoir[rd.base + v] : 0u;
            if (rv != 0u || zero_order || !vox_empty<K>(c)) {
                const uint32_t w3 = d_philox(v, fr, 0u, 0u, k0, k1).w;
                const bool calm =
                    rv == 0u && !zero_order && calm_voxel<K>(c, w3, quiet, P.T.QS, one, g23, a2, P.T.tau);
                if (!calm) dec[atomicAdd(n_pend, 1u)] = v;
            }
        }
        __syncthreads();
        const uint32_t np = *n_pend;
        if (warp < (uint32_t)NSSA) {
            float* const ws = reinterpret_cast<float*>(sm + L.ws) + (size_t)warp * SSA_WARP_SCRATCH;
            for (uint32_t q = warp; q < np; q += NSSA) {
                const uint32_t v = dec[q];
                Vox<K> r = cur[v];
                const uint32_t rv = P.reservoir ? (uint32_t)P.reservoir[rd.base + v] : 0u;
                const uint32_t w3 = d_philox(v, fr, 0u, 0u, k0, k1).w;
                react_voxel_warp<K>(r, rv, v, fr, k0, k1, rd.rate_mult, ci, P.T, nullptr, counts, s_diag, w3, ws);
                if (lane == 0u) cur[v] = r;
                __syncwarp();
            }
        }
        if (all_react) {
            // reactions may fill empty voxels: the lists and marks start afresh from the lattice
            for (uint32_t i = tid; i < mark_words; i += NT) {
                mark_cur[i] = 0u;
                mark_nx[i] = 0u;
            }
            for (uint32_t v = tid; v < V; v += NT) nx[v] = vox_zero<K>();
            nw_prev = 0u;
            __syncthreads();
            for (uint32_t base = warp * 32u; base < V; base += NT) {
                const uint32_t v = base + lane;
                const bool occupied = v < V && !vox_empty<K>(cur[v]);
                if (occupied) set_mark(mark_cur, v);
                warp_append(occupied, v, lists(b ^ 1u), &cnt[b ^ 1u], lane);
            }
            b ^= 1u;
        }
        __syncthreads();
    }

    for (uint32_t v = tid; v < V; v += NT) st_vox_g<K>(P.dst + (rd.base + v) * K, cur[v]);
    for (uint32_t i = tid; i < PD_N; i += NT)
        if (s_diag[i]) atomicAdd(P.diag + i, s_diag[i]);
    if (blockIdx.x == 0 && tid == 0) P.stepbuf[RP.stepbuf_out] = RP.frame0 + RP.n_frames;
}

}  // namespace

size_t resident_smem(int K, uint64_t vmax, uint32_t thr_words) { return resident_layout(K, vmax, thr_words).total; }

void resident_set_attrs(int device) {
    int optin = 0;
    CS_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
    CS_CUDA(cudaFuncSetAttribute(resident_frames_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    CS_CUDA(cudaFuncSetAttribute(resident_frames_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
    CS_CUDA(cudaFuncSetAttribute(resident_frames_kernel<16>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    CS_CUDA(cudaFuncSetAttribute(resident_frames_kernel<8>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
}

void resident_launch(int K, const ResidentParams& RP, int grid, size_t smem, cudaStream_t s) {
    if (K == 16) resident_frames_kernel<16><<<grid, NT, smem, s>>>(RP);
    else resident_frames_kernel<8><<<grid, NT, smem, s>>>(RP);
    CS_LAUNCH_CHECK();
}

}  // namespace cellsim
