// device_ref.cu — reference-RNG (bit-parity) form of the RDME timestep.
//
// Reproduces the reference shaders' arithmetic exactly (res/shader/rdme.wgsl,
// cme.wgsl, final_stage.wgsl, random.wgsl) in a canonical serial order: voxels
// in linear index order, slots in index order (the reference's own GPU order
// is nondeterministic because of its spin locks and CAS slot insertion).
//
// Per frame, five launches on the handle's stream:
//   1. ref_directions  one thread per voxel: for every occupied slot, the
//      direction drawn from PCG(itime + x%y + z + slot index) against the
//      cumulative move probabilities (rdme.wgsl:138-226); 7 = no particle.
//   2. ref_gather      one thread per destination voxel: arrivals from the -x,
//      -y, -z neighbours, own departures, arrivals from the +z, +y, +x
//      neighbours, each arrival into the lowest free slot.  This equals the
//      serial order when no arrival can be rejected; a voxel for which
//      max(occupancy, nonzero slots) + arrivals > K raises `contended`.
//   3. ref_serial_copy / 4. ref_serial (one thread) run only when `contended`
//      is set and redo the diffusion in serial order with the capacity rule.
//   5. ref_cme         one thread per voxel: one-event reaction test, slot
//      rewrite with rollback, stable compaction (final_stage.wgsl:25-33),
//      species-count deltas reduced per block then added atomically.
// The lattice, occupancy and concentration buffers ping-pong between frames,
// which replaces the reference's dest->src buffer copies
// (src/simulation.rs:134-144).
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

struct DeviceRef {
    int device = 0;
    cudaStream_t stream = nullptr;
    RefParams p{};
    DevBuf<uint8_t> slots[2];
    DevBuf<uint32_t> occ[2];
    DevBuf<int32_t> conc[2];
    DevBuf<uint8_t> regions, reservoir, dirs;
    DevBuf<float> P, rates;
    DevBuf<int32_t> stoich, stat;
    DevBuf<uint32_t> reactants, diag, flag, itimes;
    DevBuf<int32_t> sample_ring;
    int cur = 0;
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

// cme.wgsl:26-120 followed by final_stage.wgsl:25-33.
__global__ void ref_cme(RefParams p, uint8_t* __restrict__ dst, uint32_t* __restrict__ occD, int32_t* __restrict__ concD,
                        const uint32_t* __restrict__ itimes, uint32_t step, int32_t* stat, uint32_t* diag) {
    extern __shared__ int32_t s_delta[];  // [S1] + 2 counters
    for (uint32_t s = threadIdx.x; s < p.S1 + 2; s += blockDim.x) s_delta[s] = 0;
    __syncthreads();
    uint64_t v = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v < p.V) {
        const uint32_t K = p.K, S1 = p.S1, R = p.R;
        const uint32_t S = S1 - 1;
        uint32_t z = (uint32_t)(v % p.Z);
        uint32_t y = (uint32_t)((v / p.Z) % p.Y);
        uint32_t x = (uint32_t)(v / p.YZ);
        int32_t* c = concD + v * S1;
        uint8_t* sl = dst + v * K;
        c[0] = 1;
        float total = 0.0f;
        for (uint32_t r = 1; r <= R; r++) {
            uint32_t prod = (uint32_t)c[p.reactants[r * 3]] * (uint32_t)c[p.reactants[r * 3 + 1]] *
                            (uint32_t)c[p.reactants[r * 3 + 2]];
            total = __fadd_rn(total, __fmul_rn(p.rates[r], __int2float_rn((int32_t)prod)));
        }
        uint8_t snap[16];
        for (uint32_t s = 0; s < K; s++) snap[s] = sl[s];
        uint32_t itime = itimes[step];
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
            int32_t new_occ = (int32_t)occD[v];
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
                    sl[j] = (uint8_t)s;
                    cc--;
                    j++;
                    if (j >= K) {
                        for (uint32_t k = 0; k < K; k++) sl[k] = snap[k];
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
                occD[v] = (uint32_t)new_occ;
                while (j < K) sl[j++] = 0;
            }
        }
        uint32_t jj = 0;
        for (uint32_t s = 0; s < K; s++) {
            uint8_t q = sl[s];
            if (q != 0) {
                sl[s] = sl[jj];
                sl[jj] = q;
                jj++;
            }
        }
    }
    __syncthreads();
    for (uint32_t s = threadIdx.x; s < p.S1; s += blockDim.x)
        if (s_delta[s]) atomicAdd(stat + s, s_delta[s]);
    if (threadIdx.x == 0) {
        if (s_delta[p.S1]) atomicAdd(diag + DIAG_FIRED, (uint32_t)s_delta[p.S1]);
        if (s_delta[p.S1 + 1]) atomicAdd(diag + DIAG_ROLLBACKS, (uint32_t)s_delta[p.S1 + 1]);
    }
}

// ------------------------------------------------------------------ host side

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
    for (int b = 0; b < 2; b++) {
        d->slots[b].alloc(VK);
        d->occ[b].alloc(m.V);
        d->conc[b].alloc(VS);
    }
    d->regions.alloc(m.V);
    d->reservoir.alloc(m.V);
    d->dirs.alloc(VK);
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
    d->cur = 0;
    CS_CUDA(cudaMemcpy(d->slots[0].p, s8.data(), VK, cudaMemcpyHostToDevice));
    CS_CUDA(cudaMemcpy(d->occ[0].p, occ, d->p.V * sizeof(uint32_t), cudaMemcpyHostToDevice));
    CS_CUDA(cudaMemcpy(d->conc[0].p, conc, VS * sizeof(int32_t), cudaMemcpyHostToDevice));
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
    v.slots = d->slots[d->cur].p;
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
        CS_CUDA(cudaMemcpy(s8.data(), d->slots[d->cur].p, VK, cudaMemcpyDeviceToHost));
        for (uint64_t i = 0; i < VK; i++) slots[i] = s8[i];
    }
    if (occ) CS_CUDA(cudaMemcpy(occ, d->occ[d->cur].p, d->p.V * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (conc) CS_CUDA(cudaMemcpy(conc, d->conc[d->cur].p, VS * sizeof(int32_t), cudaMemcpyDeviceToHost));
}

// Enqueues the five launches of one frame reading itimes[k].
static void ref_enqueue_frame(DeviceRef* d, uint32_t k) {
    const RefParams& p = d->p;
    const int TB = 256;
    unsigned nb = (unsigned)((p.V + TB - 1) / TB);
    size_t smem = (p.S1 + 2) * sizeof(int32_t);
    int a = d->cur, b = a ^ 1;
    ref_directions<<<nb, TB, 0, d->stream>>>(p, d->slots[a].p, d->occ[a].p, d->itimes.p, k, d->dirs.p, d->diag.p,
                                             d->flag.p);
    ref_gather<<<nb, TB, 0, d->stream>>>(p, d->slots[a].p, d->occ[a].p, d->conc[a].p, d->dirs.p, d->slots[b].p,
                                         d->occ[b].p, d->conc[b].p, d->flag.p);
    ref_serial_copy<<<std::min<unsigned>(nb, 4096u), TB, 0, d->stream>>>(p, d->flag.p, d->slots[a].p, d->occ[a].p,
                                                                         d->conc[a].p, d->slots[b].p, d->occ[b].p,
                                                                         d->conc[b].p);
    ref_serial<<<1, 32, 0, d->stream>>>(p, d->flag.p, d->slots[a].p, d->occ[a].p, d->dirs.p, d->slots[b].p,
                                        d->occ[b].p, d->conc[b].p, d->diag.p);
    ref_cme<<<nb, TB, smem, d->stream>>>(p, d->slots[b].p, d->occ[b].p, d->conc[b].p, d->itimes.p, k, d->stat.p,
                                         d->diag.p);
    CS_LAUNCH_CHECK();
    d->cur = b;
}

static void ref_enqueue(DeviceRef* d, uint32_t n) {
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
    for (uint32_t k = 0; k < n_steps; k++) {
        uint64_t f = frame0 + k;
        if (si < sample_frames.size() && sample_frames[si] == f) {
            CS_CUDA(cudaMemcpyAsync(d->sample_ring.p + si * p.S1, d->stat.p, p.S1 * sizeof(int32_t),
                                    cudaMemcpyDeviceToDevice, d->stream));
            si++;
        }
        ref_enqueue_frame(d, k);
    }
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
