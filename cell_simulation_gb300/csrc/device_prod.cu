// device_prod.cu — production (Philox) RDME step: one fused, persistent
// launch per frame over a (replicate, tile) work queue.
//
// Each work item is a column of TY x TZ voxels in the (y, z) plane spanning
// x in [x0, x1) of one replicate.  The CTA rolls along x with rings of
// shared-memory planes ((TY+2) x (TZ+2) windows with a one-voxel halo for
// slots, two voxels for region codes):
//   load     plane i+1 from HBM (16-byte vector loads for K = 16), and decide
//            its x-moves while the content is in registers;
//   X sweep  plane i from raw planes i-1, i, i+1 (the only cross-plane
//            dependency), then decide y-moves of the result;
//   Y sweep  in-plane, then decide z-moves;
//   Z sweep  in-plane, then reactions (SSA within tau) and the store of the
//            interior to the destination lattice.
// Every lattice byte is read once and written once per frame (plus the halo
// re-reads of neighbouring tiles, which mostly hit L2); species-count deltas
// are reduced per CTA in shared memory and added to the per-replicate counts
// with one atomic per species per work item.
//
// Frame bookkeeping lives on the device so a captured two-frame CUDA graph
// can be replayed: the launch reads its frame number from stepbuf[parity]
// and writes frame+1 to stepbuf[parity^1]; work counters alternate the same
// way, each launch resetting the one the next launch will use.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "cuda_check.h"
#include "internal.h"
#include "brick_kernel.cuh"
#include "prod_common.cuh"
#include "prod_kernel.cuh"
#include "resident_kernel.cuh"
#include "stream_kernel.cuh"
#include "views.cuh"

namespace cellsim {

// ------------------------------------------------------------------ configs

typedef void (*ProdKernelFn)(ProdParams);

// A compiled step configuration.  kind 0: the tile pipeline alone over
// (TY x TZ tile, x-segment) items.  kind 1: the brick pass over BX x TY x 32
// bricks; when its pools can overflow, a second brick pass `spill` with
// pools as large as its box finishes the spilled bricks in `sub` groups of
// its own BX planes.  kind 2: the sweep stream, four barrier-free passes over
// bitmap word groups (stream_kernel.cuh); `variant` indexes its compiled
// launch shapes.
enum { KIND_TILE = 0, KIND_BRICK = 1, KIND_STREAM = 2, KIND_RESIDENT = 3 };

struct KernelCfg {
    int kind, K, TY, TZ, NT, BX;
    ProdKernelFn fn;
    size_t (*smem)(uint32_t S1, uint32_t thr_words);
    int spill;     // kind 1 with bounded pools: index of the configuration for spilled bricks, else -1
    uint32_t sub;  // plane groups per spilled brick in that configuration
    int variant;   // kind 2: launch shape of the passes
};

// TY = 1 marks the persistent multi-frame form (cs_tiling_describe)
static KernelCfg stream_cfg(int K, int variant) {
    return KernelCfg{KIND_STREAM, K, stream_variant_frames(variant) ? 1 : 0, 32, stream_variant_threads(variant), 0,
                     nullptr, nullptr, -1, 0, variant};
}

// the resident form: one block per replicate, every frame of a step call in one launch
static KernelCfg resident_cfg(int K) {
    return KernelCfg{KIND_RESIDENT, K, 0, 0, RESIDENT_THREADS, 0, nullptr, nullptr, -1, 0, 0};
}

template <int K, int TY, int TZ>
static size_t tile_smem(uint32_t S1, uint32_t) { return Tile<K, TY, TZ>::smem(S1); }

template <int K, int TY, int TZ, int NT, int MINB>
static KernelCfg tile_cfg() {
    return KernelCfg{KIND_TILE, K, TY, TZ, NT, 0, prod_step_kernel<K, TY, TZ, NT, MINB>, &tile_smem<K, TY, TZ>, -1, 0};
}

template <int K, int BX, int BY, int NT, int MINB, int CAP0, int CAP1, int CAP2>
static KernelCfg brick_cfg(int spill, uint32_t sub) {
    using B = Brick<K, BX, BY, NT, CAP0, CAP1, CAP2>;
    return KernelCfg{KIND_BRICK, K, BY, 32, NT, BX, brick_step_kernel<K, BX, BY, NT, MINB, CAP0, CAP1, CAP2>,
                     &B::smem, B::DENSE ? -1 : spill, sub};
}

// full-capacity pools for a brick of BX x BY x 32: never spills
template <int K, int BX, int BY, int NT, int MINB>
static KernelCfg dense_brick_cfg() {
    constexpr int N0 = (BX + 2) * (BY + 2) * 34, N1 = BX * (BY + 2) * 34, N2 = BX * BY * 34;
    return brick_cfg<K, BX, BY, NT, MINB, N0, N1, N2>(-1, 0);
}

static const std::vector<KernelCfg>& all_cfgs() {
    static const std::vector<KernelCfg> v = {
        tile_cfg<16, 8, 32, 256, 3>(),  tile_cfg<16, 4, 64, 256, 3>(), tile_cfg<16, 16, 32, 256, 1>(),
        tile_cfg<16, 8, 64, 256, 1>(),  tile_cfg<8, 8, 32, 256, 3>(),  tile_cfg<8, 4, 64, 256, 3>(),
        tile_cfg<8, 16, 32, 256, 2>(),  tile_cfg<8, 8, 64, 256, 2>(),
        // sparse bricks whose crowded bricks go to the dense 2-plane pass of the same K (entries 10,
        // 11).  With NT = 32 BX one warp owns each interior plane and runs its X/Y/Z sweeps without
        // CTA barriers; otherwise every phase runs CTA-wide.
        brick_cfg<16, 8, 8, 256, 3, 768, 768, 768>(10, 4), brick_cfg<8, 8, 8, 256, 3, 768, 768, 768>(11, 4),
        dense_brick_cfg<16, 2, 8, 256, 3>(), dense_brick_cfg<8, 2, 8, 256, 3>(),
        brick_cfg<16, 8, 8, 192, 4, 544, 544, 544>(10, 4), brick_cfg<16, 4, 8, 128, 5, 448, 448, 448>(10, 2),
        brick_cfg<16, 6, 8, 192, 4, 560, 560, 560>(10, 3), brick_cfg<8, 8, 8, 192, 4, 544, 544, 544>(11, 4),
        // small pool 1: bricks overflow after other warps have stored their planes (exercises that route)
        brick_cfg<16, 8, 8, 256, 3, 768, 128, 768>(10, 4),
        // 16-plane bricks, two CTAs of 12 warps per SM: the box is 1.49 times the interior (1.66 for
        // 8 planes) and the per-brick fixed cost is spread over twice the voxels
        brick_cfg<16, 16, 8, 384, 2, 1088, 1088, 1088>(10, 8), brick_cfg<8, 16, 8, 384, 2, 1088, 1088, 1088>(11, 8),
        // 16-plane bricks, three CTAs of 8 warps per SM (smaller pools; more bricks in flight)
        brick_cfg<16, 16, 8, 256, 3, 640, 640, 640>(10, 8), brick_cfg<8, 16, 8, 256, 3, 768, 768, 768>(11, 8),
        // four CTAs of 6 warps / six CTAs of 5 warps per SM: small pools for sparse replicates (the
        // 512-replicate ensemble), where more bricks in flight per SM beat larger pools
        brick_cfg<8, 16, 8, 192, 4, 432, 432, 432>(11, 8), brick_cfg<8, 16, 8, 160, 6, 176, 176, 176>(11, 8),
        // sweep stream: 256 threads, at least two / four blocks per SM (pass 3 of variants 2, 3: three, two)
        stream_cfg(16, 0), stream_cfg(16, 1), stream_cfg(8, 0), stream_cfg(8, 1), stream_cfg(16, 2), stream_cfg(8, 2),
        stream_cfg(16, 3), stream_cfg(8, 3),
        // sweep stream with the Y and Z sweeps fused into one launch (rows of at most 32 words), at
        // three / four blocks per SM
        stream_cfg(16, 4), stream_cfg(8, 4), stream_cfg(16, 5), stream_cfg(8, 5),
        // the fused stream as one persistent launch per step call (pass 1 and the fused pass of
        // every frame as tasks of one counter) at three blocks per SM, a pass's groups taken
        // heaviest first / in plane order
        stream_cfg(16, 6), stream_cfg(8, 6), stream_cfg(16, 7), stream_cfg(8, 7),
        // lattices that fit in one block's shared memory: the resident form
        resident_cfg(16), resident_cfg(8),
    };
    return v;
}

// Threshold tables up to this many words are staged in shared memory by the brick pass.
static constexpr uint32_t kThrSmemWords = 4096;

// ------------------------------------------------------------------ host side

struct DeviceProd {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint32_t K = 16, S1 = 1, R = 0, NC = 1, n_rep = 0;
    uint64_t total_voxels = 0;
    int num_sms = 1;
    std::vector<RepDesc> h_reps;
    DevBuf<RepDesc> reps;
    DevBuf<uint8_t> slots[2];
    DevBuf<uint32_t> occ[2];  // occupancy bitmaps of slots[0] and slots[1]
    uint64_t occ_words = 0;
    bool occ_valid = false;   // the bitmaps describe the slot buffers (false after uploads and tile frames)
    DevBuf<uint8_t> region_pad, reservoir;
    std::vector<uint8_t> h_region_pad;  // host copy of region_pad (single lattices; empty for ensembles)
    DevBuf<uint32_t> thr;
    DevBuf<uint8_t> rx_reactants, rx_ch_sp;
    DevBuf<int8_t> rx_ch_d;
    DevBuf<float> rx_rate;
    DevBuf<unsigned long long> rmask;
    DevBuf<float> one;
    DevBuf<uint32_t> quiet;
    DevBuf<float> g23;
    DevBuf<float> a2;  // pair propensities (ProdTables::a2)
    DevBuf<WorkItem> spill;  // bricks handed from the brick pass to the second pass
    DevBuf<unsigned long long> sample_ring;  // species counts at the sample frames of one cs_step_philox
    std::vector<float> h_rate;
    std::vector<uint8_t> h_rre;
    std::vector<unsigned long long> h_rmask;
    unsigned long long h_zmask[2] = {0ull, 0ull};
    DevBuf<unsigned long long> counts;
    DevBuf<uint32_t> diag, counters, stepbuf;
    DevBuf<WorkItem> items;      // batched order
    DevBuf<WorkItem> items_rep;  // grouped per replicate (plain launches)
    std::vector<uint32_t> rep_item_off;
    uint32_t n_items = 0;
    // sweep stream: word groups (rep-major), records of two pass boundaries and per-word arrays
    DevBuf<WordGroup> groups;
    std::vector<uint32_t> rep_group_off;
    uint32_t n_groups = 0;
    DevBuf<uint4> rec[3];  // two parities; fused variants: x-, y- and z-decision records in 0, 1, 2
    DevBuf<uint32_t> sw[14];
    DevBuf<uint8_t> wcode;  // per bitmap word: uniform region code of its window, or 0 (single lattices)
    DevBuf<uint2> ssa_over;  // pass 3: per-warp lists of the voxels set aside for the warp's SSA
    // the multi-frame form: per group its four neighbours and the completion values of its last
    // pass 1 and fused pass; the launch's task and exit counters; the completion base of the next
    // launch (completion values compare modulo 2^32)
    DevBuf<uint32_t> nbr, done1, done2, frames_ctr;
    DevBuf<uint32_t> plane_order;  // the sorted position of each group in build (plane) order
    uint32_t frames_seq = 0;
    uint32_t stall_group = 0xFFFFFFFFu;  // cs_debug_stall_group: the next multi-frame launch's stalled group
    std::vector<WordGroup> h_groups;
    bool groups_sorted = false;  // groups dealt heaviest first (sorted once per group build)
    int stream_per_sm[4] = {0, 0, 0, 0};  // resident blocks per SM of the current stream passes
    int stream_occ_cfg = -1;
    int frames_per_sm = 0, frames_occ_cfg = -1;  // ... of the current multi-frame kernel
    // The x-decisions of frame xdec_frame (parity xdec_cur, configuration xdec_cfg, seed epoch
    // xdec_epoch) are in the per-word arrays and rec[xdec_cur]: made by the last sweep-stream
    // frame's pass 3.  Any other change of the lattice clears xdec_valid.
    bool xdec_valid = false;
    uint64_t xdec_frame = 0, xdec_epoch = 0;
    int xdec_cur = 0, xdec_cfg = -1;
    uint64_t seed_epoch = 0;  // advanced whenever the Philox keys change
    uint64_t next_frame = 0;  // host copy of the frame number in stepbuf[cur]
    // stepbuf[cur] holds next_frame in stream order: it was uploaded, and every frame since wrote
    // its successor's number (a step call that continues from there uploads nothing)
    bool frame_known = false;
    unsigned long long* h_counts = nullptr;  // pinned read-back buffer of the counts (n_rep * S1)
    // pinned slots of the first frame number of each step call, copied in stream order; a slot
    // is reused once its event shows that its copy has run
    static constexpr int kFrameSlots = 8;
    uint32_t* h_frames = nullptr;
    cudaEvent_t frame_ev[kFrameSlots] = {};
    int frame_slot = 0;
    int cur = 0;
    ProdTables T{};
    int cfg_index = -1;
    uint32_t seg_len = 0;
    uint64_t cur_seed = 0;
    bool seed_set = false;
    cudaGraphExec_t graph = nullptr;  // two frames, parities 0 then 1
    int graph_cfg = -1;
    cudaGraphExec_t graph1[2] = {nullptr, nullptr};  // one frame of parity 0 / 1
    int graph1_cfg[2] = {-1, -1};
    ~DeviceProd() {
        if (graph) cudaGraphExecDestroy(graph);
        for (cudaGraphExec_t g1 : graph1)
            if (g1) cudaGraphExecDestroy(g1);
        if (h_counts) cudaFreeHost(h_counts);
        if (h_frames) cudaFreeHost(h_frames);
        for (cudaEvent_t e : frame_ev)
            if (e) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }
};

static uint32_t threshold_of(double D, double tau, double lambda) {
    double p = D * tau / (lambda * lambda);
    if (!(p > 0.0)) return 0u;
    if (p >= 1.0) return 0xFFFFFFFFu;
    double t = std::floor(p * 4294967296.0);
    return t >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)t;
}

// Builds the shared reaction/diffusion tables of the production path.
static void build_tables(DeviceProd* d, const Model& m) {
    d->K = m.K;
    d->S1 = m.n_species + 1;
    d->R = m.n_reactions;
    d->NC = m.nr + 1;
    if (m.K != 8 && m.K != 16) throw Error(CS_ERR_LIMIT, "the production path supports max_particles_site 8 or 16");
    if (m.nr > 254) throw Error(CS_ERR_LIMIT, "at most 254 regions on the production path");
    std::vector<uint32_t> thr((size_t)d->NC * d->NC * d->S1, 0u);
    for (uint32_t a = 1; a < d->NC; a++)
        for (uint32_t b = 1; b < d->NC; b++)
            for (uint32_t q = 0; q < d->S1; q++) {
                double D = m.diffusion[((size_t)(a - 1) * m.nr + (b - 1)) * m.np + q];
                double p = D * (double)m.tau / ((double)m.lambda * (double)m.lambda);
                if (p > 0.5) throw Error(CS_ERR_INVALID_ARG, "D*tau/lambda^2 exceeds 1/2 for some species and region pair: the per-axis sweep needs tau <= lambda^2/(2 D)");
                thr[((size_t)a * d->NC + b) * d->S1 + q] = threshold_of(D, m.tau, m.lambda);
            }
    std::vector<uint8_t> rre(3 * std::max<uint32_t>(d->R, 1), 0), csp(8 * std::max<uint32_t>(d->R, 1), 0);
    std::vector<int8_t> cdl(8 * std::max<uint32_t>(d->R, 1), 0);
    std::vector<float> rate(std::max<uint32_t>(d->R, 1), 0.0f);
    for (uint32_t r = 0; r < d->R; r++) {
        for (int j = 0; j < 3; j++) rre[3 * r + j] = (uint8_t)m.reactants[(size_t)(r + 1) * 3 + j];
        rate[r] = m.rates[r + 1];
        if (!(rate[r] >= 0.0f)) throw Error(CS_ERR_INVALID_ARG, "reaction rates must be non-negative on the production path");
        int n = 0;
        for (uint32_t s = 1; s < d->S1; s++) {
            int32_t v = m.stoich[(size_t)(r + 1) * d->S1 + s];
            if (!v) continue;
            if (n >= 8 || v < -127 || v > 127) throw Error(CS_ERR_LIMIT, "a reaction may change at most 8 species by at most 127");
            csp[8 * r + n] = (uint8_t)s;
            cdl[8 * r + n] = (int8_t)v;
            n++;
        }
    }
    if (d->R > 128) throw Error(CS_ERR_LIMIT, "at most 128 reactions on the production path");
    // candidate masks: bit r of rmask[s] when s is a reactant of reaction r
    std::vector<unsigned long long> rmask(2 * (size_t)d->S1, 0ull);
    unsigned long long zmask[2] = {0ull, 0ull};
    uint32_t n_zero = 0;
    for (uint32_t r = 0; r < d->R; r++) {
        bool any = false;
        for (int j = 0; j < 3; j++) {
            uint32_t s = rre[3 * r + j];
            if (s) { rmask[2 * s + (r >> 6)] |= 1ull << (r & 63); any = true; }
        }
        if (!any) { zmask[r >> 6] |= 1ull << (r & 63); n_zero++; }
    }
    d->thr.alloc(thr.size());
    d->rx_reactants.alloc(rre.size());
    d->rx_ch_sp.alloc(csp.size());
    d->rx_ch_d.alloc(cdl.size());
    d->rx_rate.alloc(rate.size());
    d->rmask.alloc(rmask.size());
    CS_CUDA(cudaMemcpy(d->thr.p, thr.data(), thr.size() * 4, cudaMemcpyHostToDevice));
    CS_CUDA(cudaMemcpy(d->rx_reactants.p, rre.data(), rre.size(), cudaMemcpyHostToDevice));
    CS_CUDA(cudaMemcpy(d->rx_ch_sp.p, csp.data(), csp.size(), cudaMemcpyHostToDevice));
    CS_CUDA(cudaMemcpy(d->rx_ch_d.p, cdl.data(), cdl.size(), cudaMemcpyHostToDevice));
    CS_CUDA(cudaMemcpy(d->rx_rate.p, rate.data(), rate.size() * 4, cudaMemcpyHostToDevice));
    CS_CUDA(cudaMemcpy(d->rmask.p, rmask.data(), rmask.size() * 8, cudaMemcpyHostToDevice));
    ProdTables& T = d->T;
    T.S1 = d->S1;
    T.R = d->R;
    T.NC = d->NC;
    T.K = d->K;
    T.tau = m.tau;
    T.tau_d = (double)m.tau;
    T.precision = CS_PREC_MIXED;
    T.max_events = 64;
    T.n_zero_order = n_zero;
    T.thr = d->thr.p;
    T.rx_reactants = d->rx_reactants.p;
    T.rx_rate = d->rx_rate.p;
    T.rx_ch_sp = d->rx_ch_sp.p;
    T.rx_ch_d = d->rx_ch_d.p;
    T.rmask = d->rmask.p;
    T.zmask[0] = zmask[0];
    T.zmask[1] = zmask[1];
    d->h_rate = rate;
    d->h_rre = rre;
    d->h_rmask = rmask;
    d->h_zmask[0] = zmask[0];
    d->h_zmask[1] = zmask[1];
}

// a0, max and min non-zero propensity of a voxel holding exactly one particle
// of species q (q = 0: no particle), per replicate, with the device's binary32
// operation sequence: a = (rate * mult) * ff, summed in reaction order over
// the candidate reactions.
static void build_one_table(DeviceProd* d) {
    std::vector<float> one((size_t)d->n_rep * d->S1 * 3, 0.0f);
    for (uint32_t ri = 0; ri < d->n_rep; ri++) {
        float mult = d->h_reps[ri].rate_mult;
        for (uint32_t q = 0; q < d->S1; q++) {
            unsigned long long m[2] = {d->h_zmask[0], d->h_zmask[1]};
            if (q) { m[0] |= d->h_rmask[2 * q]; m[1] |= d->h_rmask[2 * q + 1]; }
            float a0 = 0.0f, amax = 0.0f, amin = INFINITY;
            for (uint32_t r = 0; r < d->R; r++) {
                if (!((m[r >> 6] >> (r & 63)) & 1ull)) continue;
                uint32_t ff = 1;
                for (int j = 0; j < 3; j++) {
                    uint32_t s = d->h_rre[3 * r + j];
                    if (!s) continue;
                    uint32_t mm = 0;
                    for (int i = 0; i < j; i++) mm += d->h_rre[3 * r + i] == s;
                    uint32_t cnt = (q != 0 && s == q) ? 1u : 0u;
                    ff = (cnt <= mm) ? 0u : ff * (cnt - mm);
                }
                float k = d->h_rate[r] * mult;
                float a = k * (float)ff;
                a0 = a0 + a;
                if (a > 0.0f) { amax = std::fmax(amax, a); amin = std::fmin(amin, a); }
            }
            float* o = &one[((size_t)ri * d->S1 + q) * 3];
            o[0] = a0; o[1] = amax; o[2] = amin;
        }
    }
    d->one.alloc(one.size());
    CS_CUDA(cudaMemcpy(d->one.p, one.data(), one.size() * 4, cudaMemcpyHostToDevice));
    d->T.one = d->one.p;
    // Quiet thresholds.  A voxel without reservoir or zero-order reaction
    // holding one particle of species p (q = 0) or one of p and one of q has
    // total propensity a0, and its first event is rejected when
    // dt = -logf(u1) / a0 > tau, u1 = m * 2^-24 with m = (B(v,0)[3] >> 8) + 1.
    // For m <= quiet[p][q] that holds for certain: u1 <= exp(-a0 tau (1 + 2^-12))
    // gives -log(u1) >= a0 tau (1 + 2^-12), while the device's binary32 sum of
    // a0 (at most 128 terms), its logf (within 3 ulp) and the correctly
    // rounded division together lose far less than the 2^-12 margin.  Larger m
    // take the exact path.  Two-particle entries are tabulated when the table
    // stays small.
    const uint32_t S1 = d->S1;
    const uint32_t QS = (uint64_t)d->n_rep * S1 * S1 <= (1ull << 22) ? S1 : 1u;
    std::vector<uint32_t> quiet((size_t)d->n_rep * S1 * QS, 0u);
    const double tau = (double)d->T.tau;
    auto threshold = [&](double a0) -> uint32_t {
        if (!(a0 > 0.0)) return 1u << 24;  // no reaction can fire: every draw is quiet
        const double ub = std::exp(-a0 * tau * (1.0 + std::ldexp(1.0, -12))) * 16777216.0;
        return ub >= 16777215.0 ? 16777215u : (uint32_t)std::floor(ub);
    };
    std::vector<uint32_t> cnt(S1, 0u);
    for (uint32_t ri = 0; ri < d->n_rep; ri++) {
        const double mult = (double)d->h_reps[ri].rate_mult;
        for (uint32_t p = 1; p < S1; p++) {
            quiet[((size_t)ri * S1 + p) * QS] = threshold((double)one[((size_t)ri * S1 + p) * 3]);
            for (uint32_t q = 1; q < QS; q++) {
                std::fill(cnt.begin(), cnt.end(), 0u);
                cnt[p]++;
                cnt[q]++;
                double a0 = 0.0;
                for (uint32_t r = 0; r < d->R; r++) {
                    double ff = 1.0;
                    for (int j = 0; j < 3; j++) {
                        const uint32_t s = d->h_rre[3 * r + j];
                        if (!s) continue;
                        uint32_t mm = 0;
                        for (int i = 0; i < j; i++) mm += d->h_rre[3 * r + i] == s;
                        ff = cnt[s] <= mm ? 0.0 : ff * (double)(cnt[s] - mm);
                    }
                    a0 += (double)d->h_rate[r] * mult * ff;
                }
                quiet[((size_t)ri * S1 + p) * QS + q] = threshold(a0);
            }
        }
    }
    d->T.QS = QS;
    // summed second- and third-order rates per replicate (bound of fuller voxels' a0)
    std::vector<float> g23((size_t)d->n_rep * 2, 0.0f);
    for (uint32_t ri = 0; ri < d->n_rep; ri++) {
        double g2 = 0.0, g3 = 0.0;
        for (uint32_t r = 0; r < d->R; r++) {
            int order = 0;
            for (int j = 0; j < 3; j++) order += d->h_rre[3 * r + j] != 0;
            const double k = (double)d->h_rate[r] * (double)d->h_reps[ri].rate_mult;
            if (order == 2) g2 += k;
            if (order == 3) g3 += k;
        }
        // rounded up to binary32 so that the device bound never falls below the exact one
        g23[2 * ri] = std::nextafter((float)g2, INFINITY);
        g23[2 * ri + 1] = g3 > 0.0 ? std::nextafter((float)g3, INFINITY) : 0.0f;
    }
    d->g23.alloc(g23.size());
    CS_CUDA(cudaMemcpy(d->g23.p, g23.data(), g23.size() * 4, cudaMemcpyHostToDevice));
    d->T.g23 = d->g23.p;
    // second-order propensity of one particle pair (p, q) per replicate: the rates of the
    // reactions whose reactants are exactly p and q, twice for p == q (n(n-1) counts each
    // unordered pair of p twice), rounded up; tabulated beside the two-particle thresholds
    d->T.a2 = nullptr;
    if (QS == S1) {
        std::vector<float> a2((size_t)d->n_rep * S1 * S1, 0.0f);
        for (uint32_t ri = 0; ri < d->n_rep; ri++) {
            std::vector<double> acc2((size_t)S1 * S1, 0.0);
            for (uint32_t r = 0; r < d->R; r++) {
                const uint32_t sp[3] = {d->h_rre[3 * r], d->h_rre[3 * r + 1], d->h_rre[3 * r + 2]};
                uint32_t nz = 0, a = 0, b = 0;
                for (int j = 0; j < 3; j++)
                    if (sp[j]) {
                        if (nz == 0) a = sp[j];
                        else b = sp[j];
                        nz++;
                    }
                if (nz != 2) continue;
                const double k = (double)d->h_rate[r] * (double)d->h_reps[ri].rate_mult * (a == b ? 2.0 : 1.0);
                acc2[(size_t)a * S1 + b] += k;
                if (a != b) acc2[(size_t)b * S1 + a] += k;
            }
            for (size_t i = 0; i < acc2.size(); i++)
                a2[(size_t)ri * S1 * S1 + i] = acc2[i] > 0.0 ? std::nextafter((float)acc2[i], INFINITY) : 0.0f;
        }
        d->a2.alloc(a2.size());
        CS_CUDA(cudaMemcpy(d->a2.p, a2.data(), a2.size() * 4, cudaMemcpyHostToDevice));
        d->T.a2 = d->a2.p;
    }
    d->quiet.alloc(quiet.size());
    CS_CUDA(cudaMemcpy(d->quiet.p, quiet.data(), quiet.size() * 4, cudaMemcpyHostToDevice));
    d->T.quiet = d->quiet.p;
}

// Default step before any autotuning: the sweep stream of the model's K with
// four-block X sweeps and the Y and Z sweeps fused at three blocks per SM
// (the fastest on the sparse 256^3 lattice measured) where rows have at most
// 32 words, else four-block sweep passes and a three-block pass 3, else its
// first brick pass.
static int pick_default_cfg(uint32_t K, bool fused_ok) {
    const auto& c = all_cfgs();
    int first = -1, plain = -1;
    for (size_t i = 0; i < c.size(); i++) {
        if (c[i].K != (int)K) continue;
        if (c[i].kind == KIND_STREAM && c[i].variant == 4 && fused_ok) return (int)i;
        if (c[i].kind == KIND_STREAM && c[i].variant == 2) plain = (int)i;
        if (first < 0 && c[i].kind == KIND_BRICK) first = (int)i;
    }
    return plain >= 0 ? plain : first;
}

// The region code shared by every lattice voxel of brick w's region window
// (planes x0-2..x0+BX+1, rows y0-2..y0+BY+1, columns z0-2..z0+45), or 0 when
// the window holds more than one region or the host copy is absent.
static uint32_t window_code(const DeviceProd* d, const RepDesc& r, const WorkItem& w, const KernelCfg& cfg) {
    if (d->h_region_pad.empty() || (r.flags & 1u)) return 0u;
    const uint8_t* rp = d->h_region_pad.data() + r.rbase;
    const int64_t xa = std::max<int64_t>(0, (int64_t)w.x0 - 2), xb = std::min<int64_t>(r.X, (int64_t)w.x0 + cfg.BX + 2);
    const int64_t ya = std::max<int64_t>(0, (int64_t)w.y0 - 2), yb = std::min<int64_t>(r.Y, (int64_t)w.y0 + cfg.TY + 2);
    const int64_t za = std::max<int64_t>(0, (int64_t)w.z0 - 2), zb = std::min<int64_t>(r.Z, (int64_t)w.z0 + 46);
    uint32_t code = 0u;
    for (int64_t x = xa; x < xb; x++)
        for (int64_t y = ya; y < yb; y++) {
            const uint8_t* row = rp + ((uint64_t)x * r.Y + (uint64_t)y) * r.Zr + 2;  // column z + 2 holds z
            for (int64_t z = za; z < zb; z++) {
                if (code == 0u) code = row[z];
                else if (row[z] != code) return 0u;
            }
        }
    return code;
}

// Work items for the current config: (replicate, y0, z0, x-segment).  A brick
// configuration uses segments of BX planes, x fastest, so that bricks sharing
// halo planes run close together in time and the halo re-reads hit L2.
static void build_groups(DeviceProd* d);

// The fused Y and Z sweeps need every group to hold whole rows.
static bool fused_fits(const DeviceProd* d) {
    for (const RepDesc& r : d->h_reps)
        if (r.Wz > 32) return false;
    return true;
}

static void build_items(DeviceProd* d) {
    const KernelCfg& cfg = all_cfgs()[d->cfg_index];
    if (cfg.kind == KIND_RESIDENT) return;  // no work lists: one block per replicate
    if (cfg.kind == KIND_STREAM) {
        build_groups(d);
        return;
    }
    std::vector<WorkItem> all, per_rep;
    d->rep_item_off.assign(d->n_rep + 1, 0);
    // target: enough items to keep every SM busy with a few in flight
    uint64_t cols_total = 0;
    for (auto& r : d->h_reps) cols_total += (uint64_t)((r.Y + cfg.TY - 1) / cfg.TY) * ((r.Z + cfg.TZ - 1) / cfg.TZ);
    uint64_t want = (uint64_t)d->num_sms * 8;
    for (uint32_t ri = 0; ri < d->n_rep; ri++) {
        const RepDesc& r = d->h_reps[ri];
        d->rep_item_off[ri] = (uint32_t)per_rep.size();
        uint32_t seg;
        if (cfg.kind == KIND_BRICK) {
            seg = (uint32_t)cfg.BX;
        } else {
            uint32_t nseg = 1;
            if (d->seg_len) nseg = (r.X + d->seg_len - 1) / d->seg_len;
            else if (cols_total < want)
                nseg = (uint32_t)std::min<uint64_t>((want + cols_total - 1) / cols_total, std::max<uint32_t>(r.X / 16, 1));
            seg = (r.X + nseg - 1) / nseg;
        }
        for (uint32_t y0 = 0; y0 < r.Y; y0 += cfg.TY)
            for (uint32_t z0 = 0; z0 < r.Z; z0 += cfg.TZ)
                for (uint32_t x0 = 0; x0 < r.X; x0 += seg) {
                    WorkItem w{};
                    w.rep = ri; w.y0 = y0; w.z0 = z0; w.x0 = x0; w.x1 = std::min(r.X, x0 + seg);
                    if (cfg.kind == KIND_BRICK) w.pad[0] = window_code(d, r, w, cfg);
                    per_rep.push_back(w);
                }
    }
    d->rep_item_off[d->n_rep] = (uint32_t)per_rep.size();
    all = per_rep;
    if (cfg.kind == KIND_TILE) {
        // batched order: largest work first (longest processing time first)
        std::stable_sort(all.begin(), all.end(), [&](const WorkItem& a, const WorkItem& b) {
            uint64_t wa = (uint64_t)(a.x1 - a.x0), wb = (uint64_t)(b.x1 - b.x0);
            return wa > wb;
        });
    }
    d->n_items = (uint32_t)all.size();
    d->items.alloc(all.size());
    d->items_rep.alloc(per_rep.size());
    d->spill.alloc(all.size());
    CS_CUDA(cudaMemcpy(d->items.p, all.data(), all.size() * sizeof(WorkItem), cudaMemcpyHostToDevice));
    CS_CUDA(cudaMemcpy(d->items_rep.p, per_rep.data(), per_rep.size() * sizeof(WorkItem), cudaMemcpyHostToDevice));
}

// Word groups of the sweep stream: for each replicate and x plane, runs of
// whole rows that fill up to 32 lanes (rows of more than 32 words are cut
// into 32-word pieces), in replicate order.  The records of group g start
// after the capacities (32 per word) of the groups before it, so the
// records of all groups together number 32 per bitmap word.
static void build_groups(DeviceProd* d) {
    std::vector<WordGroup> gs;
    d->rep_group_off.assign(d->n_rep + 1, 0);
    uint64_t rb = 0;
    for (uint32_t ri = 0; ri < d->n_rep; ri++) {
        const RepDesc& r = d->h_reps[ri];
        d->rep_group_off[ri] = (uint32_t)gs.size();
        for (uint32_t x = 0; x < r.X; x++) {
            if (r.Wz <= 32) {
                const uint32_t per = 32 / r.Wz;
                for (uint32_t y0 = 0; y0 < r.Y; y0 += per) {
                    const WordGroup g{ri, x, y0, std::min(per, r.Y - y0), 0u, r.Wz, rb};
                    rb += (uint64_t)g.nrows * g.nk * 32u;
                    gs.push_back(g);
                }
            } else {
                for (uint32_t y = 0; y < r.Y; y++)
                    for (uint32_t k0 = 0; k0 < r.Wz; k0 += 32) {
                        const WordGroup g{ri, x, y, 1u, k0, std::min(32u, r.Wz - k0), rb};
                        rb += (uint64_t)g.nk * 32u;
                        gs.push_back(g);
                    }
            }
        }
    }
    d->rep_group_off[d->n_rep] = (uint32_t)gs.size();
    const bool fused = stream_variant_fused(all_cfgs()[d->cfg_index].variant);  // set_cfg checked that rows fit
    if (rb >= (1ull << 32) || gs.size() >= (1ull << 32))
        throw Error(CS_ERR_LIMIT, "lattice too large for the sweep-stream step (at most 2^32 records)");
    d->n_groups = (uint32_t)gs.size();
    d->n_items = d->n_groups;
    if (!d->h_region_pad.empty() && d->wcode.n == 0) {
        // uniform region code of each word's window: first per row word (z from 32k-1 to
        // 32k+32 inside the lattice), then over the 3 x 3 rows around it
        const RepDesc& r = d->h_reps[0];
        const uint64_t rows = (uint64_t)r.X * r.Y;
        std::vector<uint8_t> run(rows * r.Wz, 0), wc(rows * r.Wz, 0);
        for (uint64_t row = 0; row < rows; row++) {
            const uint8_t* rp = d->h_region_pad.data() + row * r.Zr + 2;  // column z + 2 holds z
            for (uint32_t k = 0; k < r.Wz; k++) {
                const int64_t za = std::max<int64_t>(0, 32 * (int64_t)k - 1);
                const int64_t zb = std::min<int64_t>(r.Z, 32 * (int64_t)k + 33);
                uint8_t c = rp[za];
                for (int64_t z = za + 1; z < zb && c; z++)
                    if (rp[z] != c) c = 0;
                run[row * r.Wz + k] = c;
            }
        }
        for (uint32_t x = 0; x < r.X; x++)
            for (uint32_t y = 0; y < r.Y; y++)
                for (uint32_t k = 0; k < r.Wz; k++) {
                    const uint64_t wi = ((uint64_t)x * r.Y + y) * r.Wz + k;
                    uint8_t c = run[wi];
                    for (int dx = -1; dx <= 1 && c; dx++)
                        for (int dy = -1; dy <= 1 && c; dy++) {
                            const int64_t xx = (int64_t)x + dx, yy = (int64_t)y + dy;
                            if (xx < 0 || xx >= r.X || yy < 0 || yy >= r.Y) continue;
                            if (run[((uint64_t)xx * r.Y + (uint64_t)yy) * r.Wz + k] != c) c = 0;
                        }
                    wc[wi] = c;
                }
        d->wcode.alloc(wc.size());
        CS_CUDA(cudaMemcpy(d->wcode.p, wc.data(), wc.size(), cudaMemcpyHostToDevice));
    }
    d->groups.alloc(gs.size());
    CS_CUDA(cudaMemcpy(d->groups.p, gs.data(), gs.size() * sizeof(WordGroup), cudaMemcpyHostToDevice));
    d->h_groups = std::move(gs);
    d->groups_sorted = false;
    for (int b = 0; b < (fused ? 3 : 2); b++)
        if (d->rec[b].n < 2 * rb) d->rec[b].alloc(2 * rb);  // two uint4 per record
    for (auto& a : d->sw)
        if (a.n < d->occ_words) a.alloc(d->occ_words);
    {
        // a pass-3 launch has at most 8 blocks of 256 threads per SM, and never more blocks than
        // its groups fill
        const uint64_t blocks = std::min<uint64_t>(8ull * (uint64_t)d->num_sms, ((uint64_t)d->n_groups + 7) / 8);
        const uint64_t need = std::max<uint64_t>(1, blocks) * 8ull * STREAM_SSA_OVER_PER_WARP;
        if (d->ssa_over.n < need) d->ssa_over.alloc(need);
    }
}

// Deals each replicate's word groups heaviest first (most occupied voxels in
// the current source bitmap), so that the passes end on light groups.  The
// order changes nothing else: records, words and results are indexed the same
// way.  Runs once per group build, with valid bitmaps, outside any capture.
static void sort_groups(DeviceProd* d) {
    std::vector<uint32_t> occ(d->occ_words);
    CS_CUDA(cudaMemcpyAsync(occ.data(), d->occ[d->cur].p, occ.size() * 4, cudaMemcpyDeviceToHost, d->stream));
    CS_CUDA(cudaStreamSynchronize(d->stream));
    std::vector<std::pair<uint32_t, uint32_t>> wg;  // (weight, index within the replicate's range)
    std::vector<WordGroup> out(d->h_groups.size());
    for (uint32_t ri = 0; ri < d->n_rep; ri++) {
        const RepDesc& r = d->h_reps[ri];
        const uint32_t a = d->rep_group_off[ri], b = d->rep_group_off[ri + 1];
        wg.clear();
        for (uint32_t gi = a; gi < b; gi++) {
            const WordGroup& G = d->h_groups[gi];
            uint32_t wsum = 0;
            for (uint32_t i = 0; i < G.nrows * G.nk; i++) {
                const uint64_t y = G.y0 + i / G.nk, k = G.k0 + i % G.nk;
                wsum += (uint32_t)__builtin_popcount(occ[r.obase + ((uint64_t)G.x * r.Y + y) * r.Wz + k]);
            }
            wg.emplace_back(wsum, gi);
        }
        std::stable_sort(wg.begin(), wg.end(), [](const auto& u, const auto& v) { return u.first > v.first; });
        for (uint32_t j = 0; j < wg.size(); j++) out[a + j] = d->h_groups[wg[j].second];
    }
    d->h_groups = std::move(out);
    CS_CUDA(cudaMemcpy(d->groups.p, d->h_groups.data(), d->h_groups.size() * sizeof(WordGroup), cudaMemcpyHostToDevice));
    d->groups_sorted = true;
    if (fused_fits(d)) {
        // neighbour links of the multi-frame form, by the sorted positions of the groups: with rows
        // of at most 32 words a group holds rows y0 .. y0 + 32 / Wz - 1 of plane x, and the
        // replicate's groups in build order are plane-major
        const size_t n = d->h_groups.size();
        std::vector<uint32_t> pos(n), nb(4 * n, 0xFFFFFFFFu);
        auto build_index = [&](const WordGroup& G) -> size_t {
            const RepDesc& r = d->h_reps[G.rep];
            const uint32_t per = 32 / r.Wz, gpp = (r.Y + per - 1) / per;
            return d->rep_group_off[G.rep] + (size_t)G.x * gpp + G.y0 / per;
        };
        for (size_t j = 0; j < n; j++) pos[build_index(d->h_groups[j])] = (uint32_t)j;
        for (size_t j = 0; j < n; j++) {
            const WordGroup& G = d->h_groups[j];
            const RepDesc& r = d->h_reps[G.rep];
            const uint32_t per = 32 / r.Wz, gpp = (r.Y + per - 1) / per;
            const size_t bi = build_index(G);
            if (G.x > 0) nb[4 * j + 0] = pos[bi - gpp];
            if (G.x + 1 < r.X) nb[4 * j + 1] = pos[bi + gpp];
            if (G.y0 > 0) nb[4 * j + 2] = pos[bi - 1];
            if (G.y0 / per + 1 < gpp) nb[4 * j + 3] = pos[bi + 1];
        }
        if (d->nbr.n != nb.size()) d->nbr.alloc(nb.size());
        CS_CUDA(cudaMemcpy(d->nbr.p, nb.data(), nb.size() * 4, cudaMemcpyHostToDevice));
        if (d->plane_order.n != n) d->plane_order.alloc(n);
        CS_CUDA(cudaMemcpy(d->plane_order.p, pos.data(), n * 4, cudaMemcpyHostToDevice));
        if (d->done1.n != n + 1) {
            // fresh completion values: every group done up to the base 0 (and one more entry that
            // nothing writes, for cs_debug_stall_group)
            d->done1.alloc(n + 1);
            d->done2.alloc(n + 1);
            CS_CUDA(cudaMemset(d->done1.p, 0, (n + 1) * 4));
            CS_CUDA(cudaMemset(d->done2.p, 0, (n + 1) * 4));
            d->frames_seq = 0;
        }
        if (d->frames_ctr.n == 0) {
            d->frames_ctr.alloc(2);
            CS_CUDA(cudaMemset(d->frames_ctr.p, 0, 8));
        }
    }
}

static uint32_t thr_words(const DeviceProd* d) {
    const uint32_t n = d->NC * d->NC * d->S1;
    return n <= kThrSmemWords ? n : 0u;
}

static uint64_t max_rep_voxels(const DeviceProd* d) {
    uint64_t m = 0;
    for (const RepDesc& r : d->h_reps) m = std::max<uint64_t>(m, (uint64_t)r.X * r.Y * r.Z);
    return m;
}

// The resident form needs every replicate in one block's shared memory.
static bool resident_fits(const DeviceProd* d) {
    int optin = 0;
    CS_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, d->device));
    const uint64_t v = max_rep_voxels(d);
    return v <= 0xFFFFull && resident_smem((int)d->K, v, thr_words(d)) <= (size_t)optin;  // 16-bit voxel lists
}

static size_t cfg_smem(const DeviceProd* d, const KernelCfg& cfg) {
    if (cfg.kind == KIND_RESIDENT) return resident_smem(cfg.K, max_rep_voxels(d), thr_words(d));
    if (cfg.kind == KIND_STREAM) return stream_pass_smem(cfg.variant, 2, d->S1, thr_words(d));  // the largest pass
    return cfg.smem(d->S1, thr_words(d));
}

static void set_attrs(const DeviceProd* d, const KernelCfg& cfg) {
    if (cfg.kind == KIND_RESIDENT) {
        resident_set_attrs(d->device);
        return;
    }
    if (cfg.kind == KIND_STREAM) {
        stream_set_attrs(cfg.K, cfg.variant, d->S1, thr_words(d));
        return;
    }
    CS_CUDA(cudaFuncSetAttribute(cfg.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cfg_smem(d, cfg)));
    CS_CUDA(cudaFuncSetAttribute(cfg.fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
}

// Captured frame graphs hold the launch parameters of the current configuration and precision.
static void drop_graphs(DeviceProd* d) {
    if (d->graph) {
        cudaGraphExecDestroy(d->graph);
        d->graph = nullptr;
    }
    for (cudaGraphExec_t& g1 : d->graph1)
        if (g1) {
            cudaGraphExecDestroy(g1);
            g1 = nullptr;
        }
}

static void set_cfg(DeviceProd* d, int idx) {
    const KernelCfg& cfg = all_cfgs()[idx];
    if (cfg.kind == KIND_STREAM && stream_variant_fused(cfg.variant) && !fused_fits(d))
        throw Error(CS_ERR_INVALID_ARG, "fused sweep-stream variant needs rows of at most 32 bitmap words (Z <= 1024)");
    if (cfg.kind == KIND_RESIDENT && !resident_fits(d))
        throw Error(CS_ERR_INVALID_ARG, "resident variant needs every lattice in one block's shared memory");
    set_attrs(d, cfg);
    if (cfg.spill >= 0) set_attrs(d, all_cfgs()[cfg.spill]);
    // build_items reads cfg_index; when it refuses the new configuration (a lattice too large for
    // its work lists), the previous configuration and its lists are restored
    const int prev = d->cfg_index;
    d->cfg_index = idx;
    try {
        build_items(d);
    } catch (...) {
        d->cfg_index = prev;
        if (prev >= 0) build_items(d);
        throw;
    }
    drop_graphs(d);
}

// Occupancy bitmap of one replicate's slot buffer: one warp per (x, y) row,
// one ballot per 32 voxels.
template <int K>
__global__ void occ_rebuild_kernel(const uint8_t* slots, uint32_t* occ, RepDesc rd) {
    const uint64_t rows = (uint64_t)rd.X * rd.Y;
    const int lane = threadIdx.x & 31;
    const uint64_t nwarps = (uint64_t)gridDim.x * (blockDim.x / 32);
    for (uint64_t row = (uint64_t)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); row < rows; row += nwarps) {
        const uint8_t* sr = slots + (rd.base + row * rd.Z) * K;
        for (uint32_t k = 0; k < rd.Wz; k++) {
            const uint32_t z = 32u * k + (uint32_t)lane;
            bool nz = false;
            if (z < rd.Z) {
                const uint8_t* p = sr + (uint64_t)z * K;
                if (K == 16) {
                    const uint4 t = *reinterpret_cast<const uint4*>(p);
                    nz = (t.x | t.y | t.z | t.w) != 0u;
                } else {
                    const uint2 t = *reinterpret_cast<const uint2*>(p);
                    nz = (t.x | t.y) != 0u;
                }
            }
            const uint32_t m = __ballot_sync(0xffffffffu, nz);
            if (lane == 0) occ[rd.obase + row * rd.Wz + k] = m;
        }
    }
}

static void rebuild_occupancy(DeviceProd* d) {
    for (int b = 0; b < 2; b++)
        for (const RepDesc& r : d->h_reps) {
            const uint64_t rows = (uint64_t)r.X * r.Y;
            const int blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>((rows + 7) / 8, (uint64_t)d->num_sms * 8));
            if (d->K == 16) occ_rebuild_kernel<16><<<blocks, 256, 0, d->stream>>>(d->slots[b].p, d->occ[b].p, r);
            else occ_rebuild_kernel<8><<<blocks, 256, 0, d->stream>>>(d->slots[b].p, d->occ[b].p, r);
            CS_LAUNCH_CHECK();
        }
    d->occ_valid = true;
}

static int grid_for(DeviceProd* d, const KernelCfg& cfg, uint32_t n_items) {
    int per_sm = 0;
    CS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cfg.fn, cfg.NT, cfg_smem(d, cfg)));
    if (per_sm < 1) throw Error(CS_ERR_CUDA, "production kernel does not fit on an SM");
    return (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)per_sm * d->num_sms, n_items));
}

// Counters of launch group g (0 = all replicates, 1 + r = replicate r alone)
// for frame parity p.  Brick pass: [0] work queue of the first launch, [1]
// spilled bricks, [2] work queue of the spill pass.  Sweep stream: [0..2] group
// queues of passes 1-3.
static constexpr int kCtrPerParity = 3;
static uint32_t* group_ctr(DeviceProd* d, int g, int p) { return d->counters.p + (size_t)(2 * g + p) * kCtrPerParity; }

// One pass of a sweep-stream frame of parity `parity` over all word groups
// (rep < 0) or over replicate rep's.  Records: the x-decisions of a frame of
// parity p are in rec[p]; pass 1 writes rec[p ^ 1], pass 2 rec[p], and pass 3
// (fused) the next frame's x-decisions into rec[p ^ 1].  Fused variants keep
// x-, y- and z-decisions in rec[0], rec[1] and rec[2]: their pass 2 sweeps
// along y and z and writes the next frame's x-decisions back into rec[0].
// Pass 1, the first pass of every frame, resets the other parity's work
// counters (as the brick pass does, so that the kinds can alternate); pass 3
// (fused variants: pass 2) advances the frame number.
static StreamParams stream_params(DeviceProd* d, const KernelCfg& cfg, const ProdParams& P, int rep, int parity, int pass) {
    uint32_t goff = 0, ng = d->n_groups;
    if (rep >= 0) {
        goff = d->rep_group_off[rep];
        ng = d->rep_group_off[rep + 1] - goff;
    }
    uint32_t* w[14];
    for (int i = 0; i < 14; i++) w[i] = d->sw[i].p;
    // per-word arrays of the pass boundaries: {occ, movers down, movers up, work, base}; the
    // x-decisions cover the source's occupied voxels, whose bitmap is their occ
    const SweepWords x_dec{nullptr, w[0], w[1], w[13], w[2]};
    const SweepWords x_in{const_cast<uint32_t*>(P.osrc), w[0], w[1], w[13], w[2]};
    const SweepWords y_dec{w[3], w[4], w[5], w[6], w[7]};
    const SweepWords z_dec{w[8], w[9], w[10], w[11], w[12]};
    const bool fused = stream_variant_fused(cfg.variant);
    uint4* const rx = d->rec[fused ? 0 : parity].p;       // this frame's x-decisions
    uint4* const ry = d->rec[fused ? 1 : parity ^ 1].p;   // y-decisions
    uint4* const rz = d->rec[fused ? 2 : parity].p;       // z-decisions
    uint4* const rnx = d->rec[fused ? 0 : parity ^ 1].p;  // the next frame's x-decisions
    StreamParams S{};
    S.P = P;
    S.P.items = nullptr;
    S.P.n_items = 0;
    S.P.advance = (pass == 3 || (fused && pass == 2)) ? 1u : 0u;
    S.P.n_reset = pass == 1 ? P.n_reset : 0u;
    S.groups = d->groups.p + goff;
    S.n_groups = ng;
    // passes 1-3 take their groups from the frame's three work counters (pass 0: round-robin)
    if (pass > 0) S.queue = group_ctr(d, rep < 0 ? 0 : 1 + rep, parity) + (pass - 1);
    S.wcode = d->wcode.n ? d->wcode.p : nullptr;
    S.ssa_over = d->ssa_over.p;
    switch (pass) {
        case 0: S.out = x_dec; S.rec_out = rx; break;
        case 1: S.in = x_in; S.rec_in = rx; S.out = y_dec; S.rec_out = ry; break;
        case 2:
            S.in = y_dec;
            S.rec_in = ry;
            if (fused) {  // the Y and Z sweeps: z-decisions in rec_mid, the next frame's x-decisions out
                S.rec_mid = rz;
                S.fuse = 1u;
                S.out = x_dec;
                S.rec_out = rnx;
            } else {
                S.out = z_dec;
                S.rec_out = rz;
            }
            break;
        default: S.in = z_dec; S.rec_in = rz; S.fuse = 1u; S.out = x_dec; S.rec_out = rnx; break;
    }
    S.in_occ1 = S.in.occ;
    S.odst1 = S.P.odst;
    S.dst1 = S.P.dst;
    return S;
}

static void launch_stream_pass(DeviceProd* d, const KernelCfg& cfg, const ProdParams& P, int rep, int parity, int pass) {
    StreamParams S = stream_params(d, cfg, P, rep, parity, pass);
    const uint32_t ng = S.n_groups;
    if (ng == 0) return;
    const size_t smem = stream_pass_smem(cfg.variant, pass, d->S1, thr_words(d));
    const uint32_t nw = (uint32_t)cfg.NT / 32u;
    if (d->stream_occ_cfg != d->cfg_index) {
        for (int q = 0; q < 4; q++)
            d->stream_per_sm[q] =
                stream_blocks_per_sm(cfg.K, cfg.variant, q, stream_pass_smem(cfg.variant, q, d->S1, thr_words(d)));
        d->stream_occ_cfg = d->cfg_index;
    }
    const int per_sm = d->stream_per_sm[pass];
    if (per_sm < 1) throw Error(CS_ERR_CUDA, "sweep-stream pass does not fit on an SM");
    const uint64_t want = ((uint64_t)ng + nw - 1) / nw;
    const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)per_sm * d->num_sms, want));
    if ((uint64_t)grid * nw * STREAM_SSA_OVER_PER_WARP > d->ssa_over.n)
        throw Error(CS_ERR_CUDA, "sweep-stream overflow lists smaller than the launch");
    // Groups per counter increment: 2 when every resident warp has 16 or more groups to take (the
    // ensemble's many mostly empty groups, where the same-address atomic is a large part of a
    // group's cost: 0.411 -> 0.354 ms per frame on 512 replicates of 32..96^3), else 1 (the 256^3
    // cell has about 4.5 groups per warp, and batches there leave warps idle at the tail: 0.164 ->
    // 0.190 ms at 2).
    S.batch = (uint64_t)ng >= 16ull * (uint64_t)grid * nw ? 2u : 1u;
    if (!stream_launch(cfg.K, cfg.variant, pass, grid, smem, d->stream, S))
        throw Error(CS_ERR_INVALID_ARG, "sweep-stream kernel not compiled for this K");
    CS_LAUNCH_CHECK();
}

static void fill_params(DeviceProd* d, ProdParams& P, int parity, int rep);

// Standalone pass 0 (x-decisions of every replicate) for the frame in stepbuf[cur].
static void launch_stream_pass0(DeviceProd* d) {
    const KernelCfg& cfg = all_cfgs()[d->cfg_index];
    ProdParams P{};
    fill_params(d, P, d->cur, -1);
    launch_stream_pass(d, cfg, P, -1, d->cur, 0);
}

// n frames of every replicate in the persistent multi-frame form, from the frame in stepbuf[cur]:
// one launch per chunk of frames (the tasks of a launch are counted in 32 bits).
static void launch_stream_frames(DeviceProd* d, uint32_t n) {
    const KernelCfg& cfg = all_cfgs()[d->cfg_index];
    const uint32_t ng = d->n_groups;
    if (n == 0 || ng == 0) return;
    if (d->nbr.n != 4ull * ng || d->done1.n != ng + 1u || d->plane_order.n != ng || d->frames_ctr.n < 2)
        throw Error(CS_ERR_STATE, "multi-frame sweep state missing (groups not sorted)");
    const size_t smem = stream_pass_smem(cfg.variant, 4, d->S1, thr_words(d));
    if (d->frames_occ_cfg != d->cfg_index) {
        d->frames_per_sm = stream_frames_blocks_per_sm(cfg.K, cfg.variant, smem);
        d->frames_occ_cfg = d->cfg_index;
    }
    const int per_sm = d->frames_per_sm;
    if (per_sm < 1) throw Error(CS_ERR_CUDA, "multi-frame sweep kernel does not fit on an SM");
    const int grid = per_sm * d->num_sms;
    const uint64_t over = (uint64_t)grid * ((uint32_t)cfg.NT / 32u) * STREAM_SSA_OVER_PER_WARP;
    if (d->ssa_over.n < over) d->ssa_over.alloc(over);
    ProdParams P0{}, P1{};
    fill_params(d, P0, 0, -1);
    fill_params(d, P1, 1, -1);
    FramesParams FP{};
    FP.sp[0] = stream_params(d, cfg, P0, -1, 0, 1);
    FP.sp[0].in_occ1 = P1.osrc;
    FP.sp[0].odst1 = P1.odst;
    FP.sp[0].dst1 = P1.dst;
    FP.sp[1] = stream_params(d, cfg, P0, -1, 0, 2);
    FP.sp[1].odst1 = P1.odst;
    FP.sp[1].dst1 = P1.dst;
    FP.nbr = d->nbr.p;
    FP.order = stream_variant_plane_order(cfg.variant) ? d->plane_order.p : nullptr;
    FP.done1 = d->done1.p;
    FP.done2 = d->done2.p;
    FP.tasks = d->frames_ctr.p;
    FP.exits = d->frames_ctr.p + 1;
    FP.reset = d->counters.p;
    FP.n_reset = (uint32_t)d->counters.n;
    FP.n_groups = ng;
    FP.fault = d->counts.p + (size_t)d->n_rep * d->S1;
    // tasks per launch: 2 ng per frame, and every warp fetches once past the last one, so the
    // counter stays below 2^32 with room for the largest grid
    const uint32_t chunk = (uint32_t)std::max<uint64_t>(
        1, std::min<uint64_t>((0xFFFFFFFFull - (1ull << 20)) / (2ull * ng), 1ull << 30));
    uint32_t stalled[4];
    const bool stall = d->stall_group < ng;
    if (stall) {
        // the group's neighbour links point at the entry that nothing writes, for this call
        CS_CUDA(cudaStreamSynchronize(d->stream));
        const uint32_t dummy[4] = {ng, ng, ng, ng};
        CS_CUDA(cudaMemcpy(stalled, d->nbr.p + 4ull * d->stall_group, 16, cudaMemcpyDeviceToHost));
        CS_CUDA(cudaMemcpy(d->nbr.p + 4ull * d->stall_group, dummy, 16, cudaMemcpyHostToDevice));
    }
    for (uint32_t k = 0; k < n;) {
        const uint32_t m = std::min(n - k, chunk);
        FP.n_frames = m;
        FP.cur0 = (uint32_t)d->cur;
        FP.seq = d->frames_seq;
        if (!stream_frames_launch(cfg.K, cfg.variant, grid, smem, d->stream, FP))
            throw Error(CS_ERR_INVALID_ARG, "multi-frame sweep kernel not compiled for this K");
        CS_LAUNCH_CHECK();
        d->frames_seq += m;
        d->cur = (int)(((uint32_t)d->cur + m) & 1u);
        k += m;
    }
    if (stall) {
        CS_CUDA(cudaStreamSynchronize(d->stream));
        CS_CUDA(cudaMemcpy(d->nbr.p + 4ull * d->stall_group, stalled, 16, cudaMemcpyHostToDevice));
        d->stall_group = 0xFFFFFFFFu;
    }
}

void prod_debug_stall_group(DeviceProd* d, uint32_t group) { d->stall_group = group; }

static void launch_stream_frame(DeviceProd* d, const KernelCfg& cfg, const ProdParams& P, int rep, int parity) {
    const bool fused = stream_variant_fused(cfg.variant);
    for (int pass = 1; pass <= 3; pass++)
        if (!(fused && pass == 3)) launch_stream_pass(d, cfg, P, rep, parity, pass);
}

// One frame over all replicates (batched) or over replicate `rep` alone.
static void launch_frame(DeviceProd* d, int parity, int rep) {
    const KernelCfg& cfg = all_cfgs()[d->cfg_index];
    ProdParams P{};
    fill_params(d, P, parity, rep);
    if (cfg.kind == KIND_STREAM) {
        launch_stream_frame(d, cfg, P, rep, parity);
        return;
    }
    const int g = rep < 0 ? 0 : 1 + rep;
    const uint32_t off = rep < 0 ? 0u : d->rep_item_off[rep];
    uint32_t* ctr = group_ctr(d, g, parity);
    const uint32_t n = P.n_items;
    if (cfg.spill >= 0) {
        P.spill = d->spill.p + off;
        P.n_spill = ctr + 1;
    }
    cfg.fn<<<grid_for(d, cfg, n), cfg.NT, cfg_smem(d, cfg), d->stream>>>(P);
    CS_LAUNCH_CHECK();
    if (cfg.spill >= 0) {
        // the full-capacity brick pass over the spilled bricks, cfg.sub plane groups each (usually
        // none: its CTAs take no item and exit)
        const KernelCfg& sc = all_cfgs()[cfg.spill];
        ProdParams Q = P;
        Q.items = d->spill.p + off;
        Q.n_items = 0;
        Q.n_items_dev = ctr + 1;
        Q.sub = cfg.sub;
        Q.queue = ctr + 2;
        Q.reset = nullptr;
        Q.n_reset = 0;
        Q.advance = 0u;
        Q.spill = nullptr;
        Q.n_spill = nullptr;
        sc.fn<<<grid_for(d, sc, n * cfg.sub), sc.NT, cfg_smem(d, sc), d->stream>>>(Q);
        CS_LAUNCH_CHECK();
    }
}

// Launch parameters shared by every kind for frame parity `parity`.
static void fill_params(DeviceProd* d, ProdParams& P, int parity, int rep) {
    P.T = d->T;
    P.reps = d->reps.p;
    P.parity = (uint32_t)parity;
    P.stepbuf = d->stepbuf.p;
    P.src = d->slots[parity].p;
    P.dst = d->slots[parity ^ 1].p;
    P.osrc = d->occ[parity].p;
    P.odst = d->occ[parity ^ 1].p;
    P.region_pad = d->region_pad.p;
    P.reservoir = d->reservoir.n ? d->reservoir.p : nullptr;
    P.counts = d->counts.p;
    P.diag = d->diag.p;
    const int g = rep < 0 ? 0 : 1 + rep;
    if (all_cfgs()[d->cfg_index].kind != KIND_STREAM) {  // the sweep stream has word groups, no items
        if (rep < 0) {
            P.items = d->items.p;
            P.n_items = d->n_items;
        } else {
            const uint32_t off = d->rep_item_off[rep];
            P.items = d->items_rep.p + off;
            P.n_items = d->rep_item_off[rep + 1] - off;
        }
    }
    uint32_t* ctr = group_ctr(d, g, parity);
    P.queue = ctr;
    P.reset = group_ctr(d, g, parity ^ 1);
    P.n_reset = kCtrPerParity;
    P.advance = 1u;
    P.thr_smem = thr_words(d) != 0u;
}

static DeviceProd* prod_alloc(const Model& m, int device, const std::vector<RepDesc>& reps, uint64_t total_voxels) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        throw Error(CS_ERR_CUDA, "no CUDA device available (libcellsim has no CPU fallback)");
    if (device < 0 || device >= ndev) throw Error(CS_ERR_INVALID_ARG, "device index out of range");
    DeviceGuard g(device);
    std::unique_ptr<DeviceProd> d(new DeviceProd());
    d->device = device;
    CS_CUDA(cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking));
    CS_CUDA(cudaDeviceGetAttribute(&d->num_sms, cudaDevAttrMultiProcessorCount, device));
    build_tables(d.get(), m);
    d->h_reps = reps;
    d->n_rep = (uint32_t)reps.size();
    d->total_voxels = total_voxels;
    d->reps.alloc(reps.size());
    CS_CUDA(cudaMemcpy(d->reps.p, reps.data(), reps.size() * sizeof(RepDesc), cudaMemcpyHostToDevice));
    build_one_table(d.get());
    for (int b = 0; b < 2; b++) d->slots[b].alloc(total_voxels * d->K);
    d->occ_words = 0;
    for (auto& r : d->h_reps) {
        r.Wz = (r.Z + 31) / 32;
        r.obase = d->occ_words;
        d->occ_words += (uint64_t)r.X * r.Y * r.Wz;
    }
    CS_CUDA(cudaMemcpy(d->reps.p, d->h_reps.data(), d->h_reps.size() * sizeof(RepDesc), cudaMemcpyHostToDevice));
    for (int b = 0; b < 2; b++) d->occ[b].alloc(d->occ_words);
    d->occ_valid = false;
    // the counts, then one word: dependency waits of the multi-frame kernel that timed out
    d->counts.alloc((size_t)d->n_rep * d->S1 + 1);
    d->diag.alloc(PD_N);
    d->counters.alloc((size_t)2 * kCtrPerParity * (1 + d->n_rep));
    d->stepbuf.alloc(2);
    CS_CUDA(cudaMemset(d->diag.p, 0, PD_N * 4));
    CS_CUDA(cudaMemset(d->counters.p, 0, d->counters.bytes()));
    CS_CUDA(cudaMemset(d->stepbuf.p, 0, 8));
    CS_CUDA(cudaMemset(d->counts.p, 0, d->counts.bytes()));
    int ci = pick_default_cfg(d->K, fused_fits(d.get()));
    if (ci < 0) throw Error(CS_ERR_LIMIT, "no kernel configuration for this K");
    set_cfg(d.get(), ci);
    return d.release();
}

DeviceProd* prod_create(const Model& m, int device) {
    m.check_tables();
    RepDesc r{};
    r.base = 0;
    r.rbase = 0;
    r.X = m.res[0]; r.Y = m.res[1]; r.Z = m.res[2];
    r.Zr = (uint32_t)((m.res[2] + 4 + 15) / 16 * 16);
    r.seed_lo = 0; r.seed_hi = 0;
    r.rate_mult = 1.0f;
    r.counts_index = 0;
    r.flags = 0;
    std::unique_ptr<DeviceProd> d(prod_alloc(m, device, {r}, m.V));
    DeviceGuard g(device);
    // region codes (id + 1) padded so that every tile's window row starts on a
    // 16-byte boundary: z is stored at column z + 2 of a row of Zr bytes
    const uint64_t XY = (uint64_t)m.res[0] * m.res[1];
    std::vector<uint8_t> rc(XY * r.Zr, 0);
    bool any_res = false;
    for (uint64_t row = 0; row < XY; row++)
        for (uint32_t z = 0; z < m.res[2]; z++) {
            uint64_t v = row * m.res[2] + z;
            rc[row * r.Zr + z + 2] = (uint8_t)(m.regions[v] + 1);
            any_res |= m.reservoir[v] != 0;
        }
    d->region_pad.alloc(rc.size());
    CS_CUDA(cudaMemcpy(d->region_pad.p, rc.data(), rc.size(), cudaMemcpyHostToDevice));
    d->h_region_pad = std::move(rc);
    build_items(d.get());  // brick items carry their window's region code
    if (any_res) {
        std::vector<uint8_t> r8(m.V);
        for (uint64_t v = 0; v < m.V; v++) r8[v] = (uint8_t)m.reservoir[v];
        d->reservoir.alloc(m.V);
        CS_CUDA(cudaMemcpy(d->reservoir.p, r8.data(), m.V, cudaMemcpyHostToDevice));
    }
    prod_set_lattice(d.get(), m, m.slots.data());
    return d.release();
}

void prod_destroy(DeviceProd* d) {
    if (!d) return;
    cudaSetDevice(d->device);
    if (d->stream) cudaStreamSynchronize(d->stream);
    delete d;
}

// Uploads a reference-layout lattice (u32 slots) for replicate 0, compacting
// each voxel's slots, and resets the species counts to slots + reservoirs.
void prod_set_lattice(DeviceProd* d, const Model& m, const uint32_t* slots) {
    DeviceGuard g(d->device);
    uint64_t V = m.V;
    std::vector<uint8_t> s8(V * d->K, 0);
    std::vector<long long> cnt(d->S1, 0);
    for (uint64_t v = 0; v < V; v++) {
        uint32_t j = 0;
        for (uint32_t k = 0; k < m.K; k++) {
            uint32_t q = slots[v * m.K + k];
            if (q > 255u) throw Error(CS_ERR_LIMIT, "slot value above 255");
            if (q) { s8[v * d->K + j++] = (uint8_t)q; cnt[q]++; }
        }
        if (m.reservoir[v]) cnt[m.reservoir[v]]++;
    }
    CS_CUDA(cudaStreamSynchronize(d->stream));
    d->cur = 0;
    d->frame_known = false;
    // the next frame has parity 0 whatever the last one had: its work counters start at zero
    CS_CUDA(cudaMemset(d->counters.p, 0, d->counters.bytes()));
    CS_CUDA(cudaMemcpy(d->slots[0].p, s8.data(), s8.size(), cudaMemcpyHostToDevice));
    d->occ_valid = false;
    std::vector<unsigned long long> c(d->S1);
    for (uint32_t s = 0; s < d->S1; s++) c[s] = (unsigned long long)cnt[s];
    CS_CUDA(cudaMemcpy(d->counts.p, c.data(), c.size() * 8, cudaMemcpyHostToDevice));
}

void prod_get_lattice(DeviceProd* d, const Model& m, uint32_t* slots, uint32_t* occ, int32_t* conc) {
    DeviceGuard g(d->device);
    CS_CUDA(cudaStreamSynchronize(d->stream));
    uint64_t V = m.V;
    std::vector<uint8_t> s8(V * d->K);
    CS_CUDA(cudaMemcpy(s8.data(), d->slots[d->cur].p, s8.size(), cudaMemcpyDeviceToHost));
    for (uint64_t v = 0; v < V; v++) {
        uint32_t n = 0;
        if (conc)
            for (uint32_t s = 0; s < d->S1; s++) conc[v * d->S1 + s] = 0;
        for (uint32_t k = 0; k < d->K; k++) {
            uint32_t q = s8[v * d->K + k];
            if (slots && k < m.K) slots[v * m.K + k] = q;
            if (q) {
                n++;
                if (conc) conc[v * d->S1 + q] += 1;
            }
        }
        if (occ) occ[v] = n;
        if (conc && m.reservoir[v]) conc[v * d->S1 + m.reservoir[v]] = 1;
    }
}

void prod_seed(DeviceProd* d, uint64_t seed) {
    if (d->seed_set && seed == d->cur_seed) return;
    for (auto& r : d->h_reps) {
        r.seed_lo = (uint32_t)seed;
        r.seed_hi = (uint32_t)(seed >> 32);
    }
    CS_CUDA(cudaMemcpyAsync(d->reps.p, d->h_reps.data(), d->h_reps.size() * sizeof(RepDesc), cudaMemcpyHostToDevice,
                            d->stream));
    CS_CUDA(cudaStreamSynchronize(d->stream));
    d->cur_seed = seed;
    d->seed_set = true;
    d->seed_epoch++;
}

// Runs n frames; batched = one launch per frame over all replicates (a
// captured two-frame graph replays pairs), otherwise one launch per replicate.
static void run_frames_nosync(DeviceProd* d, uint32_t n, bool batched);

static void run_frames(DeviceProd* d, uint32_t n, uint64_t frame0, bool batched) {
    if (n == 0) return;
    uint32_t f32 = (uint32_t)frame0;
    CS_CUDA(cudaMemcpyAsync(d->stepbuf.p + d->cur, &f32, 4, cudaMemcpyHostToDevice, d->stream));
    CS_CUDA(cudaStreamSynchronize(d->stream));
    d->next_frame = frame0;
    d->frame_known = true;
    run_frames_nosync(d, n, batched);
}

// Every frame of a call in one launch of the resident form: one block per replicate (batched) or
// one launch per replicate; the last frame's lattice lands in the buffer of parity cur ^ (n & 1).
static void launch_resident(DeviceProd* d, uint32_t n, bool batched) {
    ResidentParams RP{};
    fill_params(d, RP.P, d->cur, -1);
    const int out = d->cur ^ (int)(n & 1u);
    RP.P.dst = d->slots[out].p;
    RP.P.reset = d->counters.p;
    RP.P.n_reset = (uint32_t)d->counters.n;
    RP.frame0 = (uint32_t)d->next_frame;
    RP.n_frames = n;
    RP.stepbuf_out = (uint32_t)out;
    RP.vmax = (uint32_t)max_rep_voxels(d);
    RP.thr_words = thr_words(d);
    const size_t smem = resident_smem((int)d->K, RP.vmax, RP.thr_words);
    if (batched) {
        RP.rep0 = 0;
        resident_launch((int)d->K, RP, (int)d->n_rep, smem, d->stream);
    } else {
        for (uint32_t r = 0; r < d->n_rep; r++) {
            RP.rep0 = r;
            resident_launch((int)d->K, RP, 1, smem, d->stream);
        }
    }
}

// Enqueues n frames; the frame number must already be in stepbuf[cur] (and
// its host copy in next_frame).
static void run_frames_nosync(DeviceProd* d, uint32_t n, bool batched) {
    if (n == 0) return;
    if (all_cfgs()[d->cfg_index].kind == KIND_RESIDENT) {
        launch_resident(d, n, batched);
        d->cur ^= (int)(n & 1u);
        d->next_frame += n;
        d->occ_valid = false;  // the resident form keeps no occupancy bitmaps and no x-decisions
        d->xdec_valid = false;
        return;
    }
    // the brick pass and the sweep stream read and maintain the occupancy bitmaps
    const int kind = all_cfgs()[d->cfg_index].kind;
    const bool brick = kind != KIND_TILE;
    // x-decisions made by the last frame's pass 3 hold for this frame only if nothing has changed
    // the lattice, the seed, the frame number or the configuration since
    const bool xdec_ok = d->occ_valid && d->xdec_valid && d->xdec_cfg == d->cfg_index && d->xdec_cur == d->cur &&
                         d->xdec_frame == d->next_frame && d->xdec_epoch == d->seed_epoch;
    if (brick && !d->occ_valid) rebuild_occupancy(d);
    if (!brick) d->occ_valid = false;  // the tile pipeline does not keep the bitmaps
    if (kind == KIND_STREAM && !d->groups_sorted) sort_groups(d);
    d->xdec_valid = false;
    if (kind == KIND_STREAM && !xdec_ok) launch_stream_pass0(d);
    uint32_t k = 0;
    // the multi-frame form for calls of two or more frames; a single frame gains nothing from it
    // (no other frame's tasks to overlap) and runs as the captured per-pass launches of the same
    // shape (the fused passes at the same blocks per SM), which compute the same lattice
    if (batched && n >= 2 && kind == KIND_STREAM && stream_variant_frames(all_cfgs()[d->cfg_index].variant)) {
        launch_stream_frames(d, n);
        k = n;
    }
    // a single frame of parity p, from its own captured graph (a step call of one frame, as the
    // reference's per-frame step makes, costs one graph launch instead of three kernel launches)
    auto single = [&](int p) {
        if (!d->graph1[p] || d->graph1_cfg[p] != d->cfg_index) {
            if (d->graph1[p]) { cudaGraphExecDestroy(d->graph1[p]); d->graph1[p] = nullptr; }
            cudaGraph_t g;
            CS_CUDA(cudaStreamBeginCapture(d->stream, cudaStreamCaptureModeThreadLocal));
            launch_frame(d, p, -1);
            CS_CUDA(cudaStreamEndCapture(d->stream, &g));
            CS_CUDA(cudaGraphInstantiate(&d->graph1[p], g, 0));
            cudaGraphDestroy(g);
            d->graph1_cfg[p] = d->cfg_index;
        }
        CS_CUDA(cudaGraphLaunch(d->graph1[p], d->stream));
    };
    if (batched) {
        if (d->cur == 1 && k < n) {
            single(1);
            d->cur = 0;
            k++;
        }
        if (n - k >= 2) {
            if (!d->graph || d->graph_cfg != d->cfg_index) {
                if (d->graph) { cudaGraphExecDestroy(d->graph); d->graph = nullptr; }
                cudaGraph_t g;
                CS_CUDA(cudaStreamBeginCapture(d->stream, cudaStreamCaptureModeThreadLocal));
                launch_frame(d, 0, -1);
                launch_frame(d, 1, -1);
                CS_CUDA(cudaStreamEndCapture(d->stream, &g));
                CS_CUDA(cudaGraphInstantiate(&d->graph, g, 0));
                cudaGraphDestroy(g);
                d->graph_cfg = d->cfg_index;
            }
            while (n - k >= 2) {
                CS_CUDA(cudaGraphLaunch(d->graph, d->stream));
                k += 2;
            }
        }
        if (k < n) {
            single(0);
            d->cur = 1;
            k++;
        }
    } else {
        for (; k < n; k++) {
            for (uint32_t r = 0; r < d->n_rep; r++) launch_frame(d, d->cur, (int)r);
            d->cur ^= 1;
        }
    }
    d->next_frame += n;
    if (kind == KIND_STREAM) {
        // the last frame's pass 3 made the x-decisions of frame next_frame
        d->xdec_valid = true;
        d->xdec_cfg = d->cfg_index;
        d->xdec_cur = d->cur;
        d->xdec_frame = d->next_frame;
        d->xdec_epoch = d->seed_epoch;
    }
}

// The frame number of the next frame into stepbuf[cur] (the step's one
// host-to-device input, like the reference's per-frame itime write), in
// stream order and without a host wait.
static void upload_frame(DeviceProd* d, uint64_t frame0) {
    if (d->frame_known && d->next_frame == frame0) return;
    if (!d->h_frames) {
        CS_CUDA(cudaMallocHost(&d->h_frames, DeviceProd::kFrameSlots * sizeof(uint32_t)));
        for (cudaEvent_t& e : d->frame_ev) CS_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    const int s = d->frame_slot;
    d->frame_slot = (s + 1) % DeviceProd::kFrameSlots;
    CS_CUDA(cudaEventSynchronize(d->frame_ev[s]));  // the slot's previous copy has run (at once if never recorded)
    d->h_frames[s] = (uint32_t)frame0;
    CS_CUDA(cudaMemcpyAsync(d->stepbuf.p + d->cur, d->h_frames + s, 4, cudaMemcpyHostToDevice, d->stream));
    CS_CUDA(cudaEventRecord(d->frame_ev[s], d->stream));
    d->next_frame = frame0;
    d->frame_known = true;
}

void prod_step(DeviceProd* d, uint32_t n_steps, uint64_t seed, int precision, uint64_t frame0, uint32_t write_freq,
               const std::vector<uint32_t>& logging, std::vector<cs_stat_sample>& samples) {
    DeviceGuard g(d->device);
    if (n_steps == 0) return;
    prod_seed(d, seed);
    if (d->T.precision != precision) {
        d->T.precision = precision;
        drop_graphs(d);
    }
    std::vector<uint64_t> sample_frames;
    if (write_freq)
        for (uint64_t f = frame0; f < frame0 + n_steps; f++)
            if (f > 0 && f % write_freq == 0) sample_frames.push_back(f);
    // Samples are device-to-device copies of the counts into a ring, read back
    // once at the end: the frames in between are enqueued without host waits.
    uint64_t f = frame0, end = frame0 + n_steps;
    upload_frame(d, frame0);
    if (!sample_frames.empty() && d->sample_ring.n < sample_frames.size() * d->S1)
        d->sample_ring.alloc(sample_frames.size() * d->S1);
    for (size_t i = 0; i < sample_frames.size(); i++) {
        run_frames_nosync(d, (uint32_t)(sample_frames[i] - f), true);
        f = sample_frames[i];
        CS_CUDA(cudaMemcpyAsync(d->sample_ring.p + i * d->S1, d->counts.p, d->S1 * 8, cudaMemcpyDeviceToDevice,
                                d->stream));
    }
    run_frames_nosync(d, (uint32_t)(end - f), true);
    if (!sample_frames.empty()) {
        std::vector<unsigned long long> h(sample_frames.size() * d->S1);
        CS_CUDA(cudaMemcpyAsync(h.data(), d->sample_ring.p, h.size() * 8, cudaMemcpyDeviceToHost, d->stream));
        CS_CUDA(cudaStreamSynchronize(d->stream));
        for (size_t i = 0; i < sample_frames.size(); i++)
            for (uint32_t sp : logging)
                samples.push_back(cs_stat_sample{sp, (int32_t)(long long)h[i * d->S1 + sp], (uint32_t)sample_frames[i]});
    }
}

static const char* const kWaitFault =
    "the multi-frame sweep kernel abandoned frames after a dependency wait timed out; the lattice is not valid";

void prod_get_counts(DeviceProd* d, int64_t* counts) {
    DeviceGuard g(d->device);
    const size_t n = (size_t)d->n_rep * d->S1;
    if (!d->h_counts) CS_CUDA(cudaMallocHost(&d->h_counts, (n + 1) * 8));
    // the counts and the wait-timeout word in one copy
    CS_CUDA(cudaMemcpyAsync(d->h_counts, d->counts.p, (n + 1) * 8, cudaMemcpyDeviceToHost, d->stream));
    CS_CUDA(cudaStreamSynchronize(d->stream));
    if (d->h_counts[n]) throw Error(CS_ERR_CUDA, kWaitFault);
    for (size_t i = 0; i < n; i++) counts[i] = (int64_t)d->h_counts[i];
}

void prod_set_counts(DeviceProd* d, const int64_t* counts) {
    DeviceGuard g(d->device);
    std::vector<unsigned long long> h((size_t)d->n_rep * d->S1);
    for (size_t i = 0; i < h.size(); i++) h[i] = (unsigned long long)counts[i];
    CS_CUDA(cudaStreamSynchronize(d->stream));
    CS_CUDA(cudaMemcpy(d->counts.p, h.data(), h.size() * 8, cudaMemcpyHostToDevice));
}

// Replicate 0's view (the single lattice of a cs_sim).
void prod_render_view(DeviceProd* d, int32_t view, int32_t slice_axis, uint32_t slice, float* out_host, void* out_device) {
    DeviceGuard g(d->device);
    DevBuf<float> tmp;
    float* out_dev = static_cast<float*>(out_device);
    const uint64_t V = (uint64_t)d->h_reps[0].X * d->h_reps[0].Y * d->h_reps[0].Z;
    if (!out_dev) {
        tmp.alloc(V);
        out_dev = tmp.p;
    }
    const RepDesc& r = d->h_reps[0];
    ViewParams v{};
    v.slots = d->slots[d->cur].p;
    v.K = d->K;
    v.X = r.X; v.Y = r.Y; v.Z = r.Z;
    v.region_pad = (r.flags & 1u) ? nullptr : d->region_pad.p;
    v.Zr = r.Zr;
    v.reservoir = d->reservoir.n ? d->reservoir.p : nullptr;
    v.view = view;
    v.slice_axis = slice_axis;
    v.slice = slice;
    v.out = out_dev;
    render_view_kernel<<<1024, 256, 0, d->stream>>>(v);
    CS_LAUNCH_CHECK();
    if (!out_device) CS_CUDA(cudaMemcpyAsync(out_host, out_dev, V * sizeof(float), cudaMemcpyDeviceToHost, d->stream));
    CS_CUDA(cudaStreamSynchronize(d->stream));
}

void prod_get_diag(DeviceProd* d, uint32_t* diag, uint32_t n) {
    DeviceGuard g(d->device);
    uint32_t h[PD_N];
    CS_CUDA(cudaMemcpyAsync(h, d->diag.p, sizeof(h), cudaMemcpyDeviceToHost, d->stream));
    CS_CUDA(cudaStreamSynchronize(d->stream));
    for (uint32_t i = 0; i < n; i++) diag[i] = i < PD_N ? h[i] : 0u;
}

void prod_sync(DeviceProd* d) {
    DeviceGuard g(d->device);
    unsigned long long fault = 0;
    CS_CUDA(cudaMemcpyAsync(&fault, d->counts.p + (size_t)d->n_rep * d->S1, 8, cudaMemcpyDeviceToHost, d->stream));
    CS_CUDA(cudaStreamSynchronize(d->stream));
    if (fault) throw Error(CS_ERR_CUDA, kWaitFault);
}

}  // namespace cellsim

namespace cellsim {

// ------------------------------------------------------------------ ensemble

// Replicates of one model on lattices of their own resolution, filled with
// region 0 of the model and with counts[s] particles of species s placed
// uniformly at random (append-at-occupancy rule of src/lattice.rs:280-290,
// up to 100 draws per particle as in src/lattice.rs:66-95).
DeviceProd* prod_ensemble_create(const Model& m, uint32_t n, const uint32_t* res, const uint64_t* seeds, const float* mult,
                                 const uint32_t* init_counts, int device) {
    if (n == 0) throw Error(CS_ERR_INVALID_ARG, "an ensemble needs at least one replicate");
    std::vector<RepDesc> reps(n);
    uint64_t base = 0;
    for (uint32_t r = 0; r < n; r++) {
        RepDesc& d = reps[r];
        std::memset(&d, 0, sizeof(d));
        d.X = res[3 * r]; d.Y = res[3 * r + 1]; d.Z = res[3 * r + 2];
        if (!d.X || !d.Y || !d.Z) throw Error(CS_ERR_INVALID_ARG, "replicate resolution must be positive");
        uint64_t V = (uint64_t)d.X * d.Y * d.Z;
        if (V * m.K >= (1ull << 32)) throw Error(CS_ERR_LIMIT, "replicate too large (V*K must be below 2^32)");
        d.base = base;
        d.seed_lo = (uint32_t)seeds[r];
        d.seed_hi = (uint32_t)(seeds[r] >> 32);
        d.rate_mult = mult ? mult[r] : 1.0f;
        d.counts_index = r;
        d.flags = 1u;
        base += V;
    }
    std::unique_ptr<DeviceProd> d(prod_alloc(m, device, reps, base));
    DeviceGuard g(device);
    d->seed_set = true;  // per-replicate seeds, never overwritten by prod_seed
    d->cur_seed = ~0ull;
    // every replicate is region 0 throughout: codes are computed from the
    // coordinates (RepDesc flag bit 0), no region-code array is read
    d->region_pad.alloc(16);
    CS_CUDA(cudaMemset(d->region_pad.p, 0, 16));
    std::vector<unsigned long long> cnt((size_t)n * d->S1, 0ull);
    for (uint32_t r = 0; r < n; r++) {
        const RepDesc& rd = reps[r];
        uint64_t V = (uint64_t)rd.X * rd.Y * rd.Z;
        std::vector<uint8_t> s8(V * d->K, 0), occ(V, 0);
        HostRng rng;
        rng.seed(seeds[r] ^ 0xA5A5A5A5DEADBEEFull);
        for (uint32_t s = 1; s < d->S1; s++) {
            for (uint32_t i = 0; i < init_counts[s]; i++) {
                int tries = 0;
                for (; tries < 100; tries++) {
                    uint64_t v = rng.below(V);
                    if (occ[v] < d->K) {
                        s8[v * d->K + occ[v]++] = (uint8_t)s;
                        break;
                    }
                }
                if (tries == 100) throw Error(CS_ERR_CAPACITY, "could not place a particle in replicate " + std::to_string(r));
            }
            cnt[(size_t)r * d->S1 + s] = init_counts[s];
        }
        CS_CUDA(cudaMemcpy(d->slots[0].p + rd.base * d->K, s8.data(), s8.size(), cudaMemcpyHostToDevice));
    }
    d->occ_valid = false;
    CS_CUDA(cudaMemcpy(d->counts.p, cnt.data(), cnt.size() * 8, cudaMemcpyHostToDevice));
    d->cur = 0;
    return d.release();
}

void prod_ensemble_step(DeviceProd* d, uint32_t n_steps, bool batched, uint64_t frame0) {
    DeviceGuard g(d->device);
    run_frames(d, n_steps, frame0, batched);
}

void prod_set_precision(DeviceProd* d, int precision) {
    if (d->T.precision != precision) {
        d->T.precision = precision;
        drop_graphs(d);
    }
}

uint64_t prod_total_voxels(const DeviceProd* d) { return d->total_voxels; }
uint32_t prod_n_items(const DeviceProd* d) { return d->n_items; }
uint32_t prod_n_replicates(const DeviceProd* d) { return d->n_rep; }
uint32_t prod_s1(const DeviceProd* d) { return d->S1; }

// Downloads the packed slots of every replicate (K bytes per voxel).
void prod_get_slots_raw(DeviceProd* d, uint8_t* out) {
    DeviceGuard g(d->device);
    CS_CUDA(cudaStreamSynchronize(d->stream));
    CS_CUDA(cudaMemcpy(out, d->slots[d->cur].p, d->total_voxels * d->K, cudaMemcpyDeviceToHost));
}

// Tile configuration: index into the compiled (K, TY, TZ) variants and the
// x-segment length (0 = automatic).
void prod_set_tiling(DeviceProd* d, int cfg_index, uint32_t seg_len) {
    DeviceGuard g(d->device);
    const auto& c = all_cfgs();
    if (cfg_index < 0 || cfg_index >= (int)c.size() || c[cfg_index].K != (int)d->K)
        throw Error(CS_ERR_INVALID_ARG, "tile configuration does not exist for this K");
    CS_CUDA(cudaStreamSynchronize(d->stream));
    const uint32_t keep = d->seg_len;
    d->seg_len = seg_len;
    try {
        set_cfg(d, cfg_index);
    } catch (...) {
        d->seg_len = keep;  // a refused variant leaves the handle as it was
        throw;
    }
}

int prod_tiling_count() { return (int)all_cfgs().size(); }
void prod_tiling_desc(int i, int* K, int* TY, int* TZ, int* NT) {
    const auto& c = all_cfgs();
    if (i < 0 || i >= (int)c.size()) throw Error(CS_ERR_INVALID_ARG, "tile configuration index out of range");
    *K = c[i].K; *TY = c[i].TY; *TZ = c[i].TZ; *NT = c[i].NT;
}
void prod_tiling_kind(int i, int* kind, int* BX) {
    const auto& c = all_cfgs();
    if (i < 0 || i >= (int)c.size()) throw Error(CS_ERR_INVALID_ARG, "tile configuration index out of range");
    *kind = c[i].kind; *BX = c[i].BX;
}
int prod_tiling_launches(int i) {
    const auto& c = all_cfgs();
    if (i < 0 || i >= (int)c.size()) throw Error(CS_ERR_INVALID_ARG, "tile configuration index out of range");
    if (c[i].kind == KIND_RESIDENT) return 1;  // one launch per step call
    if (c[i].kind == KIND_STREAM) {
        if (stream_variant_frames(c[i].variant)) return 1;  // one launch per step call
        return stream_variant_fused(c[i].variant) ? 2 : 3;
    }
    return c[i].spill >= 0 ? 2 : 1;
}
int prod_tiling_current(const DeviceProd* d) { return d->cfg_index; }
cudaStream_t prod_stream(const DeviceProd* d) { return d->stream; }

}  // namespace cellsim

namespace cellsim {
// Runs n frames between two CUDA events recorded on the handle's stream and
// returns the elapsed device time in milliseconds (blocks until done).
float prod_time_frames(DeviceProd* d, uint32_t n, uint64_t frame0, bool batched) {
    DeviceGuard g(d->device);
    cudaEvent_t a, b;
    CS_CUDA(cudaEventCreate(&a));
    CS_CUDA(cudaEventCreate(&b));
    float ms = 0.0f;
    try {
        // the frame-number upload inside run_frames synchronises; record after it
        uint32_t f32 = (uint32_t)frame0;
        CS_CUDA(cudaMemcpyAsync(d->stepbuf.p + d->cur, &f32, 4, cudaMemcpyHostToDevice, d->stream));
        CS_CUDA(cudaStreamSynchronize(d->stream));
        d->next_frame = frame0;
        d->frame_known = true;
        CS_CUDA(cudaEventRecord(a, d->stream));
        run_frames_nosync(d, n, batched);
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
    return ms;
}
}  // namespace cellsim

namespace cellsim {
// Autotuner: times every compiled configuration for this K on the handle's
// own lattice and keeps the fastest.  Each trial starts from a device copy of
// the current state and the state is restored afterwards, so tuning does not
// advance or change the simulation (every configuration computes the same
// frame anyway).  Choices are cached per (K, species, reactions, regions,
// zero-order reactions or reservoirs present, lattice shapes, device) for the
// life of the process.
int prod_autotune(DeviceProd* d, uint32_t frames, uint64_t frame0, bool batched, float* best_ms) {
    DeviceGuard g(d->device);
    static std::mutex mu;
    static std::map<std::string, std::pair<int, float>> cache;
    cudaDeviceProp prop{};
    CS_CUDA(cudaGetDeviceProperties(&prop, d->device));
    std::string key = std::string(prop.name) + "|" + std::to_string(d->K) + "," + std::to_string(d->S1) + "," +
                      std::to_string(d->R) + "," + std::to_string(d->NC) + "," + std::to_string(batched ? 1 : 0) +
                      // reservoirs and zero-order reactions make the brick pass step every interior voxel
                      "," + std::to_string(d->T.n_zero_order != 0u ? 1 : 0) + std::to_string(d->reservoir.n ? 1 : 0);
    for (const RepDesc& r : d->h_reps) key += "|" + std::to_string(r.X) + "x" + std::to_string(r.Y) + "x" + std::to_string(r.Z);
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find(key);
        if (it != cache.end()) {
            if (d->cfg_index != it->second.first) {
                CS_CUDA(cudaStreamSynchronize(d->stream));
                d->seg_len = 0;
                set_cfg(d, it->second.first);
            }
            if (best_ms) *best_ms = it->second.second;
            return it->second.first;
        }
    }
    if (frames == 0) frames = 1;
    CS_CUDA(cudaStreamSynchronize(d->stream));
    const size_t bytes = (size_t)d->total_voxels * d->K;
    DevBuf<uint8_t> keep;
    keep.alloc(bytes);
    DevBuf<unsigned long long> keep_counts;
    keep_counts.alloc(d->counts.n);
    DevBuf<uint32_t> keep_diag;
    keep_diag.alloc(PD_N);
    const int cur0 = d->cur;
    CS_CUDA(cudaMemcpyAsync(keep.p, d->slots[cur0].p, bytes, cudaMemcpyDeviceToDevice, d->stream));
    CS_CUDA(cudaMemcpyAsync(keep_counts.p, d->counts.p, d->counts.bytes(), cudaMemcpyDeviceToDevice, d->stream));
    CS_CUDA(cudaMemcpyAsync(keep_diag.p, d->diag.p, PD_N * 4, cudaMemcpyDeviceToDevice, d->stream));
    auto restore = [&]() {
        CS_CUDA(cudaMemcpyAsync(d->slots[cur0].p, keep.p, bytes, cudaMemcpyDeviceToDevice, d->stream));
        CS_CUDA(cudaMemcpyAsync(d->counts.p, keep_counts.p, d->counts.bytes(), cudaMemcpyDeviceToDevice, d->stream));
        CS_CUDA(cudaMemcpyAsync(d->diag.p, keep_diag.p, PD_N * 4, cudaMemcpyDeviceToDevice, d->stream));
        CS_CUDA(cudaMemsetAsync(d->counters.p, 0, d->counters.bytes(), d->stream));  // parity cur0 starts afresh
        CS_CUDA(cudaStreamSynchronize(d->stream));
        d->cur = cur0;
        d->occ_valid = false;
        d->frame_known = false;
    };
    const auto& c = all_cfgs();
    int best = -1;
    float best_t = 0.0f;
    for (int i = 0; i < (int)c.size(); i++) {
        if (c[i].K != (int)d->K) continue;
        if (c[i].kind == KIND_STREAM && stream_variant_fused(c[i].variant) && !fused_fits(d)) continue;
        if (c[i].kind == KIND_RESIDENT && !resident_fits(d)) continue;
        d->seg_len = 0;
        set_cfg(d, i);
        prod_time_frames(d, 2, frame0, batched);  // warm-up: graph, bitmaps, caches
        restore();
        // the best of three trials, each after one untimed frame (the bitmap rebuild and the
        // x-decisions that every restored state needs first): variants within a few percent of
        // each other are then ranked by their steady frames, not by one noisy trial
        float t = 0.0f;
        for (int rep = 0; rep < 3; rep++) {
            prod_time_frames(d, 1, frame0, batched);
            const float r = prod_time_frames(d, frames, frame0 + 1, batched) / (float)frames;
            restore();
            if (rep == 0 || r < t) t = r;
        }
        if (best < 0 || t < best_t) { best = i; best_t = t; }
    }
    set_cfg(d, best);
    {
        std::lock_guard<std::mutex> lk(mu);
        cache[key] = {best, best_t};
    }
    if (best_ms) *best_ms = best_t;
    return best;
}
}  // namespace cellsim
