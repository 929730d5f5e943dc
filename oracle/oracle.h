/*
 * oracle.h — CPU restatements of the RDME timestep, used ONLY as test
 * infrastructure (the checker).  Nothing in the product library links,
 * loads or calls this code; only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py do.
 *
 * Parity status: parity unpinned.  The reference (javirk/cell_simulation)
 * ships no tests, no golden vectors and no CPU path, and its WGSL shaders
 * cannot run in this environment (no Vulkan, no Rust toolchain), so the
 * reference-semantics restatement below follows the shader source as read
 * (res/shader/rdme.wgsl, cme.wgsl, final_stage.wgsl, random.wgsl,
 * functions.wgsl) without outputs of the reference to check it against.  Its
 * own outputs on fixed cases are stored in tests/golden/ (make_golden.py)
 * and guard it against regressions.
 *
 * Three models live here:
 *   1. ref_semantics.c  — the reference algorithm (res/shader/rdme.wgsl,
 *      cme.wgsl, final_stage.wgsl, random.wgsl) in a canonical serial order,
 *      plus a gather formulation (OpenMP) that must agree with it.
 *   2. prod_semantics.c — a plain per-sweep restatement of this project's
 *      Philox production step (x/y/z sweeps + SSA within tau).
 *   3. ssa_fp64.c       — a well-mixed exact Gillespie direct method in FP64.
 */
#ifndef CELLSIM_ORACLE_H
#define CELLSIM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Mirrors LatticeParams (res/shader/functions.wgsl:16-23,
 * src/lattice_params.rs:15-25) and ReactionParams (functions.wgsl:25-28). */
typedef struct {
    uint32_t res[3];       /* X, Y, Z lattice resolution                    */
    uint32_t K;            /* max_particles_site, 1..16                     */
    uint32_t n_regions;    /* NReg                                          */
    uint32_t n_species;    /* S, excluding void species 0                   */
    uint32_t n_reactions;  /* R, excluding dummy row 0                      */
    float tau;
    float lambda;
} orc_params;

/* Reference table layout (logical C order, as the shaders index it). */
typedef struct {
    const uint32_t* regions;    /* [V] region id per voxel                       */
    const float* diffusion;     /* [NReg][NReg][S+1], [src][dst][species]        */
    const int32_t* stoich;      /* [R+1][S+1], row 0 = dummy                     */
    const uint32_t* reactants;  /* [R+1][3], padded with 0 (void)                */
    const float* rates;         /* [R+1]                                         */
    const uint32_t* reservoir;  /* [V] reservoir species per voxel (0 = none)    */
} orc_tables;

/* Diagnostic counters shared by the oracle and the CUDA parity path. */
enum {
    ORC_DIAG_SPILL = 0,      /* move into a voxel with occupancy >= K or no free slot (rejected) */
    ORC_DIAG_OCC_RANGE = 1,  /* voxel occupancy > K seen by the diffusion scan (clamped to K)    */
    ORC_DIAG_SLOW_STEPS = 2, /* steps resolved by the serial path (capacity contention)          */
    ORC_DIAG_ROLLBACKS = 3,  /* reaction rolled back because the voxel rewrite reached K slots   */
    ORC_DIAG_FIRED = 4,      /* voxels whose one-event test passed                               */
    ORC_DIAG_N = 8
};

/* ---- portable math / RNG (restated independently of the library) ---- */
uint32_t orc_pcg(uint32_t s);
uint32_t orc_xorshift(uint32_t s);
float orc_uniform_float(uint32_t s);
float orc_expf(float x);
float orc_logf(float x);
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* ---- 1. reference semantics ---- */
/* Runs n_steps timesteps in place.  itimes[n_steps] are the per-frame uniform
 * itime values (the reference's only RNG seed, src/uniforms.rs:24).
 * mode 0 = canonical serial order; mode 1 = gather formulation with
 * `threads` OpenMP threads (falls back to serial for a step whose capacity
 * check fails).  Returns 0 on success, <0 on bad arguments. */
int orc_ref_run(const orc_params* p, const orc_tables* t,
                uint32_t* slots, uint32_t* occ, int32_t* conc, int32_t* stat,
                uint32_t n_steps, const uint32_t* itimes, uint32_t* diag,
                int mode, int threads);

/* ---- 2. production (Philox) semantics ---- */
/* Plain full-lattice restatement of the production step (three sweeps, SSA
 * within tau) that the fused tile kernel must reproduce bit for bit.  Tables
 * are the reference layout (orc_tables); slots are K bytes per voxel,
 * compacted.  counts[S+1] is updated by the reaction deltas. */
typedef struct {
    uint32_t res[3];
    uint32_t K;            /* 8 or 16 */
    uint32_t n_regions;
    uint32_t n_species;    /* S */
    uint32_t n_reactions;  /* R */
    uint32_t precision;    /* 0 = mixed, 1 = FP32, 2 = FP64 selection always */
    uint32_t max_events;   /* per voxel per frame */
    float tau;
    float lambda;
    float rate_mult;
    uint64_t seed;
} orc_prod_params;

enum { ORC_PD_EVENTS = 0, ORC_PD_REJECT_CAP = 1, ORC_PD_EVENT_CAP = 2, ORC_PD_FP64_SEL = 3, ORC_PD_N = 8 };

int orc_prod_run(const orc_prod_params* p, const orc_tables* t, uint8_t* slots, int64_t* counts,
                 uint32_t frame0, uint32_t n_steps, uint32_t* diag);

/* Draws m in [lo, hi] (u1 = m 2^-24) with -logf(u1)/a0 <= tau. */
uint32_t orc_first_event_inside(float a0, float tau, uint32_t lo, uint32_t hi);

/* ---- 3. well-mixed FP64 SSA ---- */
/* Gillespie direct method.  reactants [R][3] (0 = void), ch_* as above,
 * rates [R] in well-mixed units (events per second per reactant tuple).
 * x[S+1] initial counts (x[0] ignored); samples written at times
 * t_samples[n_samples] into out[n_samples][S+1].  Propensity uses falling
 * factorials.  Returns number of events. */
int64_t orc_ssa_fp64(uint32_t S, uint32_t R, const uint8_t* reactants, const double* rates,
                     const uint8_t* ch_species, const int8_t* ch_delta,
                     const int64_t* x0, uint64_t seed, uint32_t n_samples,
                     const double* t_samples, int64_t* out);

#ifdef __cplusplus
}
#endif
#endif
