/*
 * cellsim.h — C ABI of libcellsim, the GB300 (sm_103a) implementation of the
 * RDME timestep of javirk/cell_simulation: lattice diffusion, per-voxel
 * reactions, slot compaction and species counts.
 *
 * This header is the drop-in boundary for the reference's wgpu compute path.
 * Every entry point names the reference interface it replaces (paths are
 * relative to the reference project).  Conventions:
 *   - every call returns cs_status (0 = CS_OK); cs_last_error() returns a
 *     thread-local message for the last failing call on this thread;
 *   - no exception, panic or abort crosses the ABI;
 *   - all arrays are caller-allocated host memory in the reference layout
 *     (logical C order, voxel index v = (x*Y + y)*Z + z, slot s at v*K + s);
 *     device memory is owned by the library;
 *   - a cs_sim handle owns one CUDA stream on one device and is not
 *     thread-safe (the reference's Simulation is used through &mut self);
 *   - there is no CPU fallback: device calls fail with CS_ERR_CUDA when no
 *     usable GPU is present.
 */
#ifndef CELLSIM_H
#define CELLSIM_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CELLSIM_ABI_VERSION 1

typedef int32_t cs_status;
enum {
    CS_OK = 0,
    CS_ERR_INVALID_ARG = 1,  /* null pointer, bad size, bad enum            */
    CS_ERR_NOT_FOUND = 2,    /* unknown region or species name              */
    CS_ERR_LIMIT = 3,        /* K, species, regions or reactions too large  */
    CS_ERR_STATE = 4,        /* call out of order (e.g. step before prepare)*/
    CS_ERR_PARSE = 5,        /* malformed JSON model                        */
    CS_ERR_IO = 6,           /* file could not be read                      */
    CS_ERR_CUDA = 7,         /* CUDA runtime error or no device             */
    CS_ERR_CAPACITY = 8,     /* host placement could not fit a particle     */
    CS_ERR_DEVICE_STATUS = 9 /* a kernel reported a failure status          */
};

typedef struct cs_sim cs_sim;
typedef struct cs_ensemble cs_ensemble;

/* LatticeParams::new(dimensions, resolution, tau, lambda),
 * src/lattice_params.rs:97-118; max_particles_site is the reference's
 * compile-time MAX_PARTICLES_SITE (src/lib.rs:15), a run-time value here
 * (1..16; the production path takes 8 or 16). */
typedef struct {
    float dims[3];
    uint32_t res[3];
    float tau;
    float lambda;
    uint32_t max_particles_site;
} cs_lattice_params;

/* RegionType, src/region.rs:10-20. */
typedef enum {
    CS_REGION_CUBE = 0,
    CS_REGION_SPHERE = 1,
    CS_REGION_SEMISPHERE = 2,
    CS_REGION_CYLINDER = 3,
    CS_REGION_SPHERICAL_SHELL = 4,
    CS_REGION_CYLINDRICAL_SHELL = 5,
    CS_REGION_CAPSID = 6
} cs_region_type;

/* Payload of a RegionType variant; fields a variant does not use are ignored. */
typedef struct {
    int32_t type;               /* cs_region_type                                   */
    const char* name;           /* Cube, Sphere, SemiSphere, Cylinder               */
    const char* shell_name;     /* SphericalShell, CylindricalShell, Capsid         */
    const char* interior_name;  /* SphericalShell, CylindricalShell, Capsid         */
    float p0[3], pf[3];         /* Cube, Cylinder, CylindricalShell                 */
    float center[3];            /* Sphere, SemiSphere, SphericalShell, Capsid       */
    float direction[3];         /* SemiSphere `direction`, Capsid `dir`             */
    float radius;               /* Sphere, SemiSphere, Cylinder                     */
    float internal_radius;      /* shells, Capsid                                   */
    float external_radius;      /* shells, Capsid                                   */
    float total_length;         /* Capsid                                           */
} cs_region_desc;

typedef enum {
    CS_RNG_REFERENCE = 0, /* the reference's PCG/xorshift stream keyed by itime; bit-exact */
    CS_RNG_PHILOX = 1     /* production path: Philox4x32-10, x/y/z sweeps, SSA within tau */
} cs_rng_mode;

typedef enum {
    CS_PREC_MIXED = 0, /* FP32 propensities/waiting times, FP64 clock, FP64 selection past 6 decades */
    CS_PREC_FP32 = 1,  /* everything FP32 (precision comparisons)                                  */
    CS_PREC_FP64 = 2   /* FP32 propensities, FP64 clock and FP64 selection always                  */
} cs_precision;

typedef struct {
    uint32_t res[3];
    uint32_t max_particles_site;
    uint32_t n_regions;
    uint32_t n_species;    /* S, excluding the void species 0 */
    uint32_t n_reactions;  /* R, excluding the dummy row 0    */
    uint32_t n_logging;
    uint64_t n_voxels;
    uint64_t frame;        /* frames stepped since prepare     */
    float tau;
    float lambda;
    float dims[3];
    int32_t rng_mode;      /* -1 before cs_prepare_for_gpu     */
    int32_t device;
} cs_info;

/* SolverStatisticSample<i32>, src/statistics.rs:4-9 (name -> species index). */
typedef struct {
    uint32_t species;
    int32_t value;
    uint32_t iteration_count;
} cs_stat_sample;

/* ---------------- lifecycle ---------------- */
const char* cs_version(void);
const char* cs_last_error(void);
/* Simulation::new, src/simulation.rs:51-97 */
cs_status cs_create(const cs_lattice_params* params, cs_sim** out);
/* Simulation::from_file, src/simulation.rs:210-232 (model part; no texture) */
cs_status cs_from_json_file(const char* path, uint64_t placement_seed, cs_sim** out);
cs_status cs_from_json_string(const char* json, uint64_t placement_seed, cs_sim** out);
void cs_destroy(cs_sim* sim);
/* Seeds the host placement RNG that replaces rand::thread_rng
 * (src/lattice.rs:65) so that models are reproducible. */
cs_status cs_seed_placement(cs_sim* sim, uint64_t seed);

/* ---------------- model building (host) ---------------- */
/* Simulation::add_region, src/simulation.rs:428-481 */
cs_status cs_add_region(cs_sim* sim, const cs_region_desc* region, float diffusion_rate);
/* Simulation::prepare_regions, src/simulation.rs:424-426 -> Regions::prepare_regions, src/region.rs:129-148 */
cs_status cs_prepare_regions(cs_sim* sim);
/* Simulation::add_particle_count, src/simulation.rs:792-814 */
cs_status cs_add_particle_count(cs_sim* sim, const char* name, const char* to_region, uint32_t count,
                                int32_t logging, int32_t is_reservoir);
/* Simulation::add_particle_concentration, src/simulation.rs:816-823 */
cs_status cs_add_particle_concentration(cs_sim* sim, const char* name, const char* to_region,
                                        float concentration, int32_t logging, int32_t is_reservoir);
/* Simulation::fill_region, src/simulation.rs:825-840 */
cs_status cs_fill_region(cs_sim* sim, const char* name, const char* to_region, int32_t logging);
/* Simulation::set_diffusion_rate, src/simulation.rs:867-874 */
cs_status cs_set_diffusion_rate(cs_sim* sim, const char* region, float rate);
/* Simulation::set_diffusion_rate_particle, src/simulation.rs:877-882 */
cs_status cs_set_diffusion_rate_particle(cs_sim* sim, const char* particle, const char* region, float rate);
/* Simulation::set_transition_rate, src/simulation.rs:885-893 */
cs_status cs_set_transition_rate(cs_sim* sim, const char* from_region, const char* to_region, float rate);
/* Simulation::set_transition_rate_particle, src/simulation.rs:896-902 */
cs_status cs_set_transition_rate_particle(cs_sim* sim, const char* particle, const char* from_region,
                                          const char* to_region, float rate);
/* Simulation::add_reaction, src/simulation.rs:904-947 */
cs_status cs_add_reaction(cs_sim* sim, const char* const* reactants, uint32_t n_reactants,
                          const char* const* products, uint32_t n_products, float k);

/* ---------------- introspection ---------------- */
cs_status cs_get_info(const cs_sim* sim, cs_info* out);
/* Copies the tables the shaders bind (src/simulation.rs:1156-1254); every
 * pointer may be NULL.  Sizes: regions[V], diffusion[NReg*NReg*(S+1)],
 * stoich[(R+1)*(S+1)], reactants[(R+1)*3], rates[R+1], reservoir[V]. */
cs_status cs_get_tables(const cs_sim* sim, uint32_t* regions, float* diffusion, int32_t* stoich,
                        uint32_t* reactants, float* rates, uint32_t* reservoir);
/* Regions::volumes, src/region.rs:90 (NReg entries). */
cs_status cs_get_region_volumes(const cs_sim* sim, uint32_t* volumes);
/* kind 0 = species name (index 0 = "void"), 1 = region name, 2 = logged species index */
cs_status cs_get_name(const cs_sim* sim, int32_t kind, uint32_t index, char* buf, uint32_t buf_len);

/* ---------------- reference-layout state (drop-in buffers) ---------------- */
/* Replaces all tables with prebuilt reference-layout arrays (the buffers
 * created in Simulation::prepare_for_gpu, src/simulation.rs:152-208).
 * Invalidates device state. */
cs_status cs_set_tables(cs_sim* sim, uint32_t n_regions, uint32_t n_species, uint32_t n_reactions,
                        const uint32_t* regions, const float* diffusion, const int32_t* stoich,
                        const uint32_t* reactants, const float* rates, const uint32_t* reservoir);
/* Lattice state: slots u32[V*K] (Lattice::lattice, src/lattice.rs:15),
 * occupancy u32[V] and concentrations i32[V*(S+1)].  occupancy and
 * concentrations may be NULL in cs_set_lattice, in which case they are
 * derived from the slots (plus 1 for each reservoir species).  After
 * cs_prepare_for_gpu the state lives on the device and these calls copy to
 * or from it. */
cs_status cs_set_lattice(cs_sim* sim, const uint32_t* slots, const uint32_t* occupancy,
                         const int32_t* concentrations);
cs_status cs_get_lattice(cs_sim* sim, uint32_t* slots, uint32_t* occupancy, int32_t* concentrations);

/* ---------------- device ---------------- */
/* Simulation::prepare_for_gpu, src/simulation.rs:152-208: allocates device
 * buffers on `device`, uploads the model and initialises the species counts
 * from the concentrations (create_statistics, src/simulation.rs:361-388). */
cs_status cs_prepare_for_gpu(cs_sim* sim, int32_t rng_mode, int32_t device);
/* Simulation::step, src/simulation.rs:99-150, driving RDME::step
 * (src/rdme.rs:46-76) and CME::step (src/cme.rs:47-79) for n_steps frames
 * in CS_RNG_REFERENCE mode.  itimes[n_steps] are the per-frame Uniform.itime
 * values (src/uniforms.rs:8-14).  Before frame f with f > 0 and
 * f % write_freq == 0 the logged species counts are sampled
 * (start_error_buffer_readbacks, src/simulation.rs:391-418); write_freq 0
 * disables sampling.  Returns after the work is enqueued. */
cs_status cs_step(cs_sim* sim, uint32_t n_steps, const uint32_t* itimes, uint32_t write_freq);
/* Production path (CS_RNG_PHILOX): n_steps frames keyed by `seed`. */
cs_status cs_step_philox(cs_sim* sim, uint32_t n_steps, uint64_t seed, uint32_t write_freq);
/* Precision form of the production path (cs_precision). */
cs_status cs_set_precision(cs_sim* sim, int32_t precision);
/* Global species counts, StatisticsGroup buffer 0 (src/statistics.rs:11-69):
 * counts[S+1]; synchronises the stream. */
cs_status cs_get_counts(cs_sim* sim, int64_t* counts);
/* Drains the recorded samples (Simulation::stats, src/simulation.rs:36). */
cs_status cs_pop_stats(cs_sim* sim, cs_stat_sample* out, uint32_t capacity, uint32_t* n_out);
/* Diagnostic counters, diag[n].  Reference-RNG path: [0] moves rejected for
 * capacity, [1] voxels whose occupancy exceeded K, [2] frames resolved in
 * serial order, [3] reaction rollbacks, [4] voxels that fired.  Production
 * path: [0] reaction events, [1] events rejected for capacity, [2] voxels that
 * hit the event cap, [3] FP64 selections, [4] bricks spilled to the second
 * brick pass, [5] bricks lost (always 0), [6] voxels that ran the SSA, [7]
 * waits of the multi-frame sweep kernel that timed out (always 0; nonzero
 * means its frames were abandoned and the lattice is not valid: cs_get_counts
 * and cs_synchronize then fail with CS_ERR_CUDA). */
cs_status cs_get_diagnostics(cs_sim* sim, uint32_t* diag, uint32_t n);
/* Waits for the handle's work.  Fails with CS_ERR_CUDA (as cs_get_counts does)
 * when the multi-frame sweep kernel abandoned frames after a dependency wait
 * timed out; the lattice is then not valid (upload a new one). */
cs_status cs_synchronize(cs_sim* sim);
/* Test hook of the multi-frame sweep kernel's bounded waits: the next
 * multi-frame launch makes word group `group` (in the current group order)
 * also wait on a completion value that nothing writes, so that its waits run
 * out, the launch abandons its frames and the host reports the error.  No
 * reference counterpart. */
cs_status cs_debug_stall_group(cs_sim* sim, uint32_t group);

/* ---------------- allocation-free reference-RNG frame ---------------- */
/* Arguments of cs_ref_frame_noalloc.  Every pointer is a device pointer on
 * `device`, owned by the caller, in the library's device layout:
 *   slots u8[V*K], occupancy u32[V], conc i32[V*(S+1)] (input frame and output
 *   frame, distinct buffers); regions and reservoir u8[V]; probabilities
 *   f32[NR][NR][S+1] holding (D[a][b][q] * tau) / (lambda * lambda) in
 *   binary32; stoich i32[(R+1)*(S+1)]; reactants u32[(R+1)*3]; rates f32[R+1];
 *   itime u32[1], this frame's seed; counts i32[S+1] and diag u32[8], updated
 *   in place. */
typedef struct {
    int32_t device;
    void* stream;  /* cudaStream_t; NULL = the legacy default stream */
    uint32_t res[3];
    uint32_t max_particles_site;
    uint32_t n_regions, n_species, n_reactions;
    float tau;
    const uint8_t* slots_in;
    const uint32_t* occupancy_in;
    const int32_t* conc_in;
    uint8_t* slots_out;
    uint32_t* occupancy_out;
    int32_t* conc_out;
    const uint8_t* regions;
    const uint8_t* reservoir;
    const float* probabilities;
    const int32_t* stoich;
    const uint32_t* reactants;
    const float* rates;
    const uint32_t* itime;
    int32_t* counts;
    uint32_t* diag;
} cs_ref_frame_noalloc_args;

/* No counterpart in the reference.  One reference-RNG frame (the same
 * kernels as cs_step) on caller-owned device buffers, for callers that must
 * not allocate device memory: hosts that manage every device byte through
 * their own arena and forbid cudaMalloc at run time, or loops that cannot
 * absorb an allocation's device synchronisation.  It calls no cudaMalloc,
 * cudaFree or allocating library routine.  Its only scratch is a fixed
 * 16 MiB + 256 B device array inside the library, held on every GPU where the
 * library is loaded until the process exits; lattices with V*K above
 * 16777216 slots are rejected with CS_ERR_LIMIT.  The first call on a device
 * looks up that array's address (make this first call before any stream
 * capture).  All calls share the array, so calls that overlap on the GPU
 * (different streams, or different host threads on the same device) race;
 * each call rewrites the scratch it reads, so back-to-back calls are safe.
 * Work is enqueued on `stream` and the call returns without waiting. */
cs_status cs_ref_frame_noalloc(const cs_ref_frame_noalloc_args* args);

/* ---------------- timing and tiling (production path) ---------------- */
/* Enqueue n frames between two CUDA events recorded on the handle's stream
 * and return the device time in milliseconds (blocks until done).  No
 * reference counterpart (the reference only prints FPS,
 * examples/no_window.rs:141-163). */
cs_status cs_step_timed(cs_sim* sim, uint32_t n_steps, const uint32_t* itimes, float* ms);
cs_status cs_step_philox_timed(cs_sim* sim, uint32_t n_steps, uint64_t seed, float* ms);
/* Compiled (K, TY, TZ, threads) variants of the step and the x-segment
 * length of a work item (0 = automatic; tile pipeline only); used by the
 * autotuner.  cs_tiling_kind: kind 0 = tile pipeline over (TY x TZ tile,
 * x-segment) items; kind 1 = sparse brick pass over brick_planes x TY x TZ
 * bricks, crowded bricks finished by a full-capacity second brick pass;
 * kind 2 = sweep stream (the default): barrier-free passes over groups of 32
 * occupancy-bitmap words (TZ = 32, brick_planes = 0; TY = 1 marks the
 * persistent form that runs every frame of a step call in one launch, TY = 0
 * the per-pass launches); kind 3 = resident form: one block of `threads`
 * per replicate holds its lattice in shared memory for every frame of a step
 * call (TY = TZ = 0; about 5,300 voxels per replicate at K = 16 and 9,000 at
 * K = 8 at most: cs_set_tiling refuses larger lattices).  Every variant
 * computes the same lattice.  cs_tiling_launches: kernel launches per frame
 * once a run is under way (the sweep stream: 3, or 2 where the Y and Z sweeps
 * are one launch, or 1 per step call in the persistent form; the last two need
 * Z <= 1024 and cs_set_tiling refuses them otherwise; the resident form: 1
 * per step call).  No reference counterpart (the reference has one
 * fixed dispatch shape per shader). */
cs_status cs_tiling_count(int32_t* n);
cs_status cs_tiling_describe(int32_t index, int32_t* K, int32_t* TY, int32_t* TZ, int32_t* threads);
cs_status cs_tiling_kind(int32_t index, int32_t* kind, int32_t* brick_planes);
cs_status cs_tiling_launches(int32_t index, int32_t* launches);
cs_status cs_set_tiling(cs_sim* sim, int32_t index, uint32_t segment_length);
cs_status cs_get_tiling(const cs_sim* sim, int32_t* index);
/* Autotuner: times every compiled variant for this K on the handle's own
 * lattice (frames_per_trial frames each, from a device copy of the current
 * state, which is restored afterwards, so the simulation does not advance),
 * selects the fastest and caches the choice per model shape and device for
 * the life of the process.  chosen_index / ms_per_frame may be NULL. */
cs_status cs_autotune(cs_sim* sim, uint32_t frames_per_trial, int32_t* chosen_index, float* ms_per_frame);

/* ---------------- checkpoint / resume ---------------- */
/* Writes the full state of a handle to a file: lattice parameters, model
 * tables, names and regions, the placement RNG, the current lattice (slots,
 * occupancy, concentrations) and species counts, the frame number, the RNG
 * mode and the precision.  Resuming with cs_checkpoint_load and stepping
 * continues bit for bit as the saved handle would (the Philox seed is passed
 * to cs_step_philox as before).  No reference counterpart (the reference keeps
 * its state only in wgpu buffers, src/simulation.rs:29-46). */
cs_status cs_checkpoint_save(cs_sim* sim, const char* path);
/* Creates a handle from a checkpoint file; a handle saved after
 * cs_prepare_for_gpu is prepared again on `device`. */
cs_status cs_checkpoint_load(const char* path, int32_t device, cs_sim** out);

/* ---------------- headless visualisation ---------------- */
/* The views of final_stage.wgsl:35-68 (the storage texture of the reference's
 * renderer) as V floats in lattice order: view 0 = majority species / 255,
 * 1 = region id / 255, 2 = reservoir species / 255; voxels with
 * res[slice_axis] - coord[slice_axis] < slice are 0.  Written to out_device
 * (caller-owned device memory, V floats) when it is not NULL, else copied to
 * out_host.  Needs cs_prepare_for_gpu. */
cs_status cs_render_view(cs_sim* sim, int32_t view, int32_t slice_axis, uint32_t slice, float* out_host, void* out_device);

/* ---------------- batched ensemble (production path) ---------------- */
/* Replicates of one model on lattices of uneven sizes, all stepped by one
 * persistent launch per frame over a (replicate, tile) work queue.  The
 * model's species, reactions and region-0 diffusion rates are shared; each
 * replicate is one region-0 lattice of resolution res[3r..3r+2] with its own
 * Philox seed and reaction-rate multiplier, filled uniformly with
 * initial_counts[s] particles of species s (initial_counts[S+1]).  No
 * reference counterpart: the reference runs one Simulation per lattice. */
cs_status cs_ensemble_create(const cs_sim* model, uint32_t n_replicates, const uint32_t* res, const uint64_t* seeds,
                             const float* rate_multipliers, const uint32_t* initial_counts, int32_t device,
                             cs_ensemble** out);
void cs_ensemble_destroy(cs_ensemble* ens);
/* batched != 0: one launch per frame for all replicates (CUDA-graph replayed);
 * batched == 0: one launch per replicate per frame (the plain path). */
cs_status cs_ensemble_step(cs_ensemble* ens, uint32_t n_steps, int32_t batched);
cs_status cs_ensemble_step_timed(cs_ensemble* ens, uint32_t n_steps, int32_t batched, float* ms);
cs_status cs_ensemble_set_precision(cs_ensemble* ens, int32_t precision);
cs_status cs_ensemble_set_tiling(cs_ensemble* ens, int32_t index, uint32_t segment_length);
cs_status cs_ensemble_autotune(cs_ensemble* ens, uint32_t frames_per_trial, int32_t* chosen_index, float* ms_per_frame);
/* counts[n_replicates][S+1] */
cs_status cs_ensemble_get_counts(cs_ensemble* ens, int64_t* counts);
/* packed slots of all replicates in order, K bytes per voxel */
cs_status cs_ensemble_get_slots(cs_ensemble* ens, uint8_t* slots);
cs_status cs_ensemble_get_diagnostics(cs_ensemble* ens, uint32_t* diag, uint32_t n);
cs_status cs_ensemble_synchronize(cs_ensemble* ens);
cs_status cs_ensemble_info(const cs_ensemble* ens, uint64_t* total_voxels, uint32_t* n_work_items);

#ifdef __cplusplus
}
#endif
#endif
