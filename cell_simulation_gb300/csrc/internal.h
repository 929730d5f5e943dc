// internal.h — host-side model and device state of libcellsim.
#pragma once
#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/cellsim.h"

namespace cellsim {

// Error carrying a cs_status across the C++ layer; converted at the ABI.
struct Error : std::runtime_error {
    cs_status code;
    Error(cs_status c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// Deterministic host RNG replacing rand::thread_rng for particle placement
// (xoshiro256** seeded through SplitMix64).
struct HostRng {
    uint64_t s[4];
    void seed(uint64_t v);
    uint64_t next();
    uint64_t below(uint64_t n);  // uniform in [0, n), n > 0
    float unit_f32();            // uniform in [0, 1)
};

struct RegionEntry {
    int32_t type;  // cs_region_type of the primitive stored (Cube/Sphere/SemiSphere/Cylinder)
    std::string name;
    float p0[3], pf[3], center[3], direction[3], radius;
};

// Host model: the state Simulation + Lattice + Regions keep on the CPU before
// prepare_for_gpu (src/simulation.rs:29-46, src/lattice.rs:14-23,
// src/region.rs:87-92).
struct Model {
    float dims[3] = {0, 0, 0};
    uint32_t res[3] = {0, 0, 0};
    float tau = 0, lambda = 0;
    uint32_t K = 8;
    uint64_t V = 0;

    // Regions
    std::vector<uint32_t> regions;  // [V]
    std::vector<RegionEntry> types;
    std::vector<uint32_t> volumes;
    std::map<uint32_t, std::vector<uint32_t>> index_buffer;
    bool regions_prepared = false;

    // diffusion_matrix [NR][NR][NP], NP = particle_names.size()
    std::vector<float> diffusion;
    uint32_t nr = 1, np = 1;

    std::vector<std::string> particle_names;  // [0] = "void"
    std::vector<uint32_t> logging;

    // stoichiometry [(R+1)][(S+1)], reactants [(R+1)][3], rates [R+1]
    std::vector<int32_t> stoich;
    std::vector<uint32_t> reactants;
    std::vector<float> rates;
    uint32_t n_species = 0, n_reactions = 0;

    // lattices[0] host state
    std::vector<uint32_t> slots;      // [V*K]
    std::vector<uint32_t> occupancy;  // [V]
    std::vector<int32_t> conc;        // [V*(S+1)], only when conc_explicit
    bool conc_explicit = false;       // set by cs_set_lattice with concentrations; otherwise derived
    std::vector<uint32_t> reservoir;  // [V]

    HostRng rng;

    void init(const cs_lattice_params& p);
    uint32_t S1() const { return n_species + 1; }
    float voxel_size(int a) const { return dims[a] / (float)res[a]; }
    float& D(uint32_t a, uint32_t b, uint32_t q) { return diffusion[((size_t)a * nr + b) * np + q]; }

    // Per-voxel concentrations: the explicit array, or counts of the slots
    // plus 1 for a voxel's reservoir species (src/lattice.rs:280-300).
    std::vector<int32_t> concentrations() const;
    int find_region(const std::string& name) const;
    int find_particle(const std::string& name) const;  // searches names[1..]
    void check_tables() const;

    // builders (src/simulation.rs)
    void add_region(const cs_region_desc& d, float diffusion_rate);
    void prepare_regions();
    void add_particle_count(const std::string& name, const std::string& to_region, uint32_t count, bool logging, bool reservoir);
    void add_particle_concentration(const std::string& name, const std::string& to_region, float concentration, bool logging, bool reservoir);
    void fill_region(const std::string& name, const std::string& to_region, bool logging);
    void set_diffusion_rate(const std::string& region, float rate);
    void set_diffusion_rate_particle(const std::string& particle, const std::string& region, float rate);
    void set_transition_rate(const std::string& from, const std::string& to, float rate);
    void set_transition_rate_particle(const std::string& particle, const std::string& from, const std::string& to, float rate);
    void add_reaction(const std::vector<std::string>& reactants, const std::vector<std::string>& products, float k);
    void load_json(const std::string& text);

private:
    void update_matrices_region(float diffusion_rate, float transition_rate);
    void add_region_cube(const std::string& name, const float p0[3], const float pf[3], float dr, float tr);
    void add_region_sphere(const std::string& name, const float c[3], float radius, float dr, float tr);
    void add_region_semisphere(const std::string& name, const float c[3], float radius, const float dir[3], float dr, float tr);
    void add_region_cylinder(const std::string& name, const float p0[3], const float pf[3], float radius, float dr, float tr);
    void join_regions(const std::string& del, const std::string& to);
    void check_collision(uint64_t v);
    void add_species_column();
    bool add_particle_site(uint64_t v, uint32_t particle);
    bool add_reservoir_site(uint64_t v, uint32_t particle);
};

struct DeviceRef;   // CS_RNG_REFERENCE device state (device_ref.cu)
struct DeviceProd;  // CS_RNG_PHILOX device state (device_prod.cu)

}  // namespace cellsim

struct cs_ensemble {
    std::unique_ptr<cellsim::DeviceProd, void (*)(cellsim::DeviceProd*)> prod{nullptr, nullptr};
    uint64_t frame = 0;
    uint32_t n_rep = 0, S1 = 1, K = 8;
    std::vector<uint32_t> res;
};

struct cs_sim {
    cellsim::Model model;
    int32_t mode = -1;
    int32_t device = 0;
    int32_t precision = CS_PREC_MIXED;
    uint64_t frame = 0;
    std::vector<cs_stat_sample> samples;
    std::unique_ptr<cellsim::DeviceRef, void (*)(cellsim::DeviceRef*)> ref{nullptr, nullptr};
    std::unique_ptr<cellsim::DeviceProd, void (*)(cellsim::DeviceProd*)> prod{nullptr, nullptr};
};

namespace cellsim {
// device_ref.cu
DeviceRef* ref_create(const Model& m, int device);
void ref_destroy(DeviceRef* d);
void ref_step(DeviceRef* d, uint32_t n_steps, const uint32_t* itimes, uint64_t frame0, uint32_t write_freq,
              const std::vector<uint32_t>& logging, std::vector<cs_stat_sample>& samples);
void ref_get_counts(DeviceRef* d, int64_t* counts);
void ref_get_lattice(DeviceRef* d, uint32_t* slots, uint32_t* occ, int32_t* conc);
void ref_set_lattice(DeviceRef* d, const uint32_t* slots, const uint32_t* occ, const int32_t* conc);
void ref_get_diag(DeviceRef* d, uint32_t* diag, uint32_t n);
void ref_sync(DeviceRef* d);
void ref_set_counts(DeviceRef* d, const int64_t* counts);
void ref_render_view(DeviceRef* d, int32_t view, int32_t slice_axis, uint32_t slice, float* out_host, void* out_device);

// device_prod.cu
DeviceProd* prod_create(const Model& m, int device);
void prod_destroy(DeviceProd* d);
void prod_step(DeviceProd* d, uint32_t n_steps, uint64_t seed, int precision, uint64_t frame0, uint32_t write_freq,
               const std::vector<uint32_t>& logging, std::vector<cs_stat_sample>& samples);
void prod_get_counts(DeviceProd* d, int64_t* counts);
void prod_get_lattice(DeviceProd* d, const Model& m, uint32_t* slots, uint32_t* occ, int32_t* conc);
void prod_set_lattice(DeviceProd* d, const Model& m, const uint32_t* slots);
void prod_get_diag(DeviceProd* d, uint32_t* diag, uint32_t n);
void prod_sync(DeviceProd* d);
void prod_debug_stall_group(DeviceProd* d, uint32_t group);

DeviceProd* prod_ensemble_create(const Model& m, uint32_t n, const uint32_t* res, const uint64_t* seeds, const float* mult,
                                 const uint32_t* init_counts, int device);
void prod_ensemble_step(DeviceProd* d, uint32_t n_steps, bool batched, uint64_t frame0);
void prod_set_precision(DeviceProd* d, int precision);
uint64_t prod_total_voxels(const DeviceProd* d);
uint32_t prod_n_items(const DeviceProd* d);
uint32_t prod_n_replicates(const DeviceProd* d);
uint32_t prod_s1(const DeviceProd* d);
void prod_get_slots_raw(DeviceProd* d, uint8_t* out);
void prod_set_tiling(DeviceProd* d, int cfg_index, uint32_t seg_len);
int prod_tiling_count();
void prod_tiling_desc(int i, int* K, int* TY, int* TZ, int* NT);
void prod_tiling_kind(int i, int* kind, int* BX);
int prod_tiling_launches(int i);
void prod_set_counts(DeviceProd* d, const int64_t* counts);
// out_device (V floats, caller-owned device memory) or, when null, out_host
void prod_render_view(DeviceProd* d, int32_t view, int32_t slice_axis, uint32_t slice, float* out_host, void* out_device);
int prod_tiling_current(const DeviceProd* d);
void prod_seed(DeviceProd* d, uint64_t seed);
float prod_time_frames(DeviceProd* d, uint32_t n, uint64_t frame0, bool batched);
int prod_autotune(DeviceProd* d, uint32_t frames, uint64_t frame0, bool batched, float* best_ms);
float ref_time_frames(DeviceRef* d, uint32_t n, const uint32_t* itimes, uint64_t frame0);
void ref_frame_noalloc(const cs_ref_frame_noalloc_args* a);

// model.cpp helpers shared with the device files
void compute_ref_probabilities(const Model& m, std::vector<float>& P);
}  // namespace cellsim
