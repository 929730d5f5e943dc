// abi.cpp — extern "C" entry points of libcellsim (include/cellsim.h).
// Every function converts C++ exceptions into a cs_status and a thread-local
// message; nothing throws across the ABI.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <new>
#include <sstream>
#include <string>

#include "internal.h"

using namespace cellsim;

namespace {
thread_local std::string g_last_error;

template <typename F>
cs_status guarded(F&& f) {
    try {
        f();
        g_last_error.clear();
        return CS_OK;
    } catch (const Error& e) {
        g_last_error = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        g_last_error = "host out of memory";
        return CS_ERR_LIMIT;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return CS_ERR_INVALID_ARG;
    } catch (...) {
        g_last_error = "unknown error";
        return CS_ERR_INVALID_ARG;
    }
}

void need(const void* p, const char* what) {
    if (!p) throw Error(CS_ERR_INVALID_ARG, std::string(what) + " is NULL");
}
std::string str(const char* s, const char* what) {
    need(s, what);
    return std::string(s);
}
void invalidate_device(cs_sim* s) {
    s->ref.reset();
    s->prod.reset();
    s->mode = -1;
}
void require_host_model(cs_sim* s) {
    if (s->mode >= 0) throw Error(CS_ERR_STATE, "the model cannot change after prepare_for_gpu");
}
cs_sim* new_sim() {
    cs_sim* s = new cs_sim();
    s->ref = std::unique_ptr<DeviceRef, void (*)(DeviceRef*)>(nullptr, ref_destroy);
    s->prod = std::unique_ptr<DeviceProd, void (*)(DeviceProd*)>(nullptr, prod_destroy);
    return s;
}
}  // namespace

extern "C" {

const char* cs_version(void) { return "cellsim-gb300 1.0 (sm_103a)"; }

const char* cs_last_error(void) { return g_last_error.c_str(); }

cs_status cs_create(const cs_lattice_params* params, cs_sim** out) {
    return guarded([&] {
        need(params, "params");
        need(out, "out");
        *out = nullptr;
        std::unique_ptr<cs_sim> s(new_sim());
        s->model.init(*params);
        *out = s.release();
    });
}

static cs_status from_json_text(const std::string& text, uint64_t seed, cs_sim** out) {
    return guarded([&] {
        need(out, "out");
        *out = nullptr;
        std::unique_ptr<cs_sim> s(new_sim());
        s->model.rng.seed(seed);
        s->model.load_json(text);
        *out = s.release();
    });
}

cs_status cs_from_json_file(const char* path, uint64_t placement_seed, cs_sim** out) {
    std::string text;
    cs_status st = guarded([&] {
        need(path, "path");
        std::ifstream f(path, std::ios::binary);
        if (!f) throw Error(CS_ERR_IO, std::string("cannot open ") + path);
        std::stringstream ss;
        ss << f.rdbuf();
        text = ss.str();
    });
    if (st != CS_OK) return st;
    return from_json_text(text, placement_seed, out);
}

cs_status cs_from_json_string(const char* json, uint64_t placement_seed, cs_sim** out) {
    if (!json) {
        g_last_error = "json is NULL";
        return CS_ERR_INVALID_ARG;
    }
    return from_json_text(std::string(json), placement_seed, out);
}

void cs_destroy(cs_sim* sim) {
    if (!sim) return;
    try {
        delete sim;
    } catch (...) {
    }
}

cs_status cs_seed_placement(cs_sim* sim, uint64_t seed) {
    return guarded([&] {
        need(sim, "sim");
        sim->model.rng.seed(seed);
    });
}

cs_status cs_add_region(cs_sim* sim, const cs_region_desc* region, float diffusion_rate) {
    return guarded([&] {
        need(sim, "sim");
        need(region, "region");
        require_host_model(sim);
        sim->model.add_region(*region, diffusion_rate);
    });
}

cs_status cs_prepare_regions(cs_sim* sim) {
    return guarded([&] {
        need(sim, "sim");
        require_host_model(sim);
        sim->model.prepare_regions();
    });
}

cs_status cs_add_particle_count(cs_sim* sim, const char* name, const char* to_region, uint32_t count, int32_t logging,
                                int32_t is_reservoir) {
    return guarded([&] {
        need(sim, "sim");
        require_host_model(sim);
        sim->model.add_particle_count(str(name, "name"), str(to_region, "to_region"), count, logging != 0, is_reservoir != 0);
    });
}

cs_status cs_add_particle_concentration(cs_sim* sim, const char* name, const char* to_region, float concentration,
                                        int32_t logging, int32_t is_reservoir) {
    return guarded([&] {
        need(sim, "sim");
        require_host_model(sim);
        sim->model.add_particle_concentration(str(name, "name"), str(to_region, "to_region"), concentration, logging != 0,
                                              is_reservoir != 0);
    });
}

cs_status cs_fill_region(cs_sim* sim, const char* name, const char* to_region, int32_t logging) {
    return guarded([&] {
        need(sim, "sim");
        require_host_model(sim);
        sim->model.fill_region(str(name, "name"), str(to_region, "to_region"), logging != 0);
    });
}

cs_status cs_set_diffusion_rate(cs_sim* sim, const char* region, float rate) {
    return guarded([&] {
        need(sim, "sim");
        require_host_model(sim);
        sim->model.set_diffusion_rate(str(region, "region"), rate);
    });
}

cs_status cs_set_diffusion_rate_particle(cs_sim* sim, const char* particle, const char* region, float rate) {
    return guarded([&] {
        need(sim, "sim");
        require_host_model(sim);
        sim->model.set_diffusion_rate_particle(str(particle, "particle"), str(region, "region"), rate);
    });
}

cs_status cs_set_transition_rate(cs_sim* sim, const char* from_region, const char* to_region, float rate) {
    return guarded([&] {
        need(sim, "sim");
        require_host_model(sim);
        sim->model.set_transition_rate(str(from_region, "from_region"), str(to_region, "to_region"), rate);
    });
}

cs_status cs_set_transition_rate_particle(cs_sim* sim, const char* particle, const char* from_region,
                                          const char* to_region, float rate) {
    return guarded([&] {
        need(sim, "sim");
        require_host_model(sim);
        sim->model.set_transition_rate_particle(str(particle, "particle"), str(from_region, "from_region"),
                                                str(to_region, "to_region"), rate);
    });
}

cs_status cs_add_reaction(cs_sim* sim, const char* const* reactants, uint32_t n_reactants, const char* const* products,
                          uint32_t n_products, float k) {
    return guarded([&] {
        need(sim, "sim");
        require_host_model(sim);
        if (n_reactants) need(reactants, "reactants");
        if (n_products) need(products, "products");
        std::vector<std::string> re, pr;
        for (uint32_t i = 0; i < n_reactants; i++) re.push_back(str(reactants[i], "reactant"));
        for (uint32_t i = 0; i < n_products; i++) pr.push_back(str(products[i], "product"));
        sim->model.add_reaction(re, pr, k);
    });
}

cs_status cs_get_info(const cs_sim* sim, cs_info* out) {
    return guarded([&] {
        need(sim, "sim");
        need(out, "out");
        const Model& m = sim->model;
        std::memset(out, 0, sizeof(*out));
        for (int i = 0; i < 3; i++) { out->res[i] = m.res[i]; out->dims[i] = m.dims[i]; }
        out->max_particles_site = m.K;
        out->n_regions = (uint32_t)m.types.size();
        out->n_species = m.n_species;
        out->n_reactions = m.n_reactions;
        out->n_logging = (uint32_t)m.logging.size();
        out->n_voxels = m.V;
        out->frame = sim->frame;
        out->tau = m.tau;
        out->lambda = m.lambda;
        out->rng_mode = sim->mode;
        out->device = sim->device;
    });
}

cs_status cs_get_tables(const cs_sim* sim, uint32_t* regions, float* diffusion, int32_t* stoich, uint32_t* reactants,
                        float* rates, uint32_t* reservoir) {
    return guarded([&] {
        need(sim, "sim");
        const Model& m = sim->model;
        if (regions) std::memcpy(regions, m.regions.data(), m.V * sizeof(uint32_t));
        if (diffusion) std::memcpy(diffusion, m.diffusion.data(), m.diffusion.size() * sizeof(float));
        if (stoich) std::memcpy(stoich, m.stoich.data(), m.stoich.size() * sizeof(int32_t));
        if (reactants) std::memcpy(reactants, m.reactants.data(), m.reactants.size() * sizeof(uint32_t));
        if (rates) std::memcpy(rates, m.rates.data(), m.rates.size() * sizeof(float));
        if (reservoir) std::memcpy(reservoir, m.reservoir.data(), m.V * sizeof(uint32_t));
    });
}

cs_status cs_get_region_volumes(const cs_sim* sim, uint32_t* volumes) {
    return guarded([&] {
        need(sim, "sim");
        need(volumes, "volumes");
        std::memcpy(volumes, sim->model.volumes.data(), sim->model.volumes.size() * sizeof(uint32_t));
    });
}

cs_status cs_get_name(const cs_sim* sim, int32_t kind, uint32_t index, char* buf, uint32_t buf_len) {
    return guarded([&] {
        need(sim, "sim");
        need(buf, "buf");
        const Model& m = sim->model;
        std::string n;
        if (kind == 0) {
            if (index >= m.particle_names.size()) throw Error(CS_ERR_INVALID_ARG, "species index out of range");
            n = m.particle_names[index];
        } else if (kind == 1) {
            if (index >= m.types.size()) throw Error(CS_ERR_INVALID_ARG, "region index out of range");
            n = m.types[index].name;
        } else if (kind == 2) {
            if (index >= m.logging.size()) throw Error(CS_ERR_INVALID_ARG, "logging index out of range");
            n = std::to_string(m.logging[index]);
        } else {
            throw Error(CS_ERR_INVALID_ARG, "kind must be 0, 1 or 2");
        }
        if (buf_len < n.size() + 1) throw Error(CS_ERR_INVALID_ARG, "buffer too small");
        std::memcpy(buf, n.c_str(), n.size() + 1);
    });
}

cs_status cs_set_tables(cs_sim* sim, uint32_t n_regions, uint32_t n_species, uint32_t n_reactions, const uint32_t* regions,
                        const float* diffusion, const int32_t* stoich, const uint32_t* reactants, const float* rates,
                        const uint32_t* reservoir) {
    return guarded([&] {
        need(sim, "sim");
        need(regions, "regions");
        need(diffusion, "diffusion");
        need(stoich, "stoich");
        need(reactants, "reactants");
        need(rates, "rates");
        if (n_regions < 1 || n_regions > 255) throw Error(CS_ERR_LIMIT, "n_regions must be in 1..255");
        if (n_species > 255) throw Error(CS_ERR_LIMIT, "at most 255 species");
        if (n_reactions > 99) throw Error(CS_ERR_LIMIT, "at most 99 reactions");
        Model& m = sim->model;
        invalidate_device(sim);
        uint32_t s1 = n_species + 1;
        m.nr = n_regions;
        m.np = s1;
        m.regions.assign(regions, regions + m.V);
        m.diffusion.assign(diffusion, diffusion + (size_t)n_regions * n_regions * s1);
        m.stoich.assign(stoich, stoich + (size_t)(n_reactions + 1) * s1);
        m.reactants.assign(reactants, reactants + (size_t)(n_reactions + 1) * 3);
        m.rates.assign(rates, rates + n_reactions + 1);
        if (reservoir) m.reservoir.assign(reservoir, reservoir + m.V);
        else m.reservoir.assign(m.V, 0u);
        // names and region list become anonymous placeholders
        while (m.particle_names.size() < s1) m.particle_names.push_back("species" + std::to_string(m.particle_names.size()));
        m.particle_names.resize(s1);
        while (m.types.size() < n_regions) {
            RegionEntry e{};
            e.type = CS_REGION_CUBE;
            e.name = "region" + std::to_string(m.types.size());
            m.types.push_back(e);
        }
        m.types.resize(n_regions);
        m.volumes.assign(n_regions, 0u);
        for (uint64_t v = 0; v < m.V; v++)
            if (m.regions[v] < n_regions) m.volumes[m.regions[v]]++;
        m.logging.erase(std::remove_if(m.logging.begin(), m.logging.end(), [&](uint32_t l) { return l > n_species; }),
                        m.logging.end());
        if (m.n_species != n_species) {
            m.conc.clear();
            m.conc_explicit = false;
            m.slots.assign(m.V * m.K, 0u);
            m.occupancy.assign(m.V, 0u);
        }
        m.n_species = n_species;
        m.n_reactions = n_reactions;
        m.prepare_regions();
        m.check_tables();
    });
}

cs_status cs_set_lattice(cs_sim* sim, const uint32_t* slots, const uint32_t* occupancy, const int32_t* concentrations) {
    return guarded([&] {
        need(sim, "sim");
        need(slots, "slots");
        Model& m = sim->model;
        uint32_t s1 = m.n_species + 1;
        std::vector<uint32_t> occ(m.V);
        for (uint64_t i = 0; i < m.V * m.K; i++)
            if (slots[i] > m.n_species) throw Error(CS_ERR_INVALID_ARG, "slot species out of range");
        if (occupancy) {
            std::memcpy(occ.data(), occupancy, m.V * sizeof(uint32_t));
        } else {
            for (uint64_t v = 0; v < m.V; v++) {
                uint32_t n = 0;
                for (uint32_t k = 0; k < m.K; k++) n += slots[v * m.K + k] != 0u;
                occ[v] = n;
            }
        }
        m.slots.assign(slots, slots + m.V * m.K);
        m.occupancy = occ;
        if (concentrations) {
            m.conc.assign(concentrations, concentrations + m.V * s1);
            m.conc_explicit = true;
        } else {
            m.conc.clear();
            m.conc_explicit = false;
        }
        if (sim->ref) {
            std::vector<int32_t> c = m.concentrations();
            ref_set_lattice(sim->ref.get(), m.slots.data(), m.occupancy.data(), c.data());
        }
        if (sim->prod) prod_set_lattice(sim->prod.get(), m, m.slots.data());
    });
}

cs_status cs_get_lattice(cs_sim* sim, uint32_t* slots, uint32_t* occupancy, int32_t* concentrations) {
    return guarded([&] {
        need(sim, "sim");
        Model& m = sim->model;
        if (sim->ref) {
            ref_get_lattice(sim->ref.get(), slots, occupancy, concentrations);
        } else if (sim->prod) {
            prod_get_lattice(sim->prod.get(), m, slots, occupancy, concentrations);
        } else {
            if (slots) std::memcpy(slots, m.slots.data(), m.slots.size() * sizeof(uint32_t));
            if (occupancy) std::memcpy(occupancy, m.occupancy.data(), m.V * sizeof(uint32_t));
            if (concentrations) {
                std::vector<int32_t> c = m.concentrations();
                std::memcpy(concentrations, c.data(), c.size() * sizeof(int32_t));
            }
        }
    });
}

cs_status cs_prepare_for_gpu(cs_sim* sim, int32_t rng_mode, int32_t device) {
    return guarded([&] {
        need(sim, "sim");
        if (rng_mode != CS_RNG_REFERENCE && rng_mode != CS_RNG_PHILOX) throw Error(CS_ERR_INVALID_ARG, "unknown rng_mode");
        invalidate_device(sim);
        if (rng_mode == CS_RNG_REFERENCE) sim->ref.reset(ref_create(sim->model, device));
        else sim->prod.reset(prod_create(sim->model, device));
        sim->mode = rng_mode;
        sim->device = device;
        sim->frame = 0;
        sim->samples.clear();
    });
}

cs_status cs_step(cs_sim* sim, uint32_t n_steps, const uint32_t* itimes, uint32_t write_freq) {
    return guarded([&] {
        need(sim, "sim");
        if (!sim->ref) throw Error(CS_ERR_STATE, "cs_step needs cs_prepare_for_gpu(CS_RNG_REFERENCE)");
        if (n_steps) need(itimes, "itimes");
        ref_step(sim->ref.get(), n_steps, itimes, sim->frame, write_freq, sim->model.logging, sim->samples);
        sim->frame += n_steps;
    });
}

cs_status cs_step_philox(cs_sim* sim, uint32_t n_steps, uint64_t seed, uint32_t write_freq) {
    return guarded([&] {
        need(sim, "sim");
        if (!sim->prod) throw Error(CS_ERR_STATE, "cs_step_philox needs cs_prepare_for_gpu(CS_RNG_PHILOX)");
        prod_step(sim->prod.get(), n_steps, seed, sim->precision, sim->frame, write_freq, sim->model.logging, sim->samples);
        sim->frame += n_steps;
    });
}

cs_status cs_set_precision(cs_sim* sim, int32_t precision) {
    return guarded([&] {
        need(sim, "sim");
        if (precision < CS_PREC_MIXED || precision > CS_PREC_FP64) throw Error(CS_ERR_INVALID_ARG, "unknown precision");
        sim->precision = precision;
    });
}

cs_status cs_get_counts(cs_sim* sim, int64_t* counts) {
    return guarded([&] {
        need(sim, "sim");
        need(counts, "counts");
        if (sim->ref) ref_get_counts(sim->ref.get(), counts);
        else if (sim->prod) prod_get_counts(sim->prod.get(), counts);
        else throw Error(CS_ERR_STATE, "counts live on the device: call cs_prepare_for_gpu first");
    });
}

cs_status cs_pop_stats(cs_sim* sim, cs_stat_sample* out, uint32_t capacity, uint32_t* n_out) {
    return guarded([&] {
        need(sim, "sim");
        need(n_out, "n_out");
        if (capacity) need(out, "out");
        uint32_t n = (uint32_t)std::min<size_t>(capacity, sim->samples.size());
        for (uint32_t i = 0; i < n; i++) out[i] = sim->samples[i];
        sim->samples.erase(sim->samples.begin(), sim->samples.begin() + n);
        *n_out = n;
    });
}

cs_status cs_get_diagnostics(cs_sim* sim, uint32_t* diag, uint32_t n) {
    return guarded([&] {
        need(sim, "sim");
        need(diag, "diag");
        if (sim->ref) ref_get_diag(sim->ref.get(), diag, n);
        else if (sim->prod) prod_get_diag(sim->prod.get(), diag, n);
        else throw Error(CS_ERR_STATE, "no device state");
    });
}

cs_status cs_synchronize(cs_sim* sim) {
    return guarded([&] {
        need(sim, "sim");
        if (sim->ref) ref_sync(sim->ref.get());
        if (sim->prod) prod_sync(sim->prod.get());
    });
}

cs_status cs_debug_stall_group(cs_sim* sim, uint32_t group) {
    return guarded([&] {
        need(sim, "sim");
        if (!sim->prod) throw Error(CS_ERR_STATE, "cs_debug_stall_group needs cs_prepare_for_gpu(CS_RNG_PHILOX)");
        prod_debug_stall_group(sim->prod.get(), group);
    });
}

cs_status cs_step_timed(cs_sim* sim, uint32_t n_steps, const uint32_t* itimes, float* ms) {
    return guarded([&] {
        need(sim, "sim");
        need(ms, "ms");
        if (!sim->ref) throw Error(CS_ERR_STATE, "cs_step_timed needs cs_prepare_for_gpu(CS_RNG_REFERENCE)");
        if (n_steps) need(itimes, "itimes");
        *ms = ref_time_frames(sim->ref.get(), n_steps, itimes, sim->frame);
        sim->frame += n_steps;
    });
}

cs_status cs_step_philox_timed(cs_sim* sim, uint32_t n_steps, uint64_t seed, float* ms) {
    return guarded([&] {
        need(sim, "sim");
        need(ms, "ms");
        if (!sim->prod) throw Error(CS_ERR_STATE, "cs_step_philox_timed needs cs_prepare_for_gpu(CS_RNG_PHILOX)");
        prod_set_precision(sim->prod.get(), sim->precision);
        prod_seed(sim->prod.get(), seed);
        *ms = prod_time_frames(sim->prod.get(), n_steps, sim->frame, true);
        sim->frame += n_steps;
    });
}

cs_status cs_tiling_count(int32_t* n) {
    return guarded([&] {
        need(n, "n");
        *n = prod_tiling_count();
    });
}

cs_status cs_tiling_describe(int32_t index, int32_t* K, int32_t* TY, int32_t* TZ, int32_t* threads) {
    return guarded([&] {
        need(K, "K"); need(TY, "TY"); need(TZ, "TZ"); need(threads, "threads");
        int k, ty, tz, nt;
        prod_tiling_desc(index, &k, &ty, &tz, &nt);
        *K = k; *TY = ty; *TZ = tz; *threads = nt;
    });
}

cs_status cs_tiling_kind(int32_t index, int32_t* kind, int32_t* brick_planes) {
    return guarded([&] {
        need(kind, "kind"); need(brick_planes, "brick_planes");
        int k, bx;
        prod_tiling_kind(index, &k, &bx);
        *kind = k; *brick_planes = bx;
    });
}

cs_status cs_tiling_launches(int32_t index, int32_t* launches) {
    return guarded([&] {
        need(launches, "launches");
        *launches = prod_tiling_launches(index);
    });
}

cs_status cs_set_tiling(cs_sim* sim, int32_t index, uint32_t segment_length) {
    return guarded([&] {
        need(sim, "sim");
        if (!sim->prod) throw Error(CS_ERR_STATE, "tiling applies to the production path (cs_prepare_for_gpu(CS_RNG_PHILOX))");
        prod_set_tiling(sim->prod.get(), index, segment_length);
    });
}

cs_status cs_autotune(cs_sim* sim, uint32_t frames_per_trial, int32_t* chosen_index, float* ms_per_frame) {
    return guarded([&] {
        need(sim, "sim");
        if (!sim->prod) throw Error(CS_ERR_STATE, "autotuning applies to the production path (cs_prepare_for_gpu(CS_RNG_PHILOX))");
        float ms = 0.0f;
        int best = prod_autotune(sim->prod.get(), frames_per_trial, sim->frame, true, &ms);
        if (chosen_index) *chosen_index = best;
        if (ms_per_frame) *ms_per_frame = ms;
    });
}

cs_status cs_get_tiling(const cs_sim* sim, int32_t* index) {
    return guarded([&] {
        need(sim, "sim");
        need(index, "index");
        if (!sim->prod) throw Error(CS_ERR_STATE, "tiling applies to the production path");
        *index = prod_tiling_current(sim->prod.get());
    });
}

cs_status cs_ensemble_create(const cs_sim* model, uint32_t n_replicates, const uint32_t* res, const uint64_t* seeds,
                             const float* rate_multipliers, const uint32_t* initial_counts, int32_t device,
                             cs_ensemble** out) {
    return guarded([&] {
        need(model, "model");
        need(res, "res");
        need(seeds, "seeds");
        need(initial_counts, "initial_counts");
        need(out, "out");
        *out = nullptr;
        std::unique_ptr<cs_ensemble> e(new cs_ensemble());
        e->prod = std::unique_ptr<DeviceProd, void (*)(DeviceProd*)>(
            prod_ensemble_create(model->model, n_replicates, res, seeds, rate_multipliers, initial_counts, device),
            prod_destroy);
        e->n_rep = n_replicates;
        e->S1 = model->model.n_species + 1;
        e->K = model->model.K;
        e->res.assign(res, res + 3 * (size_t)n_replicates);
        *out = e.release();
    });
}

void cs_ensemble_destroy(cs_ensemble* ens) {
    if (!ens) return;
    try {
        delete ens;
    } catch (...) {
    }
}

cs_status cs_ensemble_step(cs_ensemble* ens, uint32_t n_steps, int32_t batched) {
    return guarded([&] {
        need(ens, "ens");
        prod_ensemble_step(ens->prod.get(), n_steps, batched != 0, ens->frame);
        ens->frame += n_steps;
    });
}

cs_status cs_ensemble_step_timed(cs_ensemble* ens, uint32_t n_steps, int32_t batched, float* ms) {
    return guarded([&] {
        need(ens, "ens");
        need(ms, "ms");
        *ms = prod_time_frames(ens->prod.get(), n_steps, ens->frame, batched != 0);
        ens->frame += n_steps;
    });
}

cs_status cs_ensemble_set_precision(cs_ensemble* ens, int32_t precision) {
    return guarded([&] {
        need(ens, "ens");
        if (precision < CS_PREC_MIXED || precision > CS_PREC_FP64) throw Error(CS_ERR_INVALID_ARG, "unknown precision");
        prod_set_precision(ens->prod.get(), precision);
    });
}

cs_status cs_ensemble_set_tiling(cs_ensemble* ens, int32_t index, uint32_t segment_length) {
    return guarded([&] {
        need(ens, "ens");
        prod_set_tiling(ens->prod.get(), index, segment_length);
    });
}

cs_status cs_ensemble_autotune(cs_ensemble* ens, uint32_t frames_per_trial, int32_t* chosen_index, float* ms_per_frame) {
    return guarded([&] {
        need(ens, "ens");
        float ms = 0.0f;
        int best = prod_autotune(ens->prod.get(), frames_per_trial, ens->frame, true, &ms);
        if (chosen_index) *chosen_index = best;
        if (ms_per_frame) *ms_per_frame = ms;
    });
}

cs_status cs_ensemble_get_counts(cs_ensemble* ens, int64_t* counts) {
    return guarded([&] {
        need(ens, "ens");
        need(counts, "counts");
        prod_get_counts(ens->prod.get(), counts);
    });
}

cs_status cs_ensemble_get_slots(cs_ensemble* ens, uint8_t* slots) {
    return guarded([&] {
        need(ens, "ens");
        need(slots, "slots");
        prod_get_slots_raw(ens->prod.get(), slots);
    });
}

cs_status cs_ensemble_get_diagnostics(cs_ensemble* ens, uint32_t* diag, uint32_t n) {
    return guarded([&] {
        need(ens, "ens");
        need(diag, "diag");
        prod_get_diag(ens->prod.get(), diag, n);
    });
}

cs_status cs_ensemble_synchronize(cs_ensemble* ens) {
    return guarded([&] {
        need(ens, "ens");
        prod_sync(ens->prod.get());
    });
}

cs_status cs_ensemble_info(const cs_ensemble* ens, uint64_t* total_voxels, uint32_t* n_work_items) {
    return guarded([&] {
        need(ens, "ens");
        if (total_voxels) *total_voxels = prod_total_voxels(ens->prod.get());
        if (n_work_items) *n_work_items = prod_n_items(ens->prod.get());
    });
}

cs_status cs_ref_frame_noalloc(const cs_ref_frame_noalloc_args* args) {
    return guarded([&] { ref_frame_noalloc(args); });
}

}  // extern "C"

// ------------------------------------------------------------------ checkpoints and views
namespace {

// Little-endian binary stream of a checkpoint file.
struct CkWriter {
    std::FILE* f;
    void raw(const void* p, size_t n) {
        if (n && std::fwrite(p, 1, n, f) != n) throw Error(CS_ERR_INVALID_ARG, "checkpoint write failed");
    }
    template <class T>
    void pod(const T& v) { raw(&v, sizeof(T)); }
    void str(const std::string& s) {
        pod<uint64_t>(s.size());
        raw(s.data(), s.size());
    }
    template <class T>
    void vec(const std::vector<T>& v) {
        pod<uint64_t>(v.size());
        raw(v.data(), v.size() * sizeof(T));
    }
};

struct CkReader {
    std::FILE* f;
    void raw(void* p, size_t n) {
        if (n && std::fread(p, 1, n, f) != n) throw Error(CS_ERR_INVALID_ARG, "checkpoint file is truncated");
    }
    template <class T>
    T pod() {
        T v;
        raw(&v, sizeof(T));
        return v;
    }
    uint64_t count(uint64_t limit) {
        uint64_t n = pod<uint64_t>();
        if (n > limit) throw Error(CS_ERR_INVALID_ARG, "checkpoint file is corrupt (array length)");
        return n;
    }
    std::string str() {
        std::string s(count(1u << 20), '\0');
        raw(&s[0], s.size());
        return s;
    }
    template <class T>
    std::vector<T> vec(uint64_t limit) {
        std::vector<T> v(count(limit));
        raw(v.data(), v.size() * sizeof(T));
        return v;
    }
};

constexpr char kCkMagic[8] = {'C', 'S', 'I', 'M', 'C', 'K', 'P', 'T'};
constexpr uint32_t kCkVersion = 1;

}  // namespace

cs_status cs_checkpoint_save(cs_sim* sim, const char* path) {
    return guarded([&] {
        need(sim, "sim");
        need(path, "path");
        const Model& m = sim->model;
        const uint64_t V = m.V, S1 = m.S1();
        // current lattice state: the device's when prepared, else the host model's
        std::vector<uint32_t> slots(V * m.K), occ(V);
        std::vector<int32_t> conc(V * S1);
        std::vector<int64_t> counts(S1);
        if (sim->ref) {
            ref_get_lattice(sim->ref.get(), slots.data(), occ.data(), conc.data());
            ref_get_counts(sim->ref.get(), counts.data());
        } else if (sim->prod) {
            prod_get_lattice(sim->prod.get(), m, slots.data(), occ.data(), conc.data());
            prod_get_counts(sim->prod.get(), counts.data());
        } else {
            slots = m.slots;
            occ = m.occupancy;
            conc = m.concentrations();
            for (uint64_t v = 0; v < V; v++)
                for (uint64_t s = 0; s < S1; s++) counts[s] += conc[v * S1 + s];
        }
        std::FILE* f = std::fopen(path, "wb");
        if (!f) throw Error(CS_ERR_INVALID_ARG, std::string("cannot open checkpoint file for writing: ") + path);
        std::unique_ptr<std::FILE, int (*)(std::FILE*)> close(f, std::fclose);
        CkWriter w{f};
        w.raw(kCkMagic, sizeof(kCkMagic));
        w.pod(kCkVersion);
        for (int a = 0; a < 3; a++) w.pod(m.dims[a]);
        for (int a = 0; a < 3; a++) w.pod(m.res[a]);
        w.pod(m.tau);
        w.pod(m.lambda);
        w.pod(m.K);
        w.pod(m.nr);
        w.pod(m.np);
        w.pod(m.n_species);
        w.pod(m.n_reactions);
        w.pod<uint64_t>(m.particle_names.size());
        for (const auto& n : m.particle_names) w.str(n);
        w.vec(m.logging);
        w.pod<uint64_t>(m.types.size());
        for (const RegionEntry& e : m.types) {
            w.pod(e.type);
            w.str(e.name);
            w.raw(e.p0, sizeof(e.p0));
            w.raw(e.pf, sizeof(e.pf));
            w.raw(e.center, sizeof(e.center));
            w.raw(e.direction, sizeof(e.direction));
            w.pod(e.radius);
        }
        w.vec(m.volumes);
        w.pod<uint8_t>(m.regions_prepared ? 1 : 0);
        w.vec(m.regions);
        w.vec(m.diffusion);
        w.vec(m.stoich);
        w.vec(m.reactants);
        w.vec(m.rates);
        w.vec(m.reservoir);
        w.raw(m.rng.s, sizeof(m.rng.s));
        w.pod(sim->mode);
        w.pod(sim->precision);
        w.pod(sim->frame);
        w.vec(slots);
        w.vec(occ);
        w.vec(conc);
        w.vec(counts);
    });
}

cs_status cs_checkpoint_load(const char* path, int32_t device, cs_sim** out) {
    return guarded([&] {
        need(path, "path");
        need(out, "out");
        *out = nullptr;
        std::FILE* f = std::fopen(path, "rb");
        if (!f) throw Error(CS_ERR_NOT_FOUND, std::string("cannot open checkpoint file: ") + path);
        std::unique_ptr<std::FILE, int (*)(std::FILE*)> close(f, std::fclose);
        CkReader r{f};
        char magic[8];
        r.raw(magic, sizeof(magic));
        if (std::memcmp(magic, kCkMagic, sizeof(magic)) != 0) throw Error(CS_ERR_INVALID_ARG, "not a libcellsim checkpoint");
        if (r.pod<uint32_t>() != kCkVersion) throw Error(CS_ERR_INVALID_ARG, "unsupported checkpoint version");
        cs_lattice_params p{};
        for (int a = 0; a < 3; a++) p.dims[a] = r.pod<float>();
        for (int a = 0; a < 3; a++) p.res[a] = r.pod<uint32_t>();
        p.tau = r.pod<float>();
        p.lambda = r.pod<float>();
        p.max_particles_site = r.pod<uint32_t>();
        std::unique_ptr<cs_sim> s(new_sim());
        Model& m = s->model;
        m.init(p);
        const uint64_t V = m.V, lim = (1ull << 40);
        m.nr = r.pod<uint32_t>();
        m.np = r.pod<uint32_t>();
        m.n_species = r.pod<uint32_t>();
        m.n_reactions = r.pod<uint32_t>();
        m.particle_names.resize(r.count(1u << 16));
        for (auto& n : m.particle_names) n = r.str();
        m.logging = r.vec<uint32_t>(1u << 16);
        m.types.resize(r.count(1u << 16));
        for (RegionEntry& e : m.types) {
            e.type = r.pod<int32_t>();
            e.name = r.str();
            r.raw(e.p0, sizeof(e.p0));
            r.raw(e.pf, sizeof(e.pf));
            r.raw(e.center, sizeof(e.center));
            r.raw(e.direction, sizeof(e.direction));
            e.radius = r.pod<float>();
        }
        m.volumes = r.vec<uint32_t>(1u << 16);
        const bool prepared = r.pod<uint8_t>() != 0;
        m.regions = r.vec<uint32_t>(lim);
        m.diffusion = r.vec<float>(lim);
        m.stoich = r.vec<int32_t>(lim);
        m.reactants = r.vec<uint32_t>(lim);
        m.rates = r.vec<float>(lim);
        m.reservoir = r.vec<uint32_t>(lim);
        r.raw(m.rng.s, sizeof(m.rng.s));
        const int32_t mode = r.pod<int32_t>();
        s->precision = r.pod<int32_t>();
        const uint64_t frame = r.pod<uint64_t>();
        m.slots = r.vec<uint32_t>(lim);
        m.occupancy = r.vec<uint32_t>(lim);
        m.conc = r.vec<int32_t>(lim);
        const std::vector<int64_t> counts = r.vec<int64_t>(1u << 16);
        const uint64_t S1 = m.S1();
        if (m.regions.size() != V || m.reservoir.size() != V || m.slots.size() != V * m.K || m.occupancy.size() != V ||
            m.conc.size() != V * S1 || counts.size() != S1 || m.particle_names.size() != S1 ||
            m.diffusion.size() != (size_t)m.nr * m.nr * m.np || m.rates.size() != m.n_reactions + 1u)
            throw Error(CS_ERR_INVALID_ARG, "checkpoint file is inconsistent");
        m.conc_explicit = true;
        m.index_buffer.clear();
        if (prepared) {
            for (uint64_t v = 0; v < V; v++) m.index_buffer[m.regions[v]].push_back((uint32_t)v);
            m.regions_prepared = true;
        }
        if (mode == CS_RNG_REFERENCE) {
            s->ref.reset(ref_create(m, device));
            ref_set_counts(s->ref.get(), counts.data());
        } else if (mode == CS_RNG_PHILOX) {
            s->prod.reset(prod_create(m, device));
            prod_set_counts(s->prod.get(), counts.data());
        }
        s->mode = mode;
        s->device = device;
        s->frame = frame;
        *out = s.release();
    });
}

cs_status cs_render_view(cs_sim* sim, int32_t view, int32_t slice_axis, uint32_t slice, float* out_host, void* out_device) {
    return guarded([&] {
        need(sim, "sim");
        if (!out_host && !out_device) throw Error(CS_ERR_INVALID_ARG, "out_host or out_device is required");
        if (view < 0 || view > 2) throw Error(CS_ERR_INVALID_ARG, "view must be 0 (species), 1 (regions) or 2 (reservoirs)");
        if (slice_axis < 0 || slice_axis > 2) throw Error(CS_ERR_INVALID_ARG, "slice_axis must be 0, 1 or 2");
        if (sim->ref) ref_render_view(sim->ref.get(), view, slice_axis, slice, out_host, out_device);
        else if (sim->prod) prod_render_view(sim->prod.get(), view, slice_axis, slice, out_host, out_device);
        else throw Error(CS_ERR_STATE, "cs_render_view needs cs_prepare_for_gpu");
    });
}
