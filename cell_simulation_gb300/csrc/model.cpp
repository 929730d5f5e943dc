// model.cpp — host model builder mirroring the reference's Simulation API
// (src/simulation.rs, src/lattice.rs, src/region.rs).  Every rasteriser keeps
// the reference's binary32 arithmetic and loop structure so that the region
// masks come out voxel-for-voxel the same.  Compiled with -ffp-contract=off.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstring>
#include <fstream>
#include <sstream>

#include "internal.h"
#include "json.h"

namespace cellsim {

// ---------------------------------------------------------------- HostRng
static uint64_t splitmix(uint64_t& x) {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
void HostRng::seed(uint64_t v) {
    for (auto& w : s) w = splitmix(v);
}
static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
uint64_t HostRng::next() {
    uint64_t r = rotl(s[1] * 5, 7) * 9, t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
    s[2] ^= t; s[3] = rotl(s[3], 45);
    return r;
}
uint64_t HostRng::below(uint64_t n) {
    // rejection sampling on the top bits: unbiased
    uint64_t lim = (~0ull) - ((~0ull) % n);
    for (;;) {
        uint64_t r = next();
        if (r < lim) return r % n;
    }
}
float HostRng::unit_f32() { return (float)(next() >> 40) * 0x1p-24f; }

// ---------------------------------------------------------------- Model
void Model::init(const cs_lattice_params& p) {
    for (int i = 0; i < 3; i++) {
        if (p.res[i] == 0) throw Error(CS_ERR_INVALID_ARG, "lattice resolution must be positive");
        dims[i] = p.dims[i];
        res[i] = p.res[i];
    }
    if (p.max_particles_site < 1 || p.max_particles_site > 16)
        throw Error(CS_ERR_LIMIT, "max_particles_site must be in 1..16 (the reaction pass snapshots at most 16 slots, cme.wgsl:56)");
    tau = p.tau;
    lambda = p.lambda;
    K = p.max_particles_site;
    V = (uint64_t)res[0] * res[1] * res[2];
    if (V * K >= (1ull << 32)) throw Error(CS_ERR_LIMIT, "V*K must be below 2^32 (slot indices are u32 in the shaders)");
    regions.assign(V, 0u);
    RegionEntry bg{};
    bg.type = CS_REGION_CUBE;
    bg.name = "background";
    for (int i = 0; i < 3; i++) { bg.p0[i] = 0.0f; bg.pf[i] = dims[i]; }
    types = {bg};
    volumes = {(uint32_t)(res[0] * res[1] * res[2])};
    index_buffer.clear();
    regions_prepared = false;
    nr = 1;
    np = 1;
    diffusion.assign(1, 8.15E-14f / 6.0f);  // src/simulation.rs:72-73
    particle_names = {"void"};
    logging.clear();
    stoich.assign(1, 0);
    reactants.assign(3, 0u);
    rates.assign(1, 0.0f);
    n_species = 0;
    n_reactions = 0;
    slots.assign(V * K, 0u);
    occupancy.assign(V, 0u);
    conc.clear();
    conc_explicit = false;
    reservoir.assign(V, 0u);
    rng.seed(0x5EEDC0DEull);
}

int Model::find_region(const std::string& name) const {
    for (size_t i = 0; i < types.size(); i++)
        if (types[i].name == name) return (int)i;
    return -1;
}

int Model::find_particle(const std::string& name) const {
    for (size_t i = 1; i < particle_names.size(); i++)
        if (particle_names[i] == name) return (int)i;
    return -1;
}

void Model::check_tables() const {
    if (nr != types.size()) throw Error(CS_ERR_STATE, "region table size mismatch");
    if (np != n_species + 1) throw Error(CS_ERR_STATE, "diffusion matrix species dimension does not match the species count");
    for (uint64_t v = 0; v < V; v++)
        if (regions[v] >= nr) throw Error(CS_ERR_INVALID_ARG, "region id out of range at voxel " + std::to_string(v));
    for (uint32_t r = 0; r <= n_reactions; r++)
        for (int j = 0; j < 3; j++)
            if (reactants[r * 3 + j] > n_species) throw Error(CS_ERR_INVALID_ARG, "reactant index out of range");
    for (uint64_t v = 0; v < V; v++)
        if (reservoir[v] > n_species) throw Error(CS_ERR_INVALID_ARG, "reservoir species out of range");
    for (uint64_t i = 0; i < V * K; i++)
        if (slots[i] > n_species) throw Error(CS_ERR_INVALID_ARG, "slot species out of range at slot " + std::to_string(i));
}

// Tensor3::enlarge_dimension(0|1, value) on the [nr][nr][np] matrix.
void Model::update_matrices_region(float diffusion_rate, float transition_rate) {
    uint32_t nn = nr + 1;
    std::vector<float> d((size_t)nn * nn * np, transition_rate);
    for (uint32_t a = 0; a < nr; a++)
        for (uint32_t b = 0; b < nr; b++)
            for (uint32_t q = 0; q < np; q++) d[((size_t)a * nn + b) * np + q] = D(a, b, q);
    diffusion.swap(d);
    nr = nn;
    uint32_t last = (uint32_t)types.size() - 1;
    for (uint32_t q = 0; q < np; q++) D(last, last, q) = diffusion_rate;  // src/simulation.rs:541-545
}

void Model::check_collision(uint64_t v) {  // Regions::check_regions_collision, src/region.rs:121-127
    uint32_t old = regions[v];
    if (old != 0) volumes[old] -= 1u;
}

void Model::add_region_cube(const std::string& name, const float p0[3], const float pf[3], float dr, float tr) {
    // src/simulation.rs:627-658
    RegionEntry e{};
    e.type = CS_REGION_CUBE;
    e.name = name;
    for (int i = 0; i < 3; i++) { e.p0[i] = p0[i]; e.pf[i] = pf[i]; }
    if (!(p0[0] <= pf[0] && p0[1] <= pf[1] && p0[2] <= pf[2]))
        throw Error(CS_ERR_INVALID_ARG, "cube region needs p0 <= pf");
    types.push_back(e);
    uint32_t idx = (uint32_t)types.size() - 1;
    size_t st[3], en[3];
    for (int i = 0; i < 3; i++) {
        float vs = voxel_size(i);
        float a = p0[i] / vs, b = pf[i] / vs;
        st[i] = (a > 0.0f) ? (size_t)a : 0;  // `as usize` saturates
        en[i] = (b > 0.0f) ? (size_t)b : 0;
        if (en[i] > res[i]) {
            types.pop_back();
            throw Error(CS_ERR_INVALID_ARG, "cube region extends past the lattice");
        }
    }
    uint64_t volume = (uint64_t)(en[0] - st[0]) * (en[1] - st[1]) * (en[2] - st[2]);
    for (size_t x = st[0]; x < en[0]; x++)
        for (size_t y = st[1]; y < en[1]; y++)
            for (size_t z = st[2]; z < en[2]; z++) {
                uint64_t v = ((uint64_t)x * res[1] + y) * res[2] + z;
                check_collision(v);
                regions[v] = idx;
            }
    update_matrices_region(dr, tr);
    volumes.push_back((uint32_t)volume);
}

void Model::add_region_sphere(const std::string& name, const float c_in[3], float radius, float dr, float tr) {
    // src/simulation.rs:660-699; voxel-corner coordinates, dist < r^2
    RegionEntry e{};
    e.type = CS_REGION_SPHERE;
    e.name = name;
    for (int i = 0; i < 3; i++) e.center[i] = c_in[i];
    e.radius = radius;
    types.push_back(e);
    uint32_t idx = (uint32_t)types.size() - 1;
    float vs[3] = {voxel_size(0), voxel_size(1), voxel_size(2)};
    float c[3] = {c_in[0] / vs[0], c_in[1] / vs[1], c_in[2] / vs[2]};
    float r2 = radius * radius;
    float vss[3] = {vs[0] * vs[0], vs[1] * vs[1], vs[2] * vs[2]};
    float resf[3] = {(float)res[0], (float)res[1], (float)res[2]};
    uint32_t volume = 0;
    for (float x = 0.0f; x < resf[0]; x += 1.0f)
        for (float y = 0.0f; y < resf[1]; y += 1.0f)
            for (float z = 0.0f; z < resf[2]; z += 1.0f) {
                float dx = x - c[0], dy = y - c[1], dz = z - c[2];
                float d = (dx * dx) * vss[0] + (dy * dy) * vss[1];
                d = d + (dz * dz) * vss[2];
                if (d < r2) {
                    uint64_t v = ((uint64_t)x * res[1] + (uint64_t)y) * res[2] + (uint64_t)z;
                    check_collision(v);
                    regions[v] = idx;
                    volume++;
                }
            }
    update_matrices_region(dr, tr);
    volumes.push_back(volume);
}

void Model::add_region_semisphere(const std::string& name, const float c_in[3], float radius, const float dir[3], float dr,
                                  float tr) {
    // src/simulation.rs:701-743
    RegionEntry e{};
    e.type = CS_REGION_SEMISPHERE;
    e.name = name;
    for (int i = 0; i < 3; i++) { e.center[i] = c_in[i]; e.direction[i] = dir[i]; }
    e.radius = radius;
    types.push_back(e);
    uint32_t idx = (uint32_t)types.size() - 1;
    float vs[3] = {voxel_size(0), voxel_size(1), voxel_size(2)};
    float c[3] = {c_in[0] / vs[0], c_in[1] / vs[1], c_in[2] / vs[2]};
    float r2 = radius * radius;
    float vss[3] = {vs[0] * vs[0], vs[1] * vs[1], vs[2] * vs[2]};
    float resf[3] = {(float)res[0], (float)res[1], (float)res[2]};
    uint32_t volume = 0;
    for (float x = 0.0f; x < resf[0]; x += 1.0f)
        for (float y = 0.0f; y < resf[1]; y += 1.0f)
            for (float z = 0.0f; z < resf[2]; z += 1.0f) {
                float side = (x - c[0]) * dir[0] + (y - c[1]) * dir[1];
                side = side + (z - c[2]) * dir[2];
                if (side < 0.0f) continue;
                float dx = x - c[0], dy = y - c[1], dz = z - c[2];
                float d = (dx * dx) * vss[0] + (dy * dy) * vss[1];
                d = d + (dz * dz) * vss[2];
                if (d < r2) {
                    uint64_t v = ((uint64_t)x * res[1] + (uint64_t)y) * res[2] + (uint64_t)z;
                    check_collision(v);
                    regions[v] = idx;
                    volume++;
                }
            }
    update_matrices_region(dr, tr);
    volumes.push_back(volume);
}

void Model::add_region_cylinder(const std::string& name, const float p0[3], const float pf[3], float radius, float dr,
                                float tr) {
    // src/simulation.rs:550-625
    RegionEntry e{};
    e.type = CS_REGION_CYLINDER;
    e.name = name;
    for (int i = 0; i < 3; i++) { e.p0[i] = p0[i]; e.pf[i] = pf[i]; }
    e.radius = radius;
    types.push_back(e);
    uint32_t idx = (uint32_t)types.size() - 1;
    float resf[3] = {(float)res[0], (float)res[1], (float)res[2]};
    float vs[3] = {voxel_size(0), voxel_size(1), voxel_size(2)};
    float rl[3] = {radius / vs[0], radius / vs[1], radius / vs[2]};
    float ip0[3] = {p0[0] / vs[0], p0[1] / vs[1], p0[2] / vs[2]};
    float ipf[3] = {pf[0] / vs[0], pf[1] / vs[1], pf[2] / vs[2]};
    float vv[3] = {ipf[0] - ip0[0], ipf[1] - ip0[1], ipf[2] - ip0[2]};
    float v2 = vv[0] * vv[0] + vv[1] * vv[1];
    v2 = v2 + vv[2] * vv[2];
    float r_const = (radius * radius) * v2;
    float vss[3] = {vs[0] * vs[0], vs[1] * vs[1], vs[2] * vs[2]};
    uint32_t volume = 0;
    auto fmax0 = [](float a) { return std::fmax(a, 0.0f); };
    float x = fmax0(ip0[0] - rl[0]), y = fmax0(ip0[1] - rl[1]), z = fmax0(ip0[2] - rl[2]);
    float xf = std::fmin(ipf[0] + rl[0], resf[0]);
    float yf = std::fmin(ipf[1] + rl[1], resf[1]);
    float zf = std::fmin(ipf[2] + rl[2], resf[2]);
    while (x < xf) {
        while (y < yf) {
            while (z < zf) {
                float w0 = x - ipf[0], w1 = y - ipf[1], w2 = z - ipf[2];
                float proj = w0 * vv[0] + w1 * vv[1];
                proj = proj + w2 * vv[2];
                if (proj > 0.0f) { z += 1.0f; continue; }
                w0 = x - ip0[0]; w1 = y - ip0[1]; w2 = z - ip0[2];
                proj = w0 * vv[0] + w1 * vv[1];
                proj = proj + w2 * vv[2];
                if (proj < 0.0f) { z += 1.0f; continue; }
                float cp0 = w1 * vv[2] - w2 * vv[1];
                float cp1 = w2 * vv[0] - w0 * vv[2];
                float cp2 = w0 * vv[1] - w1 * vv[0];
                float cn = (cp0 * cp0) * vss[0] + (cp1 * cp1) * vss[1];
                cn = cn + (cp2 * cp2) * vss[2];
                if (cn <= r_const) {
                    uint64_t v = ((uint64_t)x * res[1] + (uint64_t)y) * res[2] + (uint64_t)z;
                    check_collision(v);
                    regions[v] = idx;
                    volume++;
                }
                z += 1.0f;
            }
            z = fmax0(ip0[2] - rl[2]);
            y += 1.0f;
        }
        y = fmax0(ip0[1] - rl[1]);
        x += 1.0f;
    }
    update_matrices_region(dr, tr);
    volumes.push_back(volume);
}

void Model::join_regions(const std::string& del, const std::string& to) {
    // src/simulation.rs:758-790
    int di = find_region(del), ti = find_region(to);
    if (di < 0 || ti < 0) throw Error(CS_ERR_NOT_FOUND, "region not found while joining '" + del + "' into '" + to + "'");
    uint32_t d = (uint32_t)di, t = (uint32_t)ti;
    for (uint64_t v = 0; v < V; v++) {
        if (regions[v] == d) regions[v] = t;
        if (regions[v] > d) regions[v] -= 1u;
    }
    // Tensor3::remove_element_at(0|1, d)
    uint32_t nn = nr - 1;
    std::vector<float> m((size_t)nn * nn * np);
    for (uint32_t a = 0, a2 = 0; a < nr; a++) {
        if (a == d) continue;
        for (uint32_t b = 0, b2 = 0; b < nr; b++) {
            if (b == d) continue;
            for (uint32_t q = 0; q < np; q++) m[((size_t)a2 * nn + b2) * np + q] = D(a, b, q);
            b2++;
        }
        a2++;
    }
    diffusion.swap(m);
    nr = nn;
    volumes[t] += volumes[d];
    types.erase(types.begin() + d);
    volumes.erase(volumes.begin() + d);
}

void Model::add_region(const cs_region_desc& r, float diffusion_rate) {
    const float tr = 0.0f;  // transition rate default, src/simulation.rs:430
    if (regions_prepared) {
        // the reference allows it, but the index buffer would be stale
        regions_prepared = false;
    }
    auto nm = [](const char* s) -> std::string {
        if (!s) throw Error(CS_ERR_INVALID_ARG, "region name is NULL");
        return std::string(s);
    };
    if (types.size() >= 255) throw Error(CS_ERR_LIMIT, "at most 255 regions");
    switch (r.type) {
        case CS_REGION_CUBE: add_region_cube(nm(r.name), r.p0, r.pf, diffusion_rate, tr); break;
        case CS_REGION_SPHERE: add_region_sphere(nm(r.name), r.center, r.radius, diffusion_rate, tr); break;
        case CS_REGION_SEMISPHERE: add_region_semisphere(nm(r.name), r.center, r.radius, r.direction, diffusion_rate, tr); break;
        case CS_REGION_CYLINDER: add_region_cylinder(nm(r.name), r.p0, r.pf, r.radius, diffusion_rate, tr); break;
        case CS_REGION_SPHERICAL_SHELL:
            add_region_sphere(nm(r.shell_name), r.center, r.external_radius, diffusion_rate, tr);
            add_region_sphere(nm(r.interior_name), r.center, r.internal_radius, diffusion_rate, tr);
            break;
        case CS_REGION_CYLINDRICAL_SHELL:
            add_region_cylinder(nm(r.shell_name), r.p0, r.pf, r.external_radius, diffusion_rate, tr);
            add_region_cylinder(nm(r.interior_name), r.p0, r.pf, r.internal_radius, diffusion_rate, tr);
            break;
        case CS_REGION_CAPSID: {
            // src/simulation.rs:449-477
            float cyl = r.total_length - 2.0f * r.external_radius;
            float p0[3], pf[3], nd[3];
            for (int i = 0; i < 3; i++) {
                p0[i] = r.center[i] - r.direction[i] * cyl / 2.0f;
                pf[i] = r.center[i] + r.direction[i] * cyl / 2.0f;
                nd[i] = -r.direction[i];
            }
            std::string shell = nm(r.shell_name), inner = nm(r.interior_name);
            add_region_cylinder(shell, p0, pf, r.external_radius, diffusion_rate, tr);
            add_region_cylinder(inner, p0, pf, r.internal_radius, diffusion_rate, tr);
            add_region_semisphere("cap1", p0, r.external_radius, nd, diffusion_rate, tr);
            add_region_semisphere("cap2", pf, r.external_radius, r.direction, diffusion_rate, tr);
            add_region_semisphere("inside1", p0, r.internal_radius, nd, diffusion_rate, tr);
            add_region_semisphere("inside2", pf, r.internal_radius, r.direction, diffusion_rate, tr);
            join_regions("cap1", shell);
            join_regions("cap2", shell);
            join_regions("inside1", inner);
            join_regions("inside2", inner);
            break;
        }
        default: throw Error(CS_ERR_INVALID_ARG, "unknown region type " + std::to_string(r.type));
    }
}

void Model::prepare_regions() {  // src/region.rs:129-148
    index_buffer.clear();
    for (uint64_t v = 0; v < V; v++) index_buffer[regions[v]].push_back((uint32_t)v);
    regions_prepared = true;
}

std::vector<int32_t> Model::concentrations() const {
    if (conc_explicit) return conc;
    uint32_t s1 = n_species + 1;
    std::vector<int32_t> c(V * s1, 0);
    for (uint64_t v = 0; v < V; v++) {
        for (uint32_t k = 0; k < K; k++) {
            uint32_t q = slots[v * K + k];
            if (q && q < s1) c[v * s1 + q] += 1;
        }
        if (reservoir[v] && reservoir[v] < s1) c[v * s1 + reservoir[v]] += 1;
    }
    return c;
}

void Model::add_species_column() {
    // concentrations.enlarge_dimension(3, 0), src/lattice.rs:64
    if (!conc_explicit) return;
    uint32_t s1 = n_species + 1, s2 = s1 + 1;
    std::vector<int32_t> c(V * s2, 0);
    for (uint64_t v = 0; v < V; v++)
        for (uint32_t s = 0; s < s1; s++) c[v * s2 + s] = conc[v * s1 + s];
    conc.swap(c);
}

bool Model::add_particle_site(uint64_t v, uint32_t particle) {  // src/lattice.rs:280-290
    if (occupancy[v] == K) return false;
    slots[v * K + occupancy[v]] = particle;
    occupancy[v] += 1;
    if (conc_explicit) conc[v * (n_species + 1) + particle] += 1;
    return true;
}

bool Model::add_reservoir_site(uint64_t v, uint32_t particle) {  // src/lattice.rs:292-300
    if (reservoir[v] > 0u) return false;
    reservoir[v] = particle;
    if (conc_explicit) conc[v * (n_species + 1) + particle] = 1;
    return true;
}

static void append_species(Model& m, const std::string& name, bool logging) {
    if (m.particle_names.size() >= 256) throw Error(CS_ERR_LIMIT, "at most 255 species (slots are stored as bytes)");
    uint32_t pidx = (uint32_t)m.particle_names.size();
    m.particle_names.push_back(name);
    // diffusion_matrix.copy_dimension(2), src/simulation.rs:804
    uint32_t nq = m.np + 1;
    std::vector<float> d((size_t)m.nr * m.nr * nq);
    for (uint32_t a = 0; a < m.nr; a++)
        for (uint32_t b = 0; b < m.nr; b++) {
            for (uint32_t q = 0; q < m.np; q++) d[((size_t)a * m.nr + b) * nq + q] = m.D(a, b, q);
            d[((size_t)a * m.nr + b) * nq + m.np] = m.D(a, b, m.np - 1);
        }
    m.diffusion.swap(d);
    m.np = nq;
    // stoichiometry_matrix.enlarge_dimension(1, 0), src/simulation.rs:807
    uint32_t s1 = m.n_species + 1, s2 = s1 + 1;
    std::vector<int32_t> st((size_t)(m.n_reactions + 1) * s2, 0);
    for (uint32_t r = 0; r <= m.n_reactions; r++)
        for (uint32_t s = 0; s < s1; s++) st[(size_t)r * s2 + s] = m.stoich[(size_t)r * s1 + s];
    m.stoich.swap(st);
    m.n_species += 1;
    if (logging) m.logging.push_back(pidx);
}

void Model::add_particle_count(const std::string& name, const std::string& to_region, uint32_t count, bool log, bool is_res) {
    // src/simulation.rs:792-814 with Lattice::init_random_particles_region, src/lattice.rs:63-97
    int ri = find_region(to_region);
    if (ri < 0) throw Error(CS_ERR_NOT_FOUND, "region not found: " + to_region);
    if (!regions_prepared) throw Error(CS_ERR_STATE, "prepare_regions must be called before adding particles");
    auto it = index_buffer.find((uint32_t)ri);
    if (it == index_buffer.end() || it->second.empty()) throw Error(CS_ERR_NOT_FOUND, "region has no voxels: " + to_region);
    if (particle_names.size() >= 256) throw Error(CS_ERR_LIMIT, "at most 255 species (slots are stored as bytes)");
    uint32_t pidx = (uint32_t)particle_names.size();
    add_species_column();
    const std::vector<uint32_t>& buf = it->second;
    // n_species is bumped in append_species; conc already has the new column
    uint32_t save_s = n_species;
    n_species += 1;  // so that conc indexing uses the new row width
    for (uint32_t i = 0; i < count; i++) {
        int tries = 0;
        while (tries < 100) {
            uint64_t v = buf[rng.below(buf.size())];
            bool ok = is_res ? add_reservoir_site(v, pidx) : add_particle_site(v, pidx);
            if (ok) break;
            tries++;
        }
        if (tries == 100) {
            n_species = save_s;
            throw Error(CS_ERR_CAPACITY, "could not add particle to region " + to_region + " (src/lattice.rs:93-95)");
        }
    }
    n_species = save_s;
    append_species(*this, name, log);
}

void Model::add_particle_concentration(const std::string& name, const std::string& to_region, float concentration, bool log,
                                       bool is_res) {
    // src/simulation.rs:816-823
    int ri = find_region(to_region);
    if (ri < 0) throw Error(CS_ERR_NOT_FOUND, "region not found: " + to_region);
    float volume = (float)volumes[ri];
    float c = concentration * volume;
    uint32_t count = (c > 0.0f) ? (c >= 4294967296.0f ? 0xFFFFFFFFu : (uint32_t)c) : 0u;
    add_particle_count(name, to_region, count, log, is_res);
}

void Model::fill_region(const std::string& name, const std::string& to_region, bool log) {
    // src/simulation.rs:825-840, src/lattice.rs:99-111
    int ri = find_region(to_region);
    if (ri < 0) throw Error(CS_ERR_NOT_FOUND, "region not found: " + to_region);
    if (!regions_prepared) throw Error(CS_ERR_STATE, "prepare_regions must be called before adding particles");
    auto it = index_buffer.find((uint32_t)ri);
    if (it == index_buffer.end()) throw Error(CS_ERR_NOT_FOUND, "region has no voxels: " + to_region);
    if (particle_names.size() >= 256) throw Error(CS_ERR_LIMIT, "at most 255 species (slots are stored as bytes)");
    uint32_t pidx = (uint32_t)particle_names.size();
    add_species_column();
    uint32_t save_s = n_species;
    n_species += 1;
    for (uint32_t v : it->second) {
        if (!add_particle_site(v, pidx)) {
            n_species = save_s;
            throw Error(CS_ERR_CAPACITY, "could not add particle to region " + to_region);
        }
    }
    n_species = save_s;
    append_species(*this, name, log);
}

void Model::set_diffusion_rate(const std::string& region, float rate) {
    int ri = find_region(region);
    if (ri < 0) throw Error(CS_ERR_NOT_FOUND, "region not found: " + region);
    for (uint32_t q = 0; q < np; q++) D(ri, ri, q) = rate;
}

static int position_of(const std::vector<std::string>& names, const std::string& n) {
    for (size_t i = 0; i < names.size(); i++)
        if (names[i] == n) return (int)i;
    return -1;
}

void Model::set_diffusion_rate_particle(const std::string& particle, const std::string& region, float rate) {
    int ri = find_region(region);
    if (ri < 0) throw Error(CS_ERR_NOT_FOUND, "region not found: " + region);
    int pi = position_of(particle_names, particle);  // iter().position, may match "void"
    if (pi < 0) throw Error(CS_ERR_NOT_FOUND, "particle not found: " + particle);
    D(ri, ri, pi) = rate;
}

void Model::set_transition_rate(const std::string& from, const std::string& to, float rate) {
    int a = find_region(from), b = find_region(to);
    if (a < 0 || b < 0) throw Error(CS_ERR_NOT_FOUND, "region not found: " + (a < 0 ? from : to));
    for (uint32_t q = 0; q < np; q++) D(a, b, q) = rate;
}

void Model::set_transition_rate_particle(const std::string& particle, const std::string& from, const std::string& to,
                                         float rate) {
    int a = find_region(from), b = find_region(to);
    if (a < 0 || b < 0) throw Error(CS_ERR_NOT_FOUND, "region not found: " + (a < 0 ? from : to));
    int pi = position_of(particle_names, particle);
    if (pi < 0) throw Error(CS_ERR_NOT_FOUND, "particle not found: " + particle);
    D(a, b, pi) = rate;
}

void Model::add_reaction(const std::vector<std::string>& re, const std::vector<std::string>& pr, float k) {
    // src/simulation.rs:904-947
    std::vector<uint32_t> ri, pi;
    for (auto& n : re) {
        int i = find_particle(n);
        if (i < 0) throw Error(CS_ERR_NOT_FOUND, "Reactant " + n + " not found");
        ri.push_back((uint32_t)i);
    }
    for (auto& n : pr) {
        int i = find_particle(n);
        if (i < 0) throw Error(CS_ERR_NOT_FOUND, "Product " + n + " not found");
        pi.push_back((uint32_t)i);
    }
    if (ri.size() > 3) throw Error(CS_ERR_LIMIT, "at most 3 reactants per reaction (reactions_idx has 3 columns)");
    if (n_reactions >= 99) throw Error(CS_ERR_LIMIT, "at most 99 reactions (MAX_REACTIONS = 100 cumulative entries, functions.wgsl:1)");
    uint32_t s1 = n_species + 1;
    stoich.resize((size_t)(n_reactions + 2) * s1, 0);
    int32_t* row = &stoich[(size_t)(n_reactions + 1) * s1];
    for (uint32_t i : ri) row[i] -= 1;
    for (uint32_t i : pi) row[i] += 1;
    while (ri.size() < 3) ri.push_back(0u);
    for (uint32_t i : ri) reactants.push_back(i);
    rates.push_back(k);
    n_reactions += 1;
}

// ---------------------------------------------------------------- JSON
static void arr3f(const JsonValue& v, float out[3], const std::string& what) {
    if (v.kind != JsonValue::Array || v.arr.size() != 3) throw Error(CS_ERR_PARSE, "'" + what + "' must be an array of 3 numbers");
    for (int i = 0; i < 3; i++) out[i] = (float)v.arr[i].as_number(what);
}

// Rust's str::parse::<f32>: optional sign, decimal with optional fraction
// and exponent, or inf/infinity/nan (case-insensitive).
static bool parse_rust_f32(const std::string& t, float& out) {
    std::string l;
    for (char c : t) l += (char)std::tolower((unsigned char)c);
    size_t i = 0;
    if (i < l.size() && (l[i] == '+' || l[i] == '-')) i++;
    std::string body = l.substr(i);
    if (body == "inf" || body == "infinity" || body == "nan") {
        out = std::strtof(t.c_str(), nullptr);
        return true;
    }
    size_t digits = 0, j = i;
    while (j < l.size() && std::isdigit((unsigned char)l[j])) { j++; digits++; }
    if (j < l.size() && l[j] == '.') {
        j++;
        while (j < l.size() && std::isdigit((unsigned char)l[j])) { j++; digits++; }
    }
    if (digits == 0) return false;
    if (j < l.size() && l[j] == 'e') {
        j++;
        if (j < l.size() && (l[j] == '+' || l[j] == '-')) j++;
        size_t ed = 0;
        while (j < l.size() && std::isdigit((unsigned char)l[j])) { j++; ed++; }
        if (ed == 0) return false;
    }
    if (j != l.size()) return false;
    out = std::strtof(t.c_str(), nullptr);
    return true;
}

void Model::load_json(const std::string& text) {
    JsonValue root;
    try {
        root = JsonParser(text).parse();
    } catch (const std::runtime_error& e) {
        throw Error(CS_ERR_PARSE, e.what());
    }
    try {
        // LatticeParams::from_json_value, src/lattice_params.rs:144-166
        const JsonValue& p = root.at("parameters");
        cs_lattice_params lp{};
        arr3f(p.at("dimensions"), lp.dims, "dimensions");
        const JsonValue& r = p.at("lattice_resolution");
        if (r.kind != JsonValue::Array || r.arr.size() != 3) throw Error(CS_ERR_PARSE, "'lattice_resolution' must be an array of 3 integers");
        for (int i = 0; i < 3; i++) lp.res[i] = (uint32_t)r.arr[i].as_u64("lattice_resolution");
        lp.lambda = (float)p.at("lambda").as_number("lambda");
        lp.tau = (float)p.at("tau").as_number("tau");
        lp.max_particles_site = p.has("max_particles_site") ? (uint32_t)p.at("max_particles_site").as_u64("max_particles_site") : 8u;
        uint64_t keep_seed[4];
        std::memcpy(keep_seed, rng.s, sizeof(keep_seed));
        init(lp);
        std::memcpy(rng.s, keep_seed, sizeof(keep_seed));
        // regions, src/simulation.rs:238-281
        const JsonValue& regs = root.at("regions");
        if (regs.kind != JsonValue::Array) throw Error(CS_ERR_PARSE, "'regions' must be an array");
        for (const JsonValue& rg : regs.arr) {
            std::string ty = rg.at("type").as_string("type");
            cs_region_desc d{};
            float dr = (float)rg.at("base_diffusion_rate").as_number("base_diffusion_rate");
            std::string n1, n2;
            if (ty == "cube") {
                d.type = CS_REGION_CUBE;
                n1 = rg.at("name").as_string("name");
                d.name = n1.c_str();
                arr3f(rg.at("p0"), d.p0, "p0");
                arr3f(rg.at("pf"), d.pf, "pf");
            } else if (ty == "capsid") {
                d.type = CS_REGION_CAPSID;
                n1 = rg.at("shell_name").as_string("shell_name");
                n2 = rg.at("interior_name").as_string("interior_name");
                d.shell_name = n1.c_str();
                d.interior_name = n2.c_str();
                arr3f(rg.at("center"), d.center, "center");
                arr3f(rg.at("dir"), d.direction, "dir");
                d.internal_radius = (float)rg.at("internal_radius").as_number("internal_radius");
                d.external_radius = (float)rg.at("external_radius").as_number("external_radius");
                d.total_length = (float)rg.at("total_length").as_number("total_length");
            } else if (ty == "sphere") {  // extension: the reference's loader reads cube and capsid only
                d.type = CS_REGION_SPHERE;
                n1 = rg.at("name").as_string("name");
                d.name = n1.c_str();
                arr3f(rg.at("center"), d.center, "center");
                d.radius = (float)rg.at("radius").as_number("radius");
            } else if (ty == "spherical_shell") {  // extension
                d.type = CS_REGION_SPHERICAL_SHELL;
                n1 = rg.at("shell_name").as_string("shell_name");
                n2 = rg.at("interior_name").as_string("interior_name");
                d.shell_name = n1.c_str();
                d.interior_name = n2.c_str();
                arr3f(rg.at("center"), d.center, "center");
                d.internal_radius = (float)rg.at("internal_radius").as_number("internal_radius");
                d.external_radius = (float)rg.at("external_radius").as_number("external_radius");
            } else if (ty == "sparse") {
                throw Error(CS_ERR_PARSE, "sparse regions are not implemented (the reference panics too, src/simulation.rs:275-276)");
            } else {
                throw Error(CS_ERR_PARSE, "region type not implemented: " + ty);
            }
            add_region(d, dr);
        }
        prepare_regions();
        // particles, src/simulation.rs:283-313
        const JsonValue& parts = root.at("particles");
        if (parts.kind != JsonValue::Array) throw Error(CS_ERR_PARSE, "'particles' must be an array");
        for (const JsonValue& pt : parts.arr) {
            std::string name = pt.at("name").as_string("name");
            std::string to = pt.at("to_region").as_string("to_region");
            bool lg = pt.at("logging").as_bool("logging");
            bool rs = pt.at("is_reservoir").as_bool("is_reservoir");
            if (pt.has("count")) {
                uint64_t c = pt.at("count").as_u64("count");
                add_particle_count(name, to, (uint32_t)c, lg, rs);
            } else if (pt.has("concentration")) {
                add_particle_concentration(name, to, (float)pt.at("concentration").as_number("concentration"), lg, rs);
            } else {
                throw Error(CS_ERR_PARSE, "Particle must have count or concentration");
            }
            if (pt.has("diffusion_rate")) {
                const JsonValue& dm = pt.at("diffusion_rate");
                if (dm.kind != JsonValue::Object) throw Error(CS_ERR_PARSE, "'diffusion_rate' must be an object");
                for (auto& kv : dm.obj) set_diffusion_rate_particle(name, kv.first, (float)kv.second.as_number("diffusion_rate"));
            }
        }
        // reactions, src/simulation.rs:315-356 (object keys in byte order)
        if (root.has("reactions")) {
            const JsonValue& rx = root.at("reactions");
            if (rx.kind != JsonValue::Object) throw Error(CS_ERR_PARSE, "'reactions' must be an object");
            for (auto& kv : rx.obj) {
                float k = (float)kv.second.as_number("reaction rate");
                std::vector<std::string> re, pr;
                bool before = true;
                std::istringstream ss(kv.first);
                std::string tok;
                while (ss >> tok) {
                    float nk;
                    if (parse_rust_f32(tok, nk)) { k = k * nk; continue; }
                    if (tok == "->") before = false;
                    else if (tok == "+") {}
                    else (before ? re : pr).push_back(tok);
                }
                add_reaction(re, pr, k);
            }
        }
    } catch (const Error&) {
        throw;
    } catch (const std::runtime_error& e) {
        throw Error(CS_ERR_PARSE, e.what());
    }
}

// Move probability D[src][dst][q] * tau / (lambda * lambda) in binary32, the
// expression of rdme.wgsl:132-136, evaluated once per table entry.
void compute_ref_probabilities(const Model& m, std::vector<float>& P) {
    uint32_t nr = m.nr, s1 = m.np;
    P.resize((size_t)nr * nr * s1);
    float l2 = m.lambda * m.lambda;
    for (uint32_t a = 0; a < nr; a++)
        for (uint32_t b = 0; b < nr; b++)
            for (uint32_t q = 0; q < s1; q++) {
                float num = m.diffusion[((size_t)a * nr + b) * s1 + q] * m.tau;
                P[((size_t)a * nr + b) * s1 + q] = num / l2;
            }
}

}  // namespace cellsim
