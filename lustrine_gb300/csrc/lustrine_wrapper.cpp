// lustrine_wrapper.cpp -- the reference's C entry points for the fluid path
// (Lustrine::Wrapper, src/LustrineWrapper.hpp:86-171) over one process-global
// simulation, as in the reference (LustrineWrapper.hpp:82).
//
// Scene construction follows the reference exactly, because the particle
// order it produces is the order simulation_bind_positions_copy returns:
//   sand grids   -> particles 0..n-1, each grid walked x -> y -> z
//                   (init_chunk_from_grid, Lustrine.cpp:676-722);
//   solid grids  -> stored from the end of the allocation backwards
//                   (Lustrine.cpp:174-235 / 465-527), so the solid id order
//                   (ascending storage index) is the reverse of creation order.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "lustrine_gb300.h"
#include "vox.h"

namespace {

lustrine_pbf* g_ctx = nullptr;
int g_status = LUSTRINE_OK;
int g_num_sand = 0;
int g_num_solid = 0;
float g_cell_size = 0.0f;

// Particle sources and sinks (Simulation::source / sink, Lustrine.cpp:745-861,
// 916-1017), host-side bookkeeping around the device step.
struct Source {
    std::vector<float> pattern;  // init_chunk_from_grid positions of the pattern grid
    float dir[3];                // normalised at creation
    float freq;
    int capacity, spawned = 0;
    float timer = 0.0f;
    bool state = true;
};
struct Sink {
    std::vector<int> cells;  // ascending cell ids of the box
    float freq;
    int despawned = 0;  // never incremented, as in the reference (Lustrine.cpp:812-816)
    float timer = 0.0f;
    bool state = true;
};
std::vector<Source> g_sources;
std::vector<Sink> g_sinks;
float g_total_time = 0.0f;
int g_remaining = 0;  // Simulation::num_remaining_sand_particles
float g_radius = 0.0f, g_diameter = 0.0f;
float g_gravity[3] = {0.0f, 0.0f, 0.0f};
float g_domain[3] = {0.0f, 0.0f, 0.0f};
int g_grid[3] = {0, 0, 0};

// init_chunk_from_grid (Lustrine.cpp:676-722).  The chunk holds
// num_occupied * sub^3 entries; cells skipped by the mask leave (0, 0, 0)
// entries at the end, as in the reference.
void chunk_positions(const GridWrapper& g, float cell_size, int sub, bool mask_out,
                     std::vector<float>& out) {
    const long long num = (long long)g.num_occupied_grid_cells * sub * sub * sub;
    const size_t base = out.size();
    out.resize(base + 3 * (size_t)std::max(num, 0LL), 0.0f);
    const float off = cell_size * 0.5f;
    const int X = g.X * sub, Y = g.Y * sub, Z = g.Z * sub;
    long long counter = 0;
    for (int x = 0; x < X; x++)
        for (int y = 0; y < Y; y++)
            for (int z = 0; z < Z; z++) {
                const int ci = (x / sub) * g.Y * g.Z + (y / sub) * g.Z + (z / sub);
                const int cell = g.cells ? g.cells[ci] : 0;
                if (cell && ((!mask_out) || cell != 1)) {
                    if (counter >= num) continue;  // occupancy beyond num_occupied: dropped
                    float* p = &out[base + 3 * (size_t)counter];
                    p[0] = (float)x * cell_size;
                    p[1] = (float)y * cell_size;
                    p[2] = (float)z * cell_size;
                    p[0] = p[0] + g.position.x;
                    p[1] = p[1] + g.position.y;
                    p[2] = p[2] + g.position.z;
                    p[0] = p[0] + off;
                    p[1] = p[1] + off;
                    p[2] = p[2] + off;
                    counter++;
                }
            }
}

void release() {
    if (g_ctx) lustrine_pbf_destroy(g_ctx);
    g_ctx = nullptr;
    g_num_sand = g_num_solid = 0;
    g_sources.clear();
    g_sinks.clear();
    g_total_time = 0.0f;
    g_remaining = 0;
}

// get_cell_indices (neighbors/Utils.hpp:13-21): clamp to [cell/2, domain -
// cell/2] (bounds formed in double, as glm::vec3(double) does), divide,
// truncate.
void cell_indices(const Vec3& p, int out[3]) {
    const float v[3] = {p.x, p.y, p.z};
    for (int a = 0; a < 3; a++) {
        const float lo = (float)((double)g_cell_size * 0.5);
        const float hi = (float)((double)g_domain[a] - (double)g_cell_size * 0.5);
        out[a] = (int)(std::min(std::max(v[a], lo), hi) / g_cell_size);
    }
}

// Lustrine::simulate (Lustrine.cpp:730-861): sources spawn before the step,
// sinks remove after it.
int simulate_frame(float dt) {
    const float dt_clamped = 0.016f;  // Lustrine.cpp:745
    for (Source& src : g_sources) src.timer += dt_clamped;
    for (Source& src : g_sources) {
        if (!(src.state && src.spawned < src.capacity && src.timer >= src.freq)) continue;
        const int num = (int)(src.pattern.size() / 3);
        if (g_remaining < num) continue;
        const float freq = src.freq;
        const float t_last = g_total_time;
        const float offset = freq - std::fmod(t_last, freq);
        const float speed = freq > 0.0f ? 1.0f * g_diameter / freq : 1.0f;
        // j = 0 of the reference's spawn loop: offset along the direction,
        // velocity direction * speed (+ gravity * 0)
        float off[3], vel[3];
        for (int a = 0; a < 3; a++) {
            const float zero = 0.0f * g_diameter * src.dir[a];
            off[a] = zero + src.dir[a] * offset;
            vel[a] = src.dir[a] * speed + g_gravity[a] * (0.0f * freq);
        }
        std::vector<float> x((size_t)num * 3), v((size_t)num * 3);
        for (int k = 0; k < num; k++)
            for (int a = 0; a < 3; a++) {
                x[3 * (size_t)k + a] = src.pattern[3 * (size_t)k + a] + off[a];
                v[3 * (size_t)k + a] = vel[a];
            }
        if (num > 0)  // Lustrine.cpp:790: a small perturbation against stacking
            for (int a = 0; a < 3; a++) v[3 * (size_t)(num / 2) + a] += 0.001f * 1.0f;
        const int rc = lustrine_pbf_spawn(g_ctx, x.data(), v.data(), num);
        if (rc) return rc;
        g_num_sand += num;
        g_remaining -= num;
        src.timer = 0.0f;
        src.spawned += num;
    }
    int rc = lustrine_pbf_step(g_ctx, dt);
    if (rc) return rc;
    std::vector<int> evict_cells;
    for (const Sink& sk : g_sinks)
        if (sk.state && sk.timer >= sk.freq) evict_cells.insert(evict_cells.end(), sk.cells.begin(), sk.cells.end());
    if (!evict_cells.empty()) {
        int removed = 0;
        rc = lustrine_pbf_despawn_cells(g_ctx, evict_cells.data(), (int)evict_cells.size(), &removed);
        if (rc) return rc;
        g_num_sand -= removed;
        g_remaining += removed;
    }
    for (Sink& sk : g_sinks) sk.timer += dt;
    g_total_time += dt_clamped;
    return LUSTRINE_OK;
}

void init_common(const SimulationParameters* prm, SimulationData* data, GridWrapper* sand, int num_sand,
                 GridWrapper* solid, int num_solid, int subdivision, float kernel_radius_scale,
                 bool mask_out) {
    g_status = LUSTRINE_OK;
    if (!prm || !data || num_sand < 0 || num_solid < 0 || (num_sand && !sand) ||
        (num_solid && !solid) || subdivision < 1) {
        // LustrineWrapper.cpp:177-180 prints and returns
        g_status = LUSTRINE_ERR_ARGS;
        return;
    }
    release();
    std::vector<float> xs, gen_solid;
    for (int i = 0; i < num_sand; i++) chunk_positions(sand[i], prm->particleDiameter, 1, false, xs);
    for (int i = 0; i < num_solid; i++)
        chunk_positions(solid[i], prm->particleDiameter, subdivision, mask_out, gen_solid);
    const int n = (int)(xs.size() / 3), ns = (int)(gen_solid.size() / 3);
    // storage order of solids: written from the end backwards
    std::vector<float> sol((size_t)ns * 3);
    for (int k = 0; k < ns; k++)
        for (int a = 0; a < 3; a++) sol[3 * (size_t)k + a] = gen_solid[3 * (size_t)(ns - 1 - k) + a];

    lustrine_pbf_params p;
    lustrine_pbf_params_reference(&p, prm->X, prm->Y, prm->Z, prm->particleRadius, kernel_radius_scale);
    // the step after init is simulate_sand (Lustrine.cpp:72,312)
    p.mode = LUSTRINE_MODE_SAND;
    // Lustrine.cpp:105-126,237: the allocation holds max(n + ns, X Y Z sub^3)
    // particles; sources may add num_remaining = total - 1 - ns - n of them
    // (room for them is reserved, up to 2^22 extra particles)
    const double guess = (double)prm->X * prm->Y * prm->Z * subdivision * subdivision * subdivision;
    const long long total = std::max<long long>((long long)n + ns, (long long)guess);
    const long long room = std::max<long long>(0, std::min<long long>(total - 1 - ns - n, 1LL << 22));
    int rc = lustrine_pbf_create(&p, n, ns, &g_ctx);
    if (!rc && room > 0) rc = lustrine_pbf_reserve(g_ctx, (int)(n + room));
    if (!rc) {  // simulate_sand's contact distance is the caller's particleDiameter
        lustrine_sand_controls c;
        lustrine_sand_controls_default(&c, prm->particleRadius);
        c.particle_diameter = prm->particleDiameter;
        rc = lustrine_pbf_set_sand_controls(g_ctx, &c);
    }
    if (!rc) rc = lustrine_pbf_upload(g_ctx, xs.data(), nullptr, sol.data());
    if (rc) {
        release();
        g_status = rc;
        return;
    }
    g_num_sand = n;
    g_num_solid = ns;
    g_cell_size = p.cell_size;
    g_remaining = (int)room;
    g_radius = prm->particleRadius;
    g_diameter = prm->particleDiameter;
    for (int a = 0; a < 3; a++) {
        g_gravity[a] = p.gravity[a];
        g_domain[a] = (float)p.domain[a];
        g_grid[a] = (int)(g_domain[a] / p.cell_size) + 1;
    }

    // Lustrine.cpp:105-126,208-217: index ranges of the reference's arrays
    long long solid_start = total - ns, solid_end = total;
    if (ns == 0) solid_start = solid_end = total - 1;  // Lustrine.cpp:219-222
    data->num_sand_particles = n;
    data->num_solid_particles = ns;
    data->start_sand_index = 0;
    data->end_sand_index = n;
    data->start_solid_index = (int)solid_start;
    data->end_solid_index = (int)solid_end;
}

}  // namespace

extern "C" {

void init_simulation(const SimulationParameters* parameters, SimulationData* data,
                     GridWrapper* sand_grids, int num_sand_grids, GridWrapper* solid_grids,
                     int num_solid_grids, int subdivision) {
    // Lustrine.cpp:188,253: kernel radius 3.1 r, solid cells equal to 1 masked out
    init_common(parameters, data, sand_grids, num_sand_grids, solid_grids, num_solid_grids, subdivision,
                3.1f, true);
}

void init_simulation_extra_parameters(const SimulationParameters* parameters, SimulationData* data,
                                      GridWrapper* sand_grids, int num_sand_grids,
                                      GridWrapper* solid_grids, int num_solid_grids, int subdivision,
                                      float kernel_radius_scale, int with_credits) {
    if (with_credits) {
        g_status = LUSTRINE_ERR_UNSUPPORTED;
        return;
    }
    init_common(parameters, data, sand_grids, num_sand_grids, solid_grids, num_solid_grids, subdivision,
                kernel_radius_scale, false);
}

// LustrineWrapper.cpp:342-346: the flags stay set for later simulate_no_flags
// calls; the sand step reads them (the fluid steps do not)
void simulate(float dt, bool attract_flag, bool blow_flag) {
    if (!g_ctx) {
        g_status = LUSTRINE_ERR_NO_SIMULATION;
        return;
    }
    lustrine_sand_controls c;
    lustrine_pbf_get_sand_controls(g_ctx, &c);
    c.attract_flag = attract_flag ? 1 : 0;
    c.blow_flag = blow_flag ? 1 : 0;
    g_status = lustrine_pbf_set_sand_controls(g_ctx, &c);
    if (!g_status) g_status = simulate_frame(dt);
}

void simulate_no_flags(float dt) { g_status = g_ctx ? simulate_frame(dt) : LUSTRINE_ERR_NO_SIMULATION; }

// The player's position for the sand step's attract and blow (the reference
// reads it from its Bullet world, which is not part of this library).
void lustrine_set_player_position(Vec3 position) {
    if (!g_ctx) {
        g_status = LUSTRINE_ERR_NO_SIMULATION;
        return;
    }
    lustrine_sand_controls c;
    lustrine_pbf_get_sand_controls(g_ctx, &c);
    c.player_position[0] = position.x;
    c.player_position[1] = position.y;
    c.player_position[2] = position.z;
    g_status = lustrine_pbf_set_sand_controls(g_ctx, &c);
}

// LustrineWrapper.cpp:679-703 / Lustrine.cpp:916-1017
int add_particle_source(GridWrapper* pattern, Vec3 direction, float freq, int capacity) {
    if (!g_ctx) {
        g_status = LUSTRINE_ERR_NO_SIMULATION;
        return -1;
    }
    if (!pattern) {
        g_status = LUSTRINE_ERR_ARGS;
        return -1;
    }
    Source src;
    chunk_positions(*pattern, g_diameter, 1, false, src.pattern);
    const float len = std::sqrt(direction.x * direction.x + direction.y * direction.y + direction.z * direction.z);
    src.dir[0] = direction.x / len;
    src.dir[1] = direction.y / len;
    src.dir[2] = direction.z / len;
    src.freq = freq;
    src.capacity = capacity < 0 ? 0x7fffffff : capacity;
    g_sources.push_back(src);
    g_status = LUSTRINE_OK;
    return (int)g_sources.size() - 1;
}

int add_particle_sink(Vec3 min_pos, Vec3 max_pos, float frequency) {
    if (!g_ctx) {
        g_status = LUSTRINE_ERR_NO_SIMULATION;
        return -1;
    }
    int lo[3], hi[3];
    cell_indices(min_pos, lo);
    cell_indices(max_pos, hi);
    Sink sk;
    sk.freq = frequency;
    for (int y = lo[1]; y <= hi[1]; y++)
        for (int x = lo[0]; x <= hi[0]; x++)
            for (int z = lo[2]; z <= hi[2]; z++) sk.cells.push_back(y * g_grid[0] * g_grid[2] + x * g_grid[2] + z);
    std::sort(sk.cells.begin(), sk.cells.end());
    g_sinks.push_back(sk);
    g_status = LUSTRINE_OK;
    return (int)g_sinks.size() - 1;
}

void set_source_state(int index, int state) {
    if (index < 0 || index >= (int)g_sources.size()) {
        g_status = LUSTRINE_ERR_ARGS;
        return;
    }
    g_sources[(size_t)index].state = state != 0;
    g_status = LUSTRINE_OK;
}

void set_sink_state(int index, int state) {
    if (index < 0 || index >= (int)g_sinks.size()) {
        g_status = LUSTRINE_ERR_ARGS;
        return;
    }
    g_sinks[(size_t)index].state = state != 0;
    g_status = LUSTRINE_OK;
}

int get_source_spawned(int index) {
    if (index < 0 || index >= (int)g_sources.size()) {
        g_status = LUSTRINE_ERR_ARGS;
        return 0;
    }
    g_status = LUSTRINE_OK;
    return g_sources[(size_t)index].spawned;
}

int get_sink_despawned(int index) {
    if (index < 0 || index >= (int)g_sinks.size()) {
        g_status = LUSTRINE_ERR_ARGS;
        return 0;
    }
    g_status = LUSTRINE_OK;
    return g_sinks[(size_t)index].despawned;
}

void simulation_bind_positions_copy(float* position_ptr) {
    if (!g_ctx) {
        g_status = LUSTRINE_ERR_NO_SIMULATION;
        return;
    }
    g_status = position_ptr ? lustrine_pbf_download(g_ctx, position_ptr, nullptr, nullptr, nullptr)
                            : LUSTRINE_ERR_ARGS;
}

void cleanup_simulation(void) {
    release();
    g_status = LUSTRINE_OK;
}

void init_grid_box(const SimulationParameters* parameters, GridWrapper* grid, int X, int Y, int Z,
                   Vec3 position, Color color, int type) {
    (void)parameters;
    if (!grid || X < 0 || Y < 0 || Z < 0) {
        g_status = LUSTRINE_ERR_ARGS;
        return;
    }
    // Lustrine.cpp:618-639 then grid_to_grid_wrapper (LustrineWrapper.cpp:116-139)
    const int cells = X * Y * Z;
    grid->cells = new int[cells > 0 ? cells : 1];
    for (int i = 0; i < cells; i++) grid->cells[i] = 1;
    grid->colors = nullptr;
    grid->color = color;
    grid->position = position;
    grid->has_one_color_per_cell = false;
    grid->X = X;
    grid->Y = Y;
    grid->Z = Z;
    grid->num_grid_cells = cells;
    grid->num_occupied_grid_cells = cells;
    grid->type = type;
    g_status = LUSTRINE_OK;
}

}  // extern "C"

namespace {

// The model as a grid in the reference's grid order (x -> y -> z,
// VoxelLoader.cpp:69-97): occupied cells hold the colour index (index_cells)
// or 1, colours are the palette colour / 255 in float (float_colors, glm's
// vec4 /= 255.0) or in double (LustrineWrapper.cpp:608-611).
void vox_to_grid(const lgb::VoxModel& m, bool index_cells, bool float_colors, GridWrapper* grid) {
    const int X = m.sx, Y = m.sy, Z = m.sz;
    const int cells = X * Y * Z;
    grid->cells = new int[cells > 0 ? cells : 1]();
    grid->colors = new Color[cells > 0 ? cells : 1]();
    grid->has_one_color_per_cell = true;
    grid->X = X;
    grid->Y = Y;
    grid->Z = Z;
    grid->num_grid_cells = cells;
    int occupied = 0;
    for (int x = 0; x < X; x++)
        for (int y = 0; y < Y; y++)
            for (int z = 0; z < Z; z++) {
                const int c = m.voxels[(size_t)x + (size_t)y * X + (size_t)z * X * Y];
                if (c == 0) continue;
                const int g = (x * Y * Z) + (y * Z) + z;
                const uint8_t* rgba = m.rgba[(c + 255) & 255];  // colour index c names entry c - 1
                grid->cells[g] = index_cells ? c : 1;
                float col[4];
                for (int a = 0; a < 4; a++)
                    col[a] = float_colors ? (float)rgba[a] / 255.0f : (float)((double)rgba[a] / 255.0);
                grid->colors[g] = Color{col[0], col[1], col[2], col[3]};
                occupied++;
            }
    grid->num_occupied_grid_cells = occupied;
}

}  // namespace

extern "C" {

void init_grid_magikavoxel(GridWrapper* grid, const char* path, Vec3 position) {
    lgb::VoxModel m;
    const int rc = grid && path ? lgb::vox_read_file(path, &m) : LUSTRINE_ERR_ARGS;
    if (!grid || m.voxels.empty()) {
        g_status = rc ? rc : LUSTRINE_ERR_ARGS;
        return;
    }
    vox_to_grid(m, true, true, grid);
    grid->type = 0;  // MaterialType SOLID (Simulation.hpp:28-31)
    grid->position = position;
    grid->color = Color{0.0f, 0.0f, 0.0f, 0.0f};
    g_status = rc;
}

void create_grid(GridWrapper* grid, const wchar_t* path, int type, int pathlen) {
    if (!grid || !path || pathlen < 0) {
        g_status = LUSTRINE_ERR_ARGS;
        return;
    }
    std::string narrow((size_t)pathlen, '\0');
    for (int i = 0; i < pathlen; i++) narrow[(size_t)i] = (char)path[i];  // LustrineWrapper.cpp:540-545
    lgb::VoxModel m;
    const int rc = lgb::vox_read_file(narrow.c_str(), &m);
    if (m.voxels.empty()) {
        g_status = rc ? rc : LUSTRINE_ERR_ARGS;
        return;
    }
    vox_to_grid(m, false, false, grid);
    grid->type = type;
    g_status = rc;
}

void lustrine_free_grid(GridWrapper* grid) {
    if (!grid) return;
    delete[] grid->cells;
    delete[] grid->colors;
    grid->cells = nullptr;
    grid->colors = nullptr;
}

int get_num_sand_particles(void) { return g_num_sand; }

int get_grid_cell_size(void) { return (int)g_cell_size; }

int query_cell_num_particles(Vec3 min, Vec3 max, bool include_solid) {
    if (!g_ctx) {
        g_status = LUSTRINE_ERR_NO_SIMULATION;
        return 0;
    }
    const float lo[3] = {min.x, min.y, min.z}, hi[3] = {max.x, max.y, max.z};
    int count = 0;
    g_status = lustrine_pbf_query_cell_count(g_ctx, lo, hi, include_solid ? 1 : 0, &count);
    return count;
}

void set_simulate_function(int index) {
    if (!g_ctx) {
        g_status = LUSTRINE_ERR_NO_SIMULATION;
        return;
    }
    if (index == 1) {
        // simulate_sand_v3 (LustrineWrapper.cpp:671-673), an in-place
        // Gauss-Seidel sweep over cell pairs, is not built here
        g_status = LUSTRINE_ERR_UNSUPPORTED;
        return;
    }
    if (index != 0 && index != 2 && index != 3) {
        g_status = LUSTRINE_ERR_ARGS;  // LustrineWrapper.cpp:674-675
        return;
    }
    lustrine_pbf_params p;
    lustrine_pbf_get_params(g_ctx, &p);
    // 0: simulate_sand (LustrineWrapper.cpp:668-670); 2, 3: the fluid steps
    p.mode = index == 0 ? LUSTRINE_MODE_SAND : index == 2 ? LUSTRINE_MODE_REFERENCE : LUSTRINE_MODE_PBF;
    g_status = lustrine_pbf_set_params(g_ctx, &p);
}

// LustrineWrapper.cpp:505-511: radii and coefficients of the sand step's
// attract and blow forces (Simulate.cpp:187-209), kept by the context until
// the next call
void set_attract_blow_parameters(float attract_radius, float blow_radius, float attract_coeff,
                                 float blow_coeff) {
    if (!g_ctx) {
        g_status = LUSTRINE_ERR_NO_SIMULATION;
        return;
    }
    lustrine_sand_controls c;
    lustrine_pbf_get_sand_controls(g_ctx, &c);
    c.attract_radius = attract_radius;
    c.blow_radius = blow_radius;
    c.attract_coeff = attract_coeff;
    c.blow_coeff = blow_coeff;
    g_status = lustrine_pbf_set_sand_controls(g_ctx, &c);
}

// LustrineWrapper.cpp:381-393.  The scene graph of a .vox file as JSON is
// not produced (it carries no particle data): the string comes back empty.
void read_vox_scene(BindingString* data, const uint8_t* buffer, int64_t size) {
    (void)buffer;
    (void)size;
    if (data) {
        data->length = 0;
        data->data = nullptr;
    }
    g_status = LUSTRINE_ERR_UNSUPPORTED;
}

void free_string(BindingString* data) {
    if (data) {
        delete[] data->data;
        data->length = 0;
        data->data = nullptr;
    }
    g_status = LUSTRINE_OK;
}

// LustrineWrapper.cpp:713-719: a host allocation of 10^9 bytes held until
// test_deallocate_1gb (the reference's probe of the host allocator).
static char* g_test_block = nullptr;

void test_allocate_1gb(void) {
    if (!g_test_block) g_test_block = new (std::nothrow) char[1000000000];
    g_status = g_test_block ? LUSTRINE_OK : LUSTRINE_ERR_NOMEM;
}

void test_deallocate_1gb(void) {
    delete[] g_test_block;
    g_test_block = nullptr;
    g_status = LUSTRINE_OK;
}

// The Bullet rigid-body world and the player (LustrineWrapper.hpp:132-157,
// 173-182) are not part of this library: every call records
// LUSTRINE_ERR_UNSUPPORTED and returns zero values, so a binding that
// declares them loads and runs.
static Vec3 unsupported_vec3() {
    g_status = LUSTRINE_ERR_UNSUPPORTED;
    return Vec3{0.0f, 0.0f, 0.0f};
}
static int unsupported_int() {
    g_status = LUSTRINE_ERR_UNSUPPORTED;
    return 0;
}
static float unsupported_float() {
    g_status = LUSTRINE_ERR_UNSUPPORTED;
    return 0.0f;
}

Vec3 get_gravity(void) { return unsupported_vec3(); }
void set_gravity(Vec3) { unsupported_int(); }
int add_box(Vec3, bool, Vec3) { return unsupported_int(); }
int add_capsule(Vec3, float, float) { return unsupported_int(); }
int add_detector_block(Vec3, Vec3) { return unsupported_int(); }
int check_collision(int, int) { return unsupported_int(); }
int do_collide(int) { return unsupported_int(); }
int do_collide_except_for(int, int) { return unsupported_int(); }
void check_collisions(int, int* indices, int* size) {
    (void)indices;
    if (size) *size = 0;
    unsupported_int();
}
int get_num_bodies(void) { return unsupported_int(); }
void apply_impulse(int, Vec3, Vec3) { unsupported_int(); }
Vec3 get_position(int) { return unsupported_vec3(); }
Vec3 get_velocity(int) { return unsupported_vec3(); }
void set_velocity(int, Vec3) { unsupported_int(); }
void set_position(int, Vec3) { unsupported_int(); }
void add_velocity(int, Vec3) { unsupported_int(); }
void set_body_no_rotation(int) { unsupported_int(); }
void set_body_frixion(int, float) { unsupported_int(); }
float get_body_frixion(int) { return unsupported_float(); }
void set_body_damping(int, float, float) { unsupported_int(); }
float get_body_damping(int) { return unsupported_float(); }
void set_player_id(int) { unsupported_int(); }
void set_player_box_scale(Vec3) { unsupported_int(); }
int is_grounded(int) { return unsupported_int(); }
void set_body_gravity(int, Vec3) { unsupported_int(); }
void set_body_no_collision_response(int) { unsupported_int(); }
int collide_with_player(int) { return unsupported_int(); }
void enable_particles_bounding_boxes(void) { unsupported_int(); }
void disable_particles_bounding_boxes(void) { unsupported_int(); }
void set_player_particles_bounding_spheres_radius_placement(float) { unsupported_int(); }

int lustrine_last_status(void) { return g_status; }

struct lustrine_pbf* lustrine_global_context(void) { return g_ctx; }

}  // extern "C"
