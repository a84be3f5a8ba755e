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
#include <vector>

#include "lustrine_gb300.h"

namespace {

lustrine_pbf* g_ctx = nullptr;
int g_status = LUSTRINE_OK;
int g_num_sand = 0;
int g_num_solid = 0;
float g_cell_size = 0.0f;

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
    int rc = lustrine_pbf_create(&p, n, ns, &g_ctx);
    if (!rc) rc = lustrine_pbf_upload(g_ctx, xs.data(), nullptr, sol.data());
    if (rc) {
        release();
        g_status = rc;
        return;
    }
    g_num_sand = n;
    g_num_solid = ns;
    g_cell_size = p.cell_size;

    // Lustrine.cpp:105-126,208-217: index ranges of the reference's arrays
    const double guess = (double)prm->X * prm->Y * prm->Z * subdivision * subdivision * subdivision;
    const long long total = std::max<long long>((long long)n + ns, (long long)guess);
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

void simulate(float dt, bool attract_flag, bool blow_flag) {
    (void)attract_flag;
    (void)blow_flag;
    g_status = g_ctx ? lustrine_pbf_step(g_ctx, dt) : LUSTRINE_ERR_NO_SIMULATION;
}

void simulate_no_flags(float dt) { g_status = g_ctx ? lustrine_pbf_step(g_ctx, dt) : LUSTRINE_ERR_NO_SIMULATION; }

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
    if (index == 0 || index == 1) {
        // simulate_sand / simulate_sand_v3 (LustrineWrapper.cpp:668-673) are not built here
        g_status = LUSTRINE_ERR_UNSUPPORTED;
        return;
    }
    if (index != 2 && index != 3) {
        g_status = LUSTRINE_ERR_ARGS;  // LustrineWrapper.cpp:674-675
        return;
    }
    lustrine_pbf_params p;
    lustrine_pbf_get_params(g_ctx, &p);
    p.mode = index == 2 ? LUSTRINE_MODE_REFERENCE : LUSTRINE_MODE_PBF;
    g_status = lustrine_pbf_set_params(g_ctx, &p);
}

int lustrine_last_status(void) { return g_status; }

struct lustrine_pbf* lustrine_global_context(void) { return g_ctx; }

}  // extern "C"
