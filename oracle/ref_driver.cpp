// ref_driver.cpp -- C entry points that drive the reference's own fluid step
// (compiled from the reference tree by `make -C oracle ref`).  TEST
// INFRASTRUCTURE: used to pin the C restatement and to write golden fixtures.
//
// Scene set-up follows the reference's C ABI path: init_grid_box
// (Lustrine.cpp:618-639) for the sand block, caller-given occupancy grids for
// solids, then init_simulation_extra_parameters (Lustrine.cpp:299-589) and
// Lustrine::simulate (Lustrine.cpp:730-861) with simulate_fun = simulate_fluid.
#include "Lustrine.hpp"
#include "Simulate.hpp"
#include "neighbors/Sorting.hpp"

#include <cstring>
#include <vector>

using namespace Lustrine;

static Simulation* g_sim = nullptr;

extern "C" {

void ref_free()
{
    if (g_sim) {
        clean_simulation(g_sim);
        delete g_sim;
        g_sim = nullptr;
    }
}

int ref_init(int X, int Y, int Z, float radius, float scale,
             int sbx, int sby, int sbz, const float* spos,
             int n_solid, const int* solid_dims, const float* solid_pos, const int* solid_cells)
{
    ref_free();
    SimulationParameters prm;
    prm.X = X; prm.Y = Y; prm.Z = Z;
    prm.particleRadius = radius;
    prm.particleDiameter = 2.0f * radius;
    std::vector<Grid> sand(1), solid((size_t)n_solid);
    init_grid_box(&prm, &sand[0], sbx, sby, sbz, glm::vec3(spos[0], spos[1], spos[2]),
                  glm::vec4(1.0f), SAND);
    size_t off = 0;
    for (int g = 0; g < n_solid; g++) {
        int gx = solid_dims[3 * g], gy = solid_dims[3 * g + 1], gz = solid_dims[3 * g + 2];
        init_grid_box(&prm, &solid[g], gx, gy, gz,
                      glm::vec3(solid_pos[3 * g], solid_pos[3 * g + 1], solid_pos[3 * g + 2]),
                      glm::vec4(1.0f), SOLID);
        int occ = 0;
        for (int c = 0; c < gx * gy * gz; c++) {
            solid[g].cells[c] = solid_cells[off + c];
            occ += solid_cells[off + c] != 0;
        }
        solid[g].num_occupied_grid_cells = occ;
        off += (size_t)gx * gy * gz;
    }
    g_sim = new Simulation();
    init_simulation_extra_parameters(&prm, g_sim, sand, solid, 1, scale, false);
    g_sim->simulate_fun = simulate_fluid;
    // The reference zeroes only the first bytes of velocities
    // (Lustrine.cpp:534); every oracle and fixture defines them as zero.
    memset(g_sim->velocities, 0, sizeof(glm::vec3) * (size_t)g_sim->ptr_solid_ordered_start);
    return g_sim->num_sand_particles;
}

void ref_set_params(float rest_density, float mass, const float* gravity, float eps,
                    float dq, float k, float n)
{
    g_sim->rest_density = rest_density;
    g_sim->mass = mass;
    g_sim->gravity = glm::vec3(gravity[0], gravity[1], gravity[2]);
    g_sim->relaxation_epsilon = eps;
    g_sim->s_corr_dq = dq;
    g_sim->s_corr_k = k;
    g_sim->s_corr_n = n;
}

// which: 0 sand start, 1 sand end, 2 solid start, 3 solid end, 4 total allocated,
// 5 num sand, 6 num solid, 7..9 grid dims, 10 num grid cells
long long ref_info(int which)
{
    switch (which) {
    case 0: return g_sim->ptr_sand_start;
    case 1: return g_sim->ptr_sand_end;
    case 2: return g_sim->ptr_solid_start;
    case 3: return g_sim->ptr_solid_end;
    case 4: return (long long)g_sim->total_allocated;
    case 5: return g_sim->num_sand_particles;
    case 6: return g_sim->num_solid_particles;
    case 7: return g_sim->gridX;
    case 8: return g_sim->gridY;
    case 9: return g_sim->gridZ;
    case 10: return g_sim->num_grid_cells;
    default: return -1;
    }
}

// f: kernelRadius, cell_size, cubic_kernel_k, cubic_kernel_l, kernelFactor, particleRadius
void ref_get_floats(float* f)
{
    f[0] = g_sim->kernelRadius;
    f[1] = g_sim->cell_size;
    f[2] = g_sim->cubic_kernel_k;
    f[3] = g_sim->cubic_kernel_l;
    f[4] = g_sim->kernelFactor;
    f[5] = g_sim->particleRadius;
}

void ref_set_state(const float* x, const float* v)
{
    int n = g_sim->ptr_sand_end;
    for (int i = 0; i < n; i++) {
        g_sim->positions[i] = glm::vec3(x[3 * i], x[3 * i + 1], x[3 * i + 2]);
        g_sim->positions_star[i] = g_sim->positions[i];
        g_sim->velocities[i] = glm::vec3(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
    }
}

void ref_get_state(float* x, float* xs, float* v, float* lam)
{
    int n = g_sim->ptr_sand_end;
    for (int i = 0; i < n; i++)
        for (int a = 0; a < 3; a++) {
            if (x) x[3 * i + a] = g_sim->positions[i][a];
            if (xs) xs[3 * i + a] = g_sim->positions_star[i][a];
            if (v) v[3 * i + a] = g_sim->velocities[i][a];
        }
    if (lam)
        for (int i = 0; i < n; i++) lam[i] = g_sim->lambdas[i];
}

void ref_get_solids(float* s)
{
    int k = 0;
    for (int i = g_sim->ptr_solid_start; i < g_sim->ptr_solid_end; i++, k++)
        for (int a = 0; a < 3; a++) s[3 * k + a] = g_sim->positions[i][a];
}

void ref_step(float dt) { Lustrine::simulate(g_sim, dt); }

// 0: simulate_fluid, 1: simulate_sand (the wrapper's set_simulate_function(0))
void ref_set_step_function(int which)
{
    g_sim->simulate_fun = which == 1 ? simulate_sand : simulate_fluid;
}

// simulate_sand's inputs outside SimulationParameters (Simulation.hpp:230-242,
// BulletPhysicsSimulation::player_position; the stubbed Bullet step leaves
// the player where it is set here).  The previous call's attract flag is a
// function static inside simulate_sand and cannot be set.
void ref_set_sand_controls(const float* player, int attract_flag, int blow_flag, float attract_radius,
                           float blow_radius, float attract_coeff, float blow_coeff)
{
    g_sim->bullet_physics_simulation.player_position = glm::vec3(player[0], player[1], player[2]);
    g_sim->attract_flag = attract_flag != 0;
    g_sim->blow_flag = blow_flag != 0;
    g_sim->attract_radius = attract_radius;
    g_sim->blow_radius = blow_radius;
    g_sim->attract_coeff = attract_coeff;
    g_sim->blow_coeff = blow_coeff;
}

void ref_get_attracted(int* out)
{
    for (int i = 0; i < g_sim->ptr_sand_end; i++) out[i] = g_sim->attracted[i];
}

void ref_set_attracted(const int* in)
{
    for (int i = 0; i < g_sim->ptr_sand_end; i++) g_sim->attracted[i] = in[i];
}

// Lustrine::init_grid_from_magika_voxel (VoxelLoader.cpp:48-99): dims[3]
// (X, Y, Z), cells[X*Y*Z], colors[4*X*Y*Z] in the grid's x -> y -> z order.
// Returns the occupied cell count, or -1 when the grid exceeds cap cells.
int ref_load_vox(const char* path, int* dims, int* cells, float* colors, int cap)
{
    Grid g;
    init_grid_from_magika_voxel(&g, path, glm::vec3(0.0f), SOLID);
    dims[0] = g.X;
    dims[1] = g.Y;
    dims[2] = g.Z;
    if (g.num_grid_cells > cap) return -1;
    for (int i = 0; i < g.num_grid_cells; i++) {
        cells[i] = g.cells[(size_t)i];
        for (int a = 0; a < 4; a++) colors[4 * i + a] = g.colors[(size_t)i][a];
    }
    return g.num_occupied_grid_cells;
}

// which: 0 particleDiameter, 1 mass
float ref_get_float(int which) { return which == 0 ? g_sim->particleDiameter : g_sim->mass; }

// Neighbour lists of the last step, solid indices mapped to n + (i - ptr_solid_start).
int ref_neighbors(int* count, int* idx, int cap)
{
    int n = g_sim->ptr_sand_end, rc = 0;
    for (int i = 0; i < n; i++) {
        const std::vector<int>& L = g_sim->neighbors[i];
        count[i] = (int)L.size();
        for (size_t k = 0; k < L.size(); k++) {
            if ((int)k >= cap) { rc = 2; break; }
            int j = L[k];
            idx[(size_t)i * cap + k] = j < g_sim->ptr_sand_end ? j : n + (j - g_sim->ptr_solid_start);
        }
    }
    return rc;
}

void ref_counting_sort(int* counts, int* keys, size_t n, size_t num_cells, int* sorted)
{
    Sorting::counting_sort(counts, keys, n, num_cells, sorted);
}

}  // extern "C"
