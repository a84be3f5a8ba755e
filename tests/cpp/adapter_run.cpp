// Runs the C++ step adapter (include/lustrine_gb300_sim.hpp) on a struct with
// the reference Simulation's field names through a sequence of steps while
// the sand count changes between them (as the reference's sources and sinks
// change ptr_sand_end on the host), writing every step's input and output
// state to a file:
//   repeated: int n, int ns, float x_in[3n], v_in[3n], solid[3ns], x_out[3n], v_out[3n]
// With a second argument "sand" it runs simulate_sand, the player attracting
// in steps 1-2 and blowing in step 3, and each record adds the attract flags
// before (int att_in[n]) and after (int att_out[n]) the step.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

struct vec3 {
    float x, y, z;
};
struct Bullet {
    vec3 player_position{0, 0, 0};
};
struct Sim {
    void (*simulate_fun)(Sim*, float) = nullptr;
    float particleRadius = 0.5f, particleDiameter = 1.0f, kernelRadius = 1.0f, kernelFactor = 0.5f,
          cell_size = 1.0f;
    float domainX = 24, domainY = 24, domainZ = 24;
    float rest_density = 24, mass = 5;
    vec3 gravity{0, -10, 0};
    float time_step = 0.01f, relaxation_epsilon = 10, s_corr_dq = 0.5f, s_corr_k = 1, s_corr_n = 4;
    vec3* velocities = nullptr;
    std::vector<float> lambdas;
    vec3* positions = nullptr;
    vec3* positions_star = nullptr;
    int ptr_sand_start = 0, ptr_sand_end = 0, ptr_solid_start = 0, ptr_solid_end = 0;
    Bullet bullet_physics_simulation;
    bool attract_flag = false, blow_flag = false;
    int* attracted = nullptr;
    float attract_radius = 1.5f, blow_radius = 2.0f, attract_coeff = 1000.0f, blow_coeff = 500.0f;
};

#include "lustrine_gb300_sim.hpp"

static unsigned lcg = 12345u;
static float jitter() {
    lcg = lcg * 1664525u + 1013904223u;
    return ((lcg >> 8) * (1.0f / 16777216.0f) - 0.5f) * 0.1f;
}

static void add_block(Sim& s, int X, int Y, int Z, float ox, float oy, float oz) {
    for (int x = 0; x < X; x++)
        for (int y = 0; y < Y; y++)
            for (int z = 0; z < Z; z++) {
                const int i = s.ptr_sand_end++;
                s.positions[i] = vec3{ox + x + 0.5f + jitter(), oy + y + 0.5f + jitter(), oz + z + 0.5f + jitter()};
                s.velocities[i] = vec3{0, 0, 0};
            }
}

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    const bool sand = argc > 2 && std::strcmp(argv[2], "sand") == 0;
    const int total = 4096, ns = 24 * 24;
    std::vector<vec3> pos(total), pstar(total), vel(total);
    std::vector<int> att(total, 0);
    Sim s;
    s.attracted = att.data();
    s.bullet_physics_simulation.player_position = vec3{10.0f, 8.0f, 10.0f};
    s.positions = pos.data();
    s.positions_star = pstar.data();
    s.velocities = vel.data();
    s.lambdas.assign(total, 0.0f);
    s.ptr_solid_start = total - ns;
    s.ptr_solid_end = total;
    for (int x = 0; x < 24; x++)
        for (int z = 0; z < 24; z++) pos[(size_t)(total - ns + x * 24 + z)] = vec3{x + 0.5f, 0.5f, z + 0.5f};
    add_block(s, 8, 8, 8, 6, 4, 6);
    s.simulate_fun = sand ? lustrine_gb300::simulate_sand<Sim> : lustrine_gb300::simulate_fluid<Sim>;
    FILE* f = std::fopen(argv[1], "wb");
    if (!f) return 2;
    // step; step; +10 (grows past 512); step; -30 (set_count); step; +600 (grows again); step
    for (int k = 0; k < 5; k++) {
        if (k == 2) add_block(s, 1, 1, 10, 2, 20, 2);
        if (k == 3) s.ptr_sand_end -= 30;
        if (k == 4) add_block(s, 10, 6, 10, 12, 14, 2);
        const int n = s.ptr_sand_end;
        std::fwrite(&n, sizeof(int), 1, f);
        std::fwrite(&ns, sizeof(int), 1, f);
        std::fwrite(pos.data(), sizeof(vec3), (size_t)n, f);
        std::fwrite(vel.data(), sizeof(vec3), (size_t)n, f);
        std::fwrite(pos.data() + (total - ns), sizeof(vec3), (size_t)ns, f);
        s.attract_flag = k == 1 || k == 2;
        s.blow_flag = k == 3;
        if (sand) std::fwrite(att.data(), sizeof(int), (size_t)n, f);
        s.simulate_fun(&s, 1.0f / 60.0f);
        if (lustrine_gb300::last_status() != LUSTRINE_OK) {
            std::fprintf(stderr, "step %d: status %d\n", k, lustrine_gb300::last_status());
            return 1;
        }
        std::fwrite(pos.data(), sizeof(vec3), (size_t)n, f);
        std::fwrite(vel.data(), sizeof(vec3), (size_t)n, f);
        if (sand) std::fwrite(att.data(), sizeof(int), (size_t)n, f);
    }
    std::fclose(f);
    lustrine_gb300::release(&s);
    return 0;
}
