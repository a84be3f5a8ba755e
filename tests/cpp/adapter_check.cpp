// Compile-and-link check of the C++ step adapters (fluid and sand) against a struct with the
// reference Simulation's field names and types (src/Simulation.hpp:135-251),
// or against the reference header itself when built with -DWITH_REFERENCE.
// Assigning the adapter to a Simulate_fun-typed pointer checks the signature.
#ifdef WITH_REFERENCE
#include "Lustrine.hpp"
using Sim = Lustrine::Simulation;
#else
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
    float domainX = 40, domainY = 40, domainZ = 40;
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
#endif
#include "lustrine_gb300_sim.hpp"

int main() {
    void (*step)(Sim*, float) = lustrine_gb300::simulate_fluid<Sim>;
    void (*sand)(Sim*, float) = lustrine_gb300::simulate_sand<Sim>;
    return step != nullptr && sand != nullptr && lustrine_gb300::last_status() == LUSTRINE_OK ? 0 : 1;
}
