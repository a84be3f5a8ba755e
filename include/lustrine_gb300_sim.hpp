// lustrine_gb300_sim.hpp -- the GB300 fluid and sand steps behind the
// reference's C++ step hook.
//
// The reference steps a Simulation through a function pointer,
// Simulation::simulate_fun (src/Simulation.hpp:22,137), called by
// Lustrine::simulate (src/Lustrine.cpp:803); its fluid step is
// Lustrine::simulate_fluid(Simulation*, float) (src/Simulate.hpp:12).
// lustrine_gb300::simulate_fluid<Simulation> has that signature:
//
//     #include "Lustrine.hpp"
//     #include "lustrine_gb300_sim.hpp"
//     sim.simulate_fun = lustrine_gb300::simulate_fluid<Lustrine::Simulation>;
//     Lustrine::simulate(&sim, dt);      // now steps on the GPU
//
// It reads and writes the Simulation fields the reference step uses, with
// the reference's layout (glm::vec3 arrays of 3 floats, sand in
// [ptr_sand_start, ptr_sand_end), solids in [ptr_solid_start, ptr_solid_end),
// Simulation.hpp:173-208) and its parameters (Simulation.hpp:144-171).  The
// header needs only those field names, so it compiles against the
// reference's Simulation or any struct with the same fields.
//
// Each call uploads positions and velocities of the sand range, runs one
// reference-semantics step (Jacobi position update) on the GPU and writes
// positions, positions_star, velocities and lambdas back.  The device
// context of a Simulation is created on its first call (solids are uploaded
// then: they are static in the fluid step) and kept until
// lustrine_gb300::release(sim); when the sand count changes (the reference's
// sources and sinks run on the host around the step) the context takes the
// new count, growing its buffers by doubling.  Errors are reported by last_status(), the
// step itself returning void like the reference's.
//
// lustrine_gb300::simulate_sand<Simulation> stands for Lustrine::simulate_sand
// (src/Simulate.cpp:156-325), the step init_simulation_extra_parameters selects
// (src/Lustrine.cpp:312).  Besides positions and velocities it uploads the
// attract flags (Simulation::attracted) and reads the attract/blow flags, radii,
// coefficients, particleDiameter and the player's position
// (bullet_physics_simulation.player_position); it writes back positions,
// positions_star, velocities and attracted in the order the step leaves them
// (re-sorted by cell, as the reference's step re-orders its arrays).
#pragma once

#include <cstring>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "lustrine_gb300.h"

namespace lustrine_gb300 {

namespace detail {
struct Entry {
    lustrine_pbf* ctx = nullptr;
    int n = 0, ns = 0, cap = 0;
    bool prev_attract = false;  // simulate_sand's previous attract flag (a re-created context forgets it)
};
inline std::unordered_map<const void*, Entry>& table() {
    static std::unordered_map<const void*, Entry> t;
    return t;
}
inline std::mutex& table_mutex() {
    static std::mutex m;
    return m;
}
inline int& status() {
    static thread_local int s = LUSTRINE_OK;
    return s;
}

template <class Simulation>
lustrine_pbf_params params_of(const Simulation* sim) {
    lustrine_pbf_params p;
    lustrine_pbf_params_reference(&p, (int)sim->domainX, (int)sim->domainY, (int)sim->domainZ,
                                  sim->particleRadius, sim->kernelRadius / sim->particleRadius);
    p.kernel_radius = sim->kernelRadius;
    p.kernel_factor = sim->kernelFactor;
    p.cell_size = sim->cell_size;
    p.rest_density = sim->rest_density;
    p.mass = sim->mass;
    p.gravity[0] = sim->gravity.x;
    p.gravity[1] = sim->gravity.y;
    p.gravity[2] = sim->gravity.z;
    p.relaxation_epsilon = sim->relaxation_epsilon;
    p.s_corr_dq = sim->s_corr_dq;
    p.s_corr_k = sim->s_corr_k;
    p.s_corr_n = sim->s_corr_n;
    p.mode = LUSTRINE_MODE_REFERENCE;
    return p;
}

// The device context of sim for mode p, holding the sand range's x and v
// (created on the first call, re-created when the solids change or the sand
// outgrows it, re-parameterised and re-counted otherwise).  Returns a status.
template <class Simulation>
int acquire(Simulation* sim, const lustrine_pbf_params& p, int n, int ns, float* x, float* v, Entry* out) {
    Entry e;
    {
        std::lock_guard<std::mutex> lock(table_mutex());
        e = table()[sim];
    }
    int rc = LUSTRINE_OK;
    if (e.ctx && (e.ns != ns || n > e.cap)) {  // solids changed, or more sand than the buffers hold
        std::lock_guard<std::mutex> lock(table_mutex());
        lustrine_pbf_destroy(e.ctx);
        e.ctx = nullptr;
    }
    if (!e.ctx) {
        // sources add sand between steps (Lustrine.cpp:745-800): room for growth
        const int cap = n > e.cap ? (e.cap ? (n > 2 * e.cap ? n : 2 * e.cap) : n) : e.cap;
        rc = lustrine_pbf_create(&p, n, ns, &e.ctx);
        if (!rc && cap > n) rc = lustrine_pbf_reserve(e.ctx, cap);
        const float* solid = ns ? reinterpret_cast<const float*>(sim->positions) + 3 * (size_t)sim->ptr_solid_start
                                : nullptr;
        if (!rc) rc = lustrine_pbf_upload(e.ctx, x, v, solid);
        if (rc) {
            if (e.ctx) lustrine_pbf_destroy(e.ctx);
            std::lock_guard<std::mutex> lock(table_mutex());
            table().erase(sim);
            return rc;
        }
        e.n = n;
        e.ns = ns;
        e.cap = cap > n ? cap : n;
    } else {
        // the game may change parameters between steps (ImGui sliders do,
        // experiments/fluid/fluid.cpp:176-189); unchanged ones keep the
        // captured step graphs
        lustrine_pbf_params cur;
        lustrine_pbf_get_params(e.ctx, &cur);
        lustrine_pbf_params want = p;
        want.use_graph = cur.use_graph;
        want.max_neighbors = cur.max_neighbors;  // the list capacity is fixed at creation
        if (std::memcmp(&cur, &want, sizeof(want)) != 0) rc = lustrine_pbf_set_params(e.ctx, &want);
        if (!rc && n != e.n) {  // sand added or removed by the host since the last step
            rc = lustrine_pbf_set_count(e.ctx, n);
            e.n = n;
        }
        if (!rc) rc = lustrine_pbf_upload_state_async(e.ctx, x, v);
    }
    std::lock_guard<std::mutex> lock(table_mutex());
    table()[sim] = e;
    *out = e;
    return rc;
}
}  // namespace detail

// Outcome of the last simulate_fluid call on this thread.
inline int last_status() { return detail::status(); }

// Free the device context of a Simulation (call before its arrays go away).
template <class Simulation>
void release(const Simulation* sim) {
    std::lock_guard<std::mutex> lock(detail::table_mutex());
    auto it = detail::table().find(sim);
    if (it != detail::table().end()) {
        lustrine_pbf_destroy(it->second.ctx);
        detail::table().erase(it);
    }
}

template <class Simulation>
void simulate_fluid(Simulation* sim, float dt) {
    const int start = sim->ptr_sand_start, end = sim->ptr_sand_end;
    const int n = end > start ? end - start : 0;
    const int ns = sim->ptr_solid_end > sim->ptr_solid_start ? sim->ptr_solid_end - sim->ptr_solid_start : 0;
    float* x = reinterpret_cast<float*>(sim->positions) + 3 * (size_t)start;
    float* v = reinterpret_cast<float*>(sim->velocities) + 3 * (size_t)start;
    detail::Entry e;
    int rc = detail::acquire(sim, detail::params_of(sim), n, ns, x, v, &e);
    if (!rc) rc = lustrine_pbf_step(e.ctx, dt);
    std::vector<float> lam((size_t)n);
    if (!rc) rc = lustrine_pbf_download(e.ctx, x, v, n ? lam.data() : nullptr, nullptr);
    if (!rc) {
        // Simulate.cpp:31-32,111: time_step holds the clamped dt; x* = x after the step
        sim->time_step = dt < 0.001f ? 0.001f : (dt > 0.01f ? 0.01f : dt);
        std::memcpy(reinterpret_cast<float*>(sim->positions_star) + 3 * (size_t)start, x,
                    sizeof(float) * 3 * (size_t)n);
        for (int i = 0; i < n && (size_t)(start + i) < sim->lambdas.size(); i++) sim->lambdas[start + i] = lam[i];
    }
    detail::status() = rc;
}

template <class Simulation>
void simulate_sand(Simulation* sim, float dt) {
    const int start = sim->ptr_sand_start, end = sim->ptr_sand_end;
    const int n = end > start ? end - start : 0;
    const int ns = sim->ptr_solid_end > sim->ptr_solid_start ? sim->ptr_solid_end - sim->ptr_solid_start : 0;
    float* x = reinterpret_cast<float*>(sim->positions) + 3 * (size_t)start;
    float* v = reinterpret_cast<float*>(sim->velocities) + 3 * (size_t)start;
    lustrine_pbf_params p = detail::params_of(sim);
    p.mode = LUSTRINE_MODE_SAND;
    p.max_neighbors = 96;
    detail::Entry e;
    int rc = detail::acquire(sim, p, n, ns, x, v, &e);
    if (!rc) {  // Simulate.cpp:183-209 inputs
        lustrine_sand_controls c;
        lustrine_sand_controls_default(&c, sim->particleRadius);
        const auto& pl = sim->bullet_physics_simulation.player_position;
        c.player_position[0] = pl.x;
        c.player_position[1] = pl.y;
        c.player_position[2] = pl.z;
        c.attract_flag = sim->attract_flag ? 1 : 0;
        c.blow_flag = sim->blow_flag ? 1 : 0;
        c.attract_radius = sim->attract_radius;
        c.blow_radius = sim->blow_radius;
        c.attract_coeff = sim->attract_coeff;
        c.blow_coeff = sim->blow_coeff;
        c.particle_diameter = sim->particleDiameter;
        rc = lustrine_pbf_set_sand_controls(e.ctx, &c);
    }
    // Simulate.cpp:188-190: the flags drop when attraction stops
    if (!rc && e.prev_attract && !sim->attract_flag)
        for (int i = 0; i < n; i++) sim->attracted[start + i] = 0;
    if (!rc && n) rc = lustrine_pbf_set_attracted(e.ctx, sim->attracted + start);
    if (!rc) rc = lustrine_pbf_step(e.ctx, dt);
    if (!rc) rc = lustrine_pbf_download(e.ctx, x, v, nullptr, nullptr);
    if (!rc && n) rc = lustrine_pbf_get_attracted(e.ctx, sim->attracted + start);
    if (!rc) {
        sim->time_step = dt;  // Simulate.cpp:170
        std::memcpy(reinterpret_cast<float*>(sim->positions_star) + 3 * (size_t)start, x,
                    sizeof(float) * 3 * (size_t)n);
        std::lock_guard<std::mutex> lock(detail::table_mutex());
        detail::table()[sim].prev_attract = sim->attract_flag;
    }
    detail::status() = rc;
}

}  // namespace lustrine_gb300
