// ref_shim.cpp -- link stubs for building the reference's fluid path on its own.
// TEST INFRASTRUCTURE (oracle/_ref only).
//
// The reference's Simulation embeds a Bullet world (Simulation.hpp:138) and its
// lifecycle calls Bullet and the rdtsc profiler.  The fluid step never reads
// anything Bullet computes: simulate_bullet (BulletPhysics.cpp:163-174) only
// reads sand positions.  These stubs stand in for the Bullet library and the
// x86-only timer so the hot-path sources link without building Bullet.
#include "BulletPhysics.hpp"
#include "profiling/Profiling.hpp"

#include <cstdlib>

namespace Lustrine {
namespace Profiling {
long long raw_cycles[LUSTRINE_MAX_NUM_MEASUREMENTS];
double raw_durations[LUSTRINE_MAX_NUM_MEASUREMENTS];
}  // namespace Profiling

namespace Bullet {
void init_bullet(Simulation*) {}
void clean_bullet(Simulation*) {}
void simulate_bullet(Simulation*, float, int, int) {}
int add_box(Simulation* s, glm::vec3, bool) { return s->num_bodies++; }
void allocate_particles_colliders(Simulation*, int, float) {}
void bind_foreign_sand_positions(Simulation* s, glm::vec3* p) { s->foreign_sand_positions = p; }
void print_resume(const Simulation*) {}
}  // namespace Bullet
}  // namespace Lustrine

void init_tsc() {}
myInt64 start_tsc(void) { return 0; }
myInt64 stop_tsc(myInt64) { return 0; }

void* btAlignedAllocInternal(size_t size, int alignment)
{
    void* p = nullptr;
    if (posix_memalign(&p, alignment < (int)sizeof(void*) ? sizeof(void*) : (size_t)alignment, size)) return nullptr;
    return p;
}
void btAlignedFreeInternal(void* ptr) { free(ptr); }
const char* btTypedConstraint::serialize(void*, btSerializer*) const { return nullptr; }
