/*
 * pbf_oracle.h -- CPU oracle for the Lustrine position-based-fluid step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the tests, the
 * smoke entry and the CPU-baseline leg of the benchmark call it to produce the
 * expected answer.  The product path (lustrine_gb300/, liblustrine_gb300.so)
 * never links, loads or calls it.
 *
 * Two step semantics are restated here, both in plain C:
 *
 *  Mode R ("reference-compatible"): the reference's own fluid step,
 *    src/Simulate.cpp:27-115 (simulate_fluid) with its neighbour search
 *    src/neighbors/Neighbors.cpp:366-450 (find_neighbors_uniform_grid),
 *    the cell mapping src/neighbors/Utils.hpp:24-33 (get_cell_id) and the
 *    cubic kernel src/Kernels.cpp:6-41.  Every float operation is done in
 *    the order the reference does it, so that (compiled with
 *    -ffp-contract=off) the result is bit-identical to the reference's own
 *    build with the same flags.  Options: Jacobi instead of the reference's
 *    in-place Gauss-Seidel update of positions_star (Simulate.cpp:96,103),
 *    and a per-axis clamp of the cell coordinates (the reference does not
 *    clamp, Utils.hpp:25,31, and overflows its cell table once a particle
 *    leaves the grid).
 *
 *  Mode P ("PBF"): the position-based-fluids solver of Macklin & Mueller
 *    (2013) that the reference's parameters describe but its step does not
 *    implement: N solver iterations, poly6 density and spiky gradient
 *    (the kernels of src/Kernels.cpp:43-67, normalised for support h and
 *    with the gradient pointing away from the neighbour), the s_corr
 *    tensile term (Simulate.cpp:7-9), a clamp to the box, static solid
 *    particles as neighbours plus a push-out constraint, XSPH viscosity
 *    (Simulation.hpp:170, declared but unused by the reference) and the
 *    velocity update.  Restated for T = double (the FP64 oracle) and
 *    T = float.
 *
 * Particle ids: fluid particles are 0..n-1, solid particles n..n+ns-1 in the
 * reference's storage order (Simulation::positions[ptr_solid_start + k] is
 * solid id n + k, Lustrine.cpp:491-508).  All vectors are packed xyz float
 * (or double) triples, the 12-byte stride of glm::vec3.
 */
#ifndef LUSTRINE_PBF_ORACLE_H
#define LUSTRINE_PBF_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    ORC_OK = 0,
    ORC_ERR_CELL_RANGE = 1,   /* a particle's cell id left [0, num_cells) */
    ORC_ERR_CAPACITY = 2,     /* a neighbour list exceeded the caller's capacity */
    ORC_ERR_ARGS = 3,
    ORC_ERR_NOMEM = 4
};

typedef struct orc_params {
    float domain[3];          /* Simulation::domainX/Y/Z (Simulation.hpp:153-155) */
    int grid[3];              /* gridX, gridY, gridZ (Lustrine.cpp:553-555) */
    float cell_size;          /* = kernel_radius (Lustrine.cpp:546) */
    float particle_radius;
    float kernel_radius;      /* h = kernel_radius_scale * radius (Lustrine.cpp:545) */
    float kernel_factor;      /* 0.5 (Simulation.hpp:147) */
    float cubic_k, cubic_l;   /* Lustrine.cpp:549-551 */
    float rest_density;
    float mass;
    float gravity[3];
    float relaxation_epsilon;
    float s_corr_dq, s_corr_k, s_corr_n;
    float c_xsph;             /* mode P only */
    float solid_contact;      /* mode P: push-out distance to a solid particle */
    int iterations;           /* mode P: solver iterations per step */
    int clamp_cells;          /* clamp cell coordinates per axis */
    int jacobi;               /* mode R: 1 = Jacobi, 0 = the reference's Gauss-Seidel */
} orc_params;

/* Fill the derived fields the way init_simulation_extra_parameters does
 * (Lustrine.cpp:383-387,543-555): h = scale * radius, cell = h, cubic
 * constants with pi in double, grid = (int)(domain / cell) + 1.  The
 * physical parameters take the reference's defaults (Simulation.hpp:147-171). */
void orc_params_reference(orc_params* p, int X, int Y, int Z, float particle_radius,
                          float kernel_radius_scale);

/* Sorting::counting_sort (src/neighbors/Sorting.cpp:12-34): stable counting
 * sort of keys[0..n) in [0, num_cells).  counts must hold num_cells + 1 ints.
 * sorted[k] receives the index of the k-th smallest key (ties in input order). */
void orc_counting_sort(int* counts, const int* keys, size_t n, size_t num_cells, int* sorted);

/* Cell id of a position (Utils.hpp:24-33), with the optional per-axis clamp.
 * Returns the id; *in_range is 0 if the id is outside [0, num_cells). */
int orc_cell_id(const orc_params* p, const float pos[3], int* in_range);

/* ---------------------------------------------------------------- mode R -- */

/* One call of simulate_fluid (Simulate.cpp:27-115) on n fluid particles and
 * ns static solids.  x, xs, v: 3n floats, updated in place.  solid: 3ns floats.
 * lambdas: n + ns floats indexed by id; entries >= n are read (the reference
 * indexes lambdas by list position, Simulate.cpp:97) and must be zero.
 * nbr_count (n ints) and nbr_idx (n * cap ints, row i = particle i) receive the
 * neighbour lists in the reference's order when non-NULL.  Returns ORC_*. */
int orc_compat_step(const orc_params* p, float dt, int n, int ns,
                    float* x, float* xs, float* v, const float* solid,
                    float* lambdas, int* nbr_count, int* nbr_idx, int cap);

/* Neighbour lists only (Neighbors.cpp:366-450) at positions xs, with the same
 * outputs as above. */
int orc_compat_neighbors(const orc_params* p, int n, int ns, const float* xs,
                         const float* solid, int* nbr_count, int* nbr_idx, int cap);

/* ---------------------------------------------------------------- mode P -- */

/* One PBF step (predict, neighbours, p->iterations x (lambda, delta-p with
 * s_corr, solid push-out and box clamp), velocity update, XSPH, commit).
 * density: n entries, the density of each fluid particle in the last
 * iteration's lambda pass (may be NULL).  lambdas: n entries (may be NULL).
 * nbr_count: n ints (may be NULL). */
int orc_pbf_step_d(const orc_params* p, double dt, int n, int ns,
                   double* x, double* v, const double* solid,
                   double* lambdas, double* density, int* nbr_count);
int orc_pbf_step_f(const orc_params* p, float dt, int n, int ns,
                   float* x, float* v, const float* solid,
                   float* lambdas, float* density, int* nbr_count);

/* Poly6 density of every fluid particle at positions xs (fluid) and solid,
 * in double.  This is the FP64 reference the mixed-precision step's density
 * error is measured against. */
int orc_pbf_density_d(const orc_params* p, int n, int ns, const double* xs,
                      const double* solid, double* density);

/* Mode P lambda pass alone at positions xs (no prediction): density and
 * lambda of every fluid particle, in double. */
int orc_pbf_lambda_d(const orc_params* p, int n, int ns, const double* xs,
                     const double* solid, double* lambdas, double* density);

/* ----------------------------------------------------------------- sand -- */

/* The inputs of simulate_sand that are not in orc_params: the player's
 * position (BulletPhysicsSimulation::player_position), the attract and blow
 * flags of this call and of the previous one (the reference keeps the
 * previous flag in a function static, Simulate.cpp:185), their radii and
 * coefficients (Simulation.hpp:239-242) and SimulationParameters's
 * particleDiameter (Lustrine.cpp:544). */
typedef struct orc_sand_controls {
    float player_position[3];
    int attract_flag, blow_flag, prev_attract_flag;
    float attract_radius, blow_radius, attract_coeff, blow_coeff;
    float particle_diameter;
} orc_sand_controls;

/* One call of simulate_sand (Simulate.cpp:156-325) on n sand particles and
 * ns static particles: integration with attract and blow, the stable
 * counting sort by cell that permutes x, v and attracted in place
 * (find_neighbors_uniform_grid_v1, Neighbors.cpp:262-361), 4 Jacobi
 * contact/friction substeps each followed by the box clamp, the velocity
 * update.  x, v: 3n floats; attracted: n ints; solid: 3ns floats.
 * nbr_count / nbr_idx (n * cap, row-major; may be NULL) receive the
 * reference's lists in its push order, itself included twice, static
 * particle k as n + k.  xs_sorted (3n floats, may be NULL) receives the
 * predicted positions in the sorted order, the positions the step binned
 * (the cells its sinks read).  Returns ORC_*. */
int orc_sand_step(const orc_params* p, const orc_sand_controls* ctl, float dt, int n, int ns,
                  float* x, float* v, int* attracted, const float* solid,
                  int* nbr_count, int* nbr_idx, int cap, float* xs_sorted);

#ifdef __cplusplus
}
#endif

#endif
