/*
 * lustrine_gb300.h -- C ABI of the GB300 position-based-fluid step.
 *
 * Two layers, both plain C (pointers and sizes; no CUDA or C++ types):
 *
 * 1. The reference's C entry points for the fluid path, same names, argument
 *    layouts and void returns as Lustrine::Wrapper (src/LustrineWrapper.hpp),
 *    over a process-global simulation, so a game binding that loads the
 *    reference's LustrineWrapper library can load this one instead.  Each
 *    records its outcome for lustrine_last_status().
 *
 * 2. lustrine_pbf_*: a context API with explicit state (arrays in, arrays
 *    out, status codes), used by layer 1 and by callers that hold their own
 *    particle arrays -- the C++ Simulation adapter in lustrine_gb300_sim.hpp,
 *    the tests and the benchmark.
 *
 * Threading: one context is driven from one host thread at a time; steps are
 * asynchronous on the context's CUDA stream and every download synchronises.
 */
#ifndef LUSTRINE_GB300_H
#define LUSTRINE_GB300_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define LUSTRINE_API __attribute__((visibility("default")))
#else
#define LUSTRINE_API
#endif

/* ------------------------------------------------------------------ status */
enum {
    LUSTRINE_OK = 0,
    LUSTRINE_ERR_ARGS = 1,           /* invalid argument */
    LUSTRINE_ERR_CUDA = 2,           /* a CUDA runtime call failed */
    LUSTRINE_ERR_NOMEM = 3,          /* device or host allocation failed */
    LUSTRINE_ERR_NBR_OVERFLOW = 4,   /* a neighbour list exceeded max_neighbors */
    LUSTRINE_ERR_CELL_RANGE = 5,     /* reference mode: a particle left the grid (clamped) */
    LUSTRINE_ERR_UNSUPPORTED = 6,    /* option not provided by this build */
    LUSTRINE_ERR_NO_SIMULATION = 7,  /* wrapper call before init_simulation */
    LUSTRINE_ERR_TIMEOUT = 8,        /* a bounded device wait gave up */
    LUSTRINE_ERR_BAD_VALUE = 9,      /* non-finite particle state */
    LUSTRINE_ERR_TOO_LARGE = 10      /* input larger than a fixed limit (a no-allocation entry
                                        point's scratch, or a context's reserved capacity) */
};

enum {
    LUSTRINE_MODE_REFERENCE = 0, /* simulate_fluid semantics (Simulate.cpp:27-115), Jacobi update */
    LUSTRINE_MODE_PBF = 1,       /* PBF: iterations, poly6/spiky, s_corr, solids, box, XSPH */
    LUSTRINE_MODE_SAND = 2       /* simulate_sand semantics (Simulate.cpp:156-325): contact and
                                    friction substeps; the particles are re-ordered by cell every
                                    step, as the reference does (Neighbors.cpp:296-300) */
};

enum {
    LUSTRINE_PRECISION_FP32 = 0,  /* absolute fp32 positions */
    LUSTRINE_PRECISION_MIXED = 1, /* int cell index + fp32 offset, Kahan density (PBF mode): the
                                     iterations work on offsets from each particle's cell, every
                                     pair adding its cell difference */
    LUSTRINE_PRECISION_MIXED_SCENE = 2 /* the same stored state (cell index + fp32 offset), Kahan
                                     density; the iterations work in fp32 on positions relative to
                                     the scene's box corner (PBF mode, dense grid, boxes of at most
                                     256 cells a side: a resolution of at most 2^-15 cell) */
};

/* ------------------------------------------------- layer 1: reference ABI */
/* Layouts of Lustrine::SimulationParameters (src/Simulation.hpp:83-92) and
 * Lustrine::Wrapper::{SimulationData, Color, Vec3, GridWrapper}
 * (src/LustrineWrapper.hpp:30-74). */
typedef struct SimulationParameters {
    int X, Y, Z;
    float particleRadius;
    float particleDiameter;
} SimulationParameters;

typedef struct SimulationData {
    int num_sand_particles;
    int num_solid_particles;
    int start_sand_index;
    int end_sand_index;
    int start_solid_index;
    int end_solid_index;
} SimulationData;

typedef struct Color {
    float r, g, b, a;
} Color;

typedef struct Vec3 {
    float x, y, z;
} Vec3;

typedef struct GridWrapper {
    int* cells;
    Color* colors;
    Color color;
    Vec3 position;
    bool has_one_color_per_cell;
    int X;
    int Y;
    int Z;
    int num_grid_cells;
    int num_occupied_grid_cells;
    int type; /* 0 solid, 1 sand (Simulation.hpp:28-32) */
} GridWrapper;

/* LustrineWrapper.hpp:86-94 / LustrineWrapper.cpp:165-221.  Builds the scene
 * with the reference's init_simulation layout (kernel radius 3.1 r, solid
 * cells whose value is 1 masked out, Lustrine.cpp:188,253).  The step after
 * init is the sand step (simulate_sand, as the reference's init selects,
 * Lustrine.cpp:72,312); set_simulate_function(2) or (3) selects a fluid step. */
LUSTRINE_API void init_simulation(const SimulationParameters* parameters, SimulationData* data,
                                  GridWrapper* sand_grids, int num_sand_grids,
                                  GridWrapper* solid_grids, int num_solid_grids, int subdivision);
/* LustrineWrapper.hpp:97-107 / LustrineWrapper.cpp:223-282 (kernel radius =
 * kernel_radius_scale * r, Lustrine.cpp:545).  with_credits is not supported
 * (the credits text is a sand-solver feature) and records LUSTRINE_ERR_UNSUPPORTED. */
LUSTRINE_API void init_simulation_extra_parameters(const SimulationParameters* parameters,
                                                   SimulationData* data, GridWrapper* sand_grids,
                                                   int num_sand_grids, GridWrapper* solid_grids,
                                                   int num_solid_grids, int subdivision,
                                                   float kernel_radius_scale, int with_credits);
/* LustrineWrapper.cpp:343-351: one frame of the selected step (sources, the
 * step, sinks, as Lustrine::simulate).  The attract/blow flags are kept for
 * later simulate_no_flags calls; the sand step reads them (attract towards and
 * blow away from the player, Simulate.cpp:187-209), the fluid steps do not. */
LUSTRINE_API void simulate(float dt, bool attract_flag, bool blow_flag);
LUSTRINE_API void simulate_no_flags(float dt);
/* LustrineWrapper.cpp:377-379: copies 3 * num_sand_particles floats of
 * particle positions.  Order: after a sand step, the order of that step's cell
 * sort (the reference's sand step re-orders its particle arrays by cell every
 * step, Neighbors.cpp:296-300, and returns them in that order); after a fluid
 * step, the order init_simulation created them in (sources append).
 * Synchronises. */
LUSTRINE_API void simulation_bind_positions_copy(float* position_ptr);
/* LustrineWrapper.cpp:353-375 */
LUSTRINE_API void cleanup_simulation(void);
/* LustrineWrapper.cpp:336-341 + Lustrine.cpp:618-639: fills grid with an
 * X * Y * Z block; allocates grid->cells with new[] like the reference (the
 * caller owns it; free with lustrine_free_grid). */
LUSTRINE_API void init_grid_box(const SimulationParameters* parameters, GridWrapper* grid, int X,
                                int Y, int Z, Vec3 position, Color color, int type);
/* LustrineWrapper.cpp:142-144 */
LUSTRINE_API int get_num_sand_particles(void);
/* LustrineWrapper.cpp:705-707 (returns the float cell size converted to int) */
LUSTRINE_API int get_grid_cell_size(void);
/* LustrineWrapper.hpp:162-169 / LustrineWrapper.cpp:679-703, Lustrine.cpp:916-1017:
 * particle sources and sinks, run by simulate around each step as
 * Lustrine::simulate does (Lustrine.cpp:745-861): a source's timer grows by
 * 0.016 per call; when it reaches freq (and the source is on, below its
 * capacity, with room left) the pattern grid's particles are appended at the
 * pattern positions shifted along the normalised direction by
 * freq - fmod(total_time, freq), with velocity direction * 2r / freq (the
 * middle particle + 0.001 per axis); after the step every sink whose timer
 * (+= dt per call, never reset) reached its frequency evicts the particles
 * binned in its cells (lustrine_pbf_despawn_cells).  Room for spawned
 * particles: the reference's allocation, max(n + ns, X Y Z sub^3) - 1 - ns
 * - n, reserved up to 2^22.  get_sink_despawned returns the reference's
 * counter, which it never increments (0).  Index arguments out of range
 * record LUSTRINE_ERR_ARGS. */
LUSTRINE_API int add_particle_source(GridWrapper* pattern, Vec3 direction, float freq, int capacity);
LUSTRINE_API int add_particle_sink(Vec3 min_pos, Vec3 max_pos, float frequency);
LUSTRINE_API void set_source_state(int index, int state);
LUSTRINE_API void set_sink_state(int index, int state);
LUSTRINE_API int get_source_spawned(int index);
LUSTRINE_API int get_sink_despawned(int index);
/* LustrineWrapper.hpp:184 / LustrineWrapper.cpp:288-291: particles in the
 * cells of the box [min, max] after the last step (lustrine_pbf_query_cell_count). */
LUSTRINE_API int query_cell_num_particles(Vec3 min, Vec3 max, bool include_solid);
/* LustrineWrapper.cpp:666-677.  0 selects simulate_sand (also the step after
 * init, Lustrine.cpp:72,312); 1, the reference's simulate_sand_v3, is not
 * provided (LUSTRINE_ERR_UNSUPPORTED, step unchanged); 2 selects the fluid
 * step with reference semantics; 3 the PBF step. */
LUSTRINE_API void set_simulate_function(int index);
/* The player's position read by the sand step's attract and blow
 * (the reference takes it from its Bullet world; new entry point). */
LUSTRINE_API void lustrine_set_player_position(Vec3 position);
/* LustrineWrapper.hpp:158 / LustrineWrapper.cpp:505-511: radii and
 * coefficients of the sand step's attract and blow forces (defaults 1.5, 2,
 * 1000, 500, Simulation.hpp), kept until the next call. */
LUSTRINE_API void set_attract_blow_parameters(float attract_radius, float blow_radius,
                                              float attract_coeff, float blow_coeff);

/* LustrineWrapper.hpp:76-79 */
typedef struct BindingString {
    int64_t length;
    char* data;
} BindingString;
/* LustrineWrapper.hpp:120-121 / LustrineWrapper.cpp:381-393.  read_vox_scene
 * (a .vox scene graph as JSON for the game; no particle data) is not built:
 * it returns an empty string (length 0, data NULL) and records
 * LUSTRINE_ERR_UNSUPPORTED.  free_string releases a string's data. */
LUSTRINE_API void read_vox_scene(BindingString* data, const uint8_t* buffer, int64_t size);
LUSTRINE_API void free_string(BindingString* data);
/* LustrineWrapper.hpp:187-188 / LustrineWrapper.cpp:713-719: allocate and
 * release a 10^9-byte host block (the reference's allocator probe);
 * LUSTRINE_ERR_NOMEM when the allocation fails. */
LUSTRINE_API void test_allocate_1gb(void);
LUSTRINE_API void test_deallocate_1gb(void);
/* The Bullet rigid-body world and the player (LustrineWrapper.hpp:132-157,
 * 173-182): not part of this library (they never change particle state, the
 * fluid and sand steps take the player's position as an input instead).  Each
 * records LUSTRINE_ERR_UNSUPPORTED and returns zero (check_collisions sets
 * *size to 0), so a binding that declares them loads and runs. */
LUSTRINE_API Vec3 get_gravity(void);
LUSTRINE_API void set_gravity(Vec3 new_gravity);
LUSTRINE_API int add_box(Vec3 position, bool is_dynamic, Vec3 half_dimensions);
LUSTRINE_API int add_capsule(Vec3 position, float radius, float height);
LUSTRINE_API int add_detector_block(Vec3 position, Vec3 half_dims);
LUSTRINE_API int check_collision(int body1, int body2);
LUSTRINE_API int do_collide(int body);
LUSTRINE_API int do_collide_except_for(int body, int exception_id);
LUSTRINE_API void check_collisions(int body, int* indices, int* size);
LUSTRINE_API int get_num_bodies(void);
LUSTRINE_API void apply_impulse(int body, Vec3 impulse, Vec3 relative_pos);
LUSTRINE_API Vec3 get_position(int body);
LUSTRINE_API Vec3 get_velocity(int body);
LUSTRINE_API void set_velocity(int body, Vec3 velocity);
LUSTRINE_API void set_position(int body, Vec3 position);
LUSTRINE_API void add_velocity(int body, Vec3 velocity);
LUSTRINE_API void set_body_no_rotation(int body);
LUSTRINE_API void set_body_frixion(int body, float frixion);
LUSTRINE_API float get_body_frixion(int body);
LUSTRINE_API void set_body_damping(int body, float linear, float angular);
LUSTRINE_API float get_body_damping(int body);
LUSTRINE_API void set_player_id(int id);
LUSTRINE_API void set_player_box_scale(Vec3 scale);
LUSTRINE_API int is_grounded(int id);
LUSTRINE_API void set_body_gravity(int id, Vec3 gravity);
LUSTRINE_API void set_body_no_collision_response(int id);
LUSTRINE_API int collide_with_player(int id);
LUSTRINE_API void enable_particles_bounding_boxes(void);
LUSTRINE_API void disable_particles_bounding_boxes(void);
LUSTRINE_API void set_player_particles_bounding_spheres_radius_placement(float radius);

/* Outcome of the last layer-1 call (LUSTRINE_OK or an error code). */
LUSTRINE_API int lustrine_last_status(void);
/* The context behind the layer-1 simulation (NULL before init_simulation). */
struct lustrine_pbf;
LUSTRINE_API struct lustrine_pbf* lustrine_global_context(void);
/* LustrineWrapper.cpp:146-151 with VoxelLoader.cpp:48-99: the first model of
 * the MagicaVoxel file at path (the first one with a voxel) as a SOLID grid at
 * position, in the grid order x -> y -> z: cells hold the voxels' colour
 * indices (0: empty), colors the palette colours / 255 (float division),
 * has_one_color_per_cell set, color zero (the reference leaves it unset).
 * A file without an RGBA palette chunk or with an index map (IMAP) gives the
 * grid with zero colours and LUSTRINE_ERR_UNSUPPORTED; a missing file or one
 * with no voxel, LUSTRINE_ERR_ARGS and the grid untouched. */
LUSTRINE_API void init_grid_magikavoxel(GridWrapper* grid, const char* path, Vec3 position);
/* LustrineWrapper.cpp:537-624: the same model with cells 1 for occupied
 * voxels, colors the palette colours / 255 divided in double, the given type;
 * position and color are left as the caller set them.  path holds pathlen wide
 * characters, each narrowed to one byte as the reference does.  (The
 * reference allocates the cells with sizeof(bool) per cell and overruns them;
 * here they are int arrays of num_grid_cells.) */
LUSTRINE_API void create_grid(GridWrapper* grid, const wchar_t* path, int type, int pathlen);
/* Frees what init_grid_box, init_grid_magikavoxel and create_grid allocated in grid. */
LUSTRINE_API void lustrine_free_grid(GridWrapper* grid);

/* --------------------------------------------------- layer 2: context API */
typedef struct lustrine_pbf_params {
    int mode;                 /* LUSTRINE_MODE_* */
    int precision;            /* LUSTRINE_PRECISION_* */
    int domain[3];            /* box X, Y, Z (Simulation::domainX/Y/Z) */
    float particle_radius;
    float kernel_radius;      /* h */
    float kernel_factor;      /* reference cubic kernel scale, 0.5 */
    float cell_size;          /* grid cell; the reference uses h */
    float rest_density;
    float mass;
    float gravity[3];
    float relaxation_epsilon;
    float s_corr_dq;          /* s_corr distance (absolute) */
    float s_corr_k;
    float s_corr_n;
    float c_xsph;             /* PBF mode */
    float solid_contact;      /* PBF mode: push-out distance to solid particles */
    int iterations;           /* PBF mode: solver iterations per step */
    int max_neighbors;        /* neighbour list capacity per particle (reference defaults: 512) */
    int clamp_cells;          /* reference mode: clamp cell coordinates to the grid */
    int use_graph;            /* replay each step from a captured CUDA graph */
    int grid_mode;            /* LUSTRINE_GRID_*: dense cell table or hashed cells (PBF mode) */
} lustrine_pbf_params;

enum {
    LUSTRINE_GRID_AUTO = 0,   /* dense unless the box has far more cells than particles */
    LUSTRINE_GRID_DENSE = 1,  /* one table entry per cell of the box */
    LUSTRINE_GRID_HASHED = 2  /* 2^k hash buckets (k from the particle count); any box size */
};

typedef struct lustrine_pbf lustrine_pbf;

/* Parameters of init_simulation_extra_parameters (Lustrine.cpp:543-555) with
 * the reference's physical defaults (Simulation.hpp:147-171). */
LUSTRINE_API void lustrine_pbf_params_reference(lustrine_pbf_params* p, int X, int Y, int Z,
                                                float particle_radius, float kernel_radius_scale);

LUSTRINE_API int lustrine_pbf_create(const lustrine_pbf_params* p, int n_fluid, int n_solid,
                                     lustrine_pbf** out);
LUSTRINE_API int lustrine_pbf_destroy(lustrine_pbf* s);
/* A batch of independent scenes stepped together (PBF mode): scene k has the
 * box domains[3k..3k+2], n_fluid[k] fluid and n_solid[k] solid particles
 * (n_solid may be NULL: none).  Same physics for all scenes (p; p->domain is
 * ignored).  The returned context works with every lustrine_pbf_* call;
 * particle ids run scene after scene (upload and download concatenate the
 * scenes in order, each in its own box coordinates).  One step advances all
 * scenes with one launch per stage. */
LUSTRINE_API int lustrine_batch_create(const lustrine_pbf_params* p, int num_scenes, const int* domains,
                                       const int* n_fluid, const int* n_solid, lustrine_pbf** out);
/* How a batch runs the part of its step after the cell sort (no counterpart
 * in the reference, which has no batches).
 * LUSTRINE_SOLVER_STAGES (the default): one launch per stage and pass for all
 * scenes.
 * LUSTRINE_SOLVER_ONCHIP: one persistent launch of thread-block clusters of
 * 16 CTAs that take bins of scenes from a work queue; a scene's lists,
 * iterations, XSPH and commit run out of its cluster's distributed shared
 * memory (4,096 particles per CTA, scenes of up to 65,536).  It applies to
 * PBF batches on a dense grid without static particles and with
 * max_neighbors <= 255 (in mixed precision, boxes of at most 256 cells a
 * side), on a GPU that runs such clusters; elsewhere set_solver(ONCHIP)
 * returns LUSTRINE_ERR_UNSUPPORTED.  In fp32 both give the same bits; in
 * mixed precision the on-chip solve iterates on positions relative to the
 * scene's box corner and commits cell + offset.  The autotuner times both. */
enum { LUSTRINE_SOLVER_STAGES = 0, LUSTRINE_SOLVER_ONCHIP = 1 };
LUSTRINE_API int lustrine_batch_set_solver(lustrine_pbf* s, int solver);
LUSTRINE_API int lustrine_batch_get_solver(const lustrine_pbf* s, int* solver);
/* The on-chip solve's launch: clusters of the persistent grid (0: the solve
 * does not apply to this batch), bins of scenes in its work queue, threads
 * per CTA (512 or 1024; the 4,096 particles of a CTA are dealt to them). */
LUSTRINE_API int lustrine_batch_onchip_layout(const lustrine_pbf* s, int* clusters, int* bins, int* threads);
LUSTRINE_API int lustrine_batch_set_onchip_threads(lustrine_pbf* s, int threads);
/* Change parameters (same precision, domain, cell size, grid mode and
 * max_neighbors as at create; the mode may change -- entering sand mode
 * from another mode clears the attract flags). */
LUSTRINE_API int lustrine_pbf_set_params(lustrine_pbf* s, const lustrine_pbf_params* p);
LUSTRINE_API int lustrine_pbf_get_params(const lustrine_pbf* s, lustrine_pbf_params* p);
LUSTRINE_API int lustrine_pbf_counts(const lustrine_pbf* s, int* n_fluid, int* n_solid);

/* State in: x, v as 3 * n_fluid floats (v may be NULL: zero), solid as
 * 3 * n_solid floats in the reference's storage order (solid id n_fluid + k).
 * _device: the pointers are device memory.  Both copy; the caller keeps
 * ownership. */
LUSTRINE_API int lustrine_pbf_upload(lustrine_pbf* s, const float* x, const float* v,
                                     const float* solid);
LUSTRINE_API int lustrine_pbf_upload_device(lustrine_pbf* s, const float* x, const float* v,
                                            const float* solid);
/* Fluid state only (x, v), host memory, asynchronous when the buffers are
 * page-locked. */
LUSTRINE_API int lustrine_pbf_upload_state_async(lustrine_pbf* s, const float* x, const float* v);

/* Advance by dt (asynchronous on the context stream). */
LUSTRINE_API int lustrine_pbf_step(lustrine_pbf* s, float dt);
LUSTRINE_API int lustrine_pbf_steps(lustrine_pbf* s, float dt, int count);
LUSTRINE_API int lustrine_pbf_synchronize(lustrine_pbf* s);

/* State out, in the caller's particle order (host pointers, any may be NULL;
 * synchronises): x, v 3 * n_fluid floats; lambdas, density n_fluid floats
 * (last lambda pass). */
LUSTRINE_API int lustrine_pbf_download(lustrine_pbf* s, float* x, float* v, float* lambdas,
                                       float* density);
/* Asynchronous x, v download into host buffers (page-locked for overlap). */
LUSTRINE_API int lustrine_pbf_download_state_async(lustrine_pbf* s, float* x, float* v);
/* One frame for a host that keeps the state in its own arrays (x, v: 3 floats
 * per particle, caller order): upload, one step, download into the same
 * arrays, synchronise.  Page-locked arrays are read and written by the
 * kernels directly; pageable ones go through staging copies. */
LUSTRINE_API int lustrine_pbf_step_host(lustrine_pbf* s, float dt, float* x, float* v);
/* Positions in double (exact for the mixed representation), host, synchronises. */
LUSTRINE_API int lustrine_pbf_download_positions_f64(lustrine_pbf* s, double* x);
/* Neighbour lists of the last step in the caller's ids (solids n_fluid + k):
 * count[n_fluid], idx[n_fluid * cap] row-major.  Synchronises. */
LUSTRINE_API int lustrine_pbf_neighbors(lustrine_pbf* s, int* count, int* idx, int cap);
/* The form the last step's lists took: LUSTRINE_LISTS_COMPACT,
 * LUSTRINE_LISTS_COMPACT_WIDE or LUSTRINE_LISTS_COLUMN (also before the
 * first step and for the on-chip solve, whose lists are column lists). */
LUSTRINE_API int lustrine_pbf_list_format(const lustrine_pbf* s, int* format);
/* FP64 reductions on the device: [0] mass, [1..3] momentum, [4] kinetic
 * energy, [5..7] centre of mass, [8] max |rho / rho0 - 1| of the last lambda
 * pass (0 in sand mode, which computes no density).  Synchronises. */
LUSTRINE_API int lustrine_pbf_reduce(lustrine_pbf* s, double out[9]);
/* Particles the last step binned in the grid cells of the box [min_pos,
 * max_pos] (Lustrine::query_cell_num_particles, Lustrine.cpp:864-914: corners
 * clamped to [cell/2, domain - cell/2] and truncated to cell indices; fluid
 * binned at the step's predicted positions; solids counted when
 * include_solid).  0 before the first step.  One scene only.  Synchronises. */
LUSTRINE_API int lustrine_pbf_query_cell_count(lustrine_pbf* s, const float min_pos[3],
                                               const float max_pos[3], int include_solid, int* count);
/* Particles entering and leaving (the device side of the reference's sources
 * and sinks, Lustrine.cpp:745-836).  One scene only.
 *
 * reserve: buffers for up to capacity fluid particles; call before the first
 * upload (LUSTRINE_ERR_UNSUPPORTED after it).  The fluid count of the
 * context stays n_fluid until particles are spawned.
 * spawn: appends m particles (host xyz triples; v may be NULL for zero) as
 * caller indices n, n+1, ...; LUSTRINE_ERR_TOO_LARGE past the capacity.
 * despawn_cells: removes the fluid particles the last step binned in the
 * listed cells (dense cell ids y*gX*gZ + x*gZ + z, repeats allowed), with
 * the reference's index semantics: in list order, ascending index within a
 * cell, every evicted index takes the data of the current last particle and
 * the count drops by one (so an eviction list that reaches the tail moves
 * and drops particles exactly as the reference does).  *removed = how many
 * the count dropped.  Hashed grids: LUSTRINE_ERR_UNSUPPORTED.
 * Both synchronise; lambdas and densities of the last step read as 0 after
 * either until the next step. */
LUSTRINE_API int lustrine_pbf_reserve(lustrine_pbf* s, int capacity);
LUSTRINE_API int lustrine_pbf_spawn(lustrine_pbf* s, const float* x, const float* v, int m);
LUSTRINE_API int lustrine_pbf_despawn_cells(lustrine_pbf* s, const int* cells, int ncells, int* removed);
/* Sets the fluid count to n (<= the capacity) for a caller that keeps the
 * state on the host and uploads all of it next (lustrine_pbf_upload_state_async);
 * the particles' contents are undefined until then. */
LUSTRINE_API int lustrine_pbf_set_count(lustrine_pbf* s, int n);
/* Device-side error bits since the last call, as a status code (synchronises). */
LUSTRINE_API int lustrine_pbf_status(lustrine_pbf* s);
/* The context's cudaStream_t, as void*. */
LUSTRINE_API int lustrine_pbf_stream(lustrine_pbf* s, void** stream);
/* One step with direct launches and a CUDA event after each stage, on the
 * context stream; stage_ms[k] receives the milliseconds of stage k (summed
 * over the solver iterations) and stage_launches[k] its event count.
 * Synchronises. */
enum {
    LUSTRINE_STAGE_PREDICT = 0, /* prediction + cell key + histogram */
    LUSTRINE_STAGE_SCAN = 1,    /* prefix scan over cells */
    LUSTRINE_STAGE_SORT = 2,    /* index scatter, stabilisation, reorder */
    LUSTRINE_STAGE_LISTS = 3,   /* neighbour lists */
    LUSTRINE_STAGE_LAMBDA = 4,  /* density constraint pass(es) */
    LUSTRINE_STAGE_DELTA = 5,   /* position correction pass(es) */
    LUSTRINE_STAGE_XSPH = 6,    /* XSPH + commit */
    LUSTRINE_STAGE_SOLVE = 7,   /* a batch's on-chip solve: lists, iterations, XSPH, commit */
    LUSTRINE_NUM_STAGES = 8
};
LUSTRINE_API int lustrine_pbf_profile_step(lustrine_pbf* s, float dt, double* stage_ms,
                                           int* stage_launches, int num_stages);
/* Launch shape of the PBF iteration kernels (lambda, delta-p, XSPH) and of
 * the neighbour-list build.  block and list_block: 64, 128 or 256 threads;
 * unroll: neighbour gathers in flight per thread of the lambda and delta-p
 * passes, 1, 2, 4 or 8; xsph_unroll: the same for the XSPH pass (0 in
 * lustrine_pbf_set_tuning: as unroll); particles_per_thread: 1 or 2 particles
 * per thread of the lambda and delta-p passes, whose lists are walked
 * together (0: 1; with 2, unroll is at most 2); solver and solver_threads:
 * batches only, LUSTRINE_SOLVER_* and the on-chip solve's threads per CTA
 * (512 or 1024; 0: unchanged); list_format: LUSTRINE_LISTS_COLUMN or
 * LUSTRINE_LISTS_COMPACT (compact lists apply in PBF mode, fp32 or
 * LUSTRINE_PRECISION_MIXED_SCENE, with max_neighbors <= 255, an s_corr_n
 * that is an integer in [0, 32], no static particles and one particle per
 * thread: 16-bit entries for scenes of at most
 * 65,535 in contexts of fewer than 2^24 fluid particles, wide records
 * otherwise; elsewhere the step keeps column lists whatever list_format
 * says). */
enum {
    LUSTRINE_LISTS_COLUMN = 0,       /* count + column-major 32-bit entries */
    LUSTRINE_LISTS_COMPACT = 1,      /* 16-byte records: count, scene's first slot, 6 (+8) 16-bit offsets */
    LUSTRINE_LISTS_COMPACT_WIDE = 2  /* reported only: 16-byte records, count and 3 (+4) 32-bit slots */
};
typedef struct lustrine_pbf_tuning {
    int block;
    int unroll;
    int list_block;
    int xsph_unroll;
    int particles_per_thread;
    int solver;
    int solver_threads;
    int list_format;
} lustrine_pbf_tuning;
LUSTRINE_API int lustrine_pbf_set_tuning(lustrine_pbf* s, const lustrine_pbf_tuning* t);
LUSTRINE_API int lustrine_pbf_get_tuning(const lustrine_pbf* s, lustrine_pbf_tuning* t);
/* Autotuner: times `steps` graph-replayed steps of every launch shape from
 * the current state (restored before each candidate and at the end), keeps
 * the fastest and returns it with its milliseconds per step: block size x
 * gathers in flight x particles per thread of the iteration passes, the list
 * build's block size, the XSPH pass's gathers in flight and, for a batch, the
 * solver (per-stage kernels, or the on-chip solve with 512 or 1024 threads
 * per CTA).  The state is unchanged on return.  Reference mode has a single
 * shape (returned as is). */
LUSTRINE_API int lustrine_pbf_autotune(lustrine_pbf* s, float dt, int steps, lustrine_pbf_tuning* best,
                                       float* best_ms);
/* Sand mode (LUSTRINE_MODE_SAND) inputs that lustrine_pbf_params does not
 * hold: the player's position (the reference reads it from its Bullet world,
 * BulletPhysicsSimulation.hpp:35), the attract and blow flags of the next
 * steps (Wrapper::simulate's arguments, LustrineWrapper.cpp:342-346), their
 * radii and coefficients (Simulation.hpp:239-242) and the particle diameter
 * of the contact constraint (SimulationParameters::particleDiameter).  The
 * previous step's attract flag, a function static in the reference
 * (Simulate.cpp:185), is kept per context. */
typedef struct lustrine_sand_controls {
    float player_position[3];
    int attract_flag;
    int blow_flag;
    float attract_radius;     /* 1.5 */
    float blow_radius;        /* 2.0 */
    float attract_coeff;      /* 1000 */
    float blow_coeff;         /* 500 */
    float particle_diameter;  /* 2 * particle_radius unless the caller says otherwise */
} lustrine_sand_controls;

/* The reference's defaults (player at the origin, no flags). */
LUSTRINE_API void lustrine_sand_controls_default(lustrine_sand_controls* c, float particle_radius);
LUSTRINE_API int lustrine_pbf_set_sand_controls(lustrine_pbf* s, const lustrine_sand_controls* c);
LUSTRINE_API int lustrine_pbf_get_sand_controls(const lustrine_pbf* s, lustrine_sand_controls* c);
/* Per-particle attract flags of sand mode (Simulation::attracted; 0 after an
 * upload), n_fluid ints in the current particle order.  Synchronises. */
LUSTRINE_API int lustrine_pbf_get_attracted(lustrine_pbf* s, int* flags);
LUSTRINE_API int lustrine_pbf_set_attracted(lustrine_pbf* s, const int* flags);

/* Kernel launches of the last step (for launch accounting); before the first
 * step, those of a step that runs its own prediction kernel.  PBF: prediction
 * (only when the previous step's commit kernel could not predict this one),
 * 2-3 scan, 2 sort, list build + 2*iterations - 1 solver passes, commit. */
LUSTRINE_API int lustrine_pbf_launches_per_step(const lustrine_pbf* s);

/* Sorting::counting_sort (src/neighbors/Sorting.cpp:12-34, declared in
 * src/neighbors/Sorting.hpp:12-18) on device arrays: a stable sort of
 * keys[0..num_positions) in [0, num_cells).  sorted_indices receives the
 * input index of the k-th smallest key (equal keys in input order) and
 * counts (num_cells + 1 ints) the state the reference leaves in its counts
 * array: the first output position of every key, then num_positions.  The
 * extra scratch is taken with cudaMallocAsync on `stream` (a cudaStream_t,
 * NULL for the default stream) and returned before the call ends; the call
 * synchronises the stream.  LUSTRINE_ERR_ARGS if a key is out of range. */
LUSTRINE_API int lustrine_counting_sort(int* counts, const int* keys, size_t num_positions,
                                        size_t num_cells, int* sorted_indices, void* stream);

/* No counterpart in the reference.  The same sort for callers that cannot
 * allocate GPU memory while they run (an engine that budgets all device
 * memory at level load and forbids allocation during a frame, where a
 * cudaMalloc or cudaFree could synchronise the device; a host whose
 * allocator policy rejects allocations outside its pool): it takes no memory
 * and takes its scratch from a fixed array in the library's device image,
 * LUSTRINE_NOALLOC_SCRATCH_BYTES on every GPU that loads the library, held
 * until the process exits.  Limits: num_positions <= LUSTRINE_NOALLOC_MAX_KEYS
 * and num_cells <= LUSTRINE_NOALLOC_MAX_CELLS, else LUSTRINE_ERR_TOO_LARGE.
 * The first call on a device looks up the array's device address (make it
 * before any stream capture) and keeps it for that device's context: do not
 * call this entry point again in a process after cudaDeviceReset of that
 * device.  All calls share the array: calls that overlap on the GPU race.  Same arguments, results and synchronisation as
 * lustrine_counting_sort. */
#define LUSTRINE_NOALLOC_MAX_KEYS (1 << 20)
#define LUSTRINE_NOALLOC_MAX_CELLS (1 << 20)
#define LUSTRINE_NOALLOC_SCRATCH_BYTES (17u << 20)
LUSTRINE_API int lustrine_counting_sort_noalloc(int* counts, const int* keys, size_t num_positions,
                                                size_t num_cells, int* sorted_indices, void* stream);

LUSTRINE_API const char* lustrine_error_string(int code);

#ifdef __cplusplus
}
#endif

#endif /* LUSTRINE_GB300_H */
