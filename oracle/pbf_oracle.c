/*
 * pbf_oracle.c -- CPU oracle for the Lustrine PBF step.  TEST INFRASTRUCTURE:
 * only the tests, the smoke entry and the benchmark's CPU-baseline leg use it.
 * See pbf_oracle.h for what is restated and where it comes from.
 *
 * Build: gcc -O2 -ffp-contract=off -fPIC -shared (oracle/Makefile).  The
 * -ffp-contract=off flag is part of the contract: the reference's float
 * arithmetic has no fused multiply-adds, and aarch64 gcc contracts by default.
 */
#include "pbf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static const double ORC_PI = 3.14159265358979323846; /* Lustrine.cpp:16 */

/* ------------------------------------------------------------ parameters -- */

void orc_params_reference(orc_params* p, int X, int Y, int Z, float particle_radius,
                          float kernel_radius_scale)
{
    memset(p, 0, sizeof(*p));
    p->domain[0] = (float)X;
    p->domain[1] = (float)Y;
    p->domain[2] = (float)Z;
    p->particle_radius = particle_radius;
    p->kernel_factor = 0.5f;                                   /* Simulation.hpp:147 */
    p->kernel_radius = kernel_radius_scale * particle_radius;  /* Lustrine.cpp:545 */
    p->cell_size = 1.0f * p->kernel_radius;                    /* Lustrine.cpp:546 */
    {
        /* Lustrine.cpp:549-551: h3 is a float holding pow(double h, 3); the
         * constants are computed in double and stored as float. */
        float h3 = (float)pow((double)p->kernel_radius, 3);
        p->cubic_k = (float)(8.0 / (ORC_PI * (double)h3));
        p->cubic_l = (float)(48.0 / (ORC_PI * (double)h3));
    }
    p->grid[0] = (int)(p->domain[0] / p->cell_size) + 1;       /* Lustrine.cpp:553-555 */
    p->grid[1] = (int)(p->domain[1] / p->cell_size) + 1;
    p->grid[2] = (int)(p->domain[2] / p->cell_size) + 1;
    p->rest_density = 24.0f;                                   /* Simulation.hpp:157-171 */
    p->mass = 5.0f;
    p->gravity[0] = 0.0f; p->gravity[1] = -10.0f; p->gravity[2] = 0.0f;
    p->relaxation_epsilon = 10.0f;
    p->s_corr_dq = 0.5f; p->s_corr_k = 1.0f; p->s_corr_n = 4.0f;
    p->c_xsph = 0.1f;
    p->solid_contact = 2.0f * particle_radius;
    p->iterations = 1;
    p->clamp_cells = 0;
    p->jacobi = 0;
}

/* --------------------------------------------------------- counting sort -- */

void orc_counting_sort(int* counts, const int* keys, size_t n, size_t num_cells, int* sorted)
{
    /* Sorting.cpp:18-33: histogram, inclusive scan over num_cells + 1 slots,
     * backward scatter (stable). */
    memset(counts, 0, (num_cells + 1) * sizeof(int));
    for (size_t i = 0; i < n; i++) counts[keys[i]]++;
    for (size_t i = 1; i <= num_cells; i++) counts[i] += counts[i - 1];
    for (long i = (long)n - 1; i >= 0; i--) {
        sorted[counts[keys[i]] - 1] = (int)i;
        counts[keys[i]]--;
    }
}

/* ------------------------------------------------------------ cell table -- */

typedef struct {
    int num_cells;
    int* start;   /* num_cells + 1: CSR offsets, particles of cell c at [start[c], start[c+1]) */
    int* items;   /* particle ids in ascending id order within each cell */
} cell_table;

static void cell_table_free(cell_table* t)
{
    free(t->start);
    free(t->items);
    t->start = t->items = NULL;
}

/* Bin keys[0..m) (cell ids already validated) into a CSR table.  Ascending id
 * within a cell reproduces the reference's insertion order: sand ids first in
 * ascending order, then solids in ascending storage order
 * (Neighbors.cpp:374-384), because solid ids follow all sand ids. */
static int cell_table_build(cell_table* t, int num_cells, const int* keys, int m)
{
    t->num_cells = num_cells;
    t->start = (int*)calloc((size_t)num_cells + 1, sizeof(int));
    t->items = (int*)malloc(sizeof(int) * (size_t)(m > 0 ? m : 1));
    if (!t->start || !t->items) { cell_table_free(t); return ORC_ERR_NOMEM; }
    for (int i = 0; i < m; i++) t->start[keys[i] + 1]++;
    for (int c = 0; c < num_cells; c++) t->start[c + 1] += t->start[c];
    {
        int* fill = (int*)malloc(sizeof(int) * (size_t)num_cells);
        if (!fill) { cell_table_free(t); return ORC_ERR_NOMEM; }
        memcpy(fill, t->start, sizeof(int) * (size_t)num_cells);
        for (int i = 0; i < m; i++) t->items[fill[keys[i]]++] = i;
        free(fill);
    }
    return ORC_OK;
}

/* -------------------------------------------------------- neighbour lists -- */

typedef struct {
    int* offsets;  /* n + 1 */
    int* items;
    size_t size, cap;
} nbr_lists;

static void nbr_free(nbr_lists* L)
{
    free(L->offsets);
    free(L->items);
    L->offsets = L->items = NULL;
}

static int nbr_push(nbr_lists* L, int j)
{
    if (L->size == L->cap) {
        size_t nc = L->cap ? L->cap * 2 : 1024;
        int* ni = (int*)realloc(L->items, nc * sizeof(int));
        if (!ni) return ORC_ERR_NOMEM;
        L->items = ni;
        L->cap = nc;
    }
    L->items[L->size++] = j;
    return ORC_OK;
}

/* --------------------------------------------------------------- mode R -- */

static inline float dot3f(const float* a, const float* b)
{
    /* glm::dot for vec3: tmp = a * b; tmp.x + tmp.y + tmp.z
     * (glm/detail/func_geometric.inl:48-55). */
    float tx = a[0] * b[0];
    float ty = a[1] * b[1];
    float tz = a[2] * b[2];
    return (tx + ty) + tz;
}

static inline float length3f(const float* a)
{
    return sqrtf(dot3f(a, a));
}

/* cubic_kernel (Kernels.cpp:6-19) */
static float cubic_W(const orc_params* p, float r)
{
    float q = (r * p->kernel_factor) / p->kernel_radius;
    float result = 0.0f;
    if ((double)q <= 1.0) {
        if ((double)q <= 0.5) {
            float q2 = q * q;
            float q3 = q2 * q;
            float a = 6.0f * q3;
            float b = 6.0f * q2;
            result = p->cubic_k * ((a - b) + 1.0f);
        } else {
            result = p->cubic_k * (2.0f * powf(1.0f - q, 3.0f));
        }
    }
    return result;
}

/* cubic_kernel_grad (Kernels.cpp:26-41) */
static void cubic_gradW(const orc_params* p, const float* r, float* out)
{
    float rl = length3f(r) * p->kernel_factor;
    float q = rl / p->kernel_radius;
    out[0] = out[1] = out[2] = 0.0f;
    if ((double)rl > 1.0e-5 && (double)q <= 1.0) {
        float s = 1.0f / (rl * p->kernel_radius);
        float gq[3] = { s * r[0], s * r[1], s * r[2] };
        float c;
        if ((double)q <= 0.5) {
            c = (p->cubic_l * q) * (3.0f * q - 2.0f);
        } else {
            float f = 1.0f - q;
            c = p->cubic_l * ((-f) * f);
        }
        out[0] = c * gq[0];
        out[1] = c * gq[1];
        out[2] = c * gq[2];
    }
}

/* s_coor (Simulate.cpp:7-9) */
static float s_corr_R(const orc_params* p, float rl)
{
    return (-p->s_corr_k) * powf(cubic_W(p, rl) / cubic_W(p, p->s_corr_dq), p->s_corr_n);
}

/* resolve_collision (Simulate.cpp:11-24) */
static float resolve_collision(float value, float lo, float hi)
{
    const float epsilon_collision = (float)0.01;
    if (value <= lo) return epsilon_collision;
    if (value > hi) return hi - epsilon_collision;
    return value;
}

int orc_cell_id(const orc_params* p, const float pos[3], int* in_range)
{
    /* get_cell_id (Utils.hpp:24-33): position /= cell_size, truncate each
     * axis, id = y * gX * gZ + x * gZ + z. */
    int cx = (int)(pos[0] / p->cell_size);
    int cy = (int)(pos[1] / p->cell_size);
    int cz = (int)(pos[2] / p->cell_size);
    const int gX = p->grid[0], gY = p->grid[1], gZ = p->grid[2];
    if (p->clamp_cells) {
        cx = cx < 0 ? 0 : (cx >= gX ? gX - 1 : cx);
        cy = cy < 0 ? 0 : (cy >= gY ? gY - 1 : cy);
        cz = cz < 0 ? 0 : (cz >= gZ ? gZ - 1 : cz);
    }
    {
        long long id = (long long)cy * gX * gZ + (long long)cx * gZ + cz;
        long long nc = (long long)gX * gY * gZ;
        if (in_range) *in_range = (id >= 0 && id < nc);
        return (int)id;
    }
}

/* All particles' positions as one array view: fluid ids [0, n) from xs,
 * solid ids [n, n + ns) from solid. */
static inline const float* pos_of(int j, int n, const float* xs, const float* solid)
{
    return j < n ? xs + 3 * (size_t)j : solid + 3 * (size_t)(j - n);
}

/* find_neighbors_uniform_grid (Neighbors.cpp:366-450): bin every particle,
 * then for each fluid particle walk the 27 cells around its own cell in
 * y -> x -> z offset order and keep every particle (itself and solids
 * included) with dot(d, d) <= h * h. */
static int compat_lists(const orc_params* p, int n, int ns, const float* xs,
                        const float* solid, nbr_lists* L)
{
    const int gX = p->grid[0], gY = p->grid[1], gZ = p->grid[2];
    const int num_cells = gX * gY * gZ;
    const int m = n + ns;
    const float h2 = p->kernel_radius * p->kernel_radius;
    int* keys = (int*)malloc(sizeof(int) * (size_t)(m > 0 ? m : 1));
    cell_table T;
    int rc = ORC_OK;
    memset(L, 0, sizeof(*L));
    if (!keys) return ORC_ERR_NOMEM;
    for (int j = 0; j < m; j++) {
        int ok;
        keys[j] = orc_cell_id(p, pos_of(j, n, xs, solid), &ok);
        if (!ok) { free(keys); return ORC_ERR_CELL_RANGE; }
    }
    rc = cell_table_build(&T, num_cells, keys, m);
    if (rc) { free(keys); return rc; }
    L->offsets = (int*)malloc(sizeof(int) * ((size_t)n + 1));
    if (!L->offsets) { free(keys); cell_table_free(&T); return ORC_ERR_NOMEM; }
    for (int i = 0; i < n && rc == ORC_OK; i++) {
        const float* self = xs + 3 * (size_t)i;
        /* The stencil is centred on the cell the particle was binned into;
         * an id that aliases past an axis end is decoded, as the reference's
         * cell loop (Neighbors.cpp:386-393) would see it. */
        int id = keys[i];
        int yy = id / (gX * gZ);
        int xx = (id % (gX * gZ)) / gZ;
        int zz = id % gZ;
        L->offsets[i] = (int)L->size;
        for (int y = -1; y <= 1 && rc == ORC_OK; y++)
            for (int x = -1; x <= 1 && rc == ORC_OK; x++)
                for (int z = -1; z <= 1 && rc == ORC_OK; z++) {
                    if (xx + x < 0 || xx + x >= gX || yy + y < 0 || yy + y >= gY ||
                        zz + z < 0 || zz + z >= gZ)
                        continue;
                    int c = (yy + y) * gX * gZ + (xx + x) * gZ + (zz + z);
                    for (int k = T.start[c]; k < T.start[c + 1]; k++) {
                        int j = T.items[k];
                        const float* other = pos_of(j, n, xs, solid);
                        float d[3] = { self[0] - other[0], self[1] - other[1], self[2] - other[2] };
                        if (dot3f(d, d) <= h2) {
                            rc = nbr_push(L, j);
                            if (rc) break;
                        }
                    }
                }
    }
    L->offsets[n] = (int)L->size;
    free(keys);
    cell_table_free(&T);
    if (rc) nbr_free(L);
    return rc;
}

static int export_lists(const nbr_lists* L, int n, int* nbr_count, int* nbr_idx, int cap)
{
    int rc = ORC_OK;
    for (int i = 0; i < n; i++) {
        int c = L->offsets[i + 1] - L->offsets[i];
        if (nbr_count) nbr_count[i] = c;
        if (nbr_idx) {
            if (c > cap) { rc = ORC_ERR_CAPACITY; c = cap; }
            memcpy(nbr_idx + (size_t)i * cap, L->items + L->offsets[i], sizeof(int) * (size_t)c);
        }
    }
    return rc;
}

int orc_compat_neighbors(const orc_params* p, int n, int ns, const float* xs,
                         const float* solid, int* nbr_count, int* nbr_idx, int cap)
{
    nbr_lists L;
    int rc;
    if (n < 0 || ns < 0) return ORC_ERR_ARGS;
    rc = compat_lists(p, n, ns, xs, solid, &L);
    if (rc) return rc;
    rc = export_lists(&L, n, nbr_count, nbr_idx, cap);
    nbr_free(&L);
    return rc;
}

int orc_compat_step(const orc_params* p, float dt, int n, int ns,
                    float* x, float* xs, float* v, const float* solid,
                    float* lambdas, int* nbr_count, int* nbr_idx, int cap)
{
    nbr_lists L;
    int rc;
    float* snap = NULL;
    if (n < 0 || ns < 0) return ORC_ERR_ARGS;

    /* Simulate.cpp:31: dt = glm::clamp(dt, 0.001f, 0.01f) */
    dt = dt < 0.001f ? 0.001f : dt;
    dt = dt > 0.01f ? 0.01f : dt;

    /* Simulate.cpp:48-51: v += gravity * mass * dt; x* = x + v * dt */
    for (int i = 0; i < n; i++) {
        float* vi = v + 3 * (size_t)i;
        for (int a = 0; a < 3; a++) {
            float gm = p->gravity[a] * p->mass;
            vi[a] = vi[a] + gm * dt;
        }
        for (int a = 0; a < 3; a++) xs[3 * (size_t)i + a] = x[3 * (size_t)i + a] + vi[a] * dt;
    }

    rc = compat_lists(p, n, ns, xs, solid, &L);
    if (rc) return rc;

    /* Simulate.cpp:58-88: lambda pass */
    for (int i = 0; i < n; i++) {
        const float* self = xs + 3 * (size_t)i;
        float density = 0.0f;
        for (int k = L.offsets[i]; k < L.offsets[i + 1]; k++) {
            const float* o = pos_of(L.items[k], n, xs, solid);
            float ij[3] = { self[0] - o[0], self[1] - o[1], self[2] - o[2] };
            float len = length3f(ij);
            density += p->mass * cubic_W(p, len);
        }
        density += p->mass * cubic_W(p, 0.0f);
        float constraint_i = (float)((double)(density / p->rest_density) - 1.0);
        float grad_sum = 0.0f;
        float gcp[3] = { 0.0f, 0.0f, 0.0f };
        const float coef = -(p->mass / p->rest_density);
        for (int k = L.offsets[i]; k < L.offsets[i + 1]; k++) {
            const float* o = pos_of(L.items[k], n, xs, solid);
            float t[3] = { self[0] - o[0], self[1] - o[1], self[2] - o[2] };
            float g[3];
            cubic_gradW(p, t, g);
            float ng[3] = { coef * g[0], coef * g[1], coef * g[2] };
            grad_sum += dot3f(ng, ng);
            gcp[0] -= ng[0];
            gcp[1] -= ng[1];
            gcp[2] -= ng[2];
        }
        grad_sum += dot3f(gcp, gcp);
        lambdas[i] = 0.0f;
        if ((double)grad_sum > 0.0) lambdas[i] = (-constraint_i) / (grad_sum + p->relaxation_epsilon);
    }

    /* Simulate.cpp:90-113: position correction, collision, velocity.  The
     * reference updates positions_star[i] in place (Gauss-Seidel); with
     * p->jacobi the neighbours are read from a snapshot instead. */
    const float* src = xs;
    if (p->jacobi) {
        snap = (float*)malloc(sizeof(float) * 3 * (size_t)(n > 0 ? n : 1));
        if (!snap) { nbr_free(&L); return ORC_ERR_NOMEM; }
        memcpy(snap, xs, sizeof(float) * 3 * (size_t)n);
        src = snap;
    }
    const int X = (int)p->domain[0], Y = (int)p->domain[1], Z = (int)p->domain[2];
    const float r = p->particle_radius;
    for (int i = 0; i < n; i++) {
        float pf[3] = { 0.0f, 0.0f, 0.0f };
        const float* self = src + 3 * (size_t)i;
        for (int k = L.offsets[i]; k < L.offsets[i + 1]; k++) {
            int jpos = k - L.offsets[i];
            const float* o = pos_of(L.items[k], n, src, solid);
            float ij[3] = { self[0] - o[0], self[1] - o[1], self[2] - o[2] };
            float g[3];
            float s = s_corr_R(p, length3f(ij));
            cubic_gradW(p, ij, g);
            /* lambdas[j] with j the list position (Simulate.cpp:97) */
            float w = (lambdas[i] + lambdas[jpos]) + s;
            pf[0] += w * g[0];
            pf[1] += w * g[1];
            pf[2] += w * g[2];
        }
        float* xi = xs + 3 * (size_t)i;
        for (int a = 0; a < 3; a++) pf[a] = pf[a] / p->rest_density;
        for (int a = 0; a < 3; a++) xi[a] = xi[a] + pf[a];
        xi[0] = resolve_collision(xi[0], r, (float)X - r);
        xi[1] = resolve_collision(xi[1], r, (float)Y - r);
        xi[2] = resolve_collision(xi[2], r, (float)Z - r);
        for (int a = 0; a < 3; a++) {
            v[3 * (size_t)i + a] = (xi[a] - x[3 * (size_t)i + a]) / dt;
            x[3 * (size_t)i + a] = xi[a];
        }
    }

    rc = export_lists(&L, n, nbr_count, nbr_idx, cap);
    free(snap);
    nbr_free(&L);
    return rc;
}

/* --------------------------------------------------------------- mode P -- */

#define T double
#define SUF(name) name##_d
#define SQRT sqrt
#define POW pow
#define FLOOR floor
#include "pbf_mode_p.inc"
#undef T
#undef SUF
#undef SQRT
#undef POW
#undef FLOOR

#define T float
#define SUF(name) name##_f
#define SQRT sqrtf
#define POW powf
#define FLOOR floorf
#include "pbf_mode_p.inc"
#undef T
#undef SUF
#undef SQRT
#undef POW
#undef FLOOR

int orc_pbf_step_d(const orc_params* p, double dt, int n, int ns,
                   double* x, double* v, const double* solid,
                   double* lambdas, double* density, int* nbr_count)
{
    return pbf_step_d(p, dt, n, ns, x, v, solid, lambdas, density, nbr_count);
}

int orc_pbf_step_f(const orc_params* p, float dt, int n, int ns,
                   float* x, float* v, const float* solid,
                   float* lambdas, float* density, int* nbr_count)
{
    return pbf_step_f(p, dt, n, ns, x, v, solid, lambdas, density, nbr_count);
}

int orc_pbf_density_d(const orc_params* p, int n, int ns, const double* xs,
                      const double* solid, double* density)
{
    return pbf_lambda_only_d(p, n, ns, xs, solid, NULL, density);
}

int orc_pbf_lambda_d(const orc_params* p, int n, int ns, const double* xs,
                     const double* solid, double* lambdas, double* density)
{
    return pbf_lambda_only_d(p, n, ns, xs, solid, lambdas, density);
}

/* ----------------------------------------------------------------- sand -- */

#include "sand_oracle.inc"
