// pbf_context.cu -- lustrine_pbf_* context API: device state, one step as a
// fixed sequence of kernel launches on the context stream, optionally
// replayed from a captured CUDA graph (one graph per state buffer parity).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <initializer_list>
#include <vector>

#include "lustrine_gb300.h"
#include "pbf_context.h"
#include "pbf_kernels.h"

using namespace lgb;

namespace {

constexpr double kPi = 3.14159265358979323846;  // Lustrine.cpp:16

template <class T>
int dalloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc((void**)p, count * sizeof(T)) == cudaSuccess ? LUSTRINE_OK : LUSTRINE_ERR_NOMEM;
}

int bits_for(int values) {
    int b = 0;
    while ((1 << b) < values) b++;
    return b;
}

}  // namespace


int lgb_cuda_status(cudaError_t e, const char* what) {
    if (getenv("LUSTRINE_DEBUG")) fprintf(stderr, "lustrine: %s: %s\n", what, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? LUSTRINE_ERR_NOMEM : LUSTRINE_ERR_CUDA;
}

extern "C" void lustrine_pbf_params_reference(lustrine_pbf_params* p, int X, int Y, int Z,
                                              float particle_radius, float kernel_radius_scale) {
    std::memset(p, 0, sizeof(*p));
    p->mode = LUSTRINE_MODE_REFERENCE;
    p->precision = LUSTRINE_PRECISION_FP32;
    p->domain[0] = X;
    p->domain[1] = Y;
    p->domain[2] = Z;
    p->particle_radius = particle_radius;
    p->kernel_radius = kernel_radius_scale * particle_radius;  // Lustrine.cpp:545
    p->kernel_factor = 0.5f;                                   // Simulation.hpp:147
    p->cell_size = 1.0f * p->kernel_radius;                    // Lustrine.cpp:546
    p->rest_density = 24.0f;                                   // Simulation.hpp:157-171
    p->mass = 5.0f;
    p->gravity[0] = 0.0f;
    p->gravity[1] = -10.0f;
    p->gravity[2] = 0.0f;
    p->relaxation_epsilon = 10.0f;
    p->s_corr_dq = 0.5f;
    p->s_corr_k = 1.0f;
    p->s_corr_n = 4.0f;
    p->c_xsph = 0.1f;
    p->solid_contact = 2.0f * particle_radius;
    p->iterations = 1;
    // the reference's lists are unbounded and grow to 34-150 entries once its
    // fluid clusters; lists cost memory only (4 B per entry and particle)
    p->max_neighbors = 512;
    p->clamp_cells = 1;
    p->use_graph = 1;
}

// Derived per-scene constants.  Reference-mode constants are computed with
// the reference's float/double mix (Lustrine.cpp:549-555).
static int derive(const lustrine_pbf_params& q, int n, int ns, StepParams* sp, CellPack* cp) {
    if (q.domain[0] <= 0 || q.domain[1] <= 0 || q.domain[2] <= 0) return LUSTRINE_ERR_ARGS;
    if (!(q.kernel_radius > 0.0f) || !(q.cell_size > 0.0f) || !(q.rest_density > 0.0f))
        return LUSTRINE_ERR_ARGS;
    if (q.max_neighbors <= 0 || q.iterations < 1 || q.iterations > 1000) return LUSTRINE_ERR_ARGS;
    if (!(q.s_corr_n >= 0.0f)) return LUSTRINE_ERR_ARGS;  // (W / W(dq))^n with W = 0 at r = h
    if (q.mode != LUSTRINE_MODE_REFERENCE && q.mode != LUSTRINE_MODE_PBF && q.mode != LUSTRINE_MODE_SAND)
        return LUSTRINE_ERR_ARGS;
    if (q.precision != LUSTRINE_PRECISION_FP32 && q.precision != LUSTRINE_PRECISION_MIXED &&
        q.precision != LUSTRINE_PRECISION_MIXED_SCENE)
        return LUSTRINE_ERR_ARGS;
    if (q.precision != LUSTRINE_PRECISION_FP32 && q.mode != LUSTRINE_MODE_PBF) return LUSTRINE_ERR_UNSUPPORTED;
    StepParams p;
    std::memset(&p, 0, sizeof(p));
    p.n = n;
    p.ns = ns;
    const float dX = (float)q.domain[0], dY = (float)q.domain[1], dZ = (float)q.domain[2];
    p.gx = (int)(dX / q.cell_size) + 1;
    p.gy = (int)(dY / q.cell_size) + 1;
    p.gz = (int)(dZ / q.cell_size) + 1;
    const long long C = (long long)p.gx * p.gy * p.gz;
    // hashed grid: requested, or (auto) when the box has far more cells than
    // particles -- up to 2^32 cells for a 4096 x 256 x 4096 box
    const long long parts = (long long)n + ns;
    const bool hashed = q.mode == LUSTRINE_MODE_PBF &&
                        (q.grid_mode == LUSTRINE_GRID_HASHED ||
                         (q.grid_mode == LUSTRINE_GRID_AUTO && (C > (1LL << 31) - 2 || C > 32 * parts + (1LL << 24))));
    if (q.grid_mode == LUSTRINE_GRID_HASHED && q.mode != LUSTRINE_MODE_PBF) return LUSTRINE_ERR_UNSUPPORTED;
    if (!hashed && C > (1LL << 31) - 2) return LUSTRINE_ERR_UNSUPPORTED;
    // the scene frame: a dense grid and boxes of at most 256 cells a side
    if (q.precision == LUSTRINE_PRECISION_MIXED_SCENE &&
        (hashed || std::max(dX, std::max(dY, dZ)) > 256.0f * q.cell_size))
        return LUSTRINE_ERR_UNSUPPORTED;
    p.frame = q.precision == LUSTRINE_PRECISION_MIXED_SCENE ? 1 : 0;
    // PBF neighbour entries hold a 25-bit slot
    if (q.mode == LUSTRINE_MODE_PBF && (n >= (1 << 25) || ns >= (1 << 25))) return LUSTRINE_ERR_UNSUPPORTED;
    if (hashed) {
        int bits = 10;
        while ((1LL << bits) < 4 * parts && bits < 30) bits++;
        p.hash_bits = bits;
        p.num_cells = 1 << bits;
    } else {
        p.num_cells = (int)C;
    }
    p.max_nbrs = q.max_neighbors;
    p.pad = 1;  // set per launch of the list build
    p.clamp_cells = q.clamp_cells;
    p.cell = q.cell_size;
    p.inv_cell = 1.0f / q.cell_size;
    p.h = q.kernel_radius;
    p.h2 = q.kernel_radius * q.kernel_radius;
    p.kfac = q.kernel_factor;
    {
        float h3 = (float)std::pow((double)q.kernel_radius, 3);
        p.cubic_k = (float)(8.0 / (kPi * (double)h3));
        p.cubic_l = (float)(48.0 / (kPi * (double)h3));
    }
    const double h = (double)q.kernel_radius;
    p.k6 = (float)(315.0 / (64.0 * kPi * std::pow(h, 9)));
    p.self_density = (float)((double)q.mass * 315.0 / (64.0 * kPi * std::pow(h, 9)) * std::pow(h, 6));
    p.ks = (float)(45.0 / (kPi * std::pow(h, 6)));
    {
        double d = h * h - (double)q.s_corr_dq * (double)q.s_corr_dq;
        double wdq = q.s_corr_dq <= q.kernel_radius ? 315.0 / (64.0 * kPi * std::pow(h, 9)) * d * d * d : 0.0;
        p.inv_w_dq = wdq > 0.0 ? (float)(1.0 / wdq) : 0.0f;
        p.inv_hdq2 = (wdq > 0.0 && q.s_corr_k != 0.0f) ? (float)(1.0 / d) : 0.0f;
    }
    p.k6m = (float)((double)q.mass * 315.0 / (64.0 * kPi * std::pow(h, 9)));
    p.mass = q.mass;
    p.rho0 = q.rest_density;
    p.mr = q.mass / q.rest_density;
    {
        const float c = p.ks * p.mr;  // float products, as the kernels formed them
        p.lam_c2 = c * c;
    }
    p.inv_rho0 = 1.0f / q.rest_density;
    p.eps = q.relaxation_epsilon;
    p.dq = q.s_corr_dq;
    p.sk = q.s_corr_k;
    p.sn = q.s_corr_n;
    p.sn_int = (q.s_corr_n >= 0.0f && q.s_corr_n <= 32.0f && std::floor(q.s_corr_n) == q.s_corr_n)
                   ? (int)q.s_corr_n
                   : -1;
    p.c_xsph = q.c_xsph;
    p.contact = q.solid_contact;
    p.gxv = q.gravity[0];
    p.gyv = q.gravity[1];
    p.gzv = q.gravity[2];
    const float r = q.particle_radius;
    if (q.mode != LUSTRINE_MODE_PBF) {
        // Simulate.cpp:35-37,106-108 (fluid), 206-208 and 298 (sand): [r, domain - r]
        p.lox = p.loy = p.loz = r;
        p.hix = (float)q.domain[0] - r;
        p.hiy = (float)q.domain[1] - r;
        p.hiz = (float)q.domain[2] - r;
    } else {
        p.lox = p.loy = p.loz = r;
        p.hix = dX - r;
        p.hiy = dY - r;
        p.hiz = dZ - r;
    }
    CellPack c;
    std::memset(&c, 0, sizeof(c));
    if (q.precision != LUSTRINE_PRECISION_FP32 || hashed) {
        // cells a clamped position can occupy: 0 .. floor(hi / cell)
        int vx = (int)std::floor(p.hix / p.cell) + 1, vy = (int)std::floor(p.hiy / p.cell) + 1,
            vz = (int)std::floor(p.hiz / p.cell) + 1;
        int bx = bits_for(vx), by = bits_for(vy), bz = bits_for(vz);
        if (bx + by + bz > 32) return LUSTRINE_ERR_UNSUPPORTED;
        c.mx = bx ? (unsigned)((1ull << bx) - 1) : 0u;
        c.my = by ? (unsigned)((1ull << by) - 1) : 0u;
        c.mz = bz ? (unsigned)((1ull << bz) - 1) : 0u;
        c.by_shift = bx;
        c.bz_shift = bx + by;
    }
    *sp = p;
    *cp = c;
    return LUSTRINE_OK;
}

lustrine_pbf::~lustrine_pbf() {
    free_buffers();
    if (fork_ev) cudaEventDestroy(fork_ev);
    if (join_ev) cudaEventDestroy(join_ev);
    if (side) cudaStreamDestroy(side);
    if (stream) cudaStreamDestroy(stream);
}

void lustrine_pbf::free_buffers() {
    for (int k = 0; k < 8; k++) {
        if (graph_exec[k]) cudaGraphExecDestroy(graph_exec[k]);
        graph_exec[k] = nullptr;
    }
    for (int k = 0; k < 2; k++) {
        if (host_graph[k]) cudaGraphExecDestroy(host_graph[k]);
        host_graph[k] = nullptr;
    }
    void* ptrs[] = {x[0], x[1], xs[0], xs[1], v[0], v[1], id[0], id[1], xs_alt, xs_pred, vtmp, key, key_sorted,
                    rank, tmp, perm, count, start, block_sums, tile_sum, solid_near, solid, solid_raw, sstart, nbr, cnt, lam,
                    lam_by_id, rho, status, red, qcount, out3, out3d, iota, slot_of, solid_id, d_scenes, d_scene_of,
                    d_solid_scene_of, cellk, cell_sorted, solid_cell, att[0], att[1], d_bins, d_scene_slot0,
                    d_queue, rec, rec2, src};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    x[0] = x[1] = xs[0] = xs[1] = v[0] = v[1] = nullptr;
    id[0] = id[1] = nullptr;
    xs_alt = xs_pred = vtmp = solid = solid_raw = lam_src = nullptr;
    key = key_sorted = rank = tmp = perm = count = start = block_sums = tile_sum = sstart = nullptr;
    nbr = cnt = status = qcount = iota = slot_of = solid_id = d_scene_of = d_solid_scene_of = nullptr;
    cellk = cell_sorted = solid_cell = nullptr;
    rec = rec2 = nullptr;
    src = nullptr;
    lists_format = LUSTRINE_LISTS_COLUMN;
    att[0] = att[1] = nullptr;
    solid_near = nullptr;
    lam = lam_by_id = rho = out3 = nullptr;
    red = out3d = nullptr;
    d_scenes = nullptr;
    d_bins = nullptr;
    d_scene_slot0 = d_queue = nullptr;
    num_bins = onchip_clusters = onchip_clusters512 = 0;
    onchip = false;
}

int lgb_write_sentinel(lustrine_pbf* s) {
    // the sentinel particle of the padded neighbour lists, at slot n
    const float4 far = make_float4(SENTINEL_POS, SENTINEL_POS, SENTINEL_POS, 0.0f);
    const int n = s->n;
    for (float4* a : {s->xs[0], s->xs[1], s->xs_alt})
        CK(cudaMemcpyAsync(a + n, &far, sizeof(float4), cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemsetAsync(s->vtmp + n, 0, sizeof(float4), s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return LUSTRINE_OK;
}

// The compact neighbour lists the context's steps can use: PBF mode in fp32
// or the scene frame (no cell codes in the entries), lists of at most
// COMPACT_MAX_NBRS entries and an s_corr exponent that is an integer in
// [0, 32] (the compact position pass is built without powf); 16-bit entries (LUSTRINE_LISTS_COMPACT) for
// fewer than COMPACT_MAX_N fluid slots in scenes of at most
// COMPACT_MAX_SCENE (one scene: the capacity), wide records
// (LUSTRINE_LISTS_COMPACT_WIDE) otherwise; LUSTRINE_LISTS_COLUMN when none.
// A step uses them when the tuning asks for them, with one particle per
// thread, and the context holds no static particles.
static int compact_capable(const lustrine_pbf* s) {
    if (s->prm.mode != LUSTRINE_MODE_PBF || (s->mixed() && !s->sp.frame)) return LUSTRINE_LISTS_COLUMN;
    if (s->sp.max_nbrs > COMPACT_MAX_NBRS || s->sp.sn_int < 0) return LUSTRINE_LISTS_COLUMN;
    int largest = s->cap;
    if (s->is_batch()) largest = *std::max_element(s->b_nfluid.begin(), s->b_nfluid.end());
    return (largest <= COMPACT_MAX_SCENE && s->cap < COMPACT_MAX_N) ? LUSTRINE_LISTS_COMPACT
                                                                     : LUSTRINE_LISTS_COMPACT_WIDE;
}

static int compact_now(const lustrine_pbf* s) {
    if (!s->rec || !s->tune.lists || s->tune.ppt != 1 || s->ns != 0) return LUSTRINE_LISTS_COLUMN;
    return compact_capable(s);
}

// Device buffers for s->cap fluid particles (s->n of them active).
static int ctx_alloc(lustrine_pbf* s) {
    const int n = s->cap, ns = s->ns, C = s->sp.num_cells, m = n > ns ? n : ns;
    int rc = LUSTRINE_OK;
    for (int k = 0; k < 2 && !rc; k++) {
        rc = rc ? rc : dalloc(&s->x[k], n);
        rc = rc ? rc : dalloc(&s->xs[k], (size_t)n + 1);  // + the sentinel slot n
        rc = rc ? rc : dalloc(&s->v[k], n);
        rc = rc ? rc : dalloc(&s->id[k], n);
        rc = rc ? rc : dalloc(&s->att[k], n);  // sand mode's attract flags
    }
    rc = rc ? rc : dalloc(&s->xs_alt, (size_t)n + 1);
    rc = rc ? rc : dalloc(&s->xs_pred, n);
    rc = rc ? rc : dalloc(&s->vtmp, (size_t)n + 1);
    rc = rc ? rc : dalloc(&s->key, m);
    rc = rc ? rc : dalloc(&s->key_sorted, m);  // m: key and key_sorted trade places after a despawn
    rc = rc ? rc : dalloc(&s->rank, m);
    rc = rc ? rc : dalloc(&s->tmp, m);
    rc = rc ? rc : dalloc(&s->perm, m);
    rc = rc ? rc : dalloc(&s->count, C);
    rc = rc ? rc : dalloc(&s->start, (size_t)C + 1);
    rc = rc ? rc : dalloc(&s->block_sums, scan_block_sums_size(C));
    rc = rc ? rc : dalloc(&s->tile_sum, 2 * (size_t)cell_scan_tiles(C));
    rc = rc ? rc : dalloc(&s->solid, ns);
    rc = rc ? rc : dalloc(&s->solid_raw, ns);
    rc = rc ? rc : dalloc(&s->sstart, (size_t)C + 1);
    const size_t list_rows = (size_t)((s->sp.max_nbrs + LIST_PAD_MAX - 1) / LIST_PAD_MAX * LIST_PAD_MAX);
    rc = rc ? rc : dalloc(&s->nbr, list_rows * (size_t)n);
    rc = rc ? rc : dalloc(&s->cnt, n);
    rc = rc ? rc : dalloc(&s->src, n);
    if (compact_capable(s) != LUSTRINE_LISTS_COLUMN) {
        rc = rc ? rc : dalloc(&s->rec, n);
        rc = rc ? rc : dalloc(&s->rec2, n);
    }
    rc = rc ? rc : dalloc(&s->lam, n);
    s->lam_by_id_len = (size_t)(n + ns > s->sp.max_nbrs ? n + ns : s->sp.max_nbrs) + 1;
    rc = rc ? rc : dalloc(&s->lam_by_id, s->lam_by_id_len);
    rc = rc ? rc : dalloc(&s->rho, n);
    rc = rc ? rc : dalloc(&s->status, 4);
    rc = rc ? rc : dalloc(&s->red, 9);
    rc = rc ? rc : dalloc(&s->qcount, 1);
    rc = rc ? rc : dalloc(&s->out3, (size_t)3 * m);
    rc = rc ? rc : dalloc(&s->out3d, (size_t)3 * n);
    rc = rc ? rc : dalloc(&s->iota, n);
    rc = rc ? rc : dalloc(&s->slot_of, n);
    rc = rc ? rc : dalloc(&s->solid_id, ns);
    if (ns > 0) {
        rc = rc ? rc : dalloc(&s->solid_near, (size_t)C);
        s->sp.solid_near = s->solid_near;
    }
    // packed cells, unsorted and sorted: the hashed grid tells cells sharing a
    // bucket apart by them; mixed precision reads a slot's cell from them
    // (shifts and masks, where the dense key would need two integer divisions)
    if (s->sp.hash_bits || s->mixed()) {
        rc = rc ? rc : dalloc(&s->cellk, m);
        rc = rc ? rc : dalloc(&s->cell_sorted, n);
        s->sp.cell_sorted = s->cell_sorted;
    }
    if (s->sp.hash_bits) rc = rc ? rc : dalloc(&s->solid_cell, ns);
    if (rc) return rc;
    if (n) {
        std::vector<int> ids((size_t)n);
        for (int i = 0; i < n; i++) ids[(size_t)i] = i;
        CK(cudaMemcpy(s->iota, ids.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice));
    }
    rc = lgb_write_sentinel(s);
    if (rc) return rc;
    CK(cudaMemsetAsync(s->lam_by_id, 0, s->lam_by_id_len * sizeof(float), s->stream));
    CK(cudaMemsetAsync(s->lam, 0, (size_t)(n ? n : 1) * sizeof(float), s->stream));
    CK(cudaMemsetAsync(s->rho, 0, (size_t)(n ? n : 1) * sizeof(float), s->stream));
    CK(cudaMemsetAsync(s->cnt, 0, (size_t)(n ? n : 1) * sizeof(int), s->stream));
    CK(cudaMemsetAsync(s->status, 0, 4 * sizeof(int), s->stream));
    CK(cudaMemsetAsync(s->sstart, 0, ((size_t)C + 1) * sizeof(int), s->stream));
    CK(cudaMemsetAsync(s->count, 0, (size_t)C * sizeof(int), s->stream));
    s->use_pdl = getenv("LUSTRINE_NO_PDL") == nullptr;
    return LUSTRINE_OK;
}

extern "C" int lustrine_pbf_create(const lustrine_pbf_params* p, int n_fluid, int n_solid,
                                   lustrine_pbf** out) {
    if (!p || !out || n_fluid < 0 || n_solid < 0) return LUSTRINE_ERR_ARGS;
    *out = nullptr;
    lustrine_pbf* s = new (std::nothrow) lustrine_pbf();
    if (!s) return LUSTRINE_ERR_NOMEM;
    s->prm = *p;
    s->n = n_fluid;
    s->cap = n_fluid;
    s->ns = n_solid;
    lustrine_sand_controls_default(&s->sand, p->particle_radius);
    int rc = derive(*p, n_fluid, n_solid, &s->sp, &s->cp);
    if (rc) {
        delete s;
        return rc;
    }
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete s;
        return LUSTRINE_ERR_CUDA;
    }
    rc = ctx_alloc(s);
    if (rc) {
        delete s;
        return rc;
    }
    *out = s;
    return LUSTRINE_OK;
}

extern "C" int lustrine_pbf_reserve(lustrine_pbf* s, int capacity) {
    if (!s || capacity < s->n) return LUSTRINE_ERR_ARGS;
    if (s->is_batch() || s->have_state) return LUSTRINE_ERR_UNSUPPORTED;
    if (capacity == s->cap) return LUSTRINE_OK;
    StepParams sp;
    CellPack cp;
    // grid table sized for the capacity (hash buckets follow the particle count)
    int rc = derive(s->prm, capacity, s->ns, &sp, &cp);
    if (rc) return rc;
    sp.n = s->n;
    CK(cudaStreamSynchronize(s->stream));
    s->free_buffers();
    s->sp = sp;
    s->cp = cp;
    s->cap = capacity;
    s->steps_done = 0;
    return ctx_alloc(s);
}

// Batch geometry: every scene's grid and box, cells numbered scene after
// scene; the mixed-precision packing is sized by the largest box per axis.
static int derive_batch(const lustrine_pbf_params& q0, const std::vector<int>& dom,
                        const std::vector<int>& nf, const std::vector<int>& nsv, StepParams* sp,
                        CellPack* cp, std::vector<SceneInfo>* table) {
    const int S = (int)nf.size();
    long long n = 0, ns = 0;
    lustrine_pbf_params q = q0;
    q.domain[0] = q.domain[1] = q.domain[2] = 1;
    q.grid_mode = LUSTRINE_GRID_DENSE;  // scenes' cells are numbered one after another
    for (int k = 0; k < S; k++) {
        if (dom[3 * k] <= 0 || dom[3 * k + 1] <= 0 || dom[3 * k + 2] <= 0 || nf[k] < 0 || nsv[k] < 0)
            return LUSTRINE_ERR_ARGS;
        for (int a = 0; a < 3; a++) q.domain[a] = std::max(q.domain[a], dom[3 * k + a]);
        n += nf[k];
        ns += nsv[k];
    }
    if (n >= (1LL << 26) || ns >= (1LL << 26)) return LUSTRINE_ERR_UNSUPPORTED;
    int rc = derive(q, (int)n, (int)ns, sp, cp);
    if (rc) return rc;
    table->clear();
    long long off = 0, slot = 0;
    const float r = q.particle_radius;
    for (int k = 0; k < S; k++) {
        SceneInfo si;
        si.slot0 = (int)slot;
        si.spare = 0;
        slot += nf[k];
        const float dX = (float)dom[3 * k], dY = (float)dom[3 * k + 1], dZ = (float)dom[3 * k + 2];
        si.gx = (int)(dX / q.cell_size) + 1;
        si.gy = (int)(dY / q.cell_size) + 1;
        si.gz = (int)(dZ / q.cell_size) + 1;
        si.cell_off = (int)off;
        si.lox = si.loy = si.loz = r;
        si.hix = dX - r;
        si.hiy = dY - r;
        si.hiz = dZ - r;
        table->push_back(si);
        off += (long long)si.gx * si.gy * si.gz;
        if (off > (1LL << 31) - 2) return LUSTRINE_ERR_UNSUPPORTED;
    }
    sp->num_cells = (int)off;
    return LUSTRINE_OK;
}

// The on-chip scene solve for a batch, where it applies: PBF mode on a dense
// grid, no static particles, every scene of at most SOLVE_MAX_SCENE particles,
// lists of at most 255 entries, in mixed precision boxes of at most
// SOLVE_MIXED_MAX_CELLS cells a side (the solve iterates on positions relative
// to the scene's box corner), and a GPU that runs clusters of SOLVE_CLUSTER
// CTAs with the solve's shared memory.  Scenes are packed into bins of
// SOLVE_CLUSTER CTAs (ceil(n / SOLVE_M) CTAs each, first fit by decreasing
// size).  The step keeps the per-stage kernels until lustrine_batch_set_solver
// (or the autotuner) selects the on-chip solve.
static int setup_onchip(lustrine_pbf* s) {
    s->onchip = false;
    s->onchip_clusters = s->onchip_clusters512 = 0;
    if (s->prm.mode != LUSTRINE_MODE_PBF || s->sp.hash_bits || s->ns > 0 || s->sp.max_nbrs > 255) return LUSTRINE_OK;
    const int S = (int)s->b_nfluid.size();
    for (int k = 0; k < S; k++)
        if (s->b_nfluid[(size_t)k] > SOLVE_MAX_SCENE) return LUSTRINE_OK;
    if (s->mixed())
        for (size_t k = 0; k < s->b_domains.size(); k++)
            if ((float)s->b_domains[k] > SOLVE_MIXED_MAX_CELLS * s->sp.cell) return LUSTRINE_OK;
    int clusters = 0, clusters512 = 0;
    scene_solve_prepare(s->mixed(), 512, &clusters512);
    if (!scene_solve_prepare(s->mixed(), 1024, &clusters) || clusters < 1) return LUSTRINE_OK;
    std::vector<int> order;
    for (int k = 0; k < S; k++)
        if (s->b_nfluid[(size_t)k] > 0) order.push_back(k);
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return s->b_nfluid[(size_t)a] > s->b_nfluid[(size_t)b]; });
    std::vector<int> room;        // free CTAs of every bin
    std::vector<SolveSlot> bins;  // SOLVE_CLUSTER per bin
    for (int k : order) {
        const int ctas = (s->b_nfluid[(size_t)k] + SOLVE_M - 1) / SOLVE_M;
        size_t b = 0;
        while (b < room.size() && room[b] < ctas) b++;
        if (b == room.size()) {
            room.push_back(SOLVE_CLUSTER);
            bins.resize(bins.size() + SOLVE_CLUSTER, SolveSlot{-1, 0, 0});
        }
        const int first = SOLVE_CLUSTER - room[b];
        for (int r = 0; r < ctas; r++) bins[b * SOLVE_CLUSTER + (size_t)(first + r)] = SolveSlot{k, r, ctas};
        room[b] -= ctas;
    }
    std::vector<int> slot0((size_t)S + 1, 0);
    for (int k = 0; k < S; k++) slot0[(size_t)k + 1] = slot0[(size_t)k] + s->b_nfluid[(size_t)k];
    s->num_bins = (int)room.size();
    int rc = dalloc(&s->d_bins, bins.size() ? bins.size() : 1);
    if (!rc) rc = dalloc(&s->d_scene_slot0, slot0.size());
    if (!rc) rc = dalloc(&s->d_queue, 2);
    if (rc) return rc;
    if (!bins.empty())
        CK(cudaMemcpy(s->d_bins, bins.data(), bins.size() * sizeof(SolveSlot), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s->d_scene_slot0, slot0.data(), slot0.size() * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemset(s->d_queue, 0, 2 * sizeof(int)));
    s->onchip_clusters = std::max(1, std::min(clusters, s->num_bins));
    s->onchip_clusters512 = clusters512 > 0 ? std::max(1, std::min(clusters512, s->num_bins)) : 0;
    s->onchip_threads = 1024;
    return LUSTRINE_OK;
}

extern "C" int lustrine_batch_create(const lustrine_pbf_params* p, int num_scenes, const int* domains,
                                     const int* n_fluid, const int* n_solid, lustrine_pbf** out) {
    if (!p || !out || num_scenes < 1 || !domains || !n_fluid) return LUSTRINE_ERR_ARGS;
    *out = nullptr;
    if (p->mode != LUSTRINE_MODE_PBF) return LUSTRINE_ERR_UNSUPPORTED;
    lustrine_pbf* s = new (std::nothrow) lustrine_pbf();
    if (!s) return LUSTRINE_ERR_NOMEM;
    s->b_domains.assign(domains, domains + 3 * (size_t)num_scenes);
    s->b_nfluid.assign(n_fluid, n_fluid + num_scenes);
    s->b_nsolid.assign((size_t)num_scenes, 0);
    if (n_solid) s->b_nsolid.assign(n_solid, n_solid + num_scenes);
    std::vector<SceneInfo> table;
    int rc = derive_batch(*p, s->b_domains, s->b_nfluid, s->b_nsolid, &s->sp, &s->cp, &table);
    if (rc) {
        delete s;
        return rc;
    }
    s->prm = *p;
    for (int a = 0; a < 3; a++) {
        int m = 1;
        for (int k = 0; k < num_scenes; k++) m = std::max(m, domains[3 * k + a]);
        s->prm.domain[a] = m;
    }
    s->n = s->sp.n;
    s->cap = s->n;
    s->ns = s->sp.ns;
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete s;
        return LUSTRINE_ERR_CUDA;
    }
    rc = ctx_alloc(s);
    // static maps: scene of every fluid and solid slot (scenes are contiguous slot ranges)
    std::vector<int> sof((size_t)s->n), ssof((size_t)s->ns);
    for (int k = 0, i = 0, j = 0; k < num_scenes; k++) {
        for (int c = 0; c < s->b_nfluid[k]; c++) sof[(size_t)i++] = k;
        for (int c = 0; c < s->b_nsolid[k]; c++) ssof[(size_t)j++] = k;
    }
    if (!rc) rc = dalloc(&s->d_scenes, table.size());
    if (!rc) rc = dalloc(&s->d_scene_of, sof.size());
    if (!rc) rc = dalloc(&s->d_solid_scene_of, ssof.size());
    if (!rc && cudaMemcpy(s->d_scenes, table.data(), table.size() * sizeof(SceneInfo), cudaMemcpyHostToDevice) != cudaSuccess)
        rc = LUSTRINE_ERR_CUDA;
    if (!rc && !sof.empty() &&
        cudaMemcpy(s->d_scene_of, sof.data(), sof.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
        rc = LUSTRINE_ERR_CUDA;
    if (!rc && !ssof.empty() &&
        cudaMemcpy(s->d_solid_scene_of, ssof.data(), ssof.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
        rc = LUSTRINE_ERR_CUDA;
    if (rc) {
        delete s;
        return rc;
    }
    s->sp.scenes = s->d_scenes;
    s->sp.scene_of = s->d_scene_of;
    s->sp.solid_scene_of = s->d_solid_scene_of;
    rc = setup_onchip(s);
    if (rc) {
        delete s;
        return rc;
    }
    *out = s;
    return LUSTRINE_OK;
}

extern "C" int lustrine_batch_set_solver(lustrine_pbf* s, int solver) {
    if (!s || !s->is_batch() || (solver != LUSTRINE_SOLVER_STAGES && solver != LUSTRINE_SOLVER_ONCHIP))
        return LUSTRINE_ERR_ARGS;
    if (solver == LUSTRINE_SOLVER_ONCHIP && !s->onchip_clusters) return LUSTRINE_ERR_UNSUPPORTED;
    if (s->onchip != (solver == LUSTRINE_SOLVER_ONCHIP)) {
        s->onchip = solver == LUSTRINE_SOLVER_ONCHIP;
        s->invalidate_graphs();
    }
    return LUSTRINE_OK;
}

extern "C" int lustrine_batch_get_solver(const lustrine_pbf* s, int* solver) {
    if (!s || !solver || !s->is_batch()) return LUSTRINE_ERR_ARGS;
    *solver = s->onchip ? LUSTRINE_SOLVER_ONCHIP : LUSTRINE_SOLVER_STAGES;
    return LUSTRINE_OK;
}

extern "C" int lustrine_batch_onchip_layout(const lustrine_pbf* s, int* clusters, int* bins, int* threads) {
    if (!s || !s->is_batch()) return LUSTRINE_ERR_ARGS;
    if (clusters) *clusters = s->onchip_threads == 512 ? s->onchip_clusters512 : s->onchip_clusters;
    if (bins) *bins = s->num_bins;
    if (threads) *threads = s->onchip_threads;
    return LUSTRINE_OK;
}

extern "C" int lustrine_batch_set_onchip_threads(lustrine_pbf* s, int threads) {
    if (!s || !s->is_batch() || (threads != 512 && threads != 1024)) return LUSTRINE_ERR_ARGS;
    if (!s->onchip_clusters || (threads == 512 && !s->onchip_clusters512)) return LUSTRINE_ERR_UNSUPPORTED;
    if (s->onchip_threads != threads) {
        s->onchip_threads = threads;
        s->invalidate_graphs();
    }
    return LUSTRINE_OK;
}

extern "C" int lustrine_pbf_destroy(lustrine_pbf* s) {
    if (!s) return LUSTRINE_ERR_ARGS;
    cudaStreamSynchronize(s->stream);
    delete s;
    return LUSTRINE_OK;
}

extern "C" int lustrine_pbf_set_params(lustrine_pbf* s, const lustrine_pbf_params* p) {
    if (!s || !p) return LUSTRINE_ERR_ARGS;
    if (p->precision != s->prm.precision ||
        p->domain[0] != s->prm.domain[0] || p->domain[1] != s->prm.domain[1] ||
        p->domain[2] != s->prm.domain[2] || p->max_neighbors != s->prm.max_neighbors ||
        p->cell_size != s->prm.cell_size || p->grid_mode != s->prm.grid_mode)
        return LUSTRINE_ERR_ARGS;
    StepParams sp;
    CellPack cp;
    int rc;
    if (s->is_batch()) {
        if (p->mode != LUSTRINE_MODE_PBF) return LUSTRINE_ERR_UNSUPPORTED;
        std::vector<SceneInfo> table;
        rc = derive_batch(*p, s->b_domains, s->b_nfluid, s->b_nsolid, &sp, &cp, &table);
        sp.scenes = s->sp.scenes;
        sp.scene_of = s->sp.scene_of;
        sp.solid_scene_of = s->sp.solid_scene_of;
        sp.dt = s->sp.dt;
        sp.inv_dt = s->sp.inv_dt;
    } else {
        rc = derive(*p, s->cap, s->ns, &sp, &cp);  // the grid table was sized for the capacity
        sp.n = s->n;
        sp.dt = s->sp.dt;
        sp.inv_dt = s->sp.inv_dt;
        sp.cell_sorted = s->sp.cell_sorted;
    }
    sp.solid_near = s->sp.solid_near;
    if (rc) return rc;
    // the grid's table (dense cells or hash buckets) was sized at creation
    if (sp.hash_bits != s->sp.hash_bits || sp.num_cells != s->sp.num_cells) return LUSTRINE_ERR_UNSUPPORTED;
    // the fluid steps re-sort the particles without the sand mode's attract
    // flags: entering sand mode from another mode starts them cleared
    if (p->mode == LUSTRINE_MODE_SAND && s->prm.mode != LUSTRINE_MODE_SAND && s->n > 0)
        CK(cudaMemsetAsync(s->att[s->cur], 0, (size_t)s->n * sizeof(int), s->stream));
    s->prm = *p;
    s->sp = sp;
    s->cp = cp;
    s->invalidate_graphs();
    return LUSTRINE_OK;
}

extern "C" int lustrine_pbf_get_params(const lustrine_pbf* s, lustrine_pbf_params* p) {
    if (!s || !p) return LUSTRINE_ERR_ARGS;
    *p = s->prm;
    return LUSTRINE_OK;
}

extern "C" int lustrine_pbf_counts(const lustrine_pbf* s, int* n_fluid, int* n_solid) {
    if (!s) return LUSTRINE_ERR_ARGS;
    if (n_fluid) *n_fluid = s->n;
    if (n_solid) *n_solid = s->ns;
    return LUSTRINE_OK;
}

void lustrine_pbf::invalidate_graphs() {
    for (int k = 0; k < 8; k++) {
        if (graph_exec[k]) cudaGraphExecDestroy(graph_exec[k]);
        graph_exec[k] = nullptr;
    }
    for (int k = 0; k < 2; k++) {
        if (host_graph[k]) cudaGraphExecDestroy(host_graph[k]);
        host_graph[k] = nullptr;
    }
    pred_ready = false;  // whatever invalidates the step may change the prediction too
    tiles_dirty = true;
    graphs_fresh = true;
}

// The tile totals a step of parity c scans (the other half is zeroed by that
// scan for the prediction of the following step).
static int* tiles_of(lustrine_pbf* s, int parity) {
    return s->tile_sum + (size_t)parity * cell_scan_tiles(s->sp.num_cells);
}

// Zero both halves of the tile totals (after a prediction was dropped).
static int clear_tiles(lustrine_pbf* s) {
    CK(cudaMemsetAsync(s->tile_sum, 0, 2 * (size_t)cell_scan_tiles(s->sp.num_cells) * sizeof(int), s->stream));
    s->tiles_dirty = false;
    return LUSTRINE_OK;
}

bool lustrine_pbf::mixed() const { return prm.precision != LUSTRINE_PRECISION_FP32; }

// Sort the static solids by cell once (ascending id within a cell).
static int setup_solids(lustrine_pbf* s) {
    const int ns = s->ns, C = s->sp.num_cells;
    StepParams p = s->sp;
    CK(cudaMemsetAsync(s->count, 0, (size_t)C * sizeof(int), s->stream));
    s->count_dirty = false;  // zero again after the scan below
    if (ns > 0) {
        if (s->prm.mode != LUSTRINE_MODE_PBF)  // get_cell_id's truncating division
            launch_key_ref(p, s->solid_raw, ns, s->key, s->rank, s->count, s->status, s->stream);
        else
            launch_key(s->mixed(), p, s->cp, s->solid_raw, ns, s->key, s->rank, s->count, s->cellk,
                       s->stream);
    }
    launch_scan(s->count, C, s->block_sums, s->sstart, s->stream);
    launch_sort_tail(s->key, s->rank, s->sstart, nullptr, ns, s->tmp, s->perm, s->stream);
    launch_gather_solid(s->perm, ns, s->solid_raw, s->solid, s->stream);
    if (p.hash_bits) launch_gather_int(s->perm, ns, s->cellk, s->solid_cell, s->stream);
    if (ns > 0) {  // PBF geometry (the reference-mode list build walks every cell)
        CK(cudaMemsetAsync(s->solid_near, 0, (size_t)C, s->stream));
        launch_mark_solid_near(s->mixed(), p, s->cp, s->solid_raw, ns, s->solid_near, s->stream);
    }
    CK(cudaGetLastError());
    return LUSTRINE_OK;
}

// Pack caller arrays (device memory, 3 floats per particle, caller order)
// into the state representation; slot k holds particle k.
static int pack_fluid(lustrine_pbf* s, const float* dx, const float* dv) {
    const int n = s->n, c = s->cur;
    s->slot_of_valid = false;
    if (!n) return LUSTRINE_OK;
    // caller order = slot order here; in a batch, particles come scene by scene
    launch_pack_pos(s->mixed(), s->sp, s->cp, dx, n, s->sp.scene_of, s->x[c], s->stream);
    if (dv)
        launch_pack_pos(false, s->sp, s->cp, dv, n, nullptr, s->v[c], s->stream);
    else
        CK(cudaMemsetAsync(s->v[c], 0, (size_t)n * sizeof(float4), s->stream));
    CK(cudaMemcpyAsync(s->id[c], s->iota, (size_t)n * sizeof(int), cudaMemcpyDeviceToDevice, s->stream));
    CK(cudaMemsetAsync(s->att[c], 0, (size_t)n * sizeof(int), s->stream));
    CK(cudaGetLastError());
    return LUSTRINE_OK;
}

static int pack_solids(lustrine_pbf* s, const float* dsolid) {
    if (s->ns > 0)
        launch_pack_pos(s->mixed(), s->sp, s->cp, dsolid, s->ns, s->sp.solid_scene_of, s->solid_raw, s->stream);
    CK(cudaGetLastError());
    int rc = setup_solids(s);
    if (rc) return rc;
    if (s->ns > 0)
        CK(cudaMemcpyAsync(s->solid_id, s->perm, (size_t)s->ns * sizeof(int), cudaMemcpyDeviceToDevice, s->stream));
    // the passes of a scene-frame context read the static particles in that frame
    if (s->ns > 0 && s->sp.frame) launch_to_scene_frame(s->sp, s->cp, s->solid, s->ns, s->stream);
    return LUSTRINE_OK;
}

extern "C" int lustrine_pbf_upload(lustrine_pbf* s, const float* x, const float* v, const float* solid) {
    if (!s || (!x && s->n > 0) || (s->ns > 0 && !solid)) return LUSTRINE_ERR_ARGS;
    const int n = s->n, ns = s->ns;
    s->cur = 0;
    s->invalidate_graphs();
    // staging: positions in out3d (6n floats), velocities and then solids in out3
    float* sx = (float*)s->out3d;
    if (n) CK(cudaMemcpyAsync(sx, x, (size_t)n * 3 * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    if (v && n) CK(cudaMemcpyAsync(s->out3, v, (size_t)n * 3 * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    int rc = pack_fluid(s, sx, v ? s->out3 : nullptr);
    if (rc) return rc;
    if (ns) CK(cudaMemcpyAsync(s->out3, solid, (size_t)ns * 3 * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    rc = pack_solids(s, s->out3);
    if (rc) return rc;
    CK(cudaStreamSynchronize(s->stream));
    s->have_state = true;
    s->lists_valid = false;
    s->cells_valid = false;
    return LUSTRINE_OK;
}

extern "C" int lustrine_pbf_upload_device(lustrine_pbf* s, const float* x, const float* v,
                                          const float* solid) {
    if (!s || (!x && s->n > 0) || (s->ns > 0 && !solid)) return LUSTRINE_ERR_ARGS;
    s->cur = 0;
    s->invalidate_graphs();
    int rc = pack_fluid(s, x, v);
    if (rc) return rc;
    rc = pack_solids(s, solid);
    if (rc) return rc;
    CK(cudaStreamSynchronize(s->stream));
    s->have_state = true;
    s->lists_valid = false;
    s->cells_valid = false;
    return LUSTRINE_OK;
}

// Device address of page-locked host memory the kernels can use directly,
// or nullptr (pageable memory goes through a staging copy).
static const void* host_view(const void* p) {
    if (!p) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

extern "C" int lustrine_pbf_upload_state_async(lustrine_pbf* s, const float* x, const float* v) {
    if (!s || !s->have_state || (!x && s->n > 0)) return LUSTRINE_ERR_ARGS;
    s->pred_ready = false;
    s->slot_of_valid = false;
    const int n = s->n;
    if (!n) return LUSTRINE_OK;
    const float* hx = (const float*)host_view(x);
    const float* hv = (const float*)host_view(v);
    if (hx && !s->is_batch() && (!v || hv)) {  // read straight from the page-locked buffers
        const int c = s->cur;
        launch_pack_state(s->mixed(), s->sp, s->cp, hx, hv, n, s->x[c], s->v[c], s->id[c], s->stream);
        CK(cudaGetLastError());
        return LUSTRINE_OK;
    }
    // Written in caller order into the current side; the next step re-sorts.
    float* sx = (float*)s->out3d;
    CK(cudaMemcpyAsync(sx, x, (size_t)n * 3 * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    if (v) CK(cudaMemcpyAsync(s->out3, v, (size_t)n * 3 * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    return pack_fluid(s, sx, v ? s->out3 : nullptr);
}

// Optional per-stage event marks for lustrine_pbf_profile_step.
struct StageMarks {
    cudaEvent_t ev[64];
    int stage[64];
    int count = 0;
    void mark(int stg, cudaStream_t st) {
        if (count < 64) {
            cudaEventRecord(ev[count], st);
            stage[count++] = stg;
        }
    }
};

// simulate_sand's per-call inputs from the caller's controls.
static SandParams sand_params(const lustrine_pbf* s) {
    const lustrine_sand_controls& c = s->sand;
    SandParams q;
    std::memset(&q, 0, sizeof(q));
    q.px = c.player_position[0];
    q.py = c.player_position[1];
    q.pz = c.player_position[2];
    q.attract = c.attract_flag != 0;
    q.blow = c.blow_flag != 0;
    q.prev_attract = s->prev_attract;
    q.attract_radius = c.attract_radius;
    q.blow_radius = c.blow_radius;
    q.attract_coeff = c.attract_coeff;
    q.blow_coeff = c.blow_coeff;
    q.radius = s->prm.particle_radius;
    q.diameter = c.particle_diameter;
    q.w = 1.0f / s->prm.mass;  // Simulate.cpp:185
    return q;
}

// Sand step (simulate_sand): integration and cell keys on side c, the stable
// sort into side o, lists, 4 contact/friction substeps ping-ponging between
// xs[o] and xs_alt; the last commits x, v and the attract flags back into
// side c, which the sort has consumed, so the committed side stays c and the
// particles are in this step's cell order (the reference re-orders its own
// arrays the same way).  The commit makes id[c] the identity: a particle's
// index is its position in that order, as in the reference.
static int enqueue_sand_step(lustrine_pbf* s, cudaStream_t st, StageMarks* mk) {
    const int c = s->cur, o = 1 - c, n = s->n, C = s->sp.num_cells;
    const StepParams& p = s->sp;
    const SandParams q = sand_params(s);
    int k = 0;
    launch_sand_predict(p, q, s->x[c], s->v[c], s->xs[c], s->att[c], s->key, s->rank, s->count, s->status, st);
    k += 1;
    if (mk) mk->mark(LUSTRINE_STAGE_PREDICT, st);
    launch_scan_tiles(s->count, C, tiles_of(s, c), s->start, st, false, tiles_of(s, o));
    k += scan_tiles_launches(C);
    if (mk) mk->mark(LUSTRINE_STAGE_SCAN, st);
    // stable by the particle's index (its slot after a sand step; a caller
    // index after sources or sinks changed the order), as the reference's
    // counting sort is (Sorting.cpp:29-32)
    launch_sort_state(s->key, s->rank, s->start, s->id[c], n, s->tmp, s->x[c], s->xs[c], nullptr, nullptr,
                      s->key_sorted, s->x[o], s->xs[o], nullptr, nullptr, s->att[c], s->att[o], nullptr, nullptr,
                      st);
    k += 2;
    if (mk) mk->mark(LUSTRINE_STAGE_SORT, st);
    launch_sand_lists(p, s->xs[o], s->key_sorted, s->start, s->solid, s->sstart, s->nbr, s->cnt, s->status, st);
    k += 1;
    if (mk) mk->mark(LUSTRINE_STAGE_LISTS, st);
    float4* a = s->xs[o];
    float4* b = s->xs_alt;
    for (int sub = 0; sub < 4; sub++) {
        const bool last = sub == 3;
        launch_sand_substep(p, q, a, b, s->x[o], s->nbr, s->cnt, s->solid, last ? s->x[c] : nullptr,
                            last ? s->v[c] : nullptr, s->att[o], s->att[c], s->id[c], st);
        k += 1;
        if (mk) mk->mark(LUSTRINE_STAGE_DELTA, st);
        float4* t = a;
        a = b;
        b = t;
    }
    return k;
}

// A page-locked host frame's download, split around the commit kernel: the
// positions it commits are the last position pass's output, so they go to
// the host on the side stream while XSPH runs; the velocities follow XSPH.
struct HostFrame {
    float* hx;
    float* hv;
};

// One step's launches.  Returns the number of kernels launched.
// predict: run the prediction kernel (else the previous step's commit
// kernel left it in xs_pred, key, rank, count); tail: the commit kernel
// predicts the next step (PBF mode only); hf: download into page-locked host
// buffers within the step (PBF fp32 only).
static int enqueue_step(lustrine_pbf* s, cudaStream_t st, StageMarks* mk = nullptr, bool predict = true,
                        bool tail = false, const HostFrame* hf = nullptr) {
    const int c = s->cur, o = 1 - c, n = s->n, C = s->sp.num_cells;
    const StepParams& p = s->sp;
    const bool mixed = s->mixed();
    int k = 0;
    if (mk) mk->mark(-1, st);
    // count[] is all zero here: zeroed at allocation and by every scan.
    // Step kernels use programmatic dependent launch.
    set_pdl(s->use_pdl);
    if (s->sand_mode()) {
        k = enqueue_sand_step(s, st, mk);
        s->lists_format = LUSTRINE_LISTS_COLUMN;
        set_pdl(false);
        return k;
    }
    const bool ref = s->prm.mode == LUSTRINE_MODE_REFERENCE;
    float4* xs_in = ref ? s->xs[c] : s->xs_pred;  // predicted positions, caller of the sort
    if (ref) {
        launch_predict_ref(p, s->x[c], s->v[c], s->xs[c], s->key, s->rank, s->count, s->status, st);
        k += 1;
    } else if (predict) {
        launch_predict(mixed, p, s->cp, s->x[c], s->v[c], xs_in, s->key, s->rank, s->count, s->cellk,
                       tiles_of(s, c), st);
        k += 1;
    }
    if (mk) mk->mark(LUSTRINE_STAGE_PREDICT, st);
    // PBF: the prediction (this step's or the previous commit kernel's)
    // counted the tile totals; the scan zeroes the other half for the next
    launch_scan_tiles(s->count, C, tiles_of(s, c), s->start, st, !ref, tiles_of(s, o));
    k += scan_tiles_launches(C, !ref);
    if (mk) mk->mark(LUSTRINE_STAGE_SCAN, st);
    // stable within a cell: by the caller's id in reference mode (the
    // reference's list order), by the previous slot otherwise
    const int* tie = s->prm.mode == LUSTRINE_MODE_REFERENCE ? s->id[c] : nullptr;
    // velocities are not carried: the last position pass recomputes them
    // (v = (x* - x) / dt) before anything reads them.  The per-stage PBF
    // step leaves the committed positions in the previous order too: the
    // sort records each new slot's previous slot and the last position pass
    // reads x there (the commit then writes the new side whole)
    const bool onchip = s->onchip && s->num_bins > 0;
    const bool keep_x = ref || onchip;
    launch_sort_state(s->key, s->rank, s->start, tie, n, s->tmp, s->x[c], xs_in, nullptr, s->id[c],
                      s->key_sorted, keep_x ? s->x[o] : nullptr, s->xs[o], s->v[o], s->id[o],
                      s->cell_sorted ? s->cellk : nullptr, s->cell_sorted, s->slot_of, keep_x ? nullptr : s->src,
                      st);
    k += 2;
    if (mk) mk->mark(LUSTRINE_STAGE_SORT, st);
    if (s->prm.mode == LUSTRINE_MODE_REFERENCE) {
        launch_lists_ref(p, s->xs[o], s->key_sorted, s->start, s->solid, s->sstart, s->nbr, s->cnt,
                         s->status, st);
        if (mk) mk->mark(LUSTRINE_STAGE_LISTS, st);
        launch_lambda_ref(p, s->xs[o], s->id[o], s->nbr, s->cnt, s->solid, s->lam_by_id, s->rho, st);
        if (mk) mk->mark(LUSTRINE_STAGE_LAMBDA, st);
        launch_delta_ref(p, s->xs[o], s->xs_alt, s->x[o], s->v[o], s->id[o], s->nbr, s->cnt, s->solid,
                         s->lam_by_id, st);
        if (mk) mk->mark(LUSTRINE_STAGE_DELTA, st);
        k += 3;
        s->lists_format = LUSTRINE_LISTS_COLUMN;
    } else if (onchip) {
        // the batch's lists, iterations, XSPH and commit in one persistent
        // launch of clusters (the lambdas end where the per-stage path leaves them)
        SolveArgs sa;
        sa.bins = s->d_bins;
        sa.num_bins = s->num_bins;
        sa.iters = s->prm.iterations;
        sa.queue = s->d_queue;
        sa.scene_slot0 = s->d_scene_slot0;
        sa.xs = s->xs[o];
        sa.x = s->x[o];
        sa.key_sorted = s->key_sorted;
        sa.start = s->start;
        sa.nbr = s->nbr;
        sa.cnt = s->cnt;
        sa.rho = s->rho;
        sa.lam_out = (s->prm.iterations % 2 == 1) ? s->xs[o] : s->xs_alt;
        sa.x_out = s->x[o];
        sa.v_out = s->v[o];
        sa.status = s->status;
        sa.xs_next = tail ? s->xs_pred : nullptr;
        sa.key = s->key;
        sa.rank = s->rank;
        sa.count = s->count;
        sa.cellk = s->cellk;
        sa.tile_count = tail ? tiles_of(s, o) : nullptr;
        launch_scene_solve(mixed, s->onchip_threads, p, s->cp, sa,
                           s->onchip_threads == 512 ? s->onchip_clusters512 : s->onchip_clusters, st);
        k += 1;
        s->lists_format = LUSTRINE_LISTS_COLUMN;
        if (mk) mk->mark(LUSTRINE_STAGE_SOLVE, st);
    } else {
        // iteration 0's lambda pass builds the neighbour lists as it goes
        // (compact records where the step allows them)
        StepParams pl = p;
        s->lists_format = compact_now(s);
        pl.rec = s->lists_format != LUSTRINE_LISTS_COLUMN ? s->rec : nullptr;
        pl.rec2 = pl.rec ? s->rec2 : nullptr;
        pl.wide = s->lists_format == LUSTRINE_LISTS_COMPACT_WIDE;
        pl.src = s->src;
        float4* a = s->xs[o];
        float4* b = s->xs_alt;
        const int iters = s->prm.iterations;
        const Tuning& tu = s->tune;
        for (int it = 0; it < iters; it++) {
            float* rho = it == iters - 1 ? s->rho : nullptr;  // densities of the last pass only
            if (it == 0) {
                launch_lists_lambda(mixed, tu, pl, s->cp, a, s->key_sorted, s->cell_sorted, s->start,
                                    s->solid, s->solid_cell, s->sstart, s->nbr, s->cnt, rho, s->status, st);
                if (mk) mk->mark(LUSTRINE_STAGE_LISTS, st);
            } else {
                launch_lambda(mixed, tu, pl, a, s->nbr, s->cnt, s->solid, rho, st);
                if (mk) mk->mark(LUSTRINE_STAGE_LAMBDA, st);
            }
            launch_delta(mixed, tu, pl, s->cp, a, b, s->nbr, s->cnt, s->solid, s->key_sorted, s->x[c],
                         it == iters - 1 ? s->vtmp : nullptr, st);
            if (mk) mk->mark(LUSTRINE_STAGE_DELTA, st);
            float4* t = a;
            a = b;
            b = t;
            k += 2;
        }
        if (hf) {  // positions out on the side stream (slots recorded by this step's sort)
            cudaEventRecord(s->fork_ev, st);
            cudaStreamWaitEvent(s->side, s->fork_ev, 0);
            launch_unpack_state(false, p, s->cp, a, nullptr, s->id[o], s->slot_of, true, n, hf->hx, nullptr,
                                s->side);
            k += 1;
        }
        launch_xsph(mixed, tu, pl, s->cp, a, s->vtmp, s->nbr, s->cnt, s->key_sorted, s->x[o], s->v[o],
                    tail ? s->xs_pred : nullptr, s->key, s->rank, s->count, s->cellk,
                    tail ? tiles_of(s, o) : nullptr, st);
        k += 1;
        if (hf) {
            if (hf->hv) {
                launch_unpack_state(false, p, s->cp, nullptr, s->v[o], s->id[o], s->slot_of, true, n, nullptr,
                                    hf->hv, st);
                k += 1;
            }
            cudaEventRecord(s->join_ev, s->side);
            cudaStreamWaitEvent(st, s->join_ev, 0);
        }
        if (mk) mk->mark(LUSTRINE_STAGE_XSPH, st);
    }
    set_pdl(false);
    return k;
}

// Host bookkeeping after the launches of a step that started on side c.
static void finish_step(lustrine_pbf* s, int c) {
    s->cur = s->sand_mode() ? c : 1 - c;  // the sand step commits into the side it started from
    s->slot_of_valid = !s->sand_mode();   // the fluid steps' sort recorded every particle's slot
    s->lists_valid = true;
    s->cells_valid = true;
    s->steps_done++;
    // PBF: iteration k's lambdas are written into xs[1 - c] for even k and
    // into xs_alt for odd k (the Jacobi ping-pong)
    s->lam_src = (s->prm.iterations % 2 == 1) ? s->xs[1 - c] : s->xs_alt;
}

// One step; tail_allowed: the commit kernel may predict the next step (a
// caller that replaces the state before it, like step_host, says no).
static int step_impl(lustrine_pbf* s, float dt, bool tail_allowed) {
    if (!s || !s->have_state) return LUSTRINE_ERR_ARGS;
    if (!(dt > 0.0f) || !std::isfinite(dt)) return LUSTRINE_ERR_ARGS;
    if (s->prm.mode == LUSTRINE_MODE_REFERENCE) {
        // Simulate.cpp:31: dt = glm::clamp(dt, 0.001f, 0.01f)
        dt = dt < 0.001f ? 0.001f : dt;
        dt = dt > 0.01f ? 0.01f : dt;
    }
    if (s->sp.dt != dt) {
        s->sp.dt = dt;
        s->sp.inv_dt = 1.0f / dt;
        s->invalidate_graphs();
    }
    if (s->sand_mode()) {
        // the captured sand step holds its controls (flags, player, previous flag)
        const SandParams q = sand_params(s);
        if (std::memcmp(&q, &s->sand_captured, sizeof(q)) != 0) {
            s->invalidate_graphs();
            s->sand_captured = q;
        }
    }
    const int c = s->cur;
    const bool pbf = s->prm.mode == LUSTRINE_MODE_PBF;
    // the previous step predicted this one unless something changed since
    const bool predict = !(pbf && s->pred_ready && s->pred_dt == dt);
    const bool tail = pbf && tail_allowed;
    if (predict && s->count_dirty)  // a histogram of a prediction that will not be used
        CK(cudaMemsetAsync(s->count, 0, (size_t)s->sp.num_cells * sizeof(int), s->stream));
    if (predict && (s->count_dirty || s->tiles_dirty)) {  // and its tile totals
        int rc = clear_tiles(s);
        if (rc) return rc;
    }
    s->count_dirty = false;
    const int gi = c + (predict ? 2 : 0) + (tail ? 4 : 0);
    // right after an invalidation, launch directly (see graphs_fresh)
    const bool use_graph = s->prm.use_graph && !(s->graphs_fresh && !s->graph_exec[gi]);
    s->graphs_fresh = false;
    if (use_graph) {
        if (!s->graph_exec[gi]) {
            cudaGraph_t g = nullptr;
            CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
            s->graph_launches[gi] = enqueue_step(s, s->stream, nullptr, predict, tail);
            cudaError_t e = cudaStreamEndCapture(s->stream, &g);
            if (e != cudaSuccess) return lgb_cuda_status(e, "cudaStreamEndCapture");
            e = cudaGraphInstantiate(&s->graph_exec[gi], g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return lgb_cuda_status(e, "cudaGraphInstantiate");
        }
        CK(cudaGraphLaunch(s->graph_exec[gi], s->stream));
        s->launches = s->graph_launches[gi];
    } else {
        s->launches = enqueue_step(s, s->stream, nullptr, predict, tail);
        CK(cudaGetLastError());
    }
    finish_step(s, c);
    s->pred_ready = tail;
    s->pred_dt = dt;
    s->count_dirty = tail;
    if (s->sand_mode()) s->prev_attract = s->sand.attract_flag != 0;  // Simulate.cpp:322
    return LUSTRINE_OK;
}

extern "C" int lustrine_pbf_step(lustrine_pbf* s, float dt) { return step_impl(s, dt, true); }

extern "C" int lustrine_pbf_steps(lustrine_pbf* s, float dt, int count) {
    if (count < 0) return LUSTRINE_ERR_ARGS;
    for (int k = 0; k < count; k++) {
        int rc = lustrine_pbf_step(s, dt);
        if (rc) return rc;
    }
    return LUSTRINE_OK;
}

extern "C" int lustrine_pbf_profile_step(lustrine_pbf* s, float dt, double* stage_ms,
                                         int* stage_launches, int num_stages) {
    if (!s || !s->have_state || !stage_ms || num_stages <= 0) return LUSTRINE_ERR_ARGS;
    if (!(dt > 0.0f) || !std::isfinite(dt)) return LUSTRINE_ERR_ARGS;
    if (s->prm.mode == LUSTRINE_MODE_REFERENCE) {
        dt = dt < 0.001f ? 0.001f : dt;
        dt = dt > 0.01f ? 0.01f : dt;
    }
    if (s->sp.dt != dt) {
        s->sp.dt = dt;
        s->sp.inv_dt = 1.0f / dt;
        s->invalidate_graphs();
    }
    if (s->count_dirty) CK(cudaMemsetAsync(s->count, 0, (size_t)s->sp.num_cells * sizeof(int), s->stream));
    s->count_dirty = false;
    s->pred_ready = false;
    int trc = clear_tiles(s);
    if (trc) return trc;
    StageMarks mk;
    for (int e = 0; e < 64; e++) CK(cudaEventCreate(&mk.ev[e]));
    s->launches = enqueue_step(s, s->stream, &mk);
    cudaError_t err = cudaGetLastError();
    if (err == cudaSuccess) err = cudaStreamSynchronize(s->stream);
    for (int k = 0; k < num_stages; k++) {
        stage_ms[k] = 0.0;
        if (stage_launches) stage_launches[k] = 0;
    }
    if (err == cudaSuccess)
        for (int e = 1; e < mk.count; e++) {
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, mk.ev[e - 1], mk.ev[e]);
            const int stg = mk.stage[e];
            if (stg >= 0 && stg < num_stages) {
                stage_ms[stg] += ms;
                if (stage_launches) stage_launches[stg] += 1;
            }
        }
    for (int e = 0; e < 64; e++) cudaEventDestroy(mk.ev[e]);
    if (err != cudaSuccess) return lgb_cuda_status(err, "profile_step");
    finish_step(s, s->cur);
    if (s->sand_mode()) s->prev_attract = s->sand.attract_flag != 0;
    return LUSTRINE_OK;
}

extern "C" int lustrine_pbf_set_tuning(lustrine_pbf* s, const lustrine_pbf_tuning* t) {
    if (!s || !t) return LUSTRINE_ERR_ARGS;
    auto ok = [](int b) { return b == 64 || b == 128 || b == 256; };
    auto ok_u = [](int u) { return u == 1 || u == 2 || u == 4 || u == 8; };
    const int xu = t->xsph_unroll ? t->xsph_unroll : t->unroll;  // 0: as the other passes
    const int ppt = t->particles_per_thread ? t->particles_per_thread : 1;
    if (!ok(t->block) || !ok(t->list_block) || !ok_u(t->unroll) || !ok_u(xu) || (ppt != 1 && ppt != 2) ||
        (ppt == 2 && t->unroll > 2) || (t->list_format != LUSTRINE_LISTS_COLUMN && t->list_format != LUSTRINE_LISTS_COMPACT))
        return LUSTRINE_ERR_ARGS;
    if (t->solver != LUSTRINE_SOLVER_STAGES && t->solver != LUSTRINE_SOLVER_ONCHIP) return LUSTRINE_ERR_ARGS;
    if (s->is_batch()) {
        int rc = lustrine_batch_set_solver(s, t->solver);
        if (rc) return rc;
        if (t->solver == LUSTRINE_SOLVER_ONCHIP && t->solver_threads) {
            rc = lustrine_batch_set_onchip_threads(s, t->solver_threads);
            if (rc) return rc;
        }
    } else if (t->solver != LUSTRINE_SOLVER_STAGES) {
        return LUSTRINE_ERR_ARGS;
    }
    s->tune = Tuning{t->block, t->unroll, t->list_block, xu, ppt, t->list_format};
    s->invalidate_graphs();
    return LUSTRINE_OK;
}

extern "C" int lustrine_pbf_get_tuning(const lustrine_pbf* s, lustrine_pbf_tuning* t) {
    if (!s || !t) return LUSTRINE_ERR_ARGS;
    t->block = s->tune.block;
    t->unroll = s->tune.unroll;
    t->list_block = s->tune.list_block;
    t->xsph_unroll = s->tune.xsph_unroll;
    t->particles_per_thread = s->tune.ppt;
    t->solver = s->onchip ? LUSTRINE_SOLVER_ONCHIP : LUSTRINE_SOLVER_STAGES;
    t->solver_threads = s->onchip_threads;
    t->list_format = s->tune.lists;
    return LUSTRINE_OK;
}

// Copies of the committed state, so every candidate starts from it.
struct Snapshot {
    float4 *x = nullptr, *v = nullptr;
    int* id = nullptr;
    ~Snapshot() {
        cudaFree(x);
        cudaFree(v);
        cudaFree(id);
    }
};

static int snapshot_take(lustrine_pbf* s, Snapshot& sn) {
    const size_t n = (size_t)(s->n ? s->n : 1);
    CK(cudaMalloc((void**)&sn.x, n * sizeof(float4)));
    CK(cudaMalloc((void**)&sn.v, n * sizeof(float4)));
    CK(cudaMalloc((void**)&sn.id, n * sizeof(int)));
    const int c = s->cur;
    CK(cudaMemcpyAsync(sn.x, s->x[c], (size_t)s->n * sizeof(float4), cudaMemcpyDeviceToDevice, s->stream));
    CK(cudaMemcpyAsync(sn.v, s->v[c], (size_t)s->n * sizeof(float4), cudaMemcpyDeviceToDevice, s->stream));
    CK(cudaMemcpyAsync(sn.id, s->id[c], (size_t)s->n * sizeof(int), cudaMemcpyDeviceToDevice, s->stream));
    return LUSTRINE_OK;
}

static int snapshot_restore(lustrine_pbf* s, const Snapshot& sn, int side) {
    s->cur = side;
    s->pred_ready = false;
    CK(cudaMemcpyAsync(s->x[side], sn.x, (size_t)s->n * sizeof(float4), cudaMemcpyDeviceToDevice, s->stream));
    CK(cudaMemcpyAsync(s->v[side], sn.v, (size_t)s->n * sizeof(float4), cudaMemcpyDeviceToDevice, s->stream));
    CK(cudaMemcpyAsync(s->id[side], sn.id, (size_t)s->n * sizeof(int), cudaMemcpyDeviceToDevice, s->stream));
    return LUSTRINE_OK;
}

// Milliseconds per step of `steps` graph-replayed steps from the snapshot
// with the current tuning (two untimed steps capture both parities' graphs).
// Milliseconds per step of the current launch shape: the median over three
// timings of `steps` graph-replayed steps, each from the snapshot (one
// timing is at the mercy of clock and scheduling noise; the shapes differ by
// a few per cent).
static int time_candidate(lustrine_pbf* s, const Snapshot& sn, int side, float dt, int steps, float* ms) {
    int rc = snapshot_restore(s, sn, side);
    if (rc) return rc;
    // untimed steps capture the graphs the timed ones replay (both parities,
    // with and without a prediction of their own), the first one included
    s->graphs_fresh = false;
    for (int k = 0; k < 3; k++)
        if ((rc = lustrine_pbf_step(s, dt))) return rc;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float t[3] = {0.0f, 0.0f, 0.0f};
    cudaError_t e = cudaSuccess;
    for (int r = 0; r < 3 && !rc && e == cudaSuccess; r++) {
        if ((rc = snapshot_restore(s, sn, side))) break;
        cudaEventRecord(e0, s->stream);
        for (int k = 0; k < steps && !rc; k++) rc = lustrine_pbf_step(s, dt);
        cudaEventRecord(e1, s->stream);
        e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t[r], e0, e1);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if (e != cudaSuccess) return lgb_cuda_status(e, "autotune timing");
    std::sort(t, t + 3);
    *ms = t[1] / (float)steps;
    return LUSTRINE_OK;
}

extern "C" int lustrine_pbf_autotune(lustrine_pbf* s, float dt, int steps, lustrine_pbf_tuning* best,
                                     float* best_ms) {
    if (!s || !s->have_state || steps < 1 || !(dt > 0.0f)) return LUSTRINE_ERR_ARGS;
    if (s->prm.mode != LUSTRINE_MODE_PBF || s->n == 0) {
        // the reference-semantics kernels have a single launch shape
        if (best) lustrine_pbf_get_tuning(s, best);
        if (best_ms) *best_ms = 0.0f;
        return LUSTRINE_OK;
    }
    const int use_graph = s->prm.use_graph;
    s->prm.use_graph = 1;
    Snapshot sn;
    int rc = snapshot_take(s, sn);
    const int side = s->cur;
    Tuning keep = s->tune, top = s->tune;
    const bool keep_onchip = s->onchip;
    const int keep_threads = s->onchip_threads;
    s->onchip = false;  // the per-stage kernels' shapes first
    float top_ms = 3.4e38f;
    static const int blocks[3] = {64, 128, 256};
    static const int unrolls[4] = {1, 2, 4, 8};
    // the iteration kernels' shape first (block x gathers in flight x
    // particles per thread x list format, compact first where it can
    // apply), then the list build's block size
    const int formats = s->rec && s->ns == 0 && compact_capable(s) != LUSTRINE_LISTS_COLUMN ? 2 : 1;
    for (int lf = 0; lf < formats && !rc; lf++)
        for (int bi = 0; bi < 3 && !rc; bi++)
            for (int ui = 0; ui < 4 && !rc; ui++)
                for (int pi = 1; pi <= 2 && !rc; pi++) {
                    const int lists = formats == 2 ? 1 - lf : keep.lists;
                    if (pi == 2 && (unrolls[ui] > 2 || (formats == 2 && lists == 1))) continue;
                    s->tune = Tuning{blocks[bi], unrolls[ui], keep.list_block, unrolls[ui], pi, lists};
                    s->invalidate_graphs();
                    float ms = 0.0f;
                    rc = time_candidate(s, sn, side, dt, steps, &ms);
                    if (!rc && ms < top_ms) {
                        top_ms = ms;
                        top = s->tune;
                    }
                }
    for (int bi = 0; bi < 3 && !rc; bi++) {
        s->tune = Tuning{top.block, top.unroll, blocks[bi], top.xsph_unroll, top.ppt, top.lists};
        s->invalidate_graphs();
        float ms = 0.0f;
        rc = time_candidate(s, sn, side, dt, steps, &ms);
        if (!rc && ms < top_ms) {
            top_ms = ms;
            top = s->tune;
        }
    }
    // then the XSPH pass's gathers in flight (it gains from more than the others)
    for (int ui = 0; ui < 4 && !rc; ui++) {
        if (unrolls[ui] == top.xsph_unroll) continue;
        s->tune = Tuning{top.block, top.unroll, top.list_block, unrolls[ui], top.ppt, top.lists};
        s->invalidate_graphs();
        float ms = 0.0f;
        rc = time_candidate(s, sn, side, dt, steps, &ms);
        if (!rc && ms < top_ms) {
            top_ms = ms;
            top = s->tune;
        }
    }
    // a batch: the on-chip solve (both CTA widths) against the best per-stage shape
    bool top_onchip = false;
    int top_threads = keep_threads;
    if (!rc && s->onchip_clusters > 0) {
        s->tune = top;
        for (int threads : {512, 1024}) {
            if (threads == 512 && !s->onchip_clusters512) continue;
            s->onchip = true;
            s->onchip_threads = threads;
            s->invalidate_graphs();
            float ms = 0.0f;
            rc = time_candidate(s, sn, side, dt, steps, &ms);
            if (rc) break;
            if (ms < top_ms) {
                top_ms = ms;
                top_onchip = true;
                top_threads = threads;
            }
        }
    }
    s->tune = rc ? keep : top;
    s->onchip = rc ? keep_onchip : top_onchip;
    s->onchip_threads = rc ? keep_threads : top_threads;
    s->invalidate_graphs();
    s->prm.use_graph = use_graph;
    int rc2 = snapshot_restore(s, sn, side);
    if (!rc) rc = rc2;
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (!rc && e != cudaSuccess) rc = lgb_cuda_status(e, "autotune");
    if (best) lustrine_pbf_get_tuning(s, best);
    if (best_ms) *best_ms = top_ms;
    return rc;
}

extern "C" int lustrine_pbf_synchronize(lustrine_pbf* s) {
    if (!s) return LUSTRINE_ERR_ARGS;
    CK(cudaStreamSynchronize(s->stream));
    return LUSTRINE_OK;
}

// Device-side unpermute of the current state into out3 (positions) /
// out3d (velocities) in caller order.
static void unpermute_state(lustrine_pbf* s, bool pos, bool vel) {
    const int c = s->cur;
    if (pos) launch_unpermute_pos(s->mixed(), s->sp, s->cp, s->x[c], s->id[c], s->n, s->out3, s->stream);
    if (vel)
        launch_unpermute_pos(false, s->sp, s->cp, s->v[c], s->id[c], s->n, (float*)s->out3d, s->stream);
}

extern "C" int lustrine_pbf_download(lustrine_pbf* s, float* x, float* v, float* lambdas, float* density) {
    if (!s || !s->have_state) return LUSTRINE_ERR_ARGS;
    const int n = s->n;
    if (!n) return LUSTRINE_OK;
    const size_t b3 = (size_t)n * 3 * sizeof(float);
    unpermute_state(s, x != nullptr, v != nullptr);
    if (x) CK(cudaMemcpyAsync(x, s->out3, b3, cudaMemcpyDeviceToHost, s->stream));
    if (v) CK(cudaMemcpyAsync(v, s->out3d, b3, cudaMemcpyDeviceToHost, s->stream));
    if (lambdas || density) {
        std::vector<int> ids((size_t)n);
        CK(cudaMemcpyAsync(ids.data(), s->id[s->cur], (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, s->stream));
        std::vector<float> lam((size_t)n), rho((size_t)n);
        const bool ref = s->prm.mode == LUSTRINE_MODE_REFERENCE;
        if (lambdas) {
            if (ref)
                CK(cudaMemcpyAsync(lambdas, s->lam_by_id, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
            else if (s->lam_src)  // PBF: lambdas are the w of the last pass's positions
                CK(cudaMemcpy2DAsync(lam.data(), sizeof(float),
                                     reinterpret_cast<const char*>(s->lam_src) + 3 * sizeof(float),
                                     sizeof(float4), sizeof(float), (size_t)n, cudaMemcpyDeviceToHost,
                                     s->stream));
        }
        if (density) CK(cudaMemcpyAsync(rho.data(), s->rho, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
        for (int k = 0; k < n; k++) {
            const int i = ids[(size_t)k];
            if (lambdas && !ref) lambdas[i] = lam[(size_t)k];
            if (density) density[i] = rho[(size_t)k];
        }
    }
    CK(cudaStreamSynchronize(s->stream));
    return LUSTRINE_OK;
}

extern "C" int lustrine_pbf_download_state_async(lustrine_pbf* s, float* x, float* v) {
    if (!s || !s->have_state) return LUSTRINE_ERR_ARGS;
    const int n = s->n;
    if (!n) return LUSTRINE_OK;
    float* hx = (float*)host_view(x);
    float* hv = (float*)host_view(v);
    if ((!x || hx) && (!v || hv)) {  // write straight into the page-locked buffers
        const int c = s->cur;
        launch_unpack_state(s->mixed(), s->sp, s->cp, s->x[c], s->v[c], s->id[c], s->slot_of, s->slot_of_valid, n,
                            hx, hv, s->stream);
        s->slot_of_valid = true;
        CK(cudaGetLastError());
        return LUSTRINE_OK;
    }
    const size_t b3 = (size_t)n * 3 * sizeof(float);
    unpermute_state(s, x != nullptr, v != nullptr);
    if (x) CK(cudaMemcpyAsync(x, s->out3, b3, cudaMemcpyDeviceToHost, s->stream));
    if (v) CK(cudaMemcpyAsync(v, s->out3d, b3, cudaMemcpyDeviceToHost, s->stream));
    return LUSTRINE_OK;
}

// One frame of a host that keeps the state: upload, step, download, wait.
extern "C" int lustrine_pbf_step_host(lustrine_pbf* s, float dt, float* x, float* v) {
    if (!s || !x) return LUSTRINE_ERR_ARGS;
    const float* hx = (const float*)host_view(x);
    const float* hv = (const float*)host_view(v);
    if (s->prm.mode == LUSTRINE_MODE_PBF && !s->is_batch() && s->have_state && s->n > 0 && hx && (!v || hv) &&
        dt > 0.0f && std::isfinite(dt)) {
        // page-locked arrays: the upload is fused with the step's prediction,
        // the rest of the step runs from that prediction, and the download
        // reads the slots the sort recorded
        if (s->sp.dt != dt) {
            s->sp.dt = dt;
            s->sp.inv_dt = 1.0f / dt;
            s->invalidate_graphs();
        }
        if (s->count_dirty) CK(cudaMemsetAsync(s->count, 0, (size_t)s->sp.num_cells * sizeof(int), s->stream));
        if (s->count_dirty || s->tiles_dirty) {
            int rc = clear_tiles(s);
            if (rc) return rc;
        }
        s->count_dirty = false;
        const int c = s->cur;
        if (!s->mixed() && s->prm.use_graph) {
            // the whole frame as one graph for this buffer pair: upload fused
            // with the prediction, the step, the positions downloaded while
            // the commit kernel runs, then the velocities
            if (!s->side) {
                CK(cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking));
                CK(cudaEventCreateWithFlags(&s->fork_ev, cudaEventDisableTiming));
                CK(cudaEventCreateWithFlags(&s->join_ev, cudaEventDisableTiming));
            }
            if (!s->host_graph[c] || s->host_graph_ptr[c][0] != hx || s->host_graph_ptr[c][1] != hv) {
                if (s->host_graph[c]) cudaGraphExecDestroy(s->host_graph[c]);
                s->host_graph[c] = nullptr;
                cudaGraph_t g = nullptr;
                CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
                launch_pack_predict(false, s->sp, s->cp, hx, hv, s->n, s->x[c], s->id[c], s->xs_pred, s->key,
                                    s->rank, s->count, s->cellk, tiles_of(s, c), s->stream);
                const HostFrame hf{const_cast<float*>(hx), const_cast<float*>(hv)};
                const int k = 1 + enqueue_step(s, s->stream, nullptr, false, false, &hf);
                cudaError_t e = cudaStreamEndCapture(s->stream, &g);
                if (e != cudaSuccess) return lgb_cuda_status(e, "cudaStreamEndCapture (host frame)");
                e = cudaGraphInstantiate(&s->host_graph[c], g, 0);
                cudaGraphDestroy(g);
                if (e != cudaSuccess) return lgb_cuda_status(e, "cudaGraphInstantiate (host frame)");
                s->host_graph_ptr[c][0] = hx;
                s->host_graph_ptr[c][1] = hv;
                s->host_graph_launches[c] = k;
            }
            CK(cudaGraphLaunch(s->host_graph[c], s->stream));
            s->launches = s->host_graph_launches[c];
            finish_step(s, c);
            s->pred_ready = false;
            s->pred_dt = dt;
            s->count_dirty = false;
            CK(cudaStreamSynchronize(s->stream));
            return LUSTRINE_OK;
        }
        launch_pack_predict(s->mixed(), s->sp, s->cp, hx, hv, s->n, s->x[c], s->id[c], s->xs_pred, s->key, s->rank,
                            s->count, s->cellk, tiles_of(s, c), s->stream);
        CK(cudaGetLastError());
        s->pred_ready = true;
        s->pred_dt = dt;
        int rc = step_impl(s, dt, false);
        if (!rc) rc = lustrine_pbf_download_state_async(s, x, v);
        if (!rc) CK(cudaStreamSynchronize(s->stream));
        return rc;
    }
    int rc = lustrine_pbf_upload_state_async(s, x, v);
    if (!rc) rc = step_impl(s, dt, false);  // the next frame replaces the state
    if (!rc) rc = lustrine_pbf_download_state_async(s, x, v);
    if (!rc) CK(cudaStreamSynchronize(s->stream));
    return rc;
}

extern "C" int lustrine_pbf_download_positions_f64(lustrine_pbf* s, double* x) {
    if (!s || !s->have_state || !x) return LUSTRINE_ERR_ARGS;
    const int n = s->n;
    if (!n) return LUSTRINE_OK;
    launch_unpermute_pos_d(s->mixed(), s->sp, s->cp, s->x[s->cur], s->id[s->cur], n, s->out3d, s->stream);
    CK(cudaMemcpyAsync(x, s->out3d, (size_t)n * 3 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return LUSTRINE_OK;
}

extern "C" int lustrine_pbf_neighbors(lustrine_pbf* s, int* count, int* idx, int cap) {
    if (!s || !count || (idx && cap <= 0)) return LUSTRINE_ERR_ARGS;
    if (!s->lists_valid) return LUSTRINE_ERR_ARGS;
    const int n = s->n, maxn = s->sp.max_nbrs;
    if (!n) return LUSTRINE_OK;
    std::vector<int> cnt((size_t)n), ids((size_t)n), nbr((size_t)maxn * n), sid((size_t)s->ns);
    // Lists refer to the sorted slots of the state the step started from:
    // the committed side's id array maps fluid slots; solid slots map back
    // through the solid sort permutation.
    const bool compact = s->lists_format != LUSTRINE_LISTS_COLUMN;
    std::vector<uint4> rec(compact ? (size_t)n : 0), rec2(rec.size());
    if (compact) {
        CK(cudaMemcpyAsync(rec.data(), s->rec, (size_t)n * sizeof(uint4), cudaMemcpyDeviceToHost, s->stream));
        CK(cudaMemcpyAsync(rec2.data(), s->rec2, (size_t)n * sizeof(uint4), cudaMemcpyDeviceToHost, s->stream));
    } else
        CK(cudaMemcpyAsync(cnt.data(), s->cnt, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(ids.data(), s->id[s->cur], (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(nbr.data(), s->nbr, (size_t)maxn * n * sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    if (s->ns) CK(cudaMemcpyAsync(sid.data(), s->solid_id, (size_t)s->ns * sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    if (compact) {
        // compact records into the column form: count, the records' entries
        // (16-bit: the scene's first slot + offset; wide: the slot; the
        // second record is written only for lists longer than its first),
        // the rest from the overflow rows
        const bool wide = s->lists_format == LUSTRINE_LISTS_COMPACT_WIDE;
        const int R = wide ? WIDE_RECORDS : COMPACT_RECORDS;
        std::vector<int> col((size_t)maxn * n);
        for (int k = 0; k < n; k++) {
            const uint4 r = rec[(size_t)k], x = rec2[(size_t)k];
            const unsigned w[7] = {r.y, r.z, r.w, x.x, x.y, x.z, x.w};
            const int c = wide ? (int)r.x : (int)(r.x & 0xFFu), base = wide ? 0 : (int)(r.x >> 8);
            cnt[(size_t)k] = c;
            for (int e = 0; e < c; e++)
                col[(size_t)e * n + k] = e >= R ? nbr[(size_t)(e - R) * n + k]
                                         : wide ? (int)w[e]
                                                : base + (int)((w[e >> 1] >> ((e & 1) * 16)) & 0xFFFFu);
        }
        nbr.swap(col);
    }
    int rc = LUSTRINE_OK;
    // reference-semantics lists: slot t >= 0 or static slot -1 - u; the sand
    // lists leave the particle itself out (the reference lists it twice)
    const bool ref = s->prm.mode != LUSTRINE_MODE_PBF;
    for (int k = 0; k < n; k++) {
        const int i = ids[(size_t)k];
        const int c = cnt[(size_t)k];
        // PBF lists leave the particle itself out; it is reported first
        const int self = s->prm.mode == LUSTRINE_MODE_PBF ? 1 : 0;
        count[i] = c + self;
        if (!idx) continue;
        if (c + self > cap) rc = LUSTRINE_ERR_NBR_OVERFLOW;
        if (self) idx[(size_t)i * cap] = i;
        for (int e = 0; e < c && e + self < cap; e++) {
            int j = nbr[(size_t)e * n + k];
            if (ref)
                idx[(size_t)i * cap + e] = j >= 0 ? ids[(size_t)j] : n + sid[(size_t)(-1 - j)];
            else  // PBF entry: slot in bits 0-24, solid flag in bit 31
                idx[(size_t)i * cap + e + 1] = j >= 0 ? ids[(size_t)(j & 0x1FFFFFF)] : n + sid[(size_t)(j & 0x1FFFFFF)];
        }
    }
    return rc;
}

extern "C" int lustrine_pbf_list_format(const lustrine_pbf* s, int* format) {
    if (!s || !format) return LUSTRINE_ERR_ARGS;
    *format = s->lists_format;
    return LUSTRINE_OK;
}

extern "C" int lustrine_pbf_reduce(lustrine_pbf* s, double out[9]) {
    if (!s || !s->have_state || !out) return LUSTRINE_ERR_ARGS;
    const int c = s->cur;
    // densities exist after a fluid step (the sand step computes none)
    const bool dens = s->steps_done && !s->sand_mode();
    launch_reduce(s->mixed(), s->sp, s->cp, s->x[c], s->v[c], dens ? s->rho : nullptr, s->red,
                  s->stream);
    CK(cudaMemcpyAsync(out, s->red, 9 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    if (out[0] > 0.0)
        for (int k = 5; k < 8; k++) out[k] /= out[0];
    return LUSTRINE_OK;
}

// Lustrine.cpp:864-914 with get_cell_indices (neighbors/Utils.hpp:13-21): the
// corners are clamped to [cell / 2, domain - cell / 2] per axis (float,
// bounds formed in double as glm does) and truncated to cell indices; the
// count is that of the particles the last step binned in those cells.
extern "C" int lustrine_pbf_query_cell_count(lustrine_pbf* s, const float min_pos[3],
                                             const float max_pos[3], int include_solid, int* count) {
    if (!s || !min_pos || !max_pos || !count) return LUSTRINE_ERR_ARGS;
    if (s->is_batch()) return LUSTRINE_ERR_UNSUPPORTED;
    *count = 0;
    const float cell = s->prm.cell_size;
    const int g[3] = {s->sp.gx, s->sp.gy, s->sp.gz};
    int box[6];
    for (int a = 0; a < 3; a++) {
        const float lo = (float)((double)cell * 0.5);
        const float hi = (float)((double)(float)s->prm.domain[a] - (double)cell * 0.5);
        int i0 = (int)(std::fmin(std::fmax(min_pos[a], lo), hi) / cell);
        int i1 = (int)(std::fmin(std::fmax(max_pos[a], lo), hi) / cell);
        i0 = std::min(std::max(i0, 0), g[a] - 1);
        i1 = std::min(std::max(i1, 0), g[a] - 1);
        box[2 * a] = i0;
        box[2 * a + 1] = i1;
    }
    // an empty range (min above max on an axis) counts nothing, as the
    // reference's loops do
    if (box[0] > box[1] || box[2] > box[3] || box[4] > box[5]) return LUSTRINE_OK;
    if (!s->cells_valid) return LUSTRINE_OK;  // no step yet: the cell table is empty
    CK(cudaMemsetAsync(s->qcount, 0, sizeof(int), s->stream));
    const bool solids = include_solid && s->ns > 0;
    launch_query_cells(s->sp, s->cp, box, s->start, solids ? s->sstart : nullptr, s->cell_sorted,
                       solids ? s->solid_cell : nullptr, s->qcount, s->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(count, s->qcount, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return LUSTRINE_OK;
}

extern "C" int lustrine_pbf_status(lustrine_pbf* s) {
    if (!s) return LUSTRINE_ERR_ARGS;
    int st[4] = {0, 0, 0, 0};
    CK(cudaMemcpyAsync(st, s->status, sizeof(st), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaMemsetAsync(s->status, 0, sizeof(st), s->stream));
    CK(cudaStreamSynchronize(s->stream));
    if (st[0] & ST_TIMEOUT) return LUSTRINE_ERR_TIMEOUT;
    if (st[0] & ST_NBR_OVERFLOW) return LUSTRINE_ERR_NBR_OVERFLOW;
    if (st[0] & ST_CELL_RANGE) return LUSTRINE_ERR_CELL_RANGE;
    if (st[0] & ST_BAD_VALUE) return LUSTRINE_ERR_BAD_VALUE;
    return LUSTRINE_OK;
}

extern "C" void lustrine_sand_controls_default(lustrine_sand_controls* c, float particle_radius) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    // Simulation.hpp:239-242; the player starts at the origin (BulletPhysicsSimulation.hpp:35)
    c->attract_radius = 1.5f;
    c->blow_radius = 2.0f;
    c->attract_coeff = 1000.0f;
    c->blow_coeff = 500.0f;
    c->particle_diameter = 2.0f * particle_radius;
}

extern "C" int lustrine_pbf_set_sand_controls(lustrine_pbf* s, const lustrine_sand_controls* c) {
    if (!s || !c || !(c->particle_diameter >= 0.0f)) return LUSTRINE_ERR_ARGS;
    s->sand = *c;
    s->sand_controls_set = true;
    return LUSTRINE_OK;
}

extern "C" int lustrine_pbf_get_sand_controls(const lustrine_pbf* s, lustrine_sand_controls* c) {
    if (!s || !c) return LUSTRINE_ERR_ARGS;
    *c = s->sand;
    return LUSTRINE_OK;
}

extern "C" int lustrine_pbf_get_attracted(lustrine_pbf* s, int* flags) {
    if (!s || (!flags && s->n)) return LUSTRINE_ERR_ARGS;
    if (!s->n) return LUSTRINE_OK;
    CK(cudaMemcpyAsync(flags, s->att[s->cur], (size_t)s->n * sizeof(int), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return LUSTRINE_OK;
}

extern "C" int lustrine_pbf_set_attracted(lustrine_pbf* s, const int* flags) {
    if (!s || (!flags && s->n)) return LUSTRINE_ERR_ARGS;
    if (!s->n) return LUSTRINE_OK;
    CK(cudaMemcpyAsync(s->att[s->cur], flags, (size_t)s->n * sizeof(int), cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return LUSTRINE_OK;
}

extern "C" int lustrine_pbf_stream(lustrine_pbf* s, void** stream) {
    if (!s || !stream) return LUSTRINE_ERR_ARGS;
    *stream = (void*)s->stream;
    return LUSTRINE_OK;
}

extern "C" int lustrine_pbf_launches_per_step(const lustrine_pbf* s) {
    if (!s) return -1;
    if (s->launches > 0) return s->launches;
    // before any step: a step that predicts for itself
    const int scan = scan_tiles_launches(s->sp.num_cells);
    if (s->prm.mode == LUSTRINE_MODE_REFERENCE) return 1 + scan + 2 + 3;
    if (s->prm.mode == LUSTRINE_MODE_SAND) return 1 + scan + 2 + 1 + 4;
    return 1 + scan_tiles_launches(s->sp.num_cells, true) + 2 + 2 * s->prm.iterations + 1;
}

extern "C" const char* lustrine_error_string(int code) {
    switch (code) {
    case LUSTRINE_OK: return "ok";
    case LUSTRINE_ERR_ARGS: return "invalid argument";
    case LUSTRINE_ERR_CUDA: return "CUDA runtime error";
    case LUSTRINE_ERR_NOMEM: return "out of memory";
    case LUSTRINE_ERR_NBR_OVERFLOW: return "neighbour list capacity exceeded";
    case LUSTRINE_ERR_CELL_RANGE: return "particle left the grid (cell clamped)";
    case LUSTRINE_ERR_UNSUPPORTED: return "unsupported option";
    case LUSTRINE_ERR_NO_SIMULATION: return "no simulation initialised";
    case LUSTRINE_ERR_TIMEOUT: return "device wait timed out";
    case LUSTRINE_ERR_BAD_VALUE: return "non-finite particle state";
    case LUSTRINE_ERR_TOO_LARGE: return "input exceeds the fixed scratch limit";
    default: return "unknown status";
    }
}
