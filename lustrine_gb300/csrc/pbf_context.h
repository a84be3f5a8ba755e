// pbf_context.h -- the context behind lustrine_pbf_* (host-side definition).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "lustrine_gb300.h"
#include "pbf_common.cuh"
#include "pbf_kernels.h"

int lgb_cuda_status(cudaError_t e, const char* what);

#define CK(call)                                                     \
    do {                                                             \
        cudaError_t e_ = (call);                                     \
        if (e_ != cudaSuccess) return lgb_cuda_status(e_, #call);    \
    } while (0)


struct lustrine_pbf {
    lustrine_pbf_params prm{};
    lgb::StepParams sp{};
    lgb::CellPack cp{};
    lgb::Tuning tune{128, 2, 128, 8, 1, 1};
    int n = 0, ns = 0;
    int cap = 0;  // fluid particles the buffers hold (n <= cap; sources append up to it)
    cudaStream_t stream = nullptr;

    // fluid state, two sides: the committed state is on side `cur`; a step
    // sorts it into side 1 - cur and solves there.
    float4* x[2] = {nullptr, nullptr};
    float4* xs[2] = {nullptr, nullptr};
    float4* v[2] = {nullptr, nullptr};
    int* id[2] = {nullptr, nullptr};
    int cur = 0;
    float4* xs_alt = nullptr;  // Jacobi ping-pong partner of xs
    float4* xs_pred = nullptr; // PBF: predicted positions of the next step, in the committed side's order
    float4* vtmp = nullptr;    // velocities before XSPH
    int* iota = nullptr;       // 0..n-1
    int* slot_of = nullptr;    // slot of every caller index (state download)
    bool slot_of_valid = false;  // written by the last sort of the committed side

    // counting sort
    int* key = nullptr;
    int* key_sorted = nullptr;
    int* rank = nullptr;
    int* tmp = nullptr;
    int* perm = nullptr;
    int* count = nullptr;
    int* start = nullptr;
    int* block_sums = nullptr;
    int* tile_sum = nullptr;  // per-tile totals of the step's scan, two halves (step parity)

    // static solids, sorted by cell
    float4* solid = nullptr;
    float4* solid_raw = nullptr;
    // hashed grid: packed cell of each particle (unsorted), of each sorted
    // fluid slot, of each sorted solid slot
    int* cellk = nullptr;
    int* cell_sorted = nullptr;
    int* solid_cell = nullptr;
    int* solid_id = nullptr;   // caller's solid index of each sorted slot
    unsigned char* solid_near = nullptr;  // cells within one cell of a solid (PBF list build)
    int* sstart = nullptr;

    // neighbour lists and per-particle outputs
    int* nbr = nullptr;
    int* cnt = nullptr;
    uint4* rec = nullptr;        // compact list records (allocated where compact lists can apply)
    uint4* rec2 = nullptr;       // their second records
    int* src = nullptr;          // PBF step: previous slot of each sorted slot (its committed position)
    int lists_format = LUSTRINE_LISTS_COLUMN;  // the form the last list build wrote (LUSTRINE_LISTS_*)
    float* lam = nullptr;
    float4* lam_src = nullptr;  // PBF: the buffer whose w holds the last lambdas
    float* lam_by_id = nullptr;
    size_t lam_by_id_len = 0;
    float* rho = nullptr;
    int* status = nullptr;
    double* red = nullptr;
    int* qcount = nullptr;    // cell-count query result
    float* out3 = nullptr;    // 3 * max(n, ns) floats of staging
    double* out3d = nullptr;  // 3 * n doubles of staging

    // sand mode: per-particle attract flags (two sides, carried by the sort),
    // the caller's controls, the previous step's attract flag and the
    // controls the captured sand graph was built with
    int* att[2] = {nullptr, nullptr};
    lustrine_sand_controls sand{};
    bool sand_controls_set = false;
    int prev_attract = 0;
    lgb::SandParams sand_captured{};

    // batch of independent scenes (empty for one scene)
    std::vector<int> b_domains, b_nfluid, b_nsolid;
    lgb::SceneInfo* d_scenes = nullptr;
    int* d_scene_of = nullptr;
    int* d_solid_scene_of = nullptr;
    bool is_batch() const { return !b_nfluid.empty(); }
    // on-chip scene solve of a batch (pbf_scene_solve.cu): bins of scenes,
    // the scenes' first slots, the work queue, the clusters launched
    lgb::SolveSlot* d_bins = nullptr;
    int num_bins = 0;
    int* d_scene_slot0 = nullptr;
    int* d_queue = nullptr;
    int onchip_clusters = 0;     // 0: the batch cannot take the on-chip solve (CTAs of 1024 threads)
    int onchip_clusters512 = 0;  // the same with CTAs of 512 threads
    int onchip_threads = 1024;
    bool onchip = false;         // the step uses it

    // captured steps: parity + 2 * (own prediction) + 4 * (predicts the next step)
    cudaGraphExec_t graph_exec[8] = {};
    // PBF: the last step's commit kernel predicted the next step with dt pred_dt
    bool pred_ready = false;
    float pred_dt = 0.0f;
    bool count_dirty = false;  // count[] holds that prediction's histogram
    bool tiles_dirty = true;   // tile totals may hold counts of a dropped prediction
    int launches = 0;             // kernels the last step launched
    int graph_launches[8] = {};   // kernels in each captured step
    // the step graphs were dropped since the last step: the next step runs its
    // kernels directly and only a step after it captures, so a scene whose
    // particle count or controls change every frame pays no capture
    bool graphs_fresh = true;
    long long steps_done = 0;
    bool have_state = false;
    bool use_pdl = true;  // programmatic dependent launch between step kernels
    bool lists_valid = false;
    bool cells_valid = false;  // start[] / sstart[] bin the current slots (queries, sinks)

    // page-locked host frames (lustrine_pbf_step_host, fp32): one graph per
    // step parity for the caller's last buffer pair, with the positions
    // downloaded on a side stream while the commit kernel runs
    cudaStream_t side = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    cudaGraphExec_t host_graph[2] = {nullptr, nullptr};
    const void* host_graph_ptr[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    int host_graph_launches[2] = {0, 0};

    ~lustrine_pbf();
    void free_buffers();
    void invalidate_graphs();
    bool mixed() const;
    bool sand_mode() const { return prm.mode == LUSTRINE_MODE_SAND; }
};

// Writes the sentinel particle of the padded neighbour lists at slot s->n.
int lgb_write_sentinel(lustrine_pbf* s);
