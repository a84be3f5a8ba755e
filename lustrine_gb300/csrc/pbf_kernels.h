// pbf_kernels.h -- host-side launchers of the PBF kernels (one scene).
#pragma once

#include <cuda_runtime.h>

#include "pbf_common.cuh"

namespace lgb {

// pbf_sort.cu
// Scan of the standalone sort entry points: tiles of SCAN_TILE cells, one
// block each (reduce / scan of the tile sums / down-sweep).
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;
constexpr size_t scan_block_sums_ints(size_t C) { return (C + SCAN_TILE - 1) / SCAN_TILE + 1; }
// Scratch of the standalone counting sort: count[C], the scan's tile sums,
// key[n], rank[n] (also the big cells' merge space), tmp[n], status.
constexpr size_t counting_sort_scratch_ints_for(size_t n, size_t C) {
    return C + scan_block_sums_ints(C) + 3 * n + 1;
}
// exclusive scan count -> start (C + 1 entries); zeroes count behind it
void launch_scan(int* count, int C, int* block_sums, int* start, cudaStream_t st);
int scan_block_sums_size(int C);
// scan of the step: tile totals, then tiles scanned independently (the
// totals scanned by one block in between past CELL_SCAN_MAX_TILES tiles);
// tile_sum: cell_scan_tiles(C) ints.  counted: the prediction already
// counted the tile totals into tile_sum (no totals pass); tile_zero (may be
// null): the other totals buffer, zeroed for the next prediction.
// scan_tiles_launches: kernels it issues.
int cell_scan_tiles(int C);
void launch_scan_tiles(int* count, int C, int* tile_sum, int* start, cudaStream_t st, bool counted = false,
                       int* tile_zero = nullptr);
int scan_tiles_launches(int C, bool counted = false);
// rank doubles as merge space for cells of more than a few dozen particles
void launch_sort_tail(const int* key, int* rank, const int* start, const int* tie, int n,
                      int* tmp, int* perm, cudaStream_t st);
void launch_gather_state(const int* perm, int n, const int* key, const float4* x, const float4* xs,
                         const float4* v, const int* id, int* key_out, float4* x_out,
                         float4* xs_out, float4* v_out, int* id_out, cudaStream_t st);
void launch_gather_solid(const int* perm, int n, const float4* src, float4* dst, cudaStream_t st);
// Standalone stable counting sort of caller keys (Sorting::counting_sort,
// src/neighbors/Sorting.cpp:12-34): scratch carved from one int buffer whose
// count part must be zero on entry (the scan leaves it zero again).
struct CountingSortScratch {
    int* count;       // num_cells
    int* block_sums;  // scan_block_sums_size(num_cells)
    int* key;         // n (validated keys)
    int* rank;        // n
    int* tmp;         // n
    int* status;      // 1
};
size_t counting_sort_scratch_ints(int n, int num_cells);
CountingSortScratch counting_sort_scratch(int* base, int n, int num_cells);
// start: num_cells + 1 exclusive offsets; sorted: n input indices in stable key order
void launch_counting_sort(const int* keys, int n, int num_cells, CountingSortScratch w, int* start,
                          int* sorted, cudaStream_t st);
// index scatter + stabilisation fused with the reorder of the particle state
// (v may be nullptr: not carried; aux: an optional int per particle carried
// into the new order, e.g. the packed cells of a hashed grid; x_out nullptr:
// x stays in the previous order and src_out receives each new slot's previous
// slot instead)
void launch_sort_state(const int* key, int* rank, const int* start, const int* tie, int n,
                       int* tmp, const float4* x, const float4* xs, const float4* v, const int* id,
                       int* key_out, float4* x_out, float4* xs_out, float4* v_out, int* id_out,
                       const int* aux, int* aux_out, int* slot_of, int* src_out, cudaStream_t st);
void launch_gather_int(const int* perm, int n, const int* src, int* dst, cudaStream_t st);

// pbf_compat.cu (reference semantics, no FMA contraction)
void launch_predict_ref(const StepParams& p, const float4* x, float4* v, float4* xs, int* key,
                        int* rank, int* count, int* status, cudaStream_t st);
void launch_key_ref(const StepParams& p, const float4* pos, int m, int* key, int* rank, int* count,
                    int* status, cudaStream_t st);
void launch_lists_ref(const StepParams& p, const float4* xs, const int* key, const int* fstart,
                      const float4* solid, const int* sstart, int* nbr, int* cnt, int* status,
                      cudaStream_t st);
void launch_lambda_ref(const StepParams& p, const float4* xs, const int* id, const int* nbr,
                       const int* cnt, const float4* solid, float* lam_by_id, float* rho,
                       cudaStream_t st);
void launch_delta_ref(const StepParams& p, const float4* xs, float4* xs_out, float4* x, float4* v,
                      const int* id, const int* nbr, const int* cnt, const float4* solid,
                      const float* lam_by_id, cudaStream_t st);

// sand.cu (simulate_sand semantics, no FMA contraction)
void launch_sand_predict(const StepParams& p, const SandParams& q, const float4* x, float4* v, float4* xs,
                         int* att, int* key, int* rank, int* count, int* status, cudaStream_t st);
void launch_sand_lists(const StepParams& p, const float4* xs, const int* key, const int* fstart,
                       const float4* solid, const int* sstart, int* nbr, int* cnt, int* status,
                       cudaStream_t st);
// x_commit == nullptr: write star_out; otherwise commit x, v, the flags and
// the identity index of every slot
void launch_sand_substep(const StepParams& p, const SandParams& q, const float4* tmp_in, float4* star_out,
                         const float4* xpre, const int* nbr, const int* cnt, const float4* solid,
                         float4* x_commit, float4* v_commit, const int* att_in, int* att_commit,
                         int* id_commit, cudaStream_t st);

// pbf_solver.cu (PBF; mixed = cell index + offset representation)
// cellk: packed cell of every particle on a hashed grid (nullptr when dense)
// tile_count (may be null): per-tile totals of the step's cell scan, counted
// as the histogram is (one atomic per tile a warp touches)
void launch_predict(bool mixed, const StepParams& p, const CellPack& cp, const float4* x, const float4* v,
                    float4* xs, int* key, int* rank, int* count, int* cellk, int* tile_count, cudaStream_t st);
void launch_key(bool mixed, const StepParams& p, const CellPack& cp, const float4* pos, int m,
                int* key, int* rank, int* count, int* cellk, cudaStream_t st);
// near[key] = 1 for every cell (bucket) within one cell of a static particle
// (near: num_cells bytes, zero on entry)
void launch_mark_solid_near(bool mixed, const StepParams& p, const CellPack& cp, const float4* pos, int m,
                            unsigned char* near, cudaStream_t st);
// neighbour lists + first lambda pass (lambda stored in xs.w)
void launch_lists_lambda(bool mixed, const Tuning& tu, const StepParams& p, const CellPack& cp,
                         float4* xs, const int* key_sorted, const int* cell_sorted, const int* fstart,
                         const float4* solid, const int* solid_cell, const int* sstart, int* nbr,
                         int* cnt, float* rho, int* status, cudaStream_t st);
void launch_lambda(bool mixed, const Tuning& tu, const StepParams& p, float4* xs, const int* nbr,
                   const int* cnt, const float4* solid, float* rho, cudaStream_t st);
void launch_delta(bool mixed, const Tuning& tu, const StepParams& p, const CellPack& cp,
                  const float4* xs, float4* xs_out, const int* nbr, const int* cnt,
                  const float4* solid, const int* key_sorted, const float4* x, float4* v_out,
                  cudaStream_t st);
// XSPH and commit; with xs_next (not nullptr) also the next step's
// prediction from the committed state (as launch_predict with the same dt)
void launch_xsph(bool mixed, const Tuning& tu, const StepParams& p, const CellPack& cp,
                 const float4* xs, const float4* v_in, const int* nbr, const int* cnt,
                 const int* key_sorted, float4* x_out, float4* v_out, float4* xs_next, int* key,
                 int* rank, int* count, int* cellk, int* tile_count, cudaStream_t st);
// The same passes over compact lists (p.rec set; pbf_compact.cu).  B: the
// list build's block size; p.pad: the passes' largest chunk.
void launch_lists_compact(int B, const StepParams& p, const CellPack& cp, float4* xs, const int* key_sorted,
                          const int* cell_sorted, const int* fstart, const float4* solid, const int* solid_cell,
                          const int* sstart, int* nbr, int* cnt, float* rho, int* status, cudaStream_t st);
void launch_lambda_compact(const Tuning& tu, const StepParams& p, float4* xs, const int* nbr, const int* cnt,
                           const float4* solid, float* rho, cudaStream_t st);
void launch_delta_compact(const Tuning& tu, const StepParams& p, const CellPack& cp, const float4* xs,
                          float4* xs_out, const int* nbr, const int* cnt, const float4* solid,
                          const int* key_sorted, const float4* x, float4* v_out, cudaStream_t st);
// tx.unroll: the XSPH pass's gathers in flight
void launch_xsph_compact(const Tuning& tx, const StepParams& p, const CellPack& cp, const float4* xs,
                         const float4* v_in, const int* nbr, const int* cnt, const int* key_sorted, float4* x_out,
                         float4* v_out, float4* xs_next, int* key, int* rank, int* count, int* cellk,
                         int* tile_count, cudaStream_t st);
void launch_unpermute_pos(bool mixed, const StepParams& p, const CellPack& cp, const float4* a,
                          const int* id, int n, float* out, cudaStream_t st);
void launch_unpermute_pos_d(bool mixed, const StepParams& p, const CellPack& cp, const float4* a,
                            const int* id, int n, double* out, cudaStream_t st);
// cell + offset positions (w: packed cell) into the scene frame, w kept
void launch_to_scene_frame(const StepParams& p, const CellPack& cp, float4* a, int m, cudaStream_t st);
void launch_pack_pos(bool mixed, const StepParams& p, const CellPack& cp, const float* in, int n,
                     const int* scene_of,
                     float4* out, cudaStream_t st);
// count of the particles the last step binned in the cells x0..x1, y0..y1,
// z0..z1 (box[6], inclusive, inside the grid), added to *out (device int);
// sstart / solid_cell nullptr: fluid only
void launch_query_cells(const StepParams& p, const CellPack& cp, const int box[6], const int* fstart,
                        const int* sstart, const int* cell_sorted, const int* solid_cell, int* out,
                        cudaStream_t st);
// state from / into host-visible memory (page-locked host buffers read and
// written by the kernels): hv may be nullptr (zero velocities / not written)
void launch_pack_state(bool mixed, const StepParams& p, const CellPack& cp, const float* hx, const float* hv,
                       int n, float4* x, float4* v, int* id, cudaStream_t st);
// slot_of_valid: slot_of already maps every caller index to its slot (the
// last sort wrote it); otherwise it is rebuilt from id first
void launch_unpack_state(bool mixed, const StepParams& p, const CellPack& cp, const float4* x, const float4* v,
                         const int* id, int* slot_of, bool slot_of_valid, int n, float* hx, float* hv,
                         cudaStream_t st);
// a host frame's upload fused with the step's prediction (slot = caller index)
void launch_pack_predict(bool mixed, const StepParams& p, const CellPack& cp, const float* hx, const float* hv,
                         int n, float4* x, int* id, float4* xs, int* key, int* rank, int* count, int* cellk,
                         int* tile_count, cudaStream_t st);
void launch_reduce(bool mixed, const StepParams& p, const CellPack& cp, const float4* x,
                   const float4* v, const float* rho, double* out, cudaStream_t st);

// pbf_scene_solve.cu: a batch's lists, iterations, XSPH and commit out of the
// distributed shared memory of thread-block clusters (PBF, dense grid, no
// static particles, scenes of at most SOLVE_MAX_SCENE particles)
constexpr int SOLVE_M = 4096;         // particles per CTA (threads per CTA: 512 or 1024)
constexpr int SOLVE_M_SHIFT = 12;
constexpr int SOLVE_CAP = 10;         // list entries per particle kept in shared memory
constexpr int SOLVE_CLUSTER = 16;     // CTAs per cluster
constexpr int SOLVE_MAX_SCENE = SOLVE_M * SOLVE_CLUSTER;
constexpr float SOLVE_MIXED_MAX_CELLS = 256.0f;  // mixed precision: largest box side, in cells
// One CTA of a bin: its scene (-1: none), its rank among the scene's CTAs and
// the scene's CTA count.
struct SolveSlot {
    int scene, rank, ctas;
};
struct SolveArgs {
    const SolveSlot* bins;   // num_bins x SOLVE_CLUSTER
    int num_bins;
    int iters;               // solver iterations
    int* queue;              // [0] next bin, [1] clusters done (both zero at launch)
    const int* scene_slot0;  // S + 1 first slots
    const float4* xs;        // the step's predicted positions in cell order
    const float4* x;         // committed positions in cell order
    const int* key_sorted;
    const int* start;
    int* nbr;                // the lists (slots), also written to global memory (neighbour queries)
    int* cnt;
    float* rho;              // densities of the last lambda pass (may be null)
    float4* lam_out;         // w: lambdas of the last lambda pass
    float4* x_out;           // committed state
    float4* v_out;
    int* status;
    float4* xs_next;         // the next step's prediction (null: none), as predict_one
    int* key;
    int* rank;
    int* count;
    int* cellk;
    int* tile_count;
};
size_t scene_solve_smem_bytes();
// Sets the kernel's attributes for CTAs of `threads` (512 or 1024) threads;
// returns the clusters that fit the GPU at once (0: the on-chip solve cannot
// run here).
int scene_solve_prepare(bool mixed, int threads, int* max_clusters);
void launch_scene_solve(bool mixed, int threads, const StepParams& p, const CellPack& cp, const SolveArgs& a,
                        int clusters, cudaStream_t st);

}  // namespace lgb
