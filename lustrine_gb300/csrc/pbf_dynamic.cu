// pbf_dynamic.cu -- particles entering and leaving a scene between steps:
// the device side of the reference's particle sources and sinks
// (Lustrine.cpp:745-836).
//
// Spawn appends particles after the active ones (caller indices n, n+1, ...)
// up to the context's capacity.  Despawn removes the particles the last step
// binned in given cells with the reference's index semantics: the evicted
// caller indices, cell by cell in the given order and ascending within a
// cell, each take the data of the current last particle (swap-remove,
// Lustrine.cpp:822-832).  That sequence runs on the evicted indices only (on
// the host, it is short); the device then relabels every particle's caller
// index, compacts the committed state in slot order into the other side and
// rebuilds the cell table of the surviving particles, so cell queries and
// further sinks keep working until the next step.
#include <algorithm>
#include <unordered_map>
#include <vector>

#include "lustrine_gb300.h"
#include "pbf_context.h"
#include "pbf_kernels.h"

using namespace lgb;

namespace {

constexpr int DYN_THREADS = 256;

inline int blocks(int n) { return (n + DYN_THREADS - 1) / DYN_THREADS; }

// slot range of every listed cell in the cell table
__global__ void k_cell_ranges(const int* __restrict__ start, const int* __restrict__ cells, int ncells,
                              int2* __restrict__ out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < ncells) out[k] = make_int2(start[cells[k]], start[cells[k] + 1]);
}

// caller index of every slot of the listed ranges (ranges concatenated)
__global__ void k_range_ids(const int2* __restrict__ ranges, const int* __restrict__ offsets, int nranges,
                            const int* __restrict__ id, int* __restrict__ out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nranges) return;
    const int2 r = ranges[k];
    int o = offsets[k];
    for (int t = r.x; t < r.y; t++) out[o++] = id[t];
}

// remap[q] = q for q < keep, -1 above; then the listed overrides
__global__ void k_remap_init(int* __restrict__ remap, int n, int keep) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < n) remap[q] = q < keep ? q : -1;
}
__global__ void k_remap_apply(int* __restrict__ remap, const int2* __restrict__ pairs, int npairs) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < npairs) remap[pairs[k].x] = pairs[k].y;
}

// survivors per block of slots
__global__ void __launch_bounds__(DYN_THREADS) k_keep_count(const int* __restrict__ remap,
                                                            const int* __restrict__ id, int n,
                                                            int* __restrict__ block_count) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int keep = (s < n && remap[id[s]] >= 0) ? 1 : 0;
    const int c = __syncthreads_count(keep);
    if (threadIdx.x == 0) block_count[blockIdx.x] = c;
}

// order-preserving compaction of the committed state (slot order) into the
// other side; caller indices relabelled
__global__ void __launch_bounds__(DYN_THREADS) k_keep_scatter(
    const int* __restrict__ remap, const int* __restrict__ block_offset, int n, const float4* __restrict__ x,
    const float4* __restrict__ v, const int* __restrict__ id, const int* __restrict__ key,
    const int* __restrict__ att, float4* __restrict__ x_out, float4* __restrict__ v_out, int* __restrict__ id_out,
    int* __restrict__ key_out, int* __restrict__ att_out) {
    __shared__ int warp_count[DYN_THREADS / 32];
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int nid = s < n ? remap[id[s]] : -1;
    const bool keep = nid >= 0;
    const unsigned b = __ballot_sync(0xffffffffu, keep);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) warp_count[warp] = __popc(b);
    __syncthreads();
    int before = 0;
    for (int w = 0; w < warp; w++) before += warp_count[w];
    if (!keep) return;
    const int d = block_offset[blockIdx.x] + before + __popc(b & ((1u << lane) - 1u));
    x_out[d] = x[s];
    v_out[d] = v[s];
    id_out[d] = nid;
    key_out[d] = key[s];
    att_out[d] = att[s];  // sand mode's attract flag travels with its particle
}

__global__ void k_histogram(const int* __restrict__ key, int n, int* __restrict__ count) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) atomicAdd(&count[key[s]], 1);
}

// After the active count changed: the sentinel moves, captured graphs and
// neighbour lists (stride n) are stale, lambdas / densities of the last step
// no longer match the slots.
int after_resize(lustrine_pbf* s) {
    s->sp.n = s->n;
    s->invalidate_graphs();
    s->slot_of_valid = false;
    s->lists_valid = false;
    s->lam_src = nullptr;
    if (s->n) {
        CK(cudaMemsetAsync(s->rho, 0, (size_t)s->n * sizeof(float), s->stream));
        CK(cudaMemsetAsync(s->lam_by_id, 0, s->lam_by_id_len * sizeof(float), s->stream));
    }
    return lgb_write_sentinel(s);
}

}  // namespace

extern "C" int lustrine_pbf_spawn(lustrine_pbf* s, const float* x, const float* v, int m) {
    if (!s || m < 0 || (m > 0 && !x)) return LUSTRINE_ERR_ARGS;
    if (s->is_batch()) return LUSTRINE_ERR_UNSUPPORTED;
    if (!s->have_state) return LUSTRINE_ERR_ARGS;
    if (m == 0) return LUSTRINE_OK;
    if ((long long)s->n + m > s->cap) return LUSTRINE_ERR_TOO_LARGE;
    const int n = s->n, c = s->cur;
    // staging: positions in out3d, velocities in out3 (both sized for the capacity)
    float* sx = reinterpret_cast<float*>(s->out3d);
    CK(cudaMemcpyAsync(sx, x, (size_t)m * 3 * sizeof(float), cudaMemcpyHostToDevice, s->stream));
    launch_pack_pos(s->mixed(), s->sp, s->cp, sx, m, nullptr, s->x[c] + n, s->stream);
    if (v) {
        CK(cudaMemcpyAsync(s->out3, v, (size_t)m * 3 * sizeof(float), cudaMemcpyHostToDevice, s->stream));
        launch_pack_pos(false, s->sp, s->cp, s->out3, m, nullptr, s->v[c] + n, s->stream);
    } else {
        CK(cudaMemsetAsync(s->v[c] + n, 0, (size_t)m * sizeof(float4), s->stream));
    }
    CK(cudaMemcpyAsync(s->id[c] + n, s->iota + n, (size_t)m * sizeof(int), cudaMemcpyDeviceToDevice, s->stream));
    // sand mode: spawned particles start unattracted
    CK(cudaMemsetAsync(s->att[c] + n, 0, (size_t)m * sizeof(int), s->stream));
    CK(cudaGetLastError());
    s->n = n + m;
    return after_resize(s);
}

extern "C" int lustrine_pbf_set_count(lustrine_pbf* s, int n) {
    if (!s || n < 0) return LUSTRINE_ERR_ARGS;
    if (s->is_batch()) return LUSTRINE_ERR_UNSUPPORTED;
    if (!s->have_state) return LUSTRINE_ERR_ARGS;
    if (n > s->cap) return LUSTRINE_ERR_TOO_LARGE;
    if (n == s->n) return LUSTRINE_OK;
    if (n > s->n) {  // identity labels for the new slots until the caller's state upload
        CK(cudaMemcpyAsync(s->id[s->cur] + s->n, s->iota + s->n, (size_t)(n - s->n) * sizeof(int),
                           cudaMemcpyDeviceToDevice, s->stream));
        CK(cudaMemsetAsync(s->att[s->cur] + s->n, 0, (size_t)(n - s->n) * sizeof(int), s->stream));
    }
    s->n = n;
    s->cells_valid = false;
    return after_resize(s);
}

extern "C" int lustrine_pbf_despawn_cells(lustrine_pbf* s, const int* cells, int ncells, int* removed) {
    if (!s || ncells < 0 || (ncells > 0 && !cells)) return LUSTRINE_ERR_ARGS;
    if (removed) *removed = 0;
    if (s->is_batch() || s->sp.hash_bits) return LUSTRINE_ERR_UNSUPPORTED;
    if (!s->have_state) return LUSTRINE_ERR_ARGS;
    for (int k = 0; k < ncells; k++)
        if (cells[k] < 0 || cells[k] >= s->sp.num_cells) return LUSTRINE_ERR_ARGS;
    if (ncells == 0 || !s->cells_valid || s->n == 0) return LUSTRINE_OK;
    const int n = s->n, c = s->cur, o = 1 - c, C = s->sp.num_cells;
    cudaStream_t st = s->stream;

    // 1. the binned particles of the listed cells (caller indices)
    int *d_cells = nullptr, *d_off = nullptr, *d_ids = nullptr;
    int2* d_ranges = nullptr;
    int rc = LUSTRINE_OK;
    std::vector<int2> ranges((size_t)ncells);
    std::vector<int> offsets((size_t)ncells + 1, 0), ids;
    auto fail = [&](cudaError_t e, const char* what) {
        rc = lgb_cuda_status(e, what);
        return rc;
    };
    auto cleanup = [&]() {
        cudaFree(d_cells);
        cudaFree(d_off);
        cudaFree(d_ids);
        cudaFree(d_ranges);
    };
    cudaError_t e = cudaMalloc(&d_cells, (size_t)ncells * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&d_ranges, (size_t)ncells * sizeof(int2));
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_cells, cells, (size_t)ncells * sizeof(int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        k_cell_ranges<<<blocks(ncells), DYN_THREADS, 0, st>>>(s->start, d_cells, ncells, d_ranges);
        e = cudaMemcpyAsync(ranges.data(), d_ranges, (size_t)ncells * sizeof(int2), cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        fail(e, "despawn ranges");
        cleanup();
        return rc;
    }
    for (int k = 0; k < ncells; k++) offsets[(size_t)k + 1] = offsets[(size_t)k] + (ranges[(size_t)k].y - ranges[(size_t)k].x);
    const int total = offsets[(size_t)ncells];
    if (total > 0) {
        ids.resize((size_t)total);
        e = cudaMalloc(&d_off, (size_t)ncells * sizeof(int));
        if (e == cudaSuccess) e = cudaMalloc(&d_ids, (size_t)total * sizeof(int));
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_off, offsets.data(), (size_t)ncells * sizeof(int), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) {
            k_range_ids<<<blocks(ncells), DYN_THREADS, 0, st>>>(d_ranges, d_off, ncells, s->id[c], d_ids);
            e = cudaMemcpyAsync(ids.data(), d_ids, (size_t)total * sizeof(int), cudaMemcpyDeviceToHost, st);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            fail(e, "despawn ids");
            cleanup();
            return rc;
        }
    }
    cleanup();
    if (total == 0) return LUSTRINE_OK;
    // a cell's particles in ascending caller index (the order the reference bins them)
    for (int k = 0; k < ncells; k++)
        std::sort(ids.begin() + offsets[(size_t)k], ids.begin() + offsets[(size_t)k + 1]);

    // 2. the reference's removal sequence on indices: index e takes the data
    //    of the current last index, the end moves down (Lustrine.cpp:822-832)
    std::unordered_map<int, int> at;  // index -> original particle now there
    int end = n;
    for (int k = 0; k < total && end > 0; k++) {
        const int ev = ids[(size_t)k];
        auto it = at.find(end - 1);
        at[ev] = it == at.end() ? end - 1 : it->second;
        end--;
    }
    // overrides of the identity below end: touched indices lose their
    // particle, the particles moved there take that index
    std::vector<int2> pairs;
    for (const auto& kv : at)
        if (kv.first < end) pairs.push_back(make_int2(kv.first, -1));
    for (const auto& kv : at)
        if (kv.first < end) pairs.push_back(make_int2(kv.second, kv.first));
    // apply -1 first, then moves: keep that order on the device by two launches
    const int nneg = (int)(pairs.size() / 2);

    // 3. relabel, compact into the other side, rebuild the cell table
    int* remap = s->perm;          // n ints (capacity-sized scratch)
    int* block_count = s->tmp;     // blocks(n) + 1 ints
    const int nb = blocks(n);
    std::vector<int> bc((size_t)nb + 1, 0);
    int2* d_pairs = nullptr;
    e = cudaSuccess;
    if (!pairs.empty()) {
        e = cudaMalloc(&d_pairs, pairs.size() * sizeof(int2));
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_pairs, pairs.data(), pairs.size() * sizeof(int2), cudaMemcpyHostToDevice, st);
    }
    if (e == cudaSuccess) {
        k_remap_init<<<blocks(n), DYN_THREADS, 0, st>>>(remap, n, end);
        if (nneg) {
            k_remap_apply<<<blocks(nneg), DYN_THREADS, 0, st>>>(remap, d_pairs, nneg);
            k_remap_apply<<<blocks(nneg), DYN_THREADS, 0, st>>>(remap, d_pairs + nneg, nneg);
        }
        k_keep_count<<<nb, DYN_THREADS, 0, st>>>(remap, s->id[c], n, block_count);
        e = cudaMemcpyAsync(bc.data(), block_count, (size_t)nb * sizeof(int), cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaFree(d_pairs);
        return fail(e, "despawn remap");
    }
    int run = 0;
    for (int b = 0; b < nb; b++) {
        const int t = bc[(size_t)b];
        bc[(size_t)b] = run;
        run += t;
    }
    if (run != end) {  // the relabelling must leave exactly indices 0 .. end-1
        cudaFree(d_pairs);
        return LUSTRINE_ERR_CUDA;
    }
    e = cudaMemcpyAsync(block_count, bc.data(), (size_t)nb * sizeof(int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        k_keep_scatter<<<nb, DYN_THREADS, 0, st>>>(remap, block_count, n, s->x[c], s->v[c], s->id[c],
                                                   s->key_sorted, s->att[c], s->x[o], s->v[o], s->id[o], s->key,
                                                   s->att[o]);
        std::swap(s->key, s->key_sorted);
        if (s->count_dirty)  // a histogram of the next step's prediction, dropped with it
            e = cudaMemsetAsync(s->count, 0, (size_t)C * sizeof(int), st);
        s->count_dirty = false;
        if (end > 0) k_histogram<<<blocks(end), DYN_THREADS, 0, st>>>(s->key_sorted, end, s->count);
        launch_scan(s->count, C, s->block_sums, s->start, st);  // leaves count zero
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d_pairs);
    if (e != cudaSuccess) return fail(e, "despawn compact");
    s->cur = o;
    if (removed) *removed = n - end;
    s->n = end;
    return after_resize(s);
}
