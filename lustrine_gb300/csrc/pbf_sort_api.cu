// pbf_sort_api.cu -- the reference's counting sort (Sorting::counting_sort,
// src/neighbors/Sorting.cpp:12-34) as a C entry point on device arrays.
#include <cstdio>

#include "lustrine_gb300.h"
#include "pbf_context.h"
#include "pbf_kernels.h"

using namespace lgb;

static int sort_args_ok(const int* counts, const int* keys, size_t n, size_t num_cells,
                        const int* sorted) {
    if (!counts || num_cells < 1 || num_cells > (size_t)(1 << 30)) return 0;
    if (n > (size_t)(1 << 30)) return 0;
    if (n > 0 && (!keys || !sorted)) return 0;
    return 1;
}

// Sort, then read the key-range status (the call synchronises the stream).
static int sort_with_scratch(int* counts, const int* keys, int n, int num_cells, int* sorted,
                             int* scratch, cudaStream_t st) {
    CountingSortScratch w = counting_sort_scratch(scratch, n, num_cells);
    // the histogram and the status word start at zero
    cudaError_t e = cudaMemsetAsync(w.count, 0, (size_t)num_cells * sizeof(int), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(w.status, 0, sizeof(int), st);
    if (e != cudaSuccess) return lgb_cuda_status(e, "cudaMemsetAsync");
    launch_counting_sort(keys, n, num_cells, w, counts, sorted, st);
    int bad = 0;
    e = cudaMemcpyAsync(&bad, w.status, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return lgb_cuda_status(e, "counting_sort");
    return bad ? LUSTRINE_ERR_ARGS : LUSTRINE_OK;
}

extern "C" int lustrine_counting_sort(int* counts, const int* keys, size_t num_positions,
                                      size_t num_cells, int* sorted_indices, void* stream) {
    if (!sort_args_ok(counts, keys, num_positions, num_cells, sorted_indices)) return LUSTRINE_ERR_ARGS;
    cudaStream_t st = (cudaStream_t)stream;
    const int n = (int)num_positions, C = (int)num_cells;
    int* scratch = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&scratch, counting_sort_scratch_ints(n, C) * sizeof(int), st);
    if (e != cudaSuccess) return lgb_cuda_status(e, "cudaMallocAsync");
    int rc = sort_with_scratch(counts, keys, n, C, sorted_indices, scratch, st);
    cudaFreeAsync(scratch, st);
    cudaError_t e2 = cudaStreamSynchronize(st);
    if (!rc && e2 != cudaSuccess) rc = lgb_cuda_status(e2, "cudaFreeAsync");
    return rc;
}
