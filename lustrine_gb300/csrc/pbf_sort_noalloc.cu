// pbf_sort_noalloc.cu -- the counting sort for callers that cannot allocate
// GPU memory.
//
// Some hosts of this library must not have it allocate device memory while
// they run: a game engine that budgets all GPU memory when a level loads and
// forbids allocation during a frame (cudaMalloc and cudaFree can synchronise
// the device and stall the frame), or a plugin host whose allocator policy
// rejects allocations made outside its own pool.  lustrine_counting_sort
// takes its scratch with cudaMallocAsync on every call; this variant takes it
// from one file-scope __device__ array instead, so it allocates nothing.
//
// The array is part of the library's device image: every GPU that loads the
// library holds it (LUSTRINE_NOALLOC_SCRATCH_BYTES) until the process exits.
// Host code may not use the array's name as a device address (on the host it
// names a host-side stand-in), so the first call on each device looks up its
// device address with cudaGetSymbolAddress while that device is current and
// keeps it; make that first call before any stream capture.  The kept
// address belongs to the device's context: after cudaDeviceReset (which
// unloads the library's device image) it is stale, so this entry point must
// not be called again in that process after a reset of the device.  Every call
// shares the array and leaves its contents behind: the parts that must start
// at zero are cleared on each call, and calls whose work overlaps on the GPU
// (different streams or host threads) race on it.
#include <mutex>

#include "lustrine_gb300.h"
#include "pbf_context.h"
#include "pbf_kernels.h"

using namespace lgb;

namespace {

// the sort's scratch (count[cells] + scan tile sums + key, rank, tmp[keys] +
// status) at the maxima, sized by the same layout function the sort uses
constexpr size_t kScratchInts =
    counting_sort_scratch_ints_for((size_t)LUSTRINE_NOALLOC_MAX_KEYS, (size_t)LUSTRINE_NOALLOC_MAX_CELLS);
static_assert(kScratchInts * sizeof(int) <= LUSTRINE_NOALLOC_SCRATCH_BYTES,
              "scratch array larger than the documented size");

static __device__ __align__(256) int g_scratch[LUSTRINE_NOALLOC_SCRATCH_BYTES / sizeof(int)];

constexpr int kMaxDevices = 64;
int* g_scratch_addr[kMaxDevices] = {};
std::mutex g_setup;

// Device address of g_scratch on the current device (looked up once per device).
int scratch_for_current_device(int** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return lgb_cuda_status(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return LUSTRINE_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_setup);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess) return lgb_cuda_status(e, "cudaGetSymbolAddress");
        g_scratch_addr[dev] = static_cast<int*>(p);
    }
    *out = g_scratch_addr[dev];
    return LUSTRINE_OK;
}

}  // namespace

extern "C" int lustrine_counting_sort_noalloc(int* counts, const int* keys, size_t num_positions,
                                              size_t num_cells, int* sorted_indices, void* stream) {
    if (!counts || num_cells < 1 || (num_positions > 0 && (!keys || !sorted_indices)))
        return LUSTRINE_ERR_ARGS;
    if (num_positions > (size_t)LUSTRINE_NOALLOC_MAX_KEYS || num_cells > (size_t)LUSTRINE_NOALLOC_MAX_CELLS)
        return LUSTRINE_ERR_TOO_LARGE;
    if (counting_sort_scratch_ints((int)num_positions, (int)num_cells) * sizeof(int) >
        (size_t)LUSTRINE_NOALLOC_SCRATCH_BYTES)
        return LUSTRINE_ERR_TOO_LARGE;
    int* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const int n = (int)num_positions, C = (int)num_cells;
    CountingSortScratch w = counting_sort_scratch(scratch, n, C);
    // the histogram and the status word start at zero; the rest is written
    // before it is read
    cudaError_t e = cudaMemsetAsync(w.count, 0, (size_t)C * sizeof(int), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(w.status, 0, sizeof(int), st);
    if (e != cudaSuccess) return lgb_cuda_status(e, "cudaMemsetAsync");
    launch_counting_sort(keys, n, C, w, counts, sorted_indices, st);
    int bad = 0;
    e = cudaMemcpyAsync(&bad, w.status, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return lgb_cuda_status(e, "counting_sort_noalloc");
    return bad ? LUSTRINE_ERR_ARGS : LUSTRINE_OK;
}
