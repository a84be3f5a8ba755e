// pbf_sort.cu -- cell counting sort of particles, rebuilt every step.
//
// The reference bins particles into a vector per cell (Neighbors.cpp:370-384);
// its counting sort (Sorting.cpp:12-34) is histogram -> prefix scan -> stable
// scatter.  The GPU form:
//   1. histogram: the prediction kernel does atomicAdd(count[key]) and keeps
//      the returned value as the particle's provisional rank in its cell;
//   2. exclusive scan of count over all cells: tile totals, then every tile
//      scanned from the sum of the totals before it (k_tile_sums,
//      k_scan_tiles; grids of more than CELL_SCAN_MAX_TILES tiles scan the
//      totals in one block in between); the standalone sort entry points use
//      reduce / scan of the tile sums / down-sweep; the scan also zeroes
//      count for the next step's histogram;
//   3. scatter of particle indices to start[key] + rank;
//   4. stabilisation: atomic arrival order is arbitrary, so every cell's
//      members are put in the order of a tie key (previous slot, or the
//      caller's id in compat mode) -- the result is the stable order of the
//      reference's counting sort -- and the particle state is gathered into
//      the final slot in the same kernel.  A member of a cell of at most
//      SMALL_CELL particles counts the members with a smaller tie key (O(k)
//      per particle); a larger cell is sorted by the block holding its first
//      slot: a bitonic sort in shared memory up to SORT_CAP members, beyond
//      that sorted runs of SORT_CAP merged pairwise through the rank array
//      (free once the scatter has read it) -- O(k log k) for a cell of k.
#include "pbf_common.cuh"
#include "pbf_kernels.h"

namespace lgb {

namespace {
thread_local bool t_pdl = false;
}
void set_pdl(bool on) { t_pdl = on; }
bool pdl_enabled() { return t_pdl; }

__device__ __forceinline__ int warp_inclusive_scan(int v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Exclusive scan of one value per thread across a block of THREADS threads;
// returns the exclusive prefix and writes the block total to *total.
template <int THREADS>
__device__ __forceinline__ int block_exclusive_scan(int v, int* total) {
    constexpr int W = THREADS / 32;
    __shared__ int warp_sums[W + 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int inc = warp_inclusive_scan(v);
    if (lane == 31) warp_sums[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        int w = lane < W ? warp_sums[lane] : 0;
        int wi = warp_inclusive_scan(w);
        if (lane < W) warp_sums[lane] = wi - w;
        if (lane == W - 1) warp_sums[W] = wi;
    }
    __syncthreads();
    int res = inc - v + warp_sums[warp];
    *total = warp_sums[W];
    __syncthreads();
    return res;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const int* __restrict__ count, int C,
                                                              int* __restrict__ block_sums) {
    pdl_wait();
    const int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++)
        if (base + k < C) s += count[base + k];
    int total;
    block_exclusive_scan<SCAN_THREADS>(s, &total);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// One block: exclusive scan of the per-tile sums, in place; 8 sums per
// thread, so up to 8192 tiles (16.7 M cells) take one pass.
constexpr int SUMS_THREADS = 1024;
constexpr int SUMS_ITEMS = 8;
__global__ void __launch_bounds__(SUMS_THREADS) k_scan_sums(int* __restrict__ block_sums, int nb) {
    pdl_wait();
    int carry = 0;
    for (int base = 0; base < nb; base += SUMS_THREADS * SUMS_ITEMS) {
        const int first = base + threadIdx.x * SUMS_ITEMS;
        int vals[SUMS_ITEMS];
        int s = 0;
#pragma unroll
        for (int k = 0; k < SUMS_ITEMS; k++) {
            vals[k] = first + k < nb ? block_sums[first + k] : 0;
            s += vals[k];
        }
        int total;
        int ex = block_exclusive_scan<SUMS_THREADS>(s, &total) + carry;
#pragma unroll
        for (int k = 0; k < SUMS_ITEMS; k++) {
            if (first + k < nb) block_sums[first + k] = ex;
            ex += vals[k];
        }
        carry += total;
    }
}

// Down-sweep: start[c] = exclusive prefix of count; count is zeroed behind
// it, ready for the next histogram.
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_down(int* __restrict__ count, int C,
                                                            const int* __restrict__ block_sums,
                                                            int* __restrict__ start) {
    pdl_wait();
    const int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    int vals[SCAN_ITEMS];
    int s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        vals[k] = base + k < C ? count[base + k] : 0;
        s += vals[k];
    }
    int total;
    int ex = block_exclusive_scan<SCAN_THREADS>(s, &total) + block_sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        if (base + k < C) {
            start[base + k] = ex;
            if (vals[k]) count[base + k] = 0;
        }
        ex += vals[k];
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == SCAN_THREADS - 1) start[C] = ex;
}

// Exclusive scan of the step in two passes with no inter-block waits:
// k_tile_sums writes the total of every tile of CELL_TILE cells, then each
// block of k_scan_tiles finds its tile's offset by summing the totals of the
// tiles before it (at most CELL_SCAN_MAX_TILES values, L2-resident) and
// scans its tile.
__device__ __forceinline__ void load_tile_items(const int* __restrict__ count, int C, long long base,
                                                int (&v)[CELL_SCAN_ITEMS]) {
    if (base + CELL_SCAN_ITEMS <= C) {
        const int4* c4 = reinterpret_cast<const int4*>(count + base);
#pragma unroll
        for (int q = 0; q < CELL_SCAN_ITEMS / 4; q++) {
            const int4 t = c4[q];
            v[4 * q] = t.x;
            v[4 * q + 1] = t.y;
            v[4 * q + 2] = t.z;
            v[4 * q + 3] = t.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < CELL_SCAN_ITEMS; k++) v[k] = base + k < C ? count[base + k] : 0;
    }
}

__global__ void __launch_bounds__(CELL_SCAN_THREADS) k_tile_sums(const int* __restrict__ count, int C,
                                                                 int* __restrict__ tile_sum) {
    pdl_wait();
    const long long base = (long long)blockIdx.x * CELL_TILE + (long long)threadIdx.x * CELL_SCAN_ITEMS;
    int v[CELL_SCAN_ITEMS];
    load_tile_items(count, C, base, v);
    int sum = 0;
#pragma unroll
    for (int k = 0; k < CELL_SCAN_ITEMS; k++) sum += v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    __shared__ int warp_total[CELL_SCAN_THREADS / 32];
    if ((threadIdx.x & 31) == 0) warp_total[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
#pragma unroll
        for (int w = 0; w < CELL_SCAN_THREADS / 32; w++) t += warp_total[w];
        tile_sum[blockIdx.x] = t;
    }
}

// SCANNED: tile_sum already holds every tile's exclusive offset (grids of
// more than CELL_SCAN_MAX_TILES tiles scan the totals in one block first).
// tile_zero (may be null): per-tile totals that the next prediction will
// count into, zeroed here (one entry per tile).
template <bool SCANNED>
__global__ void __launch_bounds__(CELL_SCAN_THREADS) k_scan_tiles(int* __restrict__ count, int C,
                                                                  const int* __restrict__ tile_sum,
                                                                  int* __restrict__ start,
                                                                  int* __restrict__ tile_zero) {
    pdl_wait();
    const int tile = blockIdx.x;
    if (tile_zero && threadIdx.x == 0) tile_zero[tile] = 0;
    const long long base = (long long)tile * CELL_TILE + (long long)threadIdx.x * CELL_SCAN_ITEMS;
    const bool full = base + CELL_SCAN_ITEMS <= C;
    int v[CELL_SCAN_ITEMS];
    load_tile_items(count, C, base, v);
    int part = 0;
    if (!SCANNED)
        for (int j = threadIdx.x; j < tile; j += CELL_SCAN_THREADS) part += __ldg(&tile_sum[j]);
    int sum = 0;
#pragma unroll
    for (int k = 0; k < CELL_SCAN_ITEMS; k++) sum += v[k];
    int total, offset;
    block_exclusive_scan<CELL_SCAN_THREADS>(part, &offset);
    if (SCANNED) offset = __ldg(&tile_sum[tile]);
    int ex = block_exclusive_scan<CELL_SCAN_THREADS>(sum, &total) + offset;
    if (full) {
        int4* s4 = reinterpret_cast<int4*>(start + base);
        int4* c4 = reinterpret_cast<int4*>(count + base);
#pragma unroll
        for (int q = 0; q < CELL_SCAN_ITEMS / 4; q++) {
            int4 o;
            o.x = ex;
            o.y = o.x + v[4 * q];
            o.z = o.y + v[4 * q + 1];
            o.w = o.z + v[4 * q + 2];
            ex = o.w + v[4 * q + 3];
            s4[q] = o;
            if (v[4 * q] | v[4 * q + 1] | v[4 * q + 2] | v[4 * q + 3]) c4[q] = make_int4(0, 0, 0, 0);
        }
    } else {
#pragma unroll
        for (int k = 0; k < CELL_SCAN_ITEMS; k++) {
            if (base + k < C) {
                start[base + k] = ex;
                if (v[k]) count[base + k] = 0;
            }
            ex += v[k];
        }
    }
    if (tile == gridDim.x - 1 && threadIdx.x == 0) start[C] = offset + total;
}

__global__ void k_scatter_index(const int* __restrict__ key, const int* __restrict__ rank,
                                const int* __restrict__ start, int n, int* __restrict__ tmp) {
    pdl_wait();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) tmp[start[key[i]] + rank[i]] = i;
}

// ------------------------------------------------------- stabilisation --

constexpr int STAB_THREADS = 256;
constexpr int SMALL_CELL = 32;   // cells up to this size: O(k) rank per member
constexpr int SORT_CAP = 2048;   // members a block sorts in shared memory at once
constexpr int MAX_BIG_PER_BLOCK = STAB_THREADS / (SMALL_CELL + 1) + 1;

__device__ __forceinline__ int tie_of(const int* __restrict__ tie, int e) { return tie ? tie[e] : e; }

// Bitonic sort of N (a power of two <= SORT_CAP) (tie, element) pairs in
// shared memory, ascending by tie (ties are distinct; pads carry INT_MAX).
__device__ __forceinline__ void bitonic_sort_smem(int* kk, int* vv, int N) {
    for (int size = 2; size <= N; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = threadIdx.x; t < N / 2; t += blockDim.x) {
                const int lo = 2 * stride * (t / stride) + (t % stride);
                const int hi = lo + stride;
                const bool up = (lo & size) == 0;
                const int a = kk[lo], b = kk[hi];
                if ((a > b) == up) {
                    kk[lo] = b;
                    kk[hi] = a;
                    const int x = vv[lo];
                    vv[lo] = vv[hi];
                    vv[hi] = x;
                }
            }
            __syncthreads();
        }
    }
}

// Number of elements of run A (length la) that precede output position q of
// the merge of A and B (length lb), both ascending by tie; A first on equal
// ties (ties are distinct, so that never happens).
__device__ __forceinline__ int merge_split(const int* __restrict__ A, int la, const int* __restrict__ B,
                                           int lb, int q, const int* __restrict__ tie) {
    int lo = max(0, q - lb), hi = min(q, la);
    while (lo < hi) {
        const int m = (lo + hi) >> 1;  // m elements of A and q - m of B before q?
        if (tie_of(tie, A[m]) < tie_of(tie, B[q - m - 1]))
            lo = m + 1;
        else
            hi = m;
    }
    return lo;
}

// Sorts the k members of the cell at slots [a, a + k) of buf (element ids in
// arrival order) by tie; returns the buffer (buf or aux) holding the sorted
// members at [a, a + k).  All threads of the block call it.
__device__ int* sort_cell(int* __restrict__ buf, int* __restrict__ aux, int a, int k,
                          const int* __restrict__ tie, int* kk, int* vv) {
    // runs of SORT_CAP sorted in shared memory, written back in place
    for (int c0 = 0; c0 < k; c0 += SORT_CAP) {
        const int m = min(SORT_CAP, k - c0);
        int N = 64;
        while (N < m) N <<= 1;
        for (int t = threadIdx.x; t < N; t += blockDim.x) {
            const int e = t < m ? buf[a + c0 + t] : -1;
            kk[t] = t < m ? tie_of(tie, e) : 0x7fffffff;
            vv[t] = e;
        }
        __syncthreads();
        bitonic_sort_smem(kk, vv, N);
        for (int t = threadIdx.x; t < m; t += blockDim.x) buf[a + c0 + t] = vv[t];
        __syncthreads();
    }
    // pairwise merges of sorted runs, ping-ponging between buf and aux; each
    // thread merges one contiguous stretch of the output from its split
    int* src = buf;
    int* dst = aux;
    for (int w = SORT_CAP; w < k; w <<= 1) {
        for (int lo = 0; lo < k; lo += 2 * w) {
            const int la = min(w, k - lo), lb = max(0, min(w, k - lo - w));
            const int len = la + lb;
            const int* A = src + a + lo;
            const int* B = A + la;
            int* O = dst + a + lo;
            const int per = (len + blockDim.x - 1) / blockDim.x;
            const int q0 = min(len, (int)threadIdx.x * per), q1 = min(len, q0 + per);
            if (q0 < q1) {
                int i = merge_split(A, la, B, lb, q0, tie), j = q0 - i;
                for (int q = q0; q < q1; q++) {
                    const bool takeA = j >= lb || (i < la && tie_of(tie, A[i]) < tie_of(tie, B[j]));
                    O[q] = takeA ? A[i++] : B[j++];
                }
            }
        }
        __syncthreads();
        int* t = src;
        src = dst;
        dst = t;
    }
    return src;
}

// Final slot of the member at slot s of a small cell (k <= SMALL_CELL):
// a + the number of members with a smaller tie.
__device__ __forceinline__ int small_rank(const int* __restrict__ tmp, const int* __restrict__ tie, int a, int b,
                                          int mine) {
    int r = 0;
    for (int t = a; t < b; t++) r += tie_of(tie, tmp[t]) < mine;
    return r;
}

// The stabilisation of one block of slots.  emit(f, i): element i goes to
// slot f.  Small cells are placed per slot; every big cell whose first slot
// is in this block's range is sorted by the whole block (the other blocks
// skip its members).
template <class Emit>
__device__ __forceinline__ void stabilize_block(int* __restrict__ tmp, int* __restrict__ aux,
                                                const int* __restrict__ key, const int* __restrict__ start,
                                                const int* __restrict__ tie, int n, Emit&& emit) {
    __shared__ int kk[SORT_CAP], vv[SORT_CAP];
    __shared__ int big_a[MAX_BIG_PER_BLOCK], big_k[MAX_BIG_PER_BLOCK];
    __shared__ int num_big;
    if (threadIdx.x == 0) num_big = 0;
    __syncthreads();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) {
        const int i = tmp[s];
        const int c = key[i];
        const int a = start[c], b = start[c + 1];
        if (b - a <= SMALL_CELL) {
            emit(a + small_rank(tmp, tie, a, b, tie_of(tie, i)), i);
        } else if (s == a) {
            const int q = atomicAdd(&num_big, 1);
            big_a[q] = a;
            big_k[q] = b - a;
        }
    }
    __syncthreads();
    for (int q = 0; q < num_big; q++) {
        const int a = big_a[q], k = big_k[q];
        const int* sorted = sort_cell(tmp, aux, a, k, tie, kk, vv);
        for (int p = threadIdx.x; p < k; p += blockDim.x) emit(a + p, sorted[a + p]);
        __syncthreads();
    }
}

// Standalone sort: perm[final slot] = element.  aux: n ints of merge space.
__global__ void __launch_bounds__(STAB_THREADS) k_stabilize(int* __restrict__ tmp, int* __restrict__ aux,
                                                            const int* __restrict__ key,
                                                            const int* __restrict__ start,
                                                            const int* __restrict__ tie, int n,
                                                            int* __restrict__ perm) {
    stabilize_block(tmp, aux, key, start, tie, n, [&](int f, int i) { perm[f] = i; });
}

// Stabilisation fused with the reorder: the slot found for particle i
// receives its state directly (no permutation array round trip).
__global__ void __launch_bounds__(STAB_THREADS) k_stabilize_gather(
    int* __restrict__ tmp, int* __restrict__ aux, const int* __restrict__ key, const int* __restrict__ start,
    const int* __restrict__ tie, int n, const float4* __restrict__ x, const float4* __restrict__ xs,
    const float4* __restrict__ v, const int* __restrict__ id, int* __restrict__ key_out,
    float4* __restrict__ x_out, float4* __restrict__ xs_out, float4* __restrict__ v_out, int* __restrict__ id_out,
    const int* __restrict__ aux_in, int* __restrict__ aux_out, int* __restrict__ slot_of,
    int* __restrict__ src_out) {
    pdl_wait();
    stabilize_block(tmp, aux, key, start, tie, n, [&](int f, int i) {
        key_out[f] = key[i];
        if (x_out) x_out[f] = x[i];
        if (src_out) src_out[f] = i;  // the committed position stays at i
        xs_out[f] = xs[i];
        if (v) v_out[f] = v[i];
        if (id) id_out[f] = id[i];
        if (aux_in) aux_out[f] = aux_in[i];
        if (slot_of) slot_of[id[i]] = f;  // the caller index's new slot (state downloads)
    });
}

__global__ void k_gather_int(const int* __restrict__ perm, int n, const int* __restrict__ src,
                             int* __restrict__ dst) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) dst[s] = src[perm[s]];
}

__global__ void k_gather_solid(const int* __restrict__ perm, int n, const float4* __restrict__ src,
                               float4* __restrict__ dst) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) dst[s] = src[perm[s]];
}

// Histogram of caller keys (standalone counting sort).  A key outside
// [0, num_cells) is recorded in *status and counted in cell 0 so that every
// access stays in bounds.
__global__ void k_key_hist(const int* __restrict__ keys, int n, int num_cells, int* __restrict__ key_out,
                           int* __restrict__ rank, int* __restrict__ count, int* status) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int k = keys[i];
    if (k < 0 || k >= num_cells) {
        set_status(status, ST_BAD_VALUE);
        k = 0;
    }
    key_out[i] = k;
    rank[i] = atomicAdd(&count[k], 1);
}

// ------------------------------------------------------------------ launch --

static inline int blocks_for(int n, int t) { return (n + t - 1) / t; }

void launch_scan(int* count, int C, int* block_sums, int* start, cudaStream_t st) {
    const int nb = blocks_for(C, SCAN_TILE);
    const bool pdl = pdl_enabled();
    launch_k(k_scan_reduce, nb, SCAN_THREADS, st, pdl, (const int*)count, C, block_sums);
    launch_k(k_scan_sums, 1, SUMS_THREADS, st, pdl, block_sums, nb);
    launch_k(k_scan_down, nb, SCAN_THREADS, st, pdl, count, C, (const int*)block_sums, start);
}

int scan_block_sums_size(int C) { return scan_block_sums_ints(C); }

int cell_scan_tiles(int C) { return blocks_for(C, CELL_TILE); }

void launch_scan_tiles(int* count, int C, int* tile_sum, int* start, cudaStream_t st, bool counted,
                       int* tile_zero) {
    const bool pdl = pdl_enabled();
    const int tiles = cell_scan_tiles(C);
    if (!counted) launch_k(k_tile_sums, tiles, CELL_SCAN_THREADS, st, pdl, (const int*)count, C, tile_sum);
    if (tiles <= CELL_SCAN_MAX_TILES) {
        launch_k(k_scan_tiles<false>, tiles, CELL_SCAN_THREADS, st, pdl, count, C, (const int*)tile_sum, start,
                 tile_zero);
    } else {
        launch_k(k_scan_sums, 1, SUMS_THREADS, st, pdl, tile_sum, tiles);  // in place, exclusive
        launch_k(k_scan_tiles<true>, tiles, CELL_SCAN_THREADS, st, pdl, count, C, (const int*)tile_sum, start,
                 tile_zero);
    }
}

int scan_tiles_launches(int C, bool counted) {
    return (cell_scan_tiles(C) <= CELL_SCAN_MAX_TILES ? 1 : 2) + (counted ? 0 : 1);
}

void launch_sort_tail(const int* key, int* rank, const int* start, const int* tie, int n,
                      int* tmp, int* perm, cudaStream_t st) {
    if (n <= 0) return;
    k_scatter_index<<<blocks_for(n, 256), 256, 0, st>>>(key, rank, start, n, tmp);
    k_stabilize<<<blocks_for(n, STAB_THREADS), STAB_THREADS, 0, st>>>(tmp, rank, key, start, tie, n, perm);
}

void launch_sort_state(const int* key, int* rank, const int* start, const int* tie, int n,
                       int* tmp, const float4* x, const float4* xs, const float4* v, const int* id,
                       int* key_out, float4* x_out, float4* xs_out, float4* v_out, int* id_out,
                       const int* aux, int* aux_out, int* slot_of, int* src_out, cudaStream_t st) {
    if (n <= 0) return;
    const bool pdl = pdl_enabled();
    launch_k(k_scatter_index, blocks_for(n, 256), 256, st, pdl, key, (const int*)rank, start, n, tmp);
    // the rank array, read by the scatter only, is the big cells' merge space
    launch_k(k_stabilize_gather, blocks_for(n, STAB_THREADS), STAB_THREADS, st, pdl, tmp, rank, key, start, tie,
             n, x, xs, v, id, key_out, x_out, xs_out, v_out, id_out, aux, aux_out, slot_of, src_out);
}

void launch_gather_solid(const int* perm, int n, const float4* src, float4* dst, cudaStream_t st) {
    if (n <= 0) return;
    k_gather_solid<<<blocks_for(n, 256), 256, 0, st>>>(perm, n, src, dst);
}

void launch_gather_int(const int* perm, int n, const int* src, int* dst, cudaStream_t st) {
    if (n <= 0) return;
    k_gather_int<<<blocks_for(n, 256), 256, 0, st>>>(perm, n, src, dst);
}

void launch_counting_sort(const int* keys, int n, int num_cells, CountingSortScratch w, int* start,
                          int* sorted, cudaStream_t st) {
    if (n > 0)
        k_key_hist<<<blocks_for(n, 256), 256, 0, st>>>(keys, n, num_cells, w.key, w.rank, w.count, w.status);
    launch_scan(w.count, num_cells, w.block_sums, start, st);
    launch_sort_tail(w.key, w.rank, start, nullptr, n, w.tmp, sorted, st);
}

size_t counting_sort_scratch_ints(int n, int num_cells) { return counting_sort_scratch_ints_for(n, num_cells); }

CountingSortScratch counting_sort_scratch(int* base, int n, int num_cells) {
    CountingSortScratch w;
    w.count = base;
    w.block_sums = w.count + num_cells;
    w.key = w.block_sums + scan_block_sums_size(num_cells);
    w.rank = w.key + n;
    w.tmp = w.rank + n;
    w.status = w.tmp + n;
    return w;
}

}  // namespace lgb
