// pbf_solver.cu -- launchers of the PBF step's kernels (pbf_passes.cuh) over
// column neighbour lists, the state transfers, the cell-count query and the
// FP64 reductions; the passes over compact lists launch from
// pbf_compact.cu.
#include "pbf_passes.cuh"

namespace lgb {

// Absolute positions (float3 triples) in the caller's id order.
template <bool MIXED>
__global__ void k_unpermute_pos(StepParams p, CellPack cp, const float4* __restrict__ a,
                                const int* __restrict__ id, int n, float* __restrict__ out) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    float4 q = a[s];
    int i = id[s];
    if (MIXED) {
        int3 c = unpack_cell(cp, q.w);
        out[3 * (size_t)i + 0] = (float)c.x * p.cell + q.x;
        out[3 * (size_t)i + 1] = (float)c.y * p.cell + q.y;
        out[3 * (size_t)i + 2] = (float)c.z * p.cell + q.z;
    } else {
        out[3 * (size_t)i + 0] = q.x;
        out[3 * (size_t)i + 1] = q.y;
        out[3 * (size_t)i + 2] = q.z;
    }
}

// Exact double positions in id order (mixed: cell * cell_size + offset in fp64).
template <bool MIXED>
__global__ void k_unpermute_pos_d(StepParams p, CellPack cp, const float4* __restrict__ a,
                                  const int* __restrict__ id, int n, double* __restrict__ out) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    float4 q = a[s];
    int i = id[s];
    double bx = 0.0, by = 0.0, bz = 0.0;
    if (MIXED) {
        int3 c = unpack_cell(cp, q.w);
        bx = (double)c.x * (double)p.cell;
        by = (double)c.y * (double)p.cell;
        bz = (double)c.z * (double)p.cell;
    }
    out[3 * (size_t)i + 0] = bx + (double)q.x;
    out[3 * (size_t)i + 1] = by + (double)q.y;
    out[3 * (size_t)i + 2] = bz + (double)q.z;
}

// Caller position into the state representation.  Mixed: the cell is
// clamped to the cells a clamped position can occupy (the packed field
// widths); the offset keeps the exact position, so a caller position outside
// the box stays where it is (it may then lie outside [0, cell)) and the next
// prediction clamps it like the plain form does.
template <bool MIXED>
__device__ __forceinline__ float4 pack_position(const StepParams& p, const CellPack& cp, const Geo& g, float x,
                                                float y, float z) {
    if (!MIXED) return make_float4(x, y, z, 0.0f);
    int cx = min(max((int)floorf(x * p.inv_cell), 0), (int)floorf(g.hix * p.inv_cell));
    int cy = min(max((int)floorf(y * p.inv_cell), 0), (int)floorf(g.hiy * p.inv_cell));
    int cz = min(max((int)floorf(z * p.inv_cell), 0), (int)floorf(g.hiz * p.inv_cell));
    return make_float4(x - (float)cx * p.cell, y - (float)cy * p.cell, z - (float)cz * p.cell,
                       pack_cell(cp, cx, cy, cz));
}

// Positions stored as cell + offset (w: the packed cell) into the scene
// frame, w kept: the static particles of a context that iterates in the
// scene frame (their cells stay in w for the cell keys).
__global__ void k_to_scene_frame(StepParams p, CellPack cp, float4* __restrict__ a, int m) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const float4 q = a[i];
    const int3 c = unpack_cell(cp, q.w);
    a[i] = make_float4(__fmaf_rn((float)c.x, p.cell, q.x), __fmaf_rn((float)c.y, p.cell, q.y),
                       __fmaf_rn((float)c.z, p.cell, q.z), q.w);
}

// Caller positions (float3, id order) into the state representation, slot = id.
// scene_of: scene of each packed element in a batch (nullptr for one scene).
template <bool MIXED>
__global__ void k_pack_pos(StepParams p, CellPack cp, const float* __restrict__ in, int n,
                           const int* __restrict__ scene_of, float4* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Geo g = (p.scenes && scene_of) ? geo_scene(p, scene_of[i]) : geo_single(p);
    out[i] = pack_position<MIXED>(p, cp, g, in[3 * (size_t)i], in[3 * (size_t)i + 1], in[3 * (size_t)i + 2]);
}

// The state straight from / into page-locked host memory, which the GPU
// reads and writes over the host link (no staging copy): caller order on the
// host, slot order on the device.  A block moves the 3 x 256 floats of its
// 256 particles through shared memory, so the host side is read and written
// as consecutive 16-byte pieces by consecutive threads (the tail of the
// array, and an array not 16-byte aligned, one float at a time).
constexpr int HOST_BLOCK = 256;

__device__ __forceinline__ void host_to_smem(const float* __restrict__ h, int n, float* sm) {
    const int first = blockIdx.x * HOST_BLOCK;
    const int m = min(HOST_BLOCK, n - first);
    const size_t base = 3 * (size_t)first;
    const int nf = 3 * m;
    if ((reinterpret_cast<size_t>(h) & 15) == 0) {
        const float4* h4 = reinterpret_cast<const float4*>(h + base);  // base is a multiple of 768 floats
        for (int t = threadIdx.x; 4 * t + 3 < nf; t += HOST_BLOCK) {
            const float4 q = h4[t];
            sm[4 * t] = q.x;
            sm[4 * t + 1] = q.y;
            sm[4 * t + 2] = q.z;
            sm[4 * t + 3] = q.w;
        }
        for (int f = (nf & ~3) + threadIdx.x; f < nf; f += HOST_BLOCK) sm[f] = h[base + f];
    } else {
        for (int f = threadIdx.x; f < nf; f += HOST_BLOCK) sm[f] = h[base + f];
    }
}

__device__ __forceinline__ void smem_to_host(const float* sm, int n, float* __restrict__ h) {
    const int first = blockIdx.x * HOST_BLOCK;
    const int m = min(HOST_BLOCK, n - first);
    const size_t base = 3 * (size_t)first;
    const int nf = 3 * m;
    if ((reinterpret_cast<size_t>(h) & 15) == 0) {
        float4* h4 = reinterpret_cast<float4*>(h + base);
        for (int t = threadIdx.x; 4 * t + 3 < nf; t += HOST_BLOCK)
            h4[t] = make_float4(sm[4 * t], sm[4 * t + 1], sm[4 * t + 2], sm[4 * t + 3]);
        for (int f = (nf & ~3) + threadIdx.x; f < nf; f += HOST_BLOCK) h[base + f] = sm[f];
    } else {
        for (int f = threadIdx.x; f < nf; f += HOST_BLOCK) h[base + f] = sm[f];
    }
}

// Upload: slot = caller index.
template <bool MIXED>
__global__ void __launch_bounds__(HOST_BLOCK) k_pack_state(StepParams p, CellPack cp, const float* __restrict__ hx,
                                                           const float* __restrict__ hv, int n,
                                                           float4* __restrict__ x, float4* __restrict__ v,
                                                           int* __restrict__ id) {
    __shared__ float sx[3 * HOST_BLOCK], sv[3 * HOST_BLOCK];
    host_to_smem(hx, n, sx);
    if (hv) host_to_smem(hv, n, sv);
    __syncthreads();
    const int i = blockIdx.x * HOST_BLOCK + threadIdx.x;
    if (i >= n) return;
    const int t = 3 * threadIdx.x;
    x[i] = pack_position<MIXED>(p, cp, geo_single(p), sx[t], sx[t + 1], sx[t + 2]);
    v[i] = hv ? make_float4(sv[t], sv[t + 1], sv[t + 2], 0.0f) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    id[i] = i;
}

// Upload fused with the step's prediction (a host frame: the state comes in
// from page-locked memory and is stepped at once): slot = caller index, x
// packed into the state, v used by the prediction only (the step recomputes
// it), then predict_one as k_predict does on the same values.
template <bool MIXED>
__global__ void __launch_bounds__(HOST_BLOCK) k_pack_predict(StepParams p, CellPack cp, const float* __restrict__ hx,
                                                             const float* __restrict__ hv, int n,
                                                             float4* __restrict__ x, int* __restrict__ id,
                                                             float4* __restrict__ xs, int* __restrict__ key,
                                                             int* __restrict__ rank, int* __restrict__ count,
                                                             int* __restrict__ cellk, int* __restrict__ tile_count) {
    __shared__ float sx[3 * HOST_BLOCK], sv[3 * HOST_BLOCK];
    host_to_smem(hx, n, sx);
    if (hv) host_to_smem(hv, n, sv);
    __syncthreads();
    const int i = blockIdx.x * HOST_BLOCK + threadIdx.x;
    if (i >= n) return;
    const int t = 3 * threadIdx.x;
    const Geo g = geo_single(p);
    const float4 xi = pack_position<MIXED>(p, cp, g, sx[t], sx[t + 1], sx[t + 2]);
    const float4 vi = hv ? make_float4(sv[t], sv[t + 1], sv[t + 2], 0.0f) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    x[i] = xi;
    id[i] = i;
    predict_one<MIXED>(p, cp, g, xi, vi, i, xs, key, rank, count, cellk, tile_count);
}

__global__ void k_slot_of(const int* __restrict__ id, int n, int* __restrict__ slot_of) {
    pdl_wait();
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) slot_of[id[s]] = s;
}

// Download: one thread per caller index gathers its slot.
template <bool MIXED>
__global__ void __launch_bounds__(HOST_BLOCK) k_unpack_state(StepParams p, CellPack cp, const float4* __restrict__ x,
                                                             const float4* __restrict__ v,
                                                             const int* __restrict__ slot_of, int n,
                                                             float* __restrict__ hx, float* __restrict__ hv) {
    pdl_wait();
    __shared__ float sx[3 * HOST_BLOCK], sv[3 * HOST_BLOCK];
    const int i = blockIdx.x * HOST_BLOCK + threadIdx.x;
    if (i < n) {
        const int s = slot_of[i];
        const int t = 3 * threadIdx.x;
        if (hx) {
            const float4 q = x[s];
            float a = q.x, b = q.y, c = q.z;
            if (MIXED) {
                const int3 cc = unpack_cell(cp, q.w);
                a += (float)cc.x * p.cell;
                b += (float)cc.y * p.cell;
                c += (float)cc.z * p.cell;
            }
            sx[t] = a;
            sx[t + 1] = b;
            sx[t + 2] = c;
        }
        if (hv) {
            const float4 u = v[s];
            sv[t] = u.x;
            sv[t + 1] = u.y;
            sv[t + 2] = u.z;
        }
    }
    __syncthreads();
    if (hx) smem_to_host(sx, n, hx);
    if (hv) smem_to_host(sv, n, hv);
}

// Particles binned in a box of cells by the last step (the sorted cell table
// of its prediction), Lustrine.cpp:864-914.  Dense grid: one thread per
// (y, x) row of the box, the row's z range being one slot range of each
// table.  Hashed grid: one thread per particle, its packed cell tested.
__global__ void k_query_rows(int gx, int gz, int x0, int x1, int y0, int y1, int z0, int z1,
                             const int* __restrict__ fstart, const int* __restrict__ sstart,
                             int* __restrict__ out) {
    const int nx = x1 - x0 + 1;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    int c = 0;
    if (r < nx * (y1 - y0 + 1)) {
        const int y = y0 + r / nx, x = x0 + r % nx;
        const int row = y * gx * gz + x * gz;
        c = fstart[row + z1 + 1] - fstart[row + z0];
        if (sstart) c += sstart[row + z1 + 1] - sstart[row + z0];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

__global__ void k_query_packed(CellPack cp, const int* __restrict__ cells, int m, int x0, int x1, int y0,
                               int y1, int z0, int z1, int* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int c = 0;
    if (i < m) {
        const unsigned u = (unsigned)cells[i];
        const int x = (int)(u & cp.mx), y = (int)((u >> cp.by_shift) & cp.my), z = (int)((u >> cp.bz_shift) & cp.mz);
        c = (x >= x0 && x <= x1 && y >= y0 && y <= y1 && z >= z0 && z <= z1) ? 1 : 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

void launch_query_cells(const StepParams& p, const CellPack& cp, const int box[6], const int* fstart,
                        const int* sstart, const int* cell_sorted, const int* solid_cell, int* out,
                        cudaStream_t st) {
    const int x0 = box[0], x1 = box[1], y0 = box[2], y1 = box[3], z0 = box[4], z1 = box[5];
    if (!p.hash_bits) {
        const int rows = (x1 - x0 + 1) * (y1 - y0 + 1);
        k_query_rows<<<(rows + 255) / 256, 256, 0, st>>>(p.gx, p.gz, x0, x1, y0, y1, z0, z1, fstart,
                                                            sstart, out);
        return;
    }
    if (p.n > 0)
        k_query_packed<<<(p.n + 255) / 256, 256, 0, st>>>(cp, cell_sorted, p.n, x0, x1, y0, y1, z0, z1, out);
    if (solid_cell && p.ns > 0)
        k_query_packed<<<(p.ns + 255) / 256, 256, 0, st>>>(cp, solid_cell, p.ns, x0, x1, y0, y1, z0, z1,
                                                              out);
}

// FP64 reductions over the fluid: [0] mass, [1..3] momentum, [4] kinetic
// energy, [5..7] mass-weighted position sum, [8] max |rho / rho0 - 1|.
__device__ __forceinline__ void atomic_max_pos_double(double* addr, double val) {
    // non-negative doubles order like their bit patterns as signed integers
    atomicMax((unsigned long long*)addr, (unsigned long long)__double_as_longlong(val));
}

template <bool MIXED>
__global__ void __launch_bounds__(256) k_reduce(StepParams p, CellPack cp, const float4* __restrict__ x,
                                                const float4* __restrict__ v,
                                                const float* __restrict__ rho, double* __restrict__ out) {
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    double emax = 0.0;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < p.n; s += gridDim.x * blockDim.x) {
        float4 q = x[s], u = v[s];
        double m = (double)p.mass;
        double px = q.x, py = q.y, pz = q.z;
        if (MIXED) {
            int3 c = unpack_cell(cp, q.w);
            px += (double)c.x * p.cell;
            py += (double)c.y * p.cell;
            pz += (double)c.z * p.cell;
        }
        acc[0] += m;
        acc[1] += m * u.x;
        acc[2] += m * u.y;
        acc[3] += m * u.z;
        acc[4] += 0.5 * m * ((double)u.x * u.x + (double)u.y * u.y + (double)u.z * u.z);
        acc[5] += m * px;
        acc[6] += m * py;
        acc[7] += m * pz;
        if (rho) emax = fmax(emax, fabs((double)rho[s] / (double)p.rho0 - 1.0));
    }
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < 8; k++) acc[k] += __shfl_down_sync(0xffffffffu, acc[k], o);
        emax = fmax(emax, __shfl_down_sync(0xffffffffu, emax, o));
    }
    __shared__ double sh[8][9];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        for (int k = 0; k < 8; k++) sh[warp][k] = acc[k];
        sh[warp][8] = emax;
    }
    __syncthreads();
    if (threadIdx.x < 9) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++)
            t = threadIdx.x == 8 ? fmax(t, sh[w][8]) : t + sh[w][threadIdx.x];
        if (threadIdx.x == 8)
            atomic_max_pos_double(&out[8], t);
        else
            atomicAdd(&out[threadIdx.x], t);
    }
}

// ------------------------------------------------------------------ launch --


// Step kernels go through launch_k (programmatic dependent launch when the
// calling context enables it); the others are launched plainly.
#define LGB_DISPATCH(MIXED_FLAG, KERNEL, GRID, BLOCK, ST, ...)                        \
    do {                                                                              \
        if (MIXED_FLAG)                                                               \
            launch_k(KERNEL<true>, GRID, BLOCK, ST, pdl_enabled(), __VA_ARGS__);      \
        else                                                                          \
            launch_k(KERNEL<false>, GRID, BLOCK, ST, pdl_enabled(), __VA_ARGS__);     \
    } while (0)

void launch_predict(bool mixed, const StepParams& p, const CellPack& cp, const float4* x, const float4* v,
                    float4* xs, int* key, int* rank, int* count, int* cellk, int* tile_count, cudaStream_t st) {
    if (p.n <= 0) return;
    LGB_DISPATCH(mixed, k_predict, blocks_for(p.n, 256), 256, st, p, cp, x, v, xs, key, rank, count, cellk,
                 tile_count);
}

void launch_mark_solid_near(bool mixed, const StepParams& p, const CellPack& cp, const float4* pos, int m,
                            unsigned char* near, cudaStream_t st) {
    if (m <= 0) return;
    LGB_DISPATCH(mixed, k_mark_solid_near, blocks_for(m, 256), 256, st, p, cp, pos, m, near);
}

void launch_key(bool mixed, const StepParams& p, const CellPack& cp, const float4* pos, int m,
                int* key, int* rank, int* count, int* cellk, cudaStream_t st) {
    if (m <= 0) return;
    LGB_DISPATCH(mixed, k_key, blocks_for(m, 256), 256, st, p, cp, pos, m, key, rank, count, cellk);
}

void launch_lists_lambda(bool mixed, const Tuning& tu, const StepParams& p, const CellPack& cp,
                         float4* xs, const int* key_sorted, const int* cell_sorted, const int* fstart,
                         const float4* solid, const int* solid_cell, const int* sstart, int* nbr,
                         int* cnt, float* rho, int* status, cudaStream_t st) {
    if (p.n <= 0) return;
    const int B = tu.list_block <= 64 ? 64 : (tu.list_block <= 128 ? 128 : 256);
    StepParams pp = p;  // lists padded for the largest chunk of the passes that read them
    const int u = tu.unroll > tu.xsph_unroll ? tu.unroll : tu.xsph_unroll;
    pp.pad = u >= 8 ? 8 : (u >= 4 ? 4 : (u >= 2 ? 2 : 1));
    const bool pdl = pdl_enabled();
#define LGB_LISTS_H(MIX, H, BB)                                                                 \
    launch_k(k_lists_lambda<MIX, H, BB>, blocks_for(p.n, BB), BB, st, pdl, pp, cp, xs, key_sorted, \
             cell_sorted, fstart, solid, solid_cell, sstart, nbr, cnt, rho, status)
#define LGB_LISTS(MIX, BB)                       \
    do {                                         \
        if (p.hash_bits) LGB_LISTS_H(MIX, true, BB); \
        else LGB_LISTS_H(MIX, false, BB);        \
    } while (0)
    if (p.rec) {  // compact lists (pbf_compact.cu)
        launch_lists_compact(B, pp, cp, xs, key_sorted, cell_sorted, fstart, solid, solid_cell, sstart, nbr, cnt,
                             rho, status, st);
    } else if (mixed && p.frame) {  // the scene frame: fp32 pair offsets, compensated sums
        if (B == 64) launch_k(k_lists_lambda<false, false, 64, true>, blocks_for(p.n, 64), 64, st, pdl, pp, cp, xs,
                              key_sorted, cell_sorted, fstart, solid, solid_cell, sstart, nbr, cnt, rho, status);
        else if (B == 128) launch_k(k_lists_lambda<false, false, 128, true>, blocks_for(p.n, 128), 128, st, pdl, pp, cp,
                                    xs, key_sorted, cell_sorted, fstart, solid, solid_cell, sstart, nbr, cnt, rho,
                                    status);
        else launch_k(k_lists_lambda<false, false, 256, true>, blocks_for(p.n, 256), 256, st, pdl, pp, cp, xs,
                      key_sorted, cell_sorted, fstart, solid, solid_cell, sstart, nbr, cnt, rho, status);
    } else if (mixed) {
        if (B == 64) LGB_LISTS(true, 64);
        else if (B == 128) LGB_LISTS(true, 128);
        else LGB_LISTS(true, 256);
    } else {
        if (B == 64) LGB_LISTS(false, 64);
        else if (B == 128) LGB_LISTS(false, 128);
        else LGB_LISTS(false, 256);
    }
#undef LGB_LISTS
#undef LGB_LISTS_H
}

void launch_lambda(bool mixed, const Tuning& tu, const StepParams& p, float4* xs, const int* nbr,
                   const int* cnt, const float4* solid, float* rho, cudaStream_t st) {
    if (p.n <= 0) return;
    const int f = ((mixed && !p.frame) ? 1 : 0) | (p.ns > 0 ? 2 : 0);
    if (p.rec)  // compact lists (pbf_compact.cu)
        launch_lambda_compact(tu, p, xs, nbr, cnt, solid, rho, st);
    else if (mixed && p.frame)  // the scene frame: one particle per thread
        TUNE_DISPATCH_FRAME(k_lambda, f | 4, tu, p.n, st, p, xs, nbr, cnt, solid, rho);
    else
        TUNE_DISPATCH_PPT(k_lambda, f, tu, p.n, st, p, xs, nbr, cnt, solid, rho);
}

void launch_delta(bool mixed, const Tuning& tu, const StepParams& p, const CellPack& cp,
                  const float4* xs, float4* xs_out, const int* nbr, const int* cnt,
                  const float4* solid, const int* key_sorted, const float4* x, float4* v_out,
                  cudaStream_t st) {
    if (p.n <= 0) return;
    const int f = ((mixed && !p.frame) ? 1 : 0) | (p.ns > 0 ? 2 : 0);
    if (p.rec)  // compact lists (pbf_compact.cu)
        launch_delta_compact(tu, p, cp, xs, xs_out, nbr, cnt, solid, key_sorted, x, v_out, st);
    else
        TUNE_DISPATCH_PPT(k_delta, f, tu, p.n, st, p, cp, xs, xs_out, nbr, cnt, solid, key_sorted, x, v_out);
}

void launch_xsph(bool mixed, const Tuning& tu, const StepParams& p, const CellPack& cp,
                 const float4* xs, const float4* v_in, const int* nbr, const int* cnt,
                 const int* key_sorted, float4* x_out, float4* v_out, float4* xs_next, int* key,
                 int* rank, int* count, int* cellk, int* tile_count, cudaStream_t st) {
    if (p.n <= 0) return;
    Tuning tx = tu;  // the XSPH pass has its own gathers in flight
    tx.unroll = tu.xsph_unroll;
    const int f = ((mixed && !p.frame) ? 1 : 0) | (p.ns > 0 ? 2 : 0);
    if (p.rec)  // compact lists (pbf_compact.cu)
        launch_xsph_compact(tx, p, cp, xs, v_in, nbr, cnt, key_sorted, x_out, v_out, xs_next, key, rank, count, cellk,
                            tile_count, st);
    else
        TUNE_DISPATCH(k_xsph, f, tx, p.n, st, p, cp, xs, v_in, nbr, cnt, key_sorted, x_out, v_out, xs_next, key,
                      rank, count, cellk, tile_count);
}

void launch_unpermute_pos(bool mixed, const StepParams& p, const CellPack& cp, const float4* a,
                          const int* id, int n, float* out, cudaStream_t st) {
    if (n <= 0) return;
    LGB_DISPATCH(mixed, k_unpermute_pos, blocks_for(n, 256), 256, st, p, cp, a, id, n, out);
}

void launch_unpermute_pos_d(bool mixed, const StepParams& p, const CellPack& cp, const float4* a,
                            const int* id, int n, double* out, cudaStream_t st) {
    if (n <= 0) return;
    LGB_DISPATCH(mixed, k_unpermute_pos_d, blocks_for(n, 256), 256, st, p, cp, a, id, n, out);
}

void launch_to_scene_frame(const StepParams& p, const CellPack& cp, float4* a, int m, cudaStream_t st) {
    if (m <= 0) return;
    k_to_scene_frame<<<blocks_for(m, 256), 256, 0, st>>>(p, cp, a, m);
}

void launch_pack_pos(bool mixed, const StepParams& p, const CellPack& cp, const float* in, int n,
                     const int* scene_of, float4* out, cudaStream_t st) {
    if (n <= 0) return;
    LGB_DISPATCH(mixed, k_pack_pos, blocks_for(n, 256), 256, st, p, cp, in, n, scene_of, out);
}

void launch_pack_state(bool mixed, const StepParams& p, const CellPack& cp, const float* hx, const float* hv,
                       int n, float4* x, float4* v, int* id, cudaStream_t st) {
    if (n <= 0) return;
    LGB_DISPATCH(mixed, k_pack_state, blocks_for(n, HOST_BLOCK), HOST_BLOCK, st, p, cp, hx, hv, n, x, v, id);
}

void launch_pack_predict(bool mixed, const StepParams& p, const CellPack& cp, const float* hx, const float* hv,
                         int n, float4* x, int* id, float4* xs, int* key, int* rank, int* count, int* cellk,
                         int* tile_count, cudaStream_t st) {
    if (n <= 0) return;
    LGB_DISPATCH(mixed, k_pack_predict, blocks_for(n, HOST_BLOCK), HOST_BLOCK, st, p, cp, hx, hv, n, x, id, xs,
                 key, rank, count, cellk, tile_count);
}

void launch_unpack_state(bool mixed, const StepParams& p, const CellPack& cp, const float4* x, const float4* v,
                         const int* id, int* slot_of, bool slot_of_valid, int n, float* hx, float* hv,
                         cudaStream_t st) {
    if (n <= 0) return;
    if (!slot_of_valid) launch_k(k_slot_of, blocks_for(n, 256), 256, st, pdl_enabled(), id, n, slot_of);
    LGB_DISPATCH(mixed, k_unpack_state, blocks_for(n, HOST_BLOCK), HOST_BLOCK, st, p, cp, x, v, (const int*)slot_of,
                 n, hx, hv);
}

void launch_reduce(bool mixed, const StepParams& p, const CellPack& cp, const float4* x,
                   const float4* v, const float* rho, double* out, cudaStream_t st) {
    cudaMemsetAsync(out, 0, 9 * sizeof(double), st);
    if (p.n <= 0) return;
    int nb = min(blocks_for(p.n, 256), 152 * 4);
    LGB_DISPATCH(mixed, k_reduce, nb, 256, st, p, cp, x, v, rho, out);
}

}  // namespace lgb
