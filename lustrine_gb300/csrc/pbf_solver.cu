// pbf_solver.cu -- the PBF step (mode P): the position-based-fluids solver the
// reference's parameters describe (Simulation.hpp:157-171: rest density,
// relaxation epsilon, s_corr, XSPH) on the poly6 / spiky kernels of
// Kernels.cpp:43-67, with N Jacobi solver iterations over neighbour lists
// built once per step.
//
// Two position representations (template parameter MIXED):
//   plain  float4 xyz = absolute position;
//   mixed  float4 xyz = offset inside the particle's cell, in [0, cell),
//          w = the cell's integer coordinates packed in 32 bits (bit-cast).
//          Neighbour offsets are (o_i - o_j) + (c_i - c_j) * cell with
//          c_i - c_j in {-1, 0, 1}, so their precision does not depend on
//          how far the particles are from the origin; density sums use
//          compensated (Kahan) accumulation.
#include "pbf_common.cuh"
#include "pbf_kernels.h"

namespace lgb {

// ---------------------------------------------------------------- helpers --

__device__ __forceinline__ int3 unpack_cell(const CellPack& cp, float w) {
    unsigned u = __float_as_uint(w);
    return make_int3((int)(u & cp.mx), (int)((u >> cp.by_shift) & cp.my),
                     (int)((u >> cp.bz_shift) & cp.mz));
}

__device__ __forceinline__ float pack_cell(const CellPack& cp, int cx, int cy, int cz) {
    unsigned u = (unsigned)cx | ((unsigned)cy << cp.by_shift) | ((unsigned)cz << cp.bz_shift);
    return __uint_as_float(u);
}

// a - b as a float3
template <bool MIXED>
__device__ __forceinline__ float3 rel(const StepParams& p, const CellPack& cp, float4 a, float4 b) {
    if (!MIXED) return make_float3(a.x - b.x, a.y - b.y, a.z - b.z);
    int3 ca = unpack_cell(cp, a.w), cb = unpack_cell(cp, b.w);
    return make_float3((a.x - b.x) + (float)(ca.x - cb.x) * p.cell,
                       (a.y - b.y) + (float)(ca.y - cb.y) * p.cell,
                       (a.z - b.z) + (float)(ca.z - cb.z) * p.cell);
}

// cell coordinates of a position (clamped into the grid)
template <bool MIXED>
__device__ __forceinline__ int3 cell_of(const StepParams& p, const CellPack& cp, float4 a) {
    if (MIXED) return unpack_cell(cp, a.w);
    int cx = (int)floorf(a.x * p.inv_cell), cy = (int)floorf(a.y * p.inv_cell),
        cz = (int)floorf(a.z * p.inv_cell);
    return make_int3(min(max(cx, 0), p.gx - 1), min(max(cy, 0), p.gy - 1),
                     min(max(cz, 0), p.gz - 1));
}

__device__ __forceinline__ int linear_cell(const StepParams& p, int3 c) {
    return c.y * p.gx * p.gz + c.x * p.gz + c.z;
}

// One axis of an absolute position clamped to [lo, hi].
__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }

// Mixed: move an (offset, cell) pair by delta, renormalise the offset into
// [0, cell) and clamp the absolute position to [lo, hi].
__device__ __forceinline__ void mixed_axis(const StepParams& p, float& o, int& c, float lo, float hi) {
    float k = floorf(o * p.inv_cell);
    if (k != 0.0f) {
        c += (int)k;
        o -= k * p.cell;
        if (o >= p.cell) { o -= p.cell; c += 1; }
        if (o < 0.0f) { o += p.cell; c -= 1; }
    }
    float a = (float)c * p.cell + o;
    if (a < lo || a > hi) {
        float t = clampf(a, lo, hi);
        int tc = (int)floorf(t * p.inv_cell);
        c = tc;
        o = t - (float)tc * p.cell;
    }
}

template <bool MIXED>
__device__ __forceinline__ float4 advance(const StepParams& p, const CellPack& cp, float4 a, float dx,
                                          float dy, float dz) {
    if (!MIXED)
        return make_float4(clampf(a.x + dx, p.lox, p.hix), clampf(a.y + dy, p.loy, p.hiy),
                           clampf(a.z + dz, p.loz, p.hiz), 0.0f);
    int3 c = unpack_cell(cp, a.w);
    float ox = a.x + dx, oy = a.y + dy, oz = a.z + dz;
    mixed_axis(p, ox, c.x, p.lox, p.hix);
    mixed_axis(p, oy, c.y, p.loy, p.hiy);
    mixed_axis(p, oz, c.z, p.loz, p.hiz);
    return make_float4(ox, oy, oz, pack_cell(cp, c.x, c.y, c.z));
}

__device__ __forceinline__ float poly6(const StepParams& p, float r2) {
    float d = p.h2 - r2;
    return r2 <= p.h2 ? p.k6 * d * d * d : 0.0f;
}

// spiky gradient magnitude factor: dW(d) = f * d
__device__ __forceinline__ float spiky_factor(const StepParams& p, float r) {
    float f = p.h - r;
    return (r > 0.0f && r <= p.h) ? -p.ks * f * f / r : 0.0f;
}

__device__ __forceinline__ float scorr(const StepParams& p, float r2) {
    float t = poly6(p, r2) * p.inv_w_dq;
    float pw;
    if (p.sn_int == 4) {
        float t2 = t * t;
        pw = t2 * t2;
    } else if (p.sn_int >= 0) {
        pw = 1.0f;
        for (int e = 0; e < p.sn_int; e++) pw *= t;
    } else {
        pw = powf(t, p.sn);
    }
    return -p.sk * pw;
}

__device__ __forceinline__ float4 load_nbr(int j, const float4* __restrict__ xs,
                                           const float4* __restrict__ solid) {
    return j >= 0 ? xs[j] : solid[-1 - j];
}

// ---------------------------------------------------------------- kernels --

// Prediction, box clamp, cell key and histogram.
template <bool MIXED>
__global__ void k_predict(StepParams p, CellPack cp, const float4* __restrict__ x,
                          float4* __restrict__ v, float4* __restrict__ xs, int* __restrict__ key,
                          int* __restrict__ rank, int* __restrict__ count) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    float4 vi = v[i];
    vi.x += p.gxv * p.dt;
    vi.y += p.gyv * p.dt;
    vi.z += p.gzv * p.dt;
    v[i] = vi;
    float4 s = advance<MIXED>(p, cp, x[i], vi.x * p.dt, vi.y * p.dt, vi.z * p.dt);
    xs[i] = s;
    int k = linear_cell(p, cell_of<MIXED>(p, cp, s));
    key[i] = k;
    rank[i] = atomicAdd(&count[k], 1);
}

template <bool MIXED>
__global__ void k_key(StepParams p, CellPack cp, const float4* __restrict__ pos, int m,
                      int* __restrict__ key, int* __restrict__ rank, int* __restrict__ count) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    int k = linear_cell(p, cell_of<MIXED>(p, cp, pos[i]));
    key[i] = k;
    rank[i] = atomicAdd(&count[k], 1);
}

// Neighbour lists: the 3 x 3 rows of cells around the particle's cell; the
// three cells of a row are consecutive ids, hence one contiguous slot range.
template <bool MIXED>
__global__ void __launch_bounds__(128) k_lists(StepParams p, CellPack cp, const float4* __restrict__ xs,
                                               const int* __restrict__ fstart,
                                               const float4* __restrict__ solid,
                                               const int* __restrict__ sstart, int* __restrict__ nbr,
                                               int* __restrict__ cnt, int* status) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= p.n) return;
    const float4 self = xs[s];
    const int3 c = cell_of<MIXED>(p, cp, self);
    const int z0 = max(c.z - 1, 0), z1 = min(c.z + 1, p.gz - 1);
    int c_n = 0;
    for (int dy = -1; dy <= 1; dy++) {
        const int y = c.y + dy;
        if (y < 0 || y >= p.gy) continue;
        for (int dx = -1; dx <= 1; dx++) {
            const int x = c.x + dx;
            if (x < 0 || x >= p.gx) continue;
            const int row = y * p.gx * p.gz + x * p.gz;
            for (int t = fstart[row + z0], e = fstart[row + z1 + 1]; t < e; t++) {
                float3 d = rel<MIXED>(p, cp, self, xs[t]);
                if (dot3(d.x, d.y, d.z) <= p.h2) {
                    if (c_n < p.max_nbrs) nbr[(size_t)c_n * p.n + s] = t;
                    c_n++;
                }
            }
            if (p.ns > 0) {
                for (int t = sstart[row + z0], e = sstart[row + z1 + 1]; t < e; t++) {
                    float3 d = rel<MIXED>(p, cp, self, solid[t]);
                    if (dot3(d.x, d.y, d.z) <= p.h2) {
                        if (c_n < p.max_nbrs) nbr[(size_t)c_n * p.n + s] = -1 - t;
                        c_n++;
                    }
                }
            }
        }
    }
    if (c_n > p.max_nbrs) {
        set_status(status, ST_NBR_OVERFLOW);
        c_n = p.max_nbrs;
    }
    cnt[s] = c_n;
}

// Density constraint and its multiplier (Macklin & Mueller eq. 1, 8, 11).
template <bool MIXED>
__global__ void __launch_bounds__(128) k_lambda(StepParams p, CellPack cp, const float4* __restrict__ xs,
                                                const int* __restrict__ nbr, const int* __restrict__ cnt,
                                                const float4* __restrict__ solid,
                                                float* __restrict__ lam, float* __restrict__ rho) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= p.n) return;
    const float4 self = xs[s];
    const int c = cnt[s];
    const float mr = p.mass / p.rho0;
    float density = 0.0f, comp = 0.0f, S = 0.0f;
    float gx = 0.0f, gy = 0.0f, gz = 0.0f;
    for (int k = 0; k < c; k++) {
        const int j = nbr[(size_t)k * p.n + s];
        float3 d = rel<MIXED>(p, cp, self, load_nbr(j, xs, solid));
        float r2 = dot3(d.x, d.y, d.z);
        float w = p.mass * poly6(p, r2);
        if (MIXED) {
            float y = w - comp;
            float t = density + y;
            comp = (t - density) - y;
            density = t;
        } else {
            density += w;
        }
        if (j == s) continue;
        float f = spiky_factor(p, sqrtf(r2)) * mr;
        float ax = f * d.x, ay = f * d.y, az = f * d.z;
        if (j >= 0) S += dot3(ax, ay, az);
        gx += ax;
        gy += ay;
        gz += az;
    }
    S += dot3(gx, gy, gz);
    lam[s] = -(density / p.rho0 - 1.0f) / (S + p.eps);
    if (rho) rho[s] = density;
}

// Position correction with s_corr, solid push-out and box clamp (Jacobi).
// The last iteration also writes v = (x* - x) / dt.
template <bool MIXED>
__global__ void __launch_bounds__(128) k_delta(StepParams p, CellPack cp, const float4* __restrict__ xs,
                                               float4* __restrict__ xs_out, const int* __restrict__ nbr,
                                               const int* __restrict__ cnt,
                                               const float4* __restrict__ solid,
                                               const float* __restrict__ lam,
                                               const float4* __restrict__ x, float4* __restrict__ v_out) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= p.n) return;
    const float4 self = xs[s];
    const float li = lam[s];
    const int c = cnt[s];
    float px = 0.0f, py = 0.0f, pz = 0.0f;
    float cx = 0.0f, cy = 0.0f, cz = 0.0f;
    int nct = 0;
    for (int k = 0; k < c; k++) {
        const int j = nbr[(size_t)k * p.n + s];
        if (j == s) continue;
        float3 d = rel<MIXED>(p, cp, self, load_nbr(j, xs, solid));
        float r2 = dot3(d.x, d.y, d.z);
        float r = sqrtf(r2);
        float lj = j >= 0 ? lam[j] : li;
        float w = (li + lj + scorr(p, r2)) * spiky_factor(p, r);
        px += w * d.x;
        py += w * d.y;
        pz += w * d.z;
        if (j < 0 && r < p.contact && r > 0.0f) {
            float q = (p.contact - r) / r;
            cx += q * d.x;
            cy += q * d.y;
            cz += q * d.z;
            nct++;
        }
    }
    const float mr = p.mass / p.rho0;
    float dx = px * mr, dy = py * mr, dz = pz * mr;
    if (nct) {
        float inv = 1.0f / (float)nct;
        dx += cx * inv;
        dy += cy * inv;
        dz += cz * inv;
    }
    float4 out = advance<MIXED>(p, cp, self, dx, dy, dz);
    xs_out[s] = out;
    if (v_out) {
        float3 d = rel<MIXED>(p, cp, out, x[s]);
        float inv_dt = 1.0f / p.dt;
        v_out[s] = make_float4(d.x * inv_dt, d.y * inv_dt, d.z * inv_dt, 0.0f);
    }
}

// XSPH viscosity (Macklin & Mueller eq. 17) and commit x = x*.
template <bool MIXED>
__global__ void __launch_bounds__(128) k_xsph(StepParams p, CellPack cp, const float4* __restrict__ xs,
                                              const float4* __restrict__ v_in,
                                              const int* __restrict__ nbr, const int* __restrict__ cnt,
                                              float4* __restrict__ x_out, float4* __restrict__ v_out) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= p.n) return;
    const float4 self = xs[s];
    const float4 vi = v_in[s];
    const int c = cnt[s];
    float ax = 0.0f, ay = 0.0f, az = 0.0f;
    if (p.c_xsph != 0.0f) {
        for (int k = 0; k < c; k++) {
            const int j = nbr[(size_t)k * p.n + s];
            if (j == s || j < 0) continue;
            float3 d = rel<MIXED>(p, cp, self, xs[j]);
            float w = poly6(p, dot3(d.x, d.y, d.z));
            float4 vj = v_in[j];
            ax += (vj.x - vi.x) * w;
            ay += (vj.y - vi.y) * w;
            az += (vj.z - vi.z) * w;
        }
    }
    v_out[s] = make_float4(vi.x + p.c_xsph * ax, vi.y + p.c_xsph * ay, vi.z + p.c_xsph * az, 0.0f);
    x_out[s] = self;
}

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

// Caller positions (float3, id order) into the state representation, slot = id.
template <bool MIXED>
__global__ void k_pack_pos(StepParams p, CellPack cp, const float* __restrict__ in, int n,
                           float4* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float x = in[3 * (size_t)i], y = in[3 * (size_t)i + 1], z = in[3 * (size_t)i + 2];
    if (!MIXED) {
        out[i] = make_float4(x, y, z, 0.0f);
        return;
    }
    // The cell is clamped to the cells a clamped position can occupy (the
    // packed field widths); the offset keeps the exact position, so a caller
    // position outside the box stays where it is (it may then lie outside
    // [0, cell)) and the next prediction clamps it like the plain form does.
    int cx = min(max((int)floorf(x * p.inv_cell), 0), (int)floorf(p.hix * p.inv_cell));
    int cy = min(max((int)floorf(y * p.inv_cell), 0), (int)floorf(p.hiy * p.inv_cell));
    int cz = min(max((int)floorf(z * p.inv_cell), 0), (int)floorf(p.hiz * p.inv_cell));
    out[i] = make_float4(x - (float)cx * p.cell, y - (float)cy * p.cell, z - (float)cz * p.cell,
                         pack_cell(cp, cx, cy, cz));
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

static inline int blocks_for(int n, int t) { return (n + t - 1) / t; }

#define LGB_DISPATCH(MIXED_FLAG, KERNEL, GRID, BLOCK, ST, ...)                        \
    do {                                                                              \
        if (MIXED_FLAG)                                                               \
            KERNEL<true><<<GRID, BLOCK, 0, ST>>>(__VA_ARGS__);                        \
        else                                                                          \
            KERNEL<false><<<GRID, BLOCK, 0, ST>>>(__VA_ARGS__);                       \
    } while (0)

void launch_predict(bool mixed, const StepParams& p, const CellPack& cp, const float4* x, float4* v,
                    float4* xs, int* key, int* rank, int* count, cudaStream_t st) {
    if (p.n <= 0) return;
    LGB_DISPATCH(mixed, k_predict, blocks_for(p.n, 256), 256, st, p, cp, x, v, xs, key, rank, count);
}

void launch_key(bool mixed, const StepParams& p, const CellPack& cp, const float4* pos, int m,
                int* key, int* rank, int* count, cudaStream_t st) {
    if (m <= 0) return;
    LGB_DISPATCH(mixed, k_key, blocks_for(m, 256), 256, st, p, cp, pos, m, key, rank, count);
}

void launch_lists(bool mixed, const StepParams& p, const CellPack& cp, const float4* xs,
                  const int* fstart, const float4* solid, const int* sstart, int* nbr, int* cnt,
                  int* status, cudaStream_t st) {
    if (p.n <= 0) return;
    LGB_DISPATCH(mixed, k_lists, blocks_for(p.n, 128), 128, st, p, cp, xs, fstart, solid, sstart, nbr,
                 cnt, status);
}

void launch_lambda(bool mixed, const StepParams& p, const CellPack& cp, const float4* xs,
                   const int* nbr, const int* cnt, const float4* solid, float* lam, float* rho,
                   cudaStream_t st) {
    if (p.n <= 0) return;
    LGB_DISPATCH(mixed, k_lambda, blocks_for(p.n, 128), 128, st, p, cp, xs, nbr, cnt, solid, lam, rho);
}

void launch_delta(bool mixed, const StepParams& p, const CellPack& cp, const float4* xs,
                  float4* xs_out, const int* nbr, const int* cnt, const float4* solid,
                  const float* lam, const float4* x, float4* v_out, cudaStream_t st) {
    if (p.n <= 0) return;
    LGB_DISPATCH(mixed, k_delta, blocks_for(p.n, 128), 128, st, p, cp, xs, xs_out, nbr, cnt, solid, lam,
                 x, v_out);
}

void launch_xsph(bool mixed, const StepParams& p, const CellPack& cp, const float4* xs,
                 const float4* v_in, const int* nbr, const int* cnt, float4* x_out, float4* v_out,
                 cudaStream_t st) {
    if (p.n <= 0) return;
    LGB_DISPATCH(mixed, k_xsph, blocks_for(p.n, 128), 128, st, p, cp, xs, v_in, nbr, cnt, x_out, v_out);
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

void launch_pack_pos(bool mixed, const StepParams& p, const CellPack& cp, const float* in, int n,
                     float4* out, cudaStream_t st) {
    if (n <= 0) return;
    LGB_DISPATCH(mixed, k_pack_pos, blocks_for(n, 256), 256, st, p, cp, in, n, out);
}

void launch_reduce(bool mixed, const StepParams& p, const CellPack& cp, const float4* x,
                   const float4* v, const float* rho, double* out, cudaStream_t st) {
    cudaMemsetAsync(out, 0, 9 * sizeof(double), st);
    if (p.n <= 0) return;
    int nb = min(blocks_for(p.n, 256), 152 * 4);
    LGB_DISPATCH(mixed, k_reduce, nb, 256, st, p, cp, x, v, rho, out);
}

}  // namespace lgb
