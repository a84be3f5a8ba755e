// pbf_compat.cu -- the reference's fluid step (mode R) on the GPU.
//
// Semantics of Lustrine::simulate_fluid (Simulate.cpp:27-115) with its
// neighbour search (Neighbors.cpp:366-450) and cubic kernel (Kernels.cpp:6-41),
// float operation for float operation.  This translation unit is compiled with
// --fmad=false: the reference's arithmetic has no fused multiply-adds, and
// with the same operation order the neighbour sets, lambdas and positions
// are bit-identical to the reference's.  The one intended difference is the
// position update, which is Jacobi (every particle reads its neighbours'
// positions from before the pass) instead of the reference's in-place
// Gauss-Seidel sweep, which has no parallel form.
#include "pbf_common.cuh"
#include "pbf_compat.cuh"
#include "pbf_kernels.h"

namespace lgb {

// cubic_kernel (Kernels.cpp:6-19)
__device__ __forceinline__ float W_ref(const StepParams& p, float r) {
    float q = (r * p.kfac) / p.h;
    float result = 0.0f;
    if (q <= 1.0f) {
        if (q <= 0.5f) {
            float q2 = q * q;
            float q3 = q2 * q;
            float a = 6.0f * q3;
            float b = 6.0f * q2;
            result = p.cubic_k * ((a - b) + 1.0f);
        } else {
            result = p.cubic_k * (2.0f * ipow_rn(1.0f - q, 3));
        }
    }
    return result;
}

// cubic_kernel_grad (Kernels.cpp:26-41); len = glm::length(r), which the
// callers already hold (the same expression, so the same bits)
__device__ __forceinline__ float3 gradW_ref(const StepParams& p, float rx, float ry, float rz, float len) {
    float rl = len * p.kfac;
    float q = rl / p.h;
    float3 out = make_float3(0.0f, 0.0f, 0.0f);
    if ((double)rl > 1.0e-5 && q <= 1.0f) {
        float s = 1.0f / (rl * p.h);
        float gx = s * rx, gy = s * ry, gz = s * rz;
        float c;
        if (q <= 0.5f) {
            c = (p.cubic_l * q) * (3.0f * q - 2.0f);
        } else {
            float f = 1.0f - q;
            c = p.cubic_l * ((-f) * f);
        }
        out = make_float3(c * gx, c * gy, c * gz);
    }
    return out;
}

// s_coor (Simulate.cpp:7-9): -k * pow(W(r) / W(dq), n)
__device__ __forceinline__ float scorr_ref(const StepParams& p, float rl, float w_dq) {
    float ratio = W_ref(p, rl) / w_dq;
    float pw = p.sn_int >= 0 ? ipow_rn(ratio, p.sn_int) : powf(ratio, p.sn);
    return (-p.sk) * pw;
}

// resolve_collision (Simulate.cpp:13-24)
__device__ __forceinline__ float resolve_collision(float value, float lo, float hi) {
    const float eps = 0.01f;
    if (value <= lo) return eps;
    if (value > hi) return hi - eps;
    return value;
}

// Simulate.cpp:48-51 plus the cell key and histogram of the counting sort.
__global__ void k_predict_ref(StepParams p, const float4* __restrict__ x, float4* __restrict__ v,
                              float4* __restrict__ xs, int* __restrict__ key,
                              int* __restrict__ rank, int* __restrict__ count, int* status) {
    pdl_wait();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    float4 xi = x[i], vi = v[i];
    float gmx = p.gxv * p.mass, gmy = p.gyv * p.mass, gmz = p.gzv * p.mass;
    vi.x = vi.x + gmx * p.dt;
    vi.y = vi.y + gmy * p.dt;
    vi.z = vi.z + gmz * p.dt;
    float4 s = make_float4(xi.x + vi.x * p.dt, xi.y + vi.y * p.dt, xi.z + vi.z * p.dt, 0.0f);
    v[i] = vi;
    xs[i] = s;
    int k = cell_ref(p, s.x, s.y, s.z, status);
    key[i] = k;
    rank[i] = atomicAdd(&count[k], 1);
}

__global__ void k_key_ref(StepParams p, const float4* __restrict__ pos, int m, int* __restrict__ key,
                          int* __restrict__ rank, int* __restrict__ count, int* status) {
    pdl_wait();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    float4 s = pos[i];
    int k = cell_ref(p, s.x, s.y, s.z, status);
    key[i] = k;
    rank[i] = atomicAdd(&count[k], 1);
}

// Neighbours in the reference's list order: the 27 cells around the
// particle's cell in y -> x -> z offset order (Neighbors.cpp:401-403); in each
// cell its fluid particles by ascending id, then its solids by ascending
// storage index (Neighbors.cpp:374-384).
__global__ void k_lists_ref(StepParams p, const float4* __restrict__ xs, const int* __restrict__ key,
                            const int* __restrict__ fstart, const float4* __restrict__ solid,
                            const int* __restrict__ sstart, int* __restrict__ nbr,
                            int* __restrict__ cnt, int* status) {
    pdl_wait();
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= p.n) return;
    const float4 self = xs[s];
    const int id = key[s];
    const int slab = p.gx * p.gz;
    const int yy = id / slab, xx = (id % slab) / p.gz, zz = id % p.gz;
    int c_n = 0;
    // a row's cells z-1 .. z+1 are consecutive ids: their fluid and solid
    // ranges come from four loads of each table; the cells are still walked
    // one by one, fluid before solids, as the reference lists them
    const int z0 = max(zz - 1, 0), z1 = min(zz + 1, p.gz - 1);
    for (int y = -1; y <= 1; y++)
        for (int x = -1; x <= 1; x++) {
            if (xx + x < 0 || xx + x >= p.gx || yy + y < 0 || yy + y >= p.gy) continue;
            const int row = (yy + y) * slab + (xx + x) * p.gz;
            int fb[4], sb[4];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const bool in = z0 + k <= z1 + 1;
                fb[k] = in ? __ldg(&fstart[row + z0 + k]) : 0;
                sb[k] = in ? __ldg(&sstart[row + z0 + k]) : 0;
            }
#pragma unroll
            for (int k = 0; k < 3; k++) {
                if (z0 + k > z1) break;
                for (int t = fb[k]; t < fb[k + 1]; t++) {
                    float4 o = xs[t];
                    float dx = self.x - o.x, dy = self.y - o.y, dz = self.z - o.z;
                    if ((dx * dx + dy * dy) + dz * dz <= p.h2) {
                        if (c_n < p.max_nbrs) nbr[(size_t)c_n * p.n + s] = t;
                        c_n++;
                    }
                }
                for (int t = sb[k]; t < sb[k + 1]; t++) {
                    float4 o = __ldg(&solid[t]);
                    float dx = self.x - o.x, dy = self.y - o.y, dz = self.z - o.z;
                    if ((dx * dx + dy * dy) + dz * dz <= p.h2) {
                        if (c_n < p.max_nbrs) nbr[(size_t)c_n * p.n + s] = -1 - t;
                        c_n++;
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

__device__ __forceinline__ float4 nbr_pos(int j, const float4* __restrict__ xs,
                                          const float4* __restrict__ solid) {
    return j >= 0 ? xs[j] : solid[-1 - j];
}

// Simulate.cpp:58-88; lambdas are stored by the caller's particle id because
// the position pass indexes them by list position (Simulate.cpp:97).  The
// reference's two loops over the list (density, then gradients) run as one:
// each sum still takes its terms in list order, so the bits are the same,
// with one gather per neighbour instead of two.
__global__ void k_lambda_ref(StepParams p, const float4* __restrict__ xs, const int* __restrict__ id,
                             const int* __restrict__ nbr, const int* __restrict__ cnt,
                             const float4* __restrict__ solid, float* __restrict__ lam_by_id,
                             float* __restrict__ rho) {
    pdl_wait();
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= p.n) return;
    const float4 self = xs[s];
    const int c = cnt[s];
    float density = 0.0f;
    float gsum = 0.0f;
    float gcx = 0.0f, gcy = 0.0f, gcz = 0.0f;
    const float coef = -(p.mass / p.rho0);
    int e_next = c > 0 ? __ldg(&nbr[s]) : 0;
    for (int k = 0; k < c; k++) {
        const int e = e_next;
        if (k + 1 < c) e_next = __ldg(&nbr[(size_t)(k + 1) * p.n + s]);  // next entry while this one is used
        float4 o = nbr_pos(e, xs, solid);
        float ix = self.x - o.x, iy = self.y - o.y, iz = self.z - o.z;
        float len = sqrtf((ix * ix + iy * iy) + iz * iz);
        density += p.mass * W_ref(p, len);
        float3 g = gradW_ref(p, ix, iy, iz, len);
        float nx = coef * g.x, ny = coef * g.y, nz = coef * g.z;
        gsum += (nx * nx + ny * ny) + nz * nz;
        gcx -= nx;
        gcy -= ny;
        gcz -= nz;
    }
    density += p.mass * W_ref(p, 0.0f);
    float constraint = (float)((double)(density / p.rho0) - 1.0);
    gsum += (gcx * gcx + gcy * gcy) + gcz * gcz;
    float lam = 0.0f;
    if (gsum > 0.0f) lam = (-constraint) / (gsum + p.eps);
    lam_by_id[id[s]] = lam;
    if (rho) rho[s] = density;
}

// Simulate.cpp:90-113 with a Jacobi read of the neighbours' positions.
__global__ void k_delta_ref(StepParams p, const float4* __restrict__ xs, float4* __restrict__ xs_out,
                            float4* __restrict__ x, float4* __restrict__ v,
                            const int* __restrict__ id, const int* __restrict__ nbr,
                            const int* __restrict__ cnt, const float4* __restrict__ solid,
                            const float* __restrict__ lam_by_id) {
    pdl_wait();
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= p.n) return;
    const float4 self = xs[s];
    const float li = lam_by_id[id[s]];
    const float w_dq = W_ref(p, p.dq);
    const int c = cnt[s];
    float px = 0.0f, py = 0.0f, pz = 0.0f;
    int e_next = c > 0 ? __ldg(&nbr[s]) : 0;
    for (int k = 0; k < c; k++) {
        const int e = e_next;
        if (k + 1 < c) e_next = __ldg(&nbr[(size_t)(k + 1) * p.n + s]);
        float4 o = nbr_pos(e, xs, solid);
        float ix = self.x - o.x, iy = self.y - o.y, iz = self.z - o.z;
        float len = sqrtf((ix * ix + iy * iy) + iz * iz);
        float sc = scorr_ref(p, len, w_dq);
        float3 g = gradW_ref(p, ix, iy, iz, len);
        float w = (li + lam_by_id[k]) + sc;
        px += w * g.x;
        py += w * g.y;
        pz += w * g.z;
    }
    px = px / p.rho0;
    py = py / p.rho0;
    pz = pz / p.rho0;
    float nx = self.x + px, ny = self.y + py, nz = self.z + pz;
    nx = resolve_collision(nx, p.lox, p.hix);
    ny = resolve_collision(ny, p.loy, p.hiy);
    nz = resolve_collision(nz, p.loz, p.hiz);
    const float4 xo = x[s];
    v[s] = make_float4((nx - xo.x) / p.dt, (ny - xo.y) / p.dt, (nz - xo.z) / p.dt, 0.0f);
    const float4 xn = make_float4(nx, ny, nz, 0.0f);
    x[s] = xn;
    xs_out[s] = xn;
}

// ------------------------------------------------------------------ launch --

static inline int blocks_for(int n, int t) { return (n + t - 1) / t; }

void launch_predict_ref(const StepParams& p, const float4* x, float4* v, float4* xs, int* key,
                        int* rank, int* count, int* status, cudaStream_t st) {
    if (p.n <= 0) return;
    launch_k(k_predict_ref, blocks_for(p.n, 256), 256, st, pdl_enabled(), p, x, v, xs, key, rank, count, status);
}

void launch_key_ref(const StepParams& p, const float4* pos, int m, int* key, int* rank, int* count,
                    int* status, cudaStream_t st) {
    if (m <= 0) return;
    launch_k(k_key_ref, blocks_for(m, 256), 256, st, pdl_enabled(), p, pos, m, key, rank, count, status);
}

void launch_lists_ref(const StepParams& p, const float4* xs, const int* key, const int* fstart,
                      const float4* solid, const int* sstart, int* nbr, int* cnt, int* status,
                      cudaStream_t st) {
    if (p.n <= 0) return;
    launch_k(k_lists_ref, blocks_for(p.n, 128), 128, st, pdl_enabled(), p, xs, key, fstart, solid, sstart, nbr,
             cnt, status);
}

void launch_lambda_ref(const StepParams& p, const float4* xs, const int* id, const int* nbr,
                       const int* cnt, const float4* solid, float* lam_by_id, float* rho,
                       cudaStream_t st) {
    if (p.n <= 0) return;
    launch_k(k_lambda_ref, blocks_for(p.n, 128), 128, st, pdl_enabled(), p, xs, id, nbr, cnt, solid, lam_by_id,
             rho);
}

void launch_delta_ref(const StepParams& p, const float4* xs, float4* xs_out, float4* x, float4* v,
                      const int* id, const int* nbr, const int* cnt, const float4* solid,
                      const float* lam_by_id, cudaStream_t st) {
    if (p.n <= 0) return;
    launch_k(k_delta_ref, blocks_for(p.n, 128), 128, st, pdl_enabled(), p, xs, xs_out, x, v, id, nbr, cnt, solid,
             lam_by_id);
}

}  // namespace lgb
