// sand.cu -- the reference's sand step (LUSTRINE_MODE_SAND) on the GPU.
//
// Semantics of Lustrine::simulate_sand (Simulate.cpp:156-325) with its
// neighbour search find_neighbors_uniform_grid_v1 (Neighbors.cpp:262-361),
// float operation for float operation.  This translation unit is compiled
// with --fmad=false and evaluates every expression in the reference's order
// (glm 0.9.9.8: dot = (x*x + y*y) + z*z, length = sqrt(dot),
// normalize = v * (1 / sqrt(dot(v, v))), clamp = min(max(v, lo), hi)), so
// positions, velocities, attract flags and list order equal the reference's
// bit for bit.  The reference's contact/friction substeps already read a
// snapshot of the positions (positions_tmp), so the GPU's Jacobi passes are
// its exact parallel form.
//
// Step: k_sand_predict (integration, attract and blow, box clamp, cell key,
// histogram) -> cell scan -> stable scatter/gather of x, x*, attract flags
// into cell order -> k_sand_lists (symmetric lists in the reference's push
// order) -> 4 x k_sand_substep; the last substep commits x, v and the flags
// back into the side the step started from.
#include "pbf_common.cuh"
#include "pbf_compat.cuh"
#include "pbf_kernels.h"

namespace lgb {

// simulate_sand's constants (Simulate.cpp:159-163)
constexpr float SAND_COLLISION = 0.8f;
constexpr float SAND_FRICTION = 0.7f;
constexpr float SAND_MU_S = 0.95f;
constexpr float SAND_MU_K = 0.9f;

__device__ __forceinline__ float sdot(float x, float y, float z) { return (x * x + y * y) + z * z; }
__device__ __forceinline__ float slen(float x, float y, float z) { return sqrtf(sdot(x, y, z)); }
__device__ __forceinline__ float sdot2(float ax, float ay, float az, float bx, float by, float bz) {
    return (ax * bx + ay * by) + az * bz;
}
// glm::max / glm::min on floats
__device__ __forceinline__ float smax(float a, float b) { return a < b ? b : a; }
__device__ __forceinline__ float smin(float a, float b) { return b < a ? b : a; }

// glm::clamp(v, vec3(r), vec3(X, Y, Z) - vec3(r)) (Simulate.cpp:208, 298)
__device__ __forceinline__ float4 sand_clamp(const StepParams& p, float x, float y, float z) {
    return make_float4(smin(smax(x, p.lox), p.hix), smin(smax(y, p.loy), p.hiy),
                       smin(smax(z, p.loz), p.hiz), 0.0f);
}

// Integration (Simulate.cpp:183-209) plus the cell key and histogram of the
// counting sort (Neighbors.cpp:275-278).
__global__ void k_sand_predict(StepParams p, SandParams q, const float4* __restrict__ x,
                               float4* __restrict__ v, float4* __restrict__ xs, int* __restrict__ att,
                               int* __restrict__ key, int* __restrict__ rank, int* __restrict__ count,
                               int* status) {
    pdl_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const float4 xi = x[i];
    float4 vi = v[i];
    vi.x = vi.x + p.gxv * p.dt;
    vi.y = vi.y + p.gyv * p.dt;
    vi.z = vi.z + p.gzv * p.dt;
    int a = att[i];
    if (q.prev_attract && !q.attract) a = 0;
    if (q.attract) {
        if (slen(q.px - xi.x, q.py - xi.y, q.pz - xi.z) < q.attract_radius) a = 1;
        if (a) {
            // towards 1.5 above the player's position
            const float ox = (q.px + 0.0f) - xi.x, oy = (q.py + 1.5f) - xi.y, oz = (q.pz + 0.0f) - xi.z;
            const float s = 1.0f / sqrtf(sdot(ox, oy, oz));
            vi.x = vi.x + ((((ox * s) * 1.0f) * q.attract_coeff) * q.radius * p.dt) * q.w;
            vi.y = vi.y + ((((oy * s) * 1.0f) * q.attract_coeff) * q.radius * p.dt) * q.w;
            vi.z = vi.z + ((((oz * s) * 1.0f) * q.attract_coeff) * q.radius * p.dt) * q.w;
        }
    }
    if (q.blow) {
        const float dx = q.px - xi.x, dy = q.py - xi.y, dz = q.pz - xi.z;
        const float ld = slen(dx, dy, dz);
        if (ld < q.blow_radius) {
            const float s = 1.0f / sqrtf(sdot(dx, dy, dz));
            // blow_kernel (Simulate.cpp:143-154)
            const float bk = ld > q.blow_radius ? 0.0f : 1.0f - ld / q.blow_radius;
            vi.x = vi.x + (((-(dx * s) * bk) * q.blow_coeff) * q.radius) * q.w;
            vi.y = vi.y + (((-(dy * s) * bk) * q.blow_coeff) * q.radius) * q.w;
            vi.z = vi.z + (((-(dz * s) * bk) * q.blow_coeff) * q.radius) * q.w;
        }
    }
    const float4 s = sand_clamp(p, xi.x + vi.x * p.dt, xi.y + vi.y * p.dt, xi.z + vi.z * p.dt);
    v[i] = vi;
    xs[i] = s;
    att[i] = a;
    const int k = cell_ref(p, s.x, s.y, s.z, status);
    key[i] = k;
    rank[i] = atomicAdd(&count[k], 1);
}

// The reference's lists in its push order (Neighbors.cpp:306-358), built per
// particle without the symmetric pushes: particle i's list is first the sand
// particles k < i whose own walk found i, in ascending k -- the 27-cell walk
// in y -> x -> z order visits cells by ascending id and the sorted slots of a
// cell ascend, so that is the walk itself restricted to slots below i, with
// the distance taken from k's side -- then its own walk over j >= i, each
// cell's static particles before its sand.  The reference also lists i
// itself twice; the substeps skip it (Simulate.cpp:226), so it is left out.
// Entries: sand slot t >= 0, static slot u as -1 - u.
__global__ void k_sand_lists(StepParams p, const float4* __restrict__ xs, const int* __restrict__ key,
                             const int* __restrict__ fstart, const float4* __restrict__ solid,
                             const int* __restrict__ sstart, int* __restrict__ nbr, int* __restrict__ cnt,
                             int* status) {
    pdl_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const float4 self = xs[i];
    const int id = key[i];
    const int slab = p.gx * p.gz;
    const int yy = id / slab;
    const int t0 = id - yy * slab;
    const int zz = t0 % p.gz, xx = t0 / p.gz;
    const int ylo = yy - 1 < 0 ? 0 : -1, yhi = yy + 1 >= p.gy ? 0 : 1;
    const int xlo = xx - 1 < 0 ? 0 : -1, xhi = xx + 1 >= p.gx ? 0 : 1;
    const int zlo = zz - 1 < 0 ? 0 : -1, zhi = zz + 1 >= p.gz ? 0 : 1;
    int c_n = 0;
    // sand below i that found i: cells up to its own (later cells hold later slots)
    for (int y = ylo; y <= 0; y++)
        for (int x = (y < 0 ? xlo : max(xlo, -1)); x <= (y < 0 ? xhi : 0); x++)
            for (int z = zlo; z <= ((y < 0 || x < 0) ? zhi : 0); z++) {
                const int c = (yy + y) * slab + (xx + x) * p.gz + (zz + z);
                const int e = min(fstart[c + 1], i);
                for (int t = fstart[c]; t < e; t++) {
                    const float4 o = xs[t];
                    if (sdot(o.x - self.x, o.y - self.y, o.z - self.z) <= p.h2) {
                        if (c_n < p.max_nbrs) nbr[(size_t)c_n * p.n + i] = t;
                        c_n++;
                    }
                }
            }
    // its own walk: static particles, then sand above i (cells from its own on)
    for (int y = ylo; y <= yhi; y++)
        for (int x = xlo; x <= xhi; x++)
            for (int z = zlo; z <= zhi; z++) {
                const int c = (yy + y) * slab + (xx + x) * p.gz + (zz + z);
                for (int u = sstart[c], e = sstart[c + 1]; u < e; u++) {
                    const float4 o = solid[u];
                    if (sdot(self.x - o.x, self.y - o.y, self.z - o.z) <= p.h2) {
                        if (c_n < p.max_nbrs) nbr[(size_t)c_n * p.n + i] = -1 - u;
                        c_n++;
                    }
                }
                if (c < id) continue;
                for (int t = max(fstart[c], i + 1), e = fstart[c + 1]; t < e; t++) {
                    const float4 o = xs[t];
                    if (sdot(self.x - o.x, self.y - o.y, self.z - o.z) <= p.h2) {
                        if (c_n < p.max_nbrs) nbr[(size_t)c_n * p.n + i] = t;
                        c_n++;
                    }
                }
            }
    if (c_n > p.max_nbrs) {
        set_status(status, ST_NBR_OVERFLOW);
        c_n = p.max_nbrs;
    }
    cnt[i] = c_n;
}

// One contact and friction term (Simulate.cpp:236-266 for a sand neighbour,
// 268-286 for a static one), subtracted from dp.
template <bool SAND_J>
__device__ __forceinline__ void sand_pair(const StepParams& p, const SandParams& q, float4 pi, float4 pj,
                                          float4 xi, float4 xj, float& dpx, float& dpy, float& dpz) {
    float ix = pi.x - pj.x, iy = pi.y - pj.y, iz = pi.z - pj.z;
    if (slen(ix, iy, iz) == 0.0f) {
        ix = 0.0f;
        iy = 0.00001f;
        iz = 0.0f;
    }
    const float len = slen(ix, iy, iz);
    if (len > q.diameter) return;
    const float s = SAND_J ? ((SAND_COLLISION * p.mass) / (p.mass + p.mass)) * (len - q.diameter)
                           : SAND_COLLISION * (len - q.diameter);
    const float tx = (s * ix) / len, ty = (s * iy) / len, tz = (s * iz) / len;
    dpx = dpx - tx;
    dpy = dpy - ty;
    dpz = dpz - tz;
    const float d = slen(tx, ty, tz);
    const float ax = pi.x - tx, ay = pi.y - ty, az = pi.z - tz;  // pi - tmp
    float rx, ry, rz, nx, ny, nz;
    if (SAND_J) {
        const float bx = pj.x + tx, by = pj.y + ty, bz = pj.z + tz;  // pj + tmp
        rx = (ax - xi.x) - (bx - xj.x);
        ry = (ay - xi.y) - (by - xj.y);
        rz = (az - xi.z) - (bz - xj.z);
        nx = ax - bx;
        ny = ay - by;
        nz = az - bz;
    } else {
        rx = (ax - xi.x) - 0.0f;
        ry = (ay - xi.y) - 0.0f;
        rz = (az - xi.z) - 0.0f;
        nx = ax - pj.x;
        ny = ay - pj.y;
        nz = az - pj.z;
    }
    const float inv = 1.0f / sqrtf(sdot(nx, ny, nz));
    nx = nx * inv;
    ny = ny * inv;
    nz = nz * inv;
    const float dr = sdot2(rx, ry, rz, nx, ny, nz);
    const float ux = rx - dr * nx, uy = ry - dr * ny, uz = rz - dr * nz;  // tangential part
    const float lt = slen(ux, uy, uz);
    if ((d * SAND_MU_S) > lt + 1e-9f) {
        dpx = dpx - SAND_FRICTION * ux;
        dpy = dpy - SAND_FRICTION * uy;
        dpz = dpz - SAND_FRICTION * uz;
    } else {
        const float r = (SAND_MU_K * d) / (lt + 1e-9f);
        const float ratio = r < 1 ? r : 1;
        dpx = dpx - (SAND_FRICTION * ux) * ratio;
        dpy = dpy - (SAND_FRICTION * uy) * ratio;
        dpz = dpz - (SAND_FRICTION * uz) * ratio;
    }
}

// One contact/friction substep (Simulate.cpp:221-303): every particle reads
// positions_tmp (tmp_in) and the pre-step positions (xpre), writes its new
// clamped position.  The last substep commits instead: x = x*,
// v = (x* - x) / dt (Simulate.cpp:309-313), the attract flags and the
// particle's index -- its slot in this step's cell order, as the reference
// re-orders its arrays -- into the side the step started from (whose
// contents the sort already consumed).
__global__ void k_sand_substep(StepParams p, SandParams q, const float4* __restrict__ tmp_in,
                               float4* __restrict__ star_out, const float4* __restrict__ xpre,
                               const int* __restrict__ nbr, const int* __restrict__ cnt,
                               const float4* __restrict__ solid, float4* __restrict__ x_commit,
                               float4* __restrict__ v_commit, const int* __restrict__ att_in,
                               int* __restrict__ att_commit, int* __restrict__ id_commit) {
    pdl_wait();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const float4 pi = tmp_in[i];
    const float4 xi = xpre[i];
    float dpx = 0.0f, dpy = 0.0f, dpz = 0.0f;
    const int c = cnt[i];
    for (int k = 0; k < c; k++) {
        const int e = nbr[(size_t)k * p.n + i];
        if (e >= 0)
            sand_pair<true>(p, q, pi, tmp_in[e], xi, xpre[e], dpx, dpy, dpz);
        else
            sand_pair<false>(p, q, pi, __ldg(&solid[-1 - e]), xi, xi, dpx, dpy, dpz);
    }
    const float4 s = sand_clamp(p, pi.x + dpx, pi.y + dpy, pi.z + dpz);
    if (!x_commit) {
        star_out[i] = s;
        return;
    }
    x_commit[i] = s;
    v_commit[i] = make_float4((s.x - xi.x) / p.dt, (s.y - xi.y) / p.dt, (s.z - xi.z) / p.dt, 0.0f);
    att_commit[i] = att_in[i];
    id_commit[i] = i;
}

// ------------------------------------------------------------------ launch --

static inline int blocks_for(int n, int t) { return (n + t - 1) / t; }

void launch_sand_predict(const StepParams& p, const SandParams& q, const float4* x, float4* v, float4* xs,
                         int* att, int* key, int* rank, int* count, int* status, cudaStream_t st) {
    if (p.n <= 0) return;
    launch_k(k_sand_predict, blocks_for(p.n, 256), 256, st, pdl_enabled(), p, q, x, v, xs, att, key, rank,
             count, status);
}

void launch_sand_lists(const StepParams& p, const float4* xs, const int* key, const int* fstart,
                       const float4* solid, const int* sstart, int* nbr, int* cnt, int* status,
                       cudaStream_t st) {
    if (p.n <= 0) return;
    launch_k(k_sand_lists, blocks_for(p.n, 128), 128, st, pdl_enabled(), p, xs, key, fstart, solid, sstart,
             nbr, cnt, status);
}

void launch_sand_substep(const StepParams& p, const SandParams& q, const float4* tmp_in, float4* star_out,
                         const float4* xpre, const int* nbr, const int* cnt, const float4* solid,
                         float4* x_commit, float4* v_commit, const int* att_in, int* att_commit,
                         int* id_commit, cudaStream_t st) {
    if (p.n <= 0) return;
    launch_k(k_sand_substep, blocks_for(p.n, 128), 128, st, pdl_enabled(), p, q, tmp_in, star_out, xpre, nbr,
             cnt, solid, x_commit, v_commit, att_in, att_commit, id_commit);
}

}  // namespace lgb
