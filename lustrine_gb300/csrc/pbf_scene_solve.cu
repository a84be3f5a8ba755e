// pbf_scene_solve.cu -- the on-chip solve of a batch of scenes: one persistent
// launch of thread-block clusters takes bins of scenes from a work queue and
// runs every scene's neighbour lists, first lambda pass, solver iterations,
// XSPH and commit (with the next step's prediction) out of distributed shared
// memory, with a cluster barrier between passes.
//
// Why: the per-stage kernels of the PBF step stream every particle's
// position, list entries and count from DRAM on each of their nine passes.  A
// scene of up to 65,536 particles fits the shared memory of one cluster of 16
// CTAs (4,096 particles per CTA: x* with lambda in w, velocities, up to
// SOLVE_CAP list entries as 16-bit scene-local indices, counts -- 212 KB), so
// once the batch's counting sort has put every scene in cell order, the rest
// of its step touches global memory only to read its sorted state and cell
// table once and to write its lists and committed state once.  A neighbour
// held by another CTA of the scene is read through the cluster's shared
// memory window (mapa + ld.shared::cluster), one held by this CTA with a
// plain shared-memory load.
//
// Work queue: the host packs the scenes into bins of at most 16 CTAs
// (ceil(n / 4096) CTAs per scene, first fit by decreasing size); each cluster
// pops bins with one atomic and runs every scene of the bin side by side (a
// CTA without a scene takes part in the barriers only).  No CTA ever waits on
// another cluster (the only waits are the cluster's own barriers), so the
// persistent grid is sized by the occupancy query and needs no co-residency
// beyond the cluster's own; the last cluster to finish zeroes the queue for
// the next step.
//
// Arithmetic: the pair terms, the lambda and density formulas, the position
// correction, XSPH and the prediction are the device functions of the
// per-stage kernels (pbf_device.cuh) in the same order, so in fp32 a scene's
// result is bitwise that of the per-stage path.  In mixed precision the
// iterations run on positions relative to the scene's own box corner
// (cell * cell_size + offset, fp32; this path takes boxes of at most
// SOLVE_MIXED_MAX_CELLS cells a side), and the committed state goes back to
// cell + offset; density sums are compensated (Kahan) as in the per-stage
// kernels.
#include <cooperative_groups.h>

#include "pbf_common.cuh"
#include "pbf_device.cuh"
#include "pbf_kernels.h"

namespace cg = cooperative_groups;

namespace lgb {

static_assert((1 << SOLVE_M_SHIFT) == SOLVE_M, "SOLVE_M is a power of two");

// Shared memory of one CTA.
struct SolveSmem {
    float4 pos[SOLVE_M];                      // x* (scene frame), w: lambda
    float4 vel[SOLVE_M];                      // staging of x* during a pass; velocities at the end
    unsigned short ent[SOLVE_CAP * SOLVE_M];  // entry k of particle l at k * SOLVE_M + l
    unsigned char cnt[SOLVE_M];               // neighbour count (entries beyond SOLVE_CAP: global lists)
    int bin;                                  // the bin the cluster works on (rank 0 holds it)
};

__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// Address of the same shared-memory location in CTA `rank` of the cluster.
__device__ __forceinline__ unsigned map_rank(unsigned addr, unsigned rank) {
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}

__device__ __forceinline__ float4 ld_cluster_f4(unsigned addr) {
    float4 v;
    asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "r"(addr));
    return v;
}

__device__ __forceinline__ int ld_cluster_s32(unsigned addr) {
    int v;
    asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(addr));
    return v;
}

// The scene a CTA works on within its bin.
struct SceneView {
    int scene;     // -1: none
    int srank;     // rank of this CTA among the scene's CTAs
    int base;      // cluster rank of the scene's first CTA
    int slot0, n;  // first slot and particle count of the scene
    Geo g;
};

// Element j (scene-local index) of a per-CTA float4 array: a shared-memory
// load when this CTA holds it, else a load through the cluster window.
__device__ __forceinline__ float4 gather4(const SceneView& sv, const float4* local, unsigned local_base, int j,
                                          int crank) {
    const int owner = sv.base + (j >> SOLVE_M_SHIFT);
    const int off = j & (SOLVE_M - 1);
    if (owner == crank) return local[off];
    return ld_cluster_f4(map_rank(local_base + (unsigned)(off * 16), (unsigned)owner));
}

// Position of a particle in the scene frame from its stored form.
template <bool MIXED>
__device__ __forceinline__ float3 scene_frame(const StepParams& p, float4 q, int3 c) {
    if (!MIXED) return make_float3(q.x, q.y, q.z);
    return make_float3(__fmaf_rn((float)c.x, p.cell, q.x), __fmaf_rn((float)c.y, p.cell, q.y),
                       __fmaf_rn((float)c.z, p.cell, q.z));
}

// Cell of the particle in sorted slot s (the step's key).
template <bool MIXED>
__device__ __forceinline__ int3 solve_cell(const StepParams& p, const CellPack& cp, const Geo& g,
                                           const int* __restrict__ key_sorted, float4 self_stored, int s) {
    if (MIXED) return slot_cell(p, cp, g, key_sorted, p.cell_sorted, s);
    return plain_cell(p, g, self_stored.x, self_stored.y, self_stored.z);
}

// Walks the list of CTA-local particle l_cta (global slot s, c entries): up
// to U gathers in flight, f(j, q) per entry in list order (j scene-local
// index, q its element of the float4 array at `local` / `base_addr`).
template <int U, class F>
__device__ __forceinline__ void for_each_nbr(const StepParams& p, const SolveSmem& sm, const SceneView& sv,
                                             const int* nbr, int l_cta, int s, int c, const float4* local,
                                             unsigned base_addr, int crank, F&& f) {
    for (int k = 0; k < c; k += U) {
        int j[U];
        float4 q[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int kk = k + u;
            if (kk < c) {
                j[u] = kk < SOLVE_CAP ? (int)sm.ent[kk * SOLVE_M + l_cta] : nbr[(size_t)kk * p.n + s] - sv.slot0;
            } else {
                j[u] = -1;
            }
        }
#pragma unroll
        for (int u = 0; u < U; u++)
            if (j[u] >= 0) q[u] = gather4(sv, local, base_addr, j[u], crank);
#pragma unroll
        for (int u = 0; u < U; u++)
            if (j[u] >= 0) f(j[u], q[u]);
    }
}

template <bool MIXED, int T>
__global__ void __launch_bounds__(T, 1) k_scene_solve(StepParams p, CellPack cp, SolveArgs a) {
    pdl_wait();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SolveSmem& sm = *reinterpret_cast<SolveSmem*>(smem_raw);
    cg::cluster_group cluster = cg::this_cluster();
    const int crank = (int)cluster.block_rank();
    const int tid = threadIdx.x;
    const unsigned pos_base = smem_u32(sm.pos);
    const unsigned vel_base = smem_u32(sm.vel);
    const int iters = a.iters;
    for (;;) {
        if (crank == 0 && tid == 0) sm.bin = atomicAdd(a.queue, 1);
        cluster.sync();
        const int bin = ld_cluster_s32(map_rank(smem_u32(&sm.bin), 0));
        cluster.sync();  // every CTA has read the bin before rank 0 pops the next
        if (bin >= a.num_bins) break;  // bins past the end: every cluster ends on one
        SceneView sv;
        const SolveSlot me = a.bins[(size_t)bin * SOLVE_CLUSTER + crank];
        sv.scene = me.scene;
        sv.srank = me.rank;
        sv.base = crank - me.rank;
        sv.slot0 = sv.scene >= 0 ? a.scene_slot0[sv.scene] : 0;
        sv.n = sv.scene >= 0 ? a.scene_slot0[sv.scene + 1] - sv.slot0 : 0;
        if (sv.scene >= 0) sv.g = geo_scene(p, sv.scene);
        const int l0 = sv.srank * SOLVE_M;  // first scene-local index of this CTA
        const int mine = sv.scene >= 0 ? min(SOLVE_M, sv.n - l0) : 0;

        // load: sorted x* into the scene frame
        for (int lc = tid; lc < mine; lc += T) {
            const int s = sv.slot0 + l0 + lc;
            const float4 q = a.xs[s];
            const int3 c = solve_cell<MIXED>(p, cp, sv.g, a.key_sorted, q, s);
            // (a scene-frame context's prediction wrote the frame already)
            const float3 f = p.frame ? make_float3(q.x, q.y, q.z) : scene_frame<MIXED>(p, q, c);
            sm.pos[lc] = make_float4(f.x, f.y, f.z, 0.0f);
        }
        cluster.sync();

        // neighbour lists (the per-stage list build's walk and entry order)
        // fused with the first lambda pass
        for (int lc = tid; lc < mine; lc += T) {
            const int s = sv.slot0 + l0 + lc;
            const float4 self = sm.pos[lc];
            const Geo& g = sv.g;
            const int3 c = solve_cell<MIXED>(p, cp, g, a.key_sorted, a.xs[s], s);
            LambdaAcc acc = lambda_init(p);
            int c_n = 0;
            const int slab = g.gx * g.gz;
            const int z0 = max(c.z - 1, 0), z1 = min(c.z + 1, g.gz - 1);
            for (int dy = -1; dy <= 1; dy++) {
                const int y = c.y + dy;
                if (y < 0 || y >= g.gy) continue;
                // the slot ranges of the three rows (dx = -1, 0, 1) of this layer
                int rb[3], re[3];
#pragma unroll
                for (int r = 0; r < 3; r++) {
                    const int xx = c.x + r - 1;
                    rb[r] = re[r] = 0;
                    if (xx >= 0 && xx < g.gx) {
                        const int row = g.off + y * slab + xx * g.gz;
                        rb[r] = __ldg(&a.start[row + z0]);
                        re[r] = __ldg(&a.start[row + z1 + 1]);
                    }
                }
#pragma unroll
                for (int r = 0; r < 3; r++) {
                    // candidates in slot order, gathered 4 at a time
                    for (int t0 = rb[r]; t0 < re[r]; t0 += 4) {
                        float4 q[4];
#pragma unroll
                        for (int u = 0; u < 4; u++)
                            if (t0 + u < re[r]) q[u] = gather4(sv, sm.pos, pos_base, t0 + u - sv.slot0, crank);
#pragma unroll
                        for (int u = 0; u < 4; u++) {
                            const int t = t0 + u;
                            if (t >= re[r] || t == s) continue;
                            const float3 d = make_float3(__fsub_rn(self.x, q[u].x), __fsub_rn(self.y, q[u].y),
                                                         __fsub_rn(self.z, q[u].z));
                            if (dot3e(d.x, d.y, d.z) <= p.h2) {
                                if (c_n < p.max_nbrs) {
                                    a.nbr[(size_t)c_n * p.n + s] = t;  // slot only (no cell code: unused here)
                                    if (c_n < SOLVE_CAP) sm.ent[c_n * SOLVE_M + lc] = (unsigned short)(t - sv.slot0);
                                }
                                c_n++;
                                lambda_accumulate<MIXED>(p, acc, d, false);
                            }
                        }
                    }
                }
            }
            if (c_n > p.max_nbrs) {
                set_status(a.status, ST_NBR_OVERFLOW);
                c_n = p.max_nbrs;
            }
            a.cnt[s] = c_n;
            sm.cnt[lc] = (unsigned char)c_n;
            const float lam = lambda_of(p, acc);
            sm.pos[lc].w = lam;  // the neighbours read xyz only in this pass
            if (iters == 1) {
                if (a.rho) a.rho[s] = density_of(p, acc);
                a.lam_out[s] = make_float4(self.x, self.y, self.z, lam);
            }
        }
        cluster.sync();

        for (int it = 0; it < iters; it++) {
            const bool last = it == iters - 1;
            // position correction (Jacobi): new x* staged in vel, copied after
            // every CTA of the scene has read the old ones
            for (int lc = tid; lc < mine; lc += T) {
                const int s = sv.slot0 + l0 + lc;
                const float4 self = sm.pos[lc];
                const float li = self.w;
                float px = 0.0f, py = 0.0f, pz = 0.0f;
                for_each_nbr<2>(p, sm, sv, a.nbr, lc, s, sm.cnt[lc], sm.pos, pos_base, crank, [&](int, float4 q) {
                    const float3 d = make_float3(__fsub_rn(self.x, q.x), __fsub_rn(self.y, q.y),
                                                 __fsub_rn(self.z, q.z));
                    const float r2 = dot3e(d.x, d.y, d.z);
                    const float inv_r = inv_r_of(r2);
                    const float r = __fmul_rn(r2, inv_r);
                    const float w = __fmul_rn(__fadd_rn(__fadd_rn(li, q.w), scorr_hd(p, hdiff(p, r2))),
                                              spiky_g(p, r, inv_r));
                    px = __fmaf_rn(w, d.x, px);
                    py = __fmaf_rn(w, d.y, py);
                    pz = __fmaf_rn(w, d.z, pz);
                });
                const float kd = __fmul_rn(-p.ks, p.mr);
                const Geo& g = sv.g;
                const float4 out = make_float4(clampf(__fadd_rn(self.x, __fmul_rn(px, kd)), g.lox, g.hix),
                                               clampf(__fadd_rn(self.y, __fmul_rn(py, kd)), g.loy, g.hiy),
                                               clampf(__fadd_rn(self.z, __fmul_rn(pz, kd)), g.loz, g.hiz), 0.0f);
                sm.vel[lc] = out;
                if (last) a.lam_out[s] = self;  // x* before the last correction, lambda of the last pass
            }
            cluster.sync();
            for (int lc = tid; lc < mine; lc += T) {
                const float4 out = sm.vel[lc];
                sm.pos[lc] = out;
                if (last) {  // v = (x* - x) / dt
                    const int s = sv.slot0 + l0 + lc;
                    const float4 xo = a.x[s];
                    float3 xf;
                    if (MIXED) {
                        xf = scene_frame<true>(p, xo, unpack_cell(cp, xo.w));
                    } else {
                        xf = make_float3(xo.x, xo.y, xo.z);
                    }
                    sm.vel[lc] = make_float4(__fmul_rn(__fsub_rn(out.x, xf.x), p.inv_dt),
                                             __fmul_rn(__fsub_rn(out.y, xf.y), p.inv_dt),
                                             __fmul_rn(__fsub_rn(out.z, xf.z), p.inv_dt), 0.0f);
                }
            }
            cluster.sync();
            if (last) break;
            // lambda pass, in place (neighbours read xyz only)
            const bool last_lambda = it + 1 == iters - 1;
            for (int lc = tid; lc < mine; lc += T) {
                const int s = sv.slot0 + l0 + lc;
                const float4 self = sm.pos[lc];
                LambdaAcc acc = lambda_init(p);
                for_each_nbr<2>(p, sm, sv, a.nbr, lc, s, sm.cnt[lc], sm.pos, pos_base, crank, [&](int, float4 q) {
                    const float3 d = make_float3(__fsub_rn(self.x, q.x), __fsub_rn(self.y, q.y),
                                                 __fsub_rn(self.z, q.z));
                    lambda_accumulate<MIXED>(p, acc, d, false);
                });
                sm.pos[lc].w = lambda_of(p, acc);
                if (last_lambda && a.rho) a.rho[s] = density_of(p, acc);
            }
            cluster.sync();
        }

        // XSPH (v_i += c sum (v_j - v_i) W) and commit, with the next step's
        // prediction when asked
        for (int lc = tid; lc < mine; lc += T) {
            const int s = sv.slot0 + l0 + lc;
            const float4 self = sm.pos[lc];
            const float4 vi = sm.vel[lc];
            float ax = 0.0f, ay = 0.0f, az = 0.0f;
            if (p.c_xsph != 0.0f) {
                for_each_nbr<2>(p, sm, sv, a.nbr, lc, s, sm.cnt[lc], sm.pos, pos_base, crank, [&](int j, float4 q) {
                    const float4 vj = gather4(sv, sm.vel, vel_base, j, crank);
                    const float3 d = make_float3(__fsub_rn(self.x, q.x), __fsub_rn(self.y, q.y),
                                                 __fsub_rn(self.z, q.z));
                    const float hd = hdiff(p, dot3e(d.x, d.y, d.z));
                    const float w = __fmul_rn(__fmul_rn(hd, hd), hd);
                    ax = __fmaf_rn(__fsub_rn(vj.x, vi.x), w, ax);
                    ay = __fmaf_rn(__fsub_rn(vj.y, vi.y), w, ay);
                    az = __fmaf_rn(__fsub_rn(vj.z, vi.z), w, az);
                });
            }
            const float cx = __fmul_rn(p.c_xsph, p.k6);
            const float4 vc = make_float4(__fmaf_rn(cx, ax, vi.x), __fmaf_rn(cx, ay, vi.y), __fmaf_rn(cx, az, vi.z),
                                          0.0f);
            float4 xc;
            if (!MIXED) {
                xc = make_float4(self.x, self.y, self.z, 0.0f);
            } else {
                const int3 cs = slot_cell(p, cp, sv.g, a.key_sorted, p.cell_sorted, s);
                xc = make_float4(__fsub_rn(self.x, __fmul_rn((float)cs.x, p.cell)),
                                 __fsub_rn(self.y, __fmul_rn((float)cs.y, p.cell)),
                                 __fsub_rn(self.z, __fmul_rn((float)cs.z, p.cell)), pack_cell(cp, cs.x, cs.y, cs.z));
            }
            a.x_out[s] = xc;
            a.v_out[s] = vc;
            if (a.xs_next)
                predict_one<MIXED>(p, cp, sv.g, xc, vc, s, a.xs_next, a.key, a.rank, a.count, a.cellk,
                                   a.tile_count);
        }
        cluster.sync();  // the bin's shared memory is free again
    }
    cluster.sync();  // no CTA leaves while another may still read its shared memory
    // the last cluster to finish re-arms the queue for the next launch
    if (crank == 0 && tid == 0) {
        __threadfence();
        if (atomicAdd(&a.queue[1], 1) == (int)(gridDim.x / SOLVE_CLUSTER) - 1) {
            a.queue[0] = 0;
            a.queue[1] = 0;
            __threadfence();
        }
    }
}

size_t scene_solve_smem_bytes() { return sizeof(SolveSmem); }

template <bool MIXED, int T>
static int prepare_one(int* max_clusters) {
    const void* fn = (const void*)k_scene_solve<MIXED, T>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SolveSmem));
    if (e == cudaSuccess) e = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *max_clusters = 0;
        return 0;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(SOLVE_CLUSTER);
    cfg.blockDim = dim3(T);
    cfg.dynamicSmemBytes = sizeof(SolveSmem);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = SOLVE_CLUSTER;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    e = cudaOccupancyMaxActiveClusters(&n, fn, &cfg);
    if (e != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    *max_clusters = n;
    return n;
}

int scene_solve_prepare(bool mixed, int threads, int* max_clusters) {
    if (threads == 512) return mixed ? prepare_one<true, 512>(max_clusters) : prepare_one<false, 512>(max_clusters);
    return mixed ? prepare_one<true, 1024>(max_clusters) : prepare_one<false, 1024>(max_clusters);
}

void launch_scene_solve(bool mixed, int threads, const StepParams& p, const CellPack& cp, const SolveArgs& a,
                        int clusters, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(clusters * SOLVE_CLUSTER));
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = sizeof(SolveSmem);
    cfg.stream = st;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = SOLVE_CLUSTER;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl_enabled() ? 2 : 1;
    if (threads == 512) {
        if (mixed)
            cudaLaunchKernelEx(&cfg, k_scene_solve<true, 512>, p, cp, a);
        else
            cudaLaunchKernelEx(&cfg, k_scene_solve<false, 512>, p, cp, a);
    } else {
        if (mixed)
            cudaLaunchKernelEx(&cfg, k_scene_solve<true, 1024>, p, cp, a);
        else
            cudaLaunchKernelEx(&cfg, k_scene_solve<false, 1024>, p, cp, a);
    }
}

}  // namespace lgb
