// pbf_passes.cuh -- the kernels of the PBF step (mode P): the
// position-based-fluids solver the reference's parameters describe
// (Simulation.hpp:157-171: rest density, relaxation epsilon, s_corr, XSPH) on
// the poly6 / spiky kernels of Kernels.cpp:43-67, with N Jacobi solver
// iterations over neighbour lists built once per step.  Templates only: the
// launchers in pbf_solver.cu (column lists) and pbf_compact.cu (compact lists)
// instantiate them.
//
// Position representations (template parameter MIXED):
//   plain  float4 xyz = absolute position;
//   mixed  xyz = offset from the particle's cell corner, the cell being the
//          sorted key of the step (fixed during the step's iterations, so an
//          offset may leave [0, cell) until the next prediction renormalises
//          it); the committed state keeps the cell packed in w.  Neighbour
//          offsets are (o_i - o_j) + (c_i - c_j) * cell with the cell
//          difference cached in the neighbour list entry, so their precision
//          does not depend on the distance to the origin; density sums use
//          compensated (Kahan) accumulation.
// During the iterations w of the predicted positions holds the particle's
// lambda, written in place by the lambda pass, so the position pass gathers
// one float4 per neighbour.
//
// Neighbour list entry (int32, column lists): bits 0-24 slot, then the
// neighbour's cell offset from the particle's cell, 2 bits per axis as d + 1
// (x in 25-26, y in 27-28, z in 29-30), bit 31 set for solids.  Compact
// lists (no cell codes, no solids): 16-byte records, see CompactLists.
//
// Grids: dense (cell id = offset + y gX gZ + x gZ + z; the three cells of a
// stencil row are consecutive ids) or hashed (the counting sort runs over
// hash buckets of cells, see cell_bucket; each slot keeps its packed cell,
// so the 27-cell walk rejects particles of other cells sharing a bucket --
// used for domains with more cells than fit a dense table).
#pragma once

#include "pbf_common.cuh"
#include "pbf_device.cuh"
#include "pbf_kernels.h"

namespace lgb {

template <bool MIXED>
__global__ void k_predict(StepParams p, CellPack cp, const float4* __restrict__ x,
                          const float4* __restrict__ v, float4* __restrict__ xs, int* __restrict__ key,
                          int* __restrict__ rank, int* __restrict__ count, int* __restrict__ cellk,
                          int* __restrict__ tile_count) {
    pdl_wait();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    predict_one<MIXED>(p, cp, geo_slot(p, i), x[i], v[i], i, xs, key, rank, count, cellk, tile_count);
}

// Cell key and histogram of static particles (solids; scene from solid_scene_of).
template <bool MIXED>
__global__ void k_key(StepParams p, CellPack cp, const float4* __restrict__ pos, int m,
                      int* __restrict__ key, int* __restrict__ rank, int* __restrict__ count,
                      int* __restrict__ cellk) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    float4 q = pos[i];
    const Geo g = p.scenes ? geo_scene(p, p.solid_scene_of[i]) : geo_single(p);
    int3 c = MIXED ? unpack_cell(cp, q.w) : plain_cell(p, g, q.x, q.y, q.z);
    int k = cell_key(p, cp, g, c, cellk, i);
    key[i] = k;
    rank[i] = atomicAdd(&count[k], 1);
}

// Cells (hash buckets) with a static particle in their 27-cell
// neighbourhood, marked once when the solids are set: the list build walks
// the solids only from those (a bucket shared with another cell is a false
// positive, which only costs a walk).
template <bool MIXED>
__global__ void k_mark_solid_near(StepParams p, CellPack cp, const float4* __restrict__ pos, int m,
                                  unsigned char* __restrict__ near) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    float4 q = pos[i];
    const Geo g = p.scenes ? geo_scene(p, p.solid_scene_of[i]) : geo_single(p);
    int3 c = MIXED ? unpack_cell(cp, q.w) : plain_cell(p, g, q.x, q.y, q.z);
    if (p.hash_bits) c = make_int3(min(c.x, (int)cp.mx), min(c.y, (int)cp.my), min(c.z, (int)cp.mz));
    for (int dy = -1; dy <= 1; dy++)
        for (int dx = -1; dx <= 1; dx++)
            for (int dz = -1; dz <= 1; dz++) {
                const int3 cn = make_int3(c.x + dx, c.y + dy, c.z + dz);
                if (cn.x < 0 || cn.y < 0 || cn.z < 0 || cn.x >= g.gx || cn.y >= g.gy || cn.z >= g.gz) continue;
                if (p.hash_bits) {
                    if (cn.x > (int)cp.mx || cn.y > (int)cp.my || cn.z > (int)cp.mz) continue;
                    near[cell_bucket(cn, p.hash_bits)] = 1;
                } else {
                    near[linear_cell(g, cn)] = 1;
                }
            }
}

// Where the list build puts a particle's entries.  Column lists: entry k of
// slot s at nbr[k * n + s] with its cell codes and solid flag.
struct ColumnLists {
    int* nbr;
    int n, s;
    __device__ __forceinline__ void put(int k, int t, int dx, int dy, int dz, bool solid) {
        nbr[(size_t)k * n + s] = entry(t, dx, dy, dz, solid);
    }
};

// Entries a compact list keeps in its two records: inline (first record),
// second record, both.
template <bool WIDE>
struct RecordFormat {
    static constexpr int INLINE = WIDE ? WIDE_INLINE : COMPACT_INLINE;
    static constexpr int EXT = WIDE ? WIDE_EXT : COMPACT_EXT;
    static constexpr int RECORDS = INLINE + EXT;
};

// Compact lists: the records' entries (16-bit offsets from the scene's
// first slot, or 32-bit slots in wide records) staged in the thread's
// COMPACT_STRIDE words of shared memory (filled with the sentinel first; a
// stride of 9 words keeps a warp's stores and loads free of bank conflicts)
// until the records are written; the rest as plain slots in the column rows
// of nbr from row 0.  No cell codes and no static particles (the step uses
// compact lists only without either).
constexpr int COMPACT_STRIDE = 9;
template <bool WIDE>
struct CompactLists {
    int* ovf;
    int n, s, base;
    unsigned* stage;  // this thread's words
    __device__ __forceinline__ void put(int k, int t, int, int, int, bool) {
        constexpr int R = RecordFormat<WIDE>::RECORDS;
        if (k >= R)
            ovf[(size_t)(k - R) * n + s] = t;
        else if (WIDE)
            stage[k] = (unsigned)t;
        else
            reinterpret_cast<unsigned short*>(stage)[k] = (unsigned short)(t - base);
    }
    // entry k < count of the list put so far (the thread reads back its own stores)
    __device__ __forceinline__ int get(int k) const {
        constexpr int R = RecordFormat<WIDE>::RECORDS;
        if (k >= R) return ovf[(size_t)(k - R) * n + s];
        if (WIDE) return (int)stage[k];
        return base + reinterpret_cast<const unsigned short*>(stage)[k];
    }
};

// 0: column lists; 1: compact; 2: compact in wide records
template <int FORMAT>
struct ListsOf {
    using T = ColumnLists;
};
template <>
struct ListsOf<1> {
    using T = CompactLists<false>;
};
template <>
struct ListsOf<2> {
    using T = CompactLists<true>;
};
__device__ __forceinline__ ColumnLists open_lists(ColumnLists*, int* nbr, int n, int s, int, unsigned*) {
    return ColumnLists{nbr, n, s};
}
template <bool WIDE>
__device__ __forceinline__ CompactLists<WIDE> open_lists(CompactLists<WIDE>*, int* nbr, int n, int s, int base,
                                                         unsigned* stage) {
    unsigned* mine = stage + COMPACT_STRIDE * threadIdx.x;
    if (WIDE) {
#pragma unroll
        for (int q = 0; q < WIDE_RECORDS; q++) mine[q] = (unsigned)n;
    } else {
#pragma unroll
        for (int q = 0; q < COMPACT_RECORDS / 2; q++) mine[q] = 0xFFFFFFFFu;
    }
    return CompactLists<WIDE>{nbr, n, s, base, mine};
}
// The count and the sentinel entries up to a multiple of the passes' chunk
// (pad divides the buffer's rows: max_nbrs rounded up to LIST_PAD_MAX).
__device__ __forceinline__ void close_lists(const StepParams& p, const ColumnLists& l, int* __restrict__ cnt,
                                            int c_n) {
    cnt[l.s] = c_n;
    for (int k = c_n; k % p.pad != 0; k++) l.nbr[(size_t)k * p.n + l.s] = sentinel_entry(p);
}
template <bool WIDE>
__device__ __forceinline__ void close_lists(const StepParams& p, const CompactLists<WIDE>& l, int*, int c_n) {
    using RF = RecordFormat<WIDE>;
    const unsigned* w = l.stage;
    const unsigned head = WIDE ? (unsigned)c_n : ((unsigned)c_n | ((unsigned)l.base << 8));
    p.rec[l.s] = make_uint4(head, w[0], w[1], w[2]);
    if (c_n > RF::INLINE) p.rec2[l.s] = make_uint4(w[3], w[4], w[5], w[6]);
    for (int k = c_n - RF::RECORDS; k > 0 && k % p.pad != 0; k++) l.ovf[(size_t)k * p.n + l.s] = p.n;
}

// A candidate within h, the c_n-th accepted.  PH 0: listed (below the
// capacity) and summed into the first lambda; PH 1: listed only (the sums
// run over the list afterwards); PH 2: summed only if past the capacity (the
// entries the list dropped, after the listed ones' sums).
template <int PH, bool KAHAN, bool SOLID, class L>
__device__ __forceinline__ void accept(const StepParams& p, LambdaAcc& a, const float3& d, int& c_n, L& out, int t,
                                       int dx, int dy, int dz) {
    if (PH != 2 && c_n < p.max_nbrs) out.put(c_n, t, dx, dy, dz, SOLID);
    if (PH == 0 || (PH == 2 && c_n >= p.max_nbrs)) lambda_accumulate<KAHAN>(p, a, d, SOLID);
    c_n++;
}

// One row (dy, dx) of the stencil: the cells z0..z1 of a row are consecutive
// ids, so their particles form one slot range, walked in one loop (a warp
// then runs as many rounds as its fullest row, not the sum over the three
// cells of its fullest cell); a candidate's dz follows from the cell bounds,
// loaded once per row.  The candidates come in the same order as cell by cell.
template <bool MIXED, bool SOLID, bool KAHAN, class L, int PH = 0>
__device__ __forceinline__ void walk_row(const StepParams& p, const float4& self, int s,
                                         const float4* __restrict__ pos, const int* __restrict__ start,
                                         int row, int zc, int gz, int dx, int dy, LambdaAcc& a, int& c_n,
                                         L& out) {
    const int z0 = max(zc - 1, 0), z1 = min(zc + 1, gz - 1);
    const int b0 = start[row + z0];
    const int b1 = start[row + z0 + 1];
    const int b2 = (z0 + 1 <= z1) ? start[row + z0 + 2] : b1;
    const int b3 = (z0 + 2 <= z1) ? start[row + z0 + 3] : b2;
    const int dz0 = z0 - zc;
    const float sx = -(float)dx * p.cell, sy = -(float)dy * p.cell;
    for (int t = b0; t < b3; t++) {
        if (!SOLID && t == s) continue;
        const int dz = dz0 + (t >= b1) + (t >= b2);
        const float4 q = SOLID ? __ldg(&pos[t]) : pos[t];
        float3 d = make_float3(__fsub_rn(self.x, q.x), __fsub_rn(self.y, q.y), __fsub_rn(self.z, q.z));
        if (MIXED) {
            d.x = __fadd_rn(d.x, sx);
            d.y = __fadd_rn(d.y, sy);
            d.z = __fadd_rn(d.z, -(float)dz * p.cell);
        }
        if (dot3e(d.x, d.y, d.z) <= p.h2) accept<PH, KAHAN, SOLID>(p, a, d, c_n, out, t, dx, dy, dz);
    }
}

// The candidates [t_begin, t_end) of one row, gathered W at a time (the
// loads of a chunk are in flight together; the tests run in slot order, so
// the list is the one walk_row builds).  W = 4; the compact list build takes
// 2 and loads each row's bounds just before the row, for fewer live
// registers (config 3 lists 0.522 -> 0.493 ms at step 50 of the run, both
// steps together).  b1, b2: the row's cell bounds, read
// in mixed precision only (the entry's dz code and the cell shift; fp32
// entries carry dz = 0, which no fp32 pass reads).
template <bool MIXED, bool SOLID, bool KAHAN, class L, int W = 4, int PH = 0>
__device__ __forceinline__ void walk_range(const StepParams& p, const float4& self, int s,
                                           const float4* __restrict__ pos, int t_begin, int t_end, int b1, int b2,
                                           int dz0, int dx, int dy, LambdaAcc& a, int& c_n, L& out) {
    const float sx = -(float)dx * p.cell, sy = -(float)dy * p.cell;
    for (int t0 = t_begin; t0 < t_end; t0 += W) {
        float4 q[W];
#pragma unroll
        for (int u = 0; u < W; u++)
            if (t0 + u < t_end) q[u] = SOLID ? __ldg(&pos[t0 + u]) : pos[t0 + u];
#pragma unroll
        for (int u = 0; u < W; u++) {
            const int t = t0 + u;
            if (t >= t_end || (!SOLID && t == s)) continue;
            const int dz = MIXED ? dz0 + (t >= b1) + (t >= b2) : 0;
            float3 d = make_float3(__fsub_rn(self.x, q[u].x), __fsub_rn(self.y, q[u].y), __fsub_rn(self.z, q[u].z));
            if (MIXED) {
                d.x = __fadd_rn(d.x, sx);
                d.y = __fadd_rn(d.y, sy);
                d.z = __fadd_rn(d.z, -(float)dz * p.cell);
            }
            if (dot3e(d.x, d.y, d.z) <= p.h2) accept<PH, KAHAN, SOLID>(p, a, d, c_n, out, t, dx, dy, dz);
        }
    }
}

// One cell of the stencil on a hashed grid: the particles of its bucket,
// kept only if they belong to that cell.
template <bool MIXED, bool SOLID, bool KAHAN, class L, int PH = 0>
__device__ __forceinline__ void walk_hashed_cell(const StepParams& p, const float4& self, int s,
                                                 const float4* __restrict__ pos,
                                                 const int* __restrict__ start,
                                                 const int* __restrict__ cells, int b, int packed,
                                                 int dx, int dy, int dz, LambdaAcc& a, int& c_n, L& out) {
    const float sx = -(float)dx * p.cell, sy = -(float)dy * p.cell, sz = -(float)dz * p.cell;
    for (int t = start[b], e = start[b + 1]; t < e; t++) {
        if ((!SOLID && t == s) || __ldg(&cells[t]) != packed) continue;
        const float4 q = SOLID ? __ldg(&pos[t]) : pos[t];
        float3 d = make_float3(__fsub_rn(self.x, q.x), __fsub_rn(self.y, q.y), __fsub_rn(self.z, q.z));
        if (MIXED) {
            d.x = __fadd_rn(d.x, sx);
            d.y = __fadd_rn(d.y, sy);
            d.z = __fadd_rn(d.z, sz);
        }
        if (dot3e(d.x, d.y, d.z) <= p.h2) accept<PH, KAHAN, SOLID>(p, a, d, c_n, out, t, dx, dy, dz);
    }
}

// The stencil's candidates of fluid slot s in cell c, in list order: on a
// dense grid the nine rows (with the static particles of each row after its
// fluid ones where the neighbourhood holds some); on a hashed grid the
// cells' buckets.  PH: what each accepted candidate does (accept()).
template <int PH, bool MIXED, bool HASHED, bool KAHAN, bool COMPACT, class Lists>
__device__ __forceinline__ void walk_stencil(const StepParams& p, const CellPack& cp, const float4& self, int s,
                                             const int3& c, const Geo& g, const float4* __restrict__ xs,
                                             const int* __restrict__ cell_sorted, const int* __restrict__ fstart,
                                             const float4* __restrict__ solid, const int* __restrict__ solid_cell,
                                             const int* __restrict__ sstart, bool solids, LambdaAcc& a, int& c_n,
                                             Lists& out) {
    const int slab = g.gx * g.gz;
    if (!HASHED && COMPACT) {
        // each row's two bounds loaded just before its walk (fewer live
        // registers than a layer's six: more resident warps)
        const int z0 = max(c.z - 1, 0), z1 = min(c.z + 1, g.gz - 1);
        for (int dy = -1; dy <= 1; dy++) {
            const int y = c.y + dy;
            if (y < 0 || y >= g.gy) continue;
            for (int dx = -1; dx <= 1; dx++) {
                const int xx = c.x + dx;
                if (xx < 0 || xx >= g.gx) continue;
                const int row = g.off + y * slab + xx * g.gz;
                walk_range<MIXED, false, KAHAN, Lists, 2, PH>(p, self, s, xs, fstart[row + z0], fstart[row + z1 + 1],
                                                              0, 0, z0 - c.z, dx, dy, a, c_n, out);
            }
        }
    } else if (!HASHED) {
        const int z0 = max(c.z - 1, 0), z1 = min(c.z + 1, g.gz - 1);
        for (int dy = -1; dy <= 1; dy++) {
            const int y = c.y + dy;
            if (y < 0 || y >= g.gy) continue;
            // the fluid slot ranges of the layer's three rows, loaded together
            int b0[3], b1[3], b2[3], b3[3];
#pragma unroll
            for (int r = 0; r < 3; r++) {
                const int xx = c.x + r - 1;
                b0[r] = b1[r] = b2[r] = b3[r] = 0;
                if (xx >= 0 && xx < g.gx) {
                    const int row = g.off + y * slab + xx * g.gz;
                    b0[r] = fstart[row + z0];
                    b3[r] = fstart[row + z1 + 1];
                    if (MIXED) {
                        b1[r] = fstart[row + z0 + 1];
                        b2[r] = (z0 + 1 <= z1) ? fstart[row + z0 + 2] : b1[r];
                    }
                }
            }
#pragma unroll
            for (int r = 0; r < 3; r++) {
                const int xx = c.x + r - 1;
                if (xx < 0 || xx >= g.gx) continue;
                walk_range<MIXED, false, KAHAN, Lists, COMPACT ? 2 : 4, PH>(p, self, s, xs, b0[r], b3[r], b1[r], b2[r],
                                                                         z0 - c.z, r - 1, dy, a, c_n, out);
                if (solids)
                    walk_row<MIXED, true, KAHAN, Lists, PH>(p, self, s, solid, sstart, g.off + y * slab + xx * g.gz,
                                                            c.z, g.gz, r - 1, dy, a, c_n, out);
            }
        }
    }
    for (int dy = -1; dy <= 1 && HASHED; dy++) {
        const int y = c.y + dy;
        if (y < 0 || y >= g.gy) continue;
        for (int dx = -1; dx <= 1; dx++) {
            const int xx = c.x + dx;
            if (xx < 0 || xx >= g.gx) continue;
            {
                // cells past the packed field widths hold no particle
                if (xx > (int)cp.mx || y > (int)cp.my) continue;
                // the dense walk's entry order: the row's fluid cells, then its solid cells
                const int z0 = max(c.z - 1, 0), z1 = min(min(c.z + 1, g.gz - 1), (int)cp.mz);
                for (int z = z0; z <= z1; z++) {
                    const int3 cn = make_int3(xx, y, z);
                    walk_hashed_cell<MIXED, false, KAHAN, Lists, PH>(p, self, s, xs, fstart, cell_sorted,
                                                                     cell_bucket(cn, p.hash_bits),
                                                                     (int)pack_bits(cp, cn), dx, dy, z - c.z, a, c_n,
                                                                     out);
                }
                if (solids)
                    for (int z = z0; z <= z1; z++) {
                        const int3 cn = make_int3(xx, y, z);
                        walk_hashed_cell<MIXED, true, KAHAN, Lists, PH>(p, self, s, solid, sstart, solid_cell,
                                                                        cell_bucket(cn, p.hash_bits),
                                                                        (int)pack_bits(cp, cn), dx, dy, z - c.z, a,
                                                                        c_n, out);
                    }
            }
        }
    }
}

// FRAME: mixed storage with the iterations in the scene frame (positions
// relative to the box corner, compensated density sums; the walk's cell is
// the step's key, which rounding of the frame position could move).
// FORMAT 1 or 2: compact lists (in wide records with 2) to p.rec (no cell
// codes, no static particles).  Column lists sum the first lambda as the
// walk accepts each candidate.  Compact lists walk first, only listing the
// accepted candidates (no sums live across the walk: fewer registers, so
// more resident warps), and then sum over the finished list, two entries'
// positions loaded together (in the cache from the walk); a list cut at the
// capacity walks once more to sum the dropped entries after the listed
// ones.  The terms and their order are the walk's, so the sums equal the
// column lists'.
template <bool MIXED, bool HASHED, bool FRAME, int FORMAT>
__device__ __forceinline__ void lists_lambda(const StepParams& p, const CellPack& cp, float4* __restrict__ xs,
                                             const int* __restrict__ key_sorted, const int* __restrict__ cell_sorted,
                                             const int* __restrict__ fstart, const float4* __restrict__ solid,
                                             const int* __restrict__ solid_cell, const int* __restrict__ sstart,
                                             int* __restrict__ nbr, int* __restrict__ cnt, float* __restrict__ rho,
                                             int* status, unsigned* stage = nullptr) {
    pdl_wait();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= p.n) return;
    const float4 self = xs[s];
    const Geo g = geo_slot(p, s);
    // fp32 on a dense grid: the cell the prediction keyed this position by
    constexpr bool KAHAN = MIXED || FRAME;
    const int3 c = (MIXED || HASHED || FRAME) ? slot_cell(p, cp, g, key_sorted, cell_sorted, s)
                                              : plain_cell(p, g, self.x, self.y, self.z);
    LambdaAcc a = lambda_init(p);
    int c_n = 0;
    constexpr bool COMPACT = FORMAT != 0;
    using Lists = typename ListsOf<FORMAT>::T;
    Lists out = open_lists((Lists*)nullptr, nbr, p.n, s, g.slot0, stage);
    // static particles only where the cell's neighbourhood holds some
    const bool solids = p.ns > 0 && p.solid_near && __ldg(&p.solid_near[__ldg(&key_sorted[s])]);
    walk_stencil<COMPACT ? 1 : 0, MIXED, HASHED, KAHAN, COMPACT>(p, cp, self, s, c, g, xs, cell_sorted, fstart, solid,
                                                                 solid_cell, sstart, solids, a, c_n, out);
    if constexpr (COMPACT) {
        // compact lists hold fluid slots only, with fp32 offsets: d as the walk formed it
        const int m = min(c_n, p.max_nbrs);
        for (int k = 0; k < m; k += 2) {
            const bool two = k + 1 < m;
            const float4 q0 = xs[out.get(k)];
            const float4 q1 = two ? xs[out.get(k + 1)] : q0;
            lambda_accumulate<KAHAN>(
                p, a, make_float3(__fsub_rn(self.x, q0.x), __fsub_rn(self.y, q0.y), __fsub_rn(self.z, q0.z)), false);
            if (two)
                lambda_accumulate<KAHAN>(
                    p, a, make_float3(__fsub_rn(self.x, q1.x), __fsub_rn(self.y, q1.y), __fsub_rn(self.z, q1.z)),
                    false);
        }
        if (c_n > p.max_nbrs) {
            int c2 = 0;
            walk_stencil<2, MIXED, HASHED, KAHAN, COMPACT>(p, cp, self, s, c, g, xs, cell_sorted, fstart, solid,
                                                           solid_cell, sstart, solids, a, c2, out);
        }
    }
    if (c_n > p.max_nbrs) {
        set_status(status, ST_NBR_OVERFLOW);
        c_n = p.max_nbrs;
    }
    close_lists(p, out, cnt, c_n);
    // lambda into w in place: neighbours read only xyz of this element here
    reinterpret_cast<float*>(xs)[4 * (size_t)s + 3] = lambda_of(p, a);
    if (rho) rho[s] = density_of(p, a);
}

template <bool MIXED, bool HASHED, int B, bool FRAME = false>
__global__ void __launch_bounds__(B) k_lists_lambda(StepParams p, CellPack cp, float4* __restrict__ xs,
                                                    const int* __restrict__ key_sorted,
                                                    const int* __restrict__ cell_sorted,
                                                    const int* __restrict__ fstart,
                                                    const float4* __restrict__ solid,
                                                    const int* __restrict__ solid_cell,
                                                    const int* __restrict__ sstart,
                                                    int* __restrict__ nbr, int* __restrict__ cnt,
                                                    float* __restrict__ rho, int* status) {
    lists_lambda<MIXED, HASHED, FRAME, 0>(p, cp, xs, key_sorted, cell_sorted, fstart, solid, solid_cell, sstart, nbr,
                                          cnt, rho, status);
}

// Compact lists (no static particles, fp32 pair offsets; WIDE: wide records).
// Held to 12 blocks of 128 threads per SM (40 registers, a few bytes
// spilled): the extra resident warps hide more of the gathers' latency
// (config 3: 0.382 -> 0.353 ms a step; a walk that loads the next row's
// bounds ahead, or 4 gathers in flight, was slower).
template <bool HASHED, int B, bool FRAME, bool WIDE>
__global__ void __launch_bounds__(B, 1536 / B) k_lists_compact(StepParams p, CellPack cp, float4* __restrict__ xs,
                                                             const int* __restrict__ key_sorted,
                                                             const int* __restrict__ cell_sorted,
                                                             const int* __restrict__ fstart,
                                                             const float4* __restrict__ solid,
                                                             const int* __restrict__ solid_cell,
                                                             const int* __restrict__ sstart,
                                                             int* __restrict__ nbr, int* __restrict__ cnt,
                                                             float* __restrict__ rho, int* status) {
    __shared__ unsigned stage[COMPACT_STRIDE * B];
    lists_lambda<false, HASHED, FRAME, WIDE ? 2 : 1>(p, cp, xs, key_sorted, cell_sorted, fstart, solid, solid_cell,
                                                     sstart, nbr, cnt, rho, status, stage);
}

// Walk a particle's list U entries at a time, calling f(entry, position)
// for each (SOL: the scene has static particles, whose entries read solid).
// E entries (U or LIST_PAD_MAX) are loaded together with the count, the
// rest a chunk ahead of their gathers: with E = LIST_PAD_MAX a list of up to
// 8 neighbours waits for one round trip to DRAM for its entries and then one
// to L2 per chunk of gathers, at the price of loading 8 entries for shorter
// lists (the position pass gains, measured; the lambda pass, with fewer
// instructions per pair to hide the latency behind, loses and keeps E = U).
// The list is padded with sentinel entries to a multiple of U (the list
// build's pad) and the buffer holds at least LIST_PAD_MAX rows (2
// LIST_PAD_MAX when a count exceeds LIST_PAD_MAX), so every entry a chunk
// below the count reads is valid and every load in bounds.
template <int U, bool SOL, int E = U, class F>
__device__ __forceinline__ void for_each_entry(const StepParams& p, const int* __restrict__ col,
                                               const int* __restrict__ cnt, int s,
                                               const float4* __restrict__ xs,
                                               const float4* __restrict__ solid, F&& f) {
    static_assert(E % U == 0 && E <= LIST_PAD_MAX, "prefetch depth");
    int e0[E];
#pragma unroll
    for (int u = 0; u < E; u++) e0[u] = __ldg(&col[(size_t)u * p.n]);
    const int c = __ldg(&cnt[s]);
    if (E > U) {
#pragma unroll
        for (int k = 0; k < E; k += U) {
            if (k >= c) return;
            float4 q[U];
#pragma unroll
            for (int u = 0; u < U; u++) q[u] = SOL ? load_entry(e0[k + u], xs, solid) : xs[entry_slot(e0[k + u])];
#pragma unroll
            for (int u = 0; u < U; u++) f(e0[k + u], q[u]);
        }
        if (c <= E) return;
    }
    // the chunks from E on (E = U: from the first), each chunk's entries
    // loaded while the one before is gathered
    int nx[U];
#pragma unroll
    for (int u = 0; u < U; u++) nx[u] = E > U ? __ldg(&col[(size_t)(E + u) * p.n]) : e0[u];
    for (int k = E > U ? E : 0; k < c; k += U) {
        int e[U];
        float4 q[U];
#pragma unroll
        for (int u = 0; u < U; u++) e[u] = nx[u];
        if (k + U < c) {
#pragma unroll
            for (int u = 0; u < U; u++) nx[u] = __ldg(&col[(size_t)(k + U + u) * p.n]);
        }
#pragma unroll
        for (int u = 0; u < U; u++) q[u] = SOL ? load_entry(e[u], xs, solid) : xs[entry_slot(e[u])];
#pragma unroll
        for (int u = 0; u < U; u++) f(e[u], q[u]);
    }
}

// P particles per thread: the lists of slots s[0..P) walked together, U
// entries of each per round, so the loads of all P lists and their gathers
// are in flight at once; f(r, entry, position) per entry of particle r in
// list order.  Past its own count a particle reads the sentinel entry (every
// pair term with it is exactly zero), so the lists may differ in length.
template <int U, int P, bool SOL, class F>
__device__ __forceinline__ void for_each_entry_p(const StepParams& p, const int* __restrict__ nbr,
                                                 const int (&s)[P], const int (&c)[P],
                                                 const float4* __restrict__ xs, const float4* __restrict__ solid,
                                                 F&& f) {
    int cmax = 0;
#pragma unroll
    for (int r = 0; r < P; r++) cmax = max(cmax, c[r]);
    const int sent = sentinel_entry(p);
    for (int k = 0; k < cmax; k += U) {
        int e[P][U];
        float4 q[P][U];
#pragma unroll
        for (int r = 0; r < P; r++)
#pragma unroll
            for (int u = 0; u < U; u++) e[r][u] = k + u < c[r] ? __ldg(&nbr[(size_t)(k + u) * p.n + s[r]]) : sent;
#pragma unroll
        for (int r = 0; r < P; r++)
#pragma unroll
            for (int u = 0; u < U; u++) q[r][u] = SOL ? load_entry(e[r][u], xs, solid) : xs[entry_slot(e[r][u])];
#pragma unroll
        for (int u = 0; u < U; u++)
#pragma unroll
            for (int r = 0; r < P; r++) f(r, e[r][u], q[r][u]);
    }
}

// Field j of a record: .y .z .w of the first, .x .y .z .w of the second.
template <bool FIRST>
__device__ __forceinline__ unsigned record_field(const uint4& r, int j) {
    const int f = j + (FIRST ? 1 : 0);
    return f == 0 ? r.x : (f == 1 ? r.y : (f == 2 ? r.z : r.w));
}

// The entries [K0, K0 + M) of a compact list from record r (K0 = 0: the
// first record), min(U, M) gathers at a time; false once the count is
// reached.
template <int U, int M, int K0, bool WIDE, class T, class G, class F>
__device__ __forceinline__ bool walk_record(const StepParams& p, const uint4& r, int c, int base, G&& gather,
                                            F&& f) {
    constexpr int V = U < M ? U : M;
    // each chunk decodes its own entries (a short list decodes only those it uses)
#pragma unroll
    for (int k = 0; k < M; k += V) {
        if (K0 + k >= c) return false;
        int sl[V];
        T q[V];
#pragma unroll
        for (int u = 0; u < V; u++)
            if (k + u < M) {
                if (WIDE) {
                    sl[u] = (int)record_field<K0 == 0>(r, k + u);
                } else {
                    const unsigned x = record_field<K0 == 0>(r, (k + u) >> 1);
                    sl[u] = compact_slot(p, base, ((k + u) & 1) ? (x >> 16) : (x & 0xFFFFu));
                }
                q[u] = gather(sl[u]);
            }
#pragma unroll
        for (int u = 0; u < V; u++)
            if (k + u < M) f(sl[u], q[u]);
    }
    return K0 + M < c;
}

// Walk a compact list (record r of slot s, r2 its second record; col =
// nbr + s, its overflow rows): gather(slot) loads what f(slot, value) needs
// of each neighbour.  A record's entries go min(U, its entries) at a time,
// all gathers of a chunk in flight together, so with U >= 4 a list of up to
// 4 neighbours (3 in wide records) waits for one round trip to DRAM (the
// record, with the particle's own loads) and one to L2 for the neighbours;
// the second record is loaded only for a longer list.  Past the count an
// entry reads the sentinel slot, whose terms are exactly zero; the overflow
// rows are padded with it to a multiple of U (the list build's pad).
template <int U, bool WIDE, class T, class G, class F>
__device__ __forceinline__ void walk_compact(const StepParams& p, const uint4& r, const uint4* __restrict__ r2,
                                             const int* __restrict__ col, G&& gather, F&& f) {
    using RF = RecordFormat<WIDE>;
    const int c = WIDE ? (int)r.x : (int)(r.x & 0xFFu);
    const int base = WIDE ? 0 : (int)(r.x >> 8);
    if (!walk_record<U, RF::INLINE, 0, WIDE, T>(p, r, c, base, gather, f)) return;
    if (!walk_record<U, RF::EXT, RF::INLINE, WIDE, T>(p, __ldg(r2), c, base, gather, f)) return;
    constexpr int R = RF::RECORDS;
    int nx[U];
#pragma unroll
    for (int u = 0; u < U; u++) nx[u] = __ldg(&col[(size_t)u * p.n]);
    for (int k = R; k < c; k += U) {
        int e[U];
        T q[U];
#pragma unroll
        for (int u = 0; u < U; u++) e[u] = nx[u];
        if (k + U < c) {
#pragma unroll
            for (int u = 0; u < U; u++) nx[u] = __ldg(&col[(size_t)(k - R + U + u) * p.n]);
        }
#pragma unroll
        for (int u = 0; u < U; u++) q[u] = gather(e[u]);
#pragma unroll
        for (int u = 0; u < U; u++) f(e[u], q[u]);
    }
}

// Lambda pass over the lists (iterations after the first); U neighbour
// gathers in flight per thread.
// F: bit 0 mixed precision, bit 1 the scene has static particles (the
// solid-free kernels skip the per-entry solid tests).
template <int F, int U, int B, int P = 1>
__global__ void __launch_bounds__(B) k_lambda(StepParams p, float4* __restrict__ xs,
                                              const int* __restrict__ nbr, const int* __restrict__ cnt,
                                              const float4* __restrict__ solid,
                                              float* __restrict__ rho) {
    // F bit 2: the scene frame (fp32 pair offsets, compensated density sums)
    // F bit 3: compact lists (fp32 pair offsets, no static particles); bit 4: in wide records
    constexpr bool MIXED = (F & 1) != 0, SOL = (F & 2) != 0, KAHAN = MIXED || (F & 4) != 0;
    constexpr bool COMPACT = (F & 8) != 0, WIDE = (F & 16) != 0;
    static_assert(!COMPACT || (!MIXED && !SOL && P == 1), "compact lists");
    pdl_wait();
    __shared__ float4 shift_tab[MIXED ? 64 : 1];
    if (MIXED) fill_shift_table(p, shift_tab);
    if (P == 1) {
        const int s = blockIdx.x * blockDim.x + threadIdx.x;
        if (s >= p.n) return;
        const float4 self = xs[s];
        LambdaAcc a = lambda_init(p);
        if (COMPACT) {
            walk_compact<U, WIDE, float4>(
                p, __ldg(&p.rec[s]), p.rec2 + s, nbr + s, [&](int t) { return xs[t]; },
                [&](int, float4 q) { lambda_accumulate<KAHAN>(p, a, rel_t<false>(self, q, 0, shift_tab), false); });
        } else {
            for_each_entry<U, SOL>(p, nbr + s, cnt, s, xs, solid, [&](int e, float4 q) {
                float3 d = rel_t<MIXED>(self, q, e, shift_tab);
                lambda_accumulate<KAHAN>(p, a, d, SOL && entry_solid(e));
            });
        }
        reinterpret_cast<float*>(xs)[4 * (size_t)s + 3] = lambda_of(p, a);
        if (rho) rho[s] = density_of(p, a);
        return;
    }
    // P slots per thread, B apart (each load of the block coalesced)
    int s[P], c[P];
    float4 self[P];
    LambdaAcc a[P];
#pragma unroll
    for (int r = 0; r < P; r++) {
        s[r] = (blockIdx.x * P + r) * B + threadIdx.x;
        const bool ok = s[r] < p.n;
        c[r] = ok ? __ldg(&cnt[s[r]]) : 0;
        self[r] = ok ? xs[s[r]] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        a[r] = lambda_init(p);
    }
    for_each_entry_p<U, P, SOL>(p, nbr, s, c, xs, solid, [&](int r, int e, float4 q) {
        float3 d = rel_t<MIXED>(self[r], q, e, shift_tab);
        lambda_accumulate<KAHAN>(p, a[r], d, SOL && entry_solid(e));
    });
#pragma unroll
    for (int r = 0; r < P; r++) {
        if (s[r] >= p.n) continue;
        reinterpret_cast<float*>(xs)[4 * (size_t)s[r] + 3] = lambda_of(p, a[r]);
        if (rho) rho[s[r]] = density_of(p, a[r]);
    }
}

// Position correction with s_corr, solid push-out and box clamp (Jacobi).
// The last iteration also writes v = (x* - x) / dt.
struct DeltaAcc {
    float px, py, pz, cx, cy, cz;
    int nct;
};

template <bool MIXED, bool SOL, bool POW = true>
__device__ __forceinline__ void delta_pair(const StepParams& p, DeltaAcc& a, const float4& self, int e, float4 q,
                                           const float4* tab) {
    const float li = self.w;
    const bool sol = SOL && entry_solid(e);
    float3 d = rel_t<MIXED>(self, q, e, tab);
    const float r2 = dot3e(d.x, d.y, d.z);
    const float inv_r = inv_r_of(r2);
    const float r = __fmul_rn(r2, inv_r);
    const float lj = sol ? li : q.w;
    const float w = __fmul_rn(__fadd_rn(__fadd_rn(li, lj), scorr_hd<POW>(p, hdiff(p, r2))), spiky_g(p, r, inv_r));
    a.px = __fmaf_rn(w, d.x, a.px);
    a.py = __fmaf_rn(w, d.y, a.py);
    a.pz = __fmaf_rn(w, d.z, a.pz);
    if (sol && r < p.contact && r2 > 0.0f) {
        const float t = __fmul_rn(__fsub_rn(p.contact, r), inv_r);
        a.cx = __fmaf_rn(t, d.x, a.cx);
        a.cy = __fmaf_rn(t, d.y, a.cy);
        a.cz = __fmaf_rn(t, d.z, a.cz);
        a.nct++;
    }
}

// dp = (m / rho0) sum (lambda_i + lambda_j + s_corr) dW, dW = -Ks g d; the
// solid push-out averaged; the box clamp; x* and (last pass) v written.
// scene: the slot's scene index (scene_index); packed: its packed cell in
// mixed precision on a sorted packed-cell array (else unused), both loaded
// before the neighbour walk.
template <bool MIXED>
__device__ __forceinline__ void delta_finish(const StepParams& p, const CellPack& cp, int s, const float4& self,
                                             const DeltaAcc& a, float4* __restrict__ xs_out,
                                             const int* __restrict__ key_sorted, const float4* __restrict__ x,
                                             float4* __restrict__ v_out, int scene, int packed) {
    const float kd = __fmul_rn(-p.ks, p.mr);
    float dx = __fmul_rn(a.px, kd), dy = __fmul_rn(a.py, kd), dz = __fmul_rn(a.pz, kd);
    if (a.nct) {
        const float inv = __frcp_rn((float)a.nct);
        dx = __fmaf_rn(a.cx, inv, dx);
        dy = __fmaf_rn(a.cy, inv, dy);
        dz = __fmaf_rn(a.cz, inv, dz);
    }
    float4 out;
    int3 cs = make_int3(0, 0, 0);
    const Geo g = geo_of(p, scene);
    if (!MIXED) {
        out = make_float4(clampf(__fadd_rn(self.x, dx), g.lox, g.hix), clampf(__fadd_rn(self.y, dy), g.loy, g.hiy),
                          clampf(__fadd_rn(self.z, dz), g.loz, g.hiz), 0.0f);
    } else {
        if (p.cell_sorted) {
            const unsigned u = (unsigned)packed;
            cs = make_int3((int)(u & cp.mx), (int)((u >> cp.by_shift) & cp.my), (int)((u >> cp.bz_shift) & cp.mz));
        } else {
            cs = slot_cell(p, cp, g, key_sorted, nullptr, s);
        }
        out = make_float4(clamp_offset(p, __fadd_rn(self.x, dx), cs.x, g.lox, g.hix),
                          clamp_offset(p, __fadd_rn(self.y, dy), cs.y, g.loy, g.hiy),
                          clamp_offset(p, __fadd_rn(self.z, dz), cs.z, g.loz, g.hiz), 0.0f);
    }
    xs_out[s] = out;
    if (v_out) {
        float4 xo = x[p.src ? __ldg(&p.src[s]) : s];  // the committed position, unsorted when src is set
        if (!MIXED && p.frame) {  // the committed state is cell + offset: into the scene frame
            const int3 co = unpack_cell(cp, xo.w);
            xo = make_float4(__fmaf_rn((float)co.x, p.cell, xo.x), __fmaf_rn((float)co.y, p.cell, xo.y),
                             __fmaf_rn((float)co.z, p.cell, xo.z), 0.0f);
        }
        float3 d = make_float3(__fsub_rn(out.x, xo.x), __fsub_rn(out.y, xo.y), __fsub_rn(out.z, xo.z));
        if (MIXED) {
            int3 co = unpack_cell(cp, xo.w);
            d.x = __fmaf_rn((float)(cs.x - co.x), p.cell, d.x);
            d.y = __fmaf_rn((float)(cs.y - co.y), p.cell, d.y);
            d.z = __fmaf_rn((float)(cs.z - co.z), p.cell, d.z);
        }
        v_out[s] = make_float4(__fmul_rn(d.x, p.inv_dt), __fmul_rn(d.y, p.inv_dt), __fmul_rn(d.z, p.inv_dt), 0.0f);
    }
}

// With one particle per thread and up to 2 gathers in flight the kernel
// fits 40 registers without spilling: 6 blocks of 256 threads per SM instead
// of 5 (a 262,144-particle pass then takes 1.12 waves of the GPU instead of
// 1.35).  Compact lists with one gather in flight fit 32 registers without
// spilling (their steps have an integer s_corr exponent: no powf): 16 blocks
// of 128 threads per SM, the whole SM's warps.  P = 2:
// two particles per thread (B apart), their lists walked together.
template <int F, int U, int B, int P = 1>
__global__ void __launch_bounds__(B, ((F & 8) && U == 1) ? 2048 / B : ((U <= 2 && P == 1) ? 1536 / B : 1))
    k_delta(StepParams p, CellPack cp, const float4* __restrict__ xs, float4* __restrict__ xs_out,
            const int* __restrict__ nbr, const int* __restrict__ cnt, const float4* __restrict__ solid,
            const int* __restrict__ key_sorted, const float4* __restrict__ x, float4* __restrict__ v_out) {
    constexpr bool MIXED = (F & 1) != 0, SOL = (F & 2) != 0, COMPACT = (F & 8) != 0, WIDE = (F & 16) != 0;
    static_assert(!COMPACT || (!MIXED && !SOL && P == 1), "compact lists");
    pdl_wait();
    __shared__ float4 shift_tab[MIXED ? 64 : 1];
    if (MIXED) fill_shift_table(p, shift_tab);
    if (P == 1) {
        const int s = blockIdx.x * blockDim.x + threadIdx.x;
        if (s >= p.n) return;
        const float4 self = xs[s];
        const uint4 rec = COMPACT ? __ldg(&p.rec[s]) : make_uint4(0u, 0u, 0u, 0u);
        const int scene = (COMPACT && !WIDE) ? scene_of_record(p, rec.x) : scene_index(p, s);
        const int packed = (MIXED && p.cell_sorted) ? __ldg(&p.cell_sorted[s]) : 0;
        DeltaAcc a{0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0};
        if (COMPACT) {
            walk_compact<U, WIDE, float4>(
                p, rec, p.rec2 + s, nbr + s, [&](int t) { return xs[t]; },
                [&](int t, float4 q) { delta_pair<false, false, false>(p, a, self, t, q, shift_tab); });
        } else {
            for_each_entry<U, SOL, LIST_PAD_MAX>(p, nbr + s, cnt, s, xs, solid, [&](int e, float4 q) {
                delta_pair<MIXED, SOL>(p, a, self, e, q, shift_tab);
            });
        }
        delta_finish<MIXED>(p, cp, s, self, a, xs_out, key_sorted, x, v_out, scene, packed);
        return;
    }
    int s[P], c[P];
    float4 self[P];
    DeltaAcc a[P];
#pragma unroll
    for (int r = 0; r < P; r++) {
        s[r] = (blockIdx.x * P + r) * B + threadIdx.x;
        const bool ok = s[r] < p.n;
        c[r] = ok ? __ldg(&cnt[s[r]]) : 0;
        self[r] = ok ? xs[s[r]] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        a[r] = DeltaAcc{0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0};
    }
    for_each_entry_p<U, P, SOL>(p, nbr, s, c, xs, solid, [&](int r, int e, float4 q) {
        delta_pair<MIXED, SOL>(p, a[r], self[r], e, q, shift_tab);
    });
#pragma unroll
    for (int r = 0; r < P; r++)
        if (s[r] < p.n)
            delta_finish<MIXED>(p, cp, s[r], self[r], a[r], xs_out, key_sorted, x, v_out, scene_index(p, s[r]),
                                (MIXED && p.cell_sorted) ? __ldg(&p.cell_sorted[s[r]]) : 0);
}

// A neighbour's predicted position and velocity (the XSPH gathers).
struct PosVel {
    float4 x, v;
};

// One XSPH pair: a += (v_j - v_i) hd^3 (the sum is scaled by c K6 once).
template <bool MIXED>
__device__ __forceinline__ void xsph_pair(const StepParams& p, const float4& self, const float4& vi,
                                          const float4& q, const float4& vj, int e, const float4* tab, float& ax,
                                          float& ay, float& az) {
    float3 d = rel_t<MIXED>(self, q, e, tab);
    const float hd = hdiff(p, dot3e(d.x, d.y, d.z));
    const float w = __fmul_rn(__fmul_rn(hd, hd), hd);
    ax = __fmaf_rn(__fsub_rn(vj.x, vi.x), w, ax);
    ay = __fmaf_rn(__fsub_rn(vj.y, vi.y), w, ay);
    az = __fmaf_rn(__fsub_rn(vj.z, vi.z), w, az);
}

// XSPH viscosity (Macklin & Mueller eq. 17) and commit x = x*.
// With xs_next, also the next step's prediction from the state it commits
// (into xs_next, key, rank, count, cellk; count is zero here, the step's
// scan having consumed it).
template <int F, int U>
__device__ __forceinline__ void xsph_commit(const StepParams& p, const CellPack& cp, const float4* __restrict__ xs,
                                            const float4* __restrict__ v_in, const int* __restrict__ nbr,
                                            const int* __restrict__ cnt, const int* __restrict__ key_sorted,
                                            float4* __restrict__ x_out, float4* __restrict__ v_out,
                                            float4* __restrict__ xs_next, int* __restrict__ key,
                                            int* __restrict__ rank, int* __restrict__ count, int* __restrict__ cellk,
                                            int* __restrict__ tile_count) {
    constexpr bool MIXED = (F & 1) != 0, SOL = (F & 2) != 0, COMPACT = (F & 8) != 0, WIDE = (F & 16) != 0;
    static_assert(!COMPACT || (!MIXED && !SOL), "compact lists");
    pdl_wait();
    __shared__ float4 shift_tab[MIXED ? 64 : 1];
    if (MIXED) fill_shift_table(p, shift_tab);
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= p.n) return;
    const float4 self = xs[s];
    const float4 vi = v_in[s];
    const int* __restrict__ col = nbr + s;
    float ax = 0.0f, ay = 0.0f, az = 0.0f;
    if (COMPACT && p.c_xsph != 0.0f) {
        walk_compact<U, WIDE, PosVel>(
            p, __ldg(&p.rec[s]), p.rec2 + s, col, [&](int t) { return PosVel{xs[t], v_in[t]}; },
            [&](int t, const PosVel& q) { xsph_pair<false>(p, self, vi, q.x, q.v, t, shift_tab, ax, ay, az); });
    } else if (p.c_xsph != 0.0f) {
        const int c = cnt[s];
        const int sent = sentinel_entry(p);
        for (int k = 0; k < c; k += U) {
            int e[U];
            float4 q[U], vj[U];
#pragma unroll
            for (int u = 0; u < U; u++) {
                const int t = __ldg(&col[(size_t)(k + u) * p.n]);  // padded list: valid below roundup(c, U)
                e[u] = (SOL && entry_solid(t)) ? sent : t;  // solids take no part (the sentinel's zero term)
            }
#pragma unroll
            for (int u = 0; u < U; u++) {
                q[u] = xs[entry_slot(e[u])];
                vj[u] = v_in[entry_slot(e[u])];
            }
#pragma unroll
            for (int u = 0; u < U; u++) xsph_pair<MIXED>(p, self, vi, q[u], vj[u], e[u], shift_tab, ax, ay, az);
        }
    }
    // v += c sum (v_j - v_i) W, W = K6 hd^3
    const float cx = __fmul_rn(p.c_xsph, p.k6);
    const float4 vc = make_float4(__fmaf_rn(cx, ax, vi.x), __fmaf_rn(cx, ay, vi.y), __fmaf_rn(cx, az, vi.z), 0.0f);
    v_out[s] = vc;
    const Geo g = (COMPACT && !WIDE) ? geo_of(p, scene_of_record(p, __ldg(reinterpret_cast<const unsigned*>(p.rec + s))))
                                     : geo_slot(p, s);
    float4 xc;
    if (!MIXED && !p.frame) {
        xc = make_float4(self.x, self.y, self.z, 0.0f);
    } else {
        const int3 cs = slot_cell(p, cp, g, key_sorted, p.cell_sorted, s);
        if (MIXED)
            xc = make_float4(self.x, self.y, self.z, pack_cell(cp, cs.x, cs.y, cs.z));
        else  // scene frame: back to the offset from the step's cell
            xc = make_float4(__fsub_rn(self.x, __fmul_rn((float)cs.x, p.cell)),
                             __fsub_rn(self.y, __fmul_rn((float)cs.y, p.cell)),
                             __fsub_rn(self.z, __fmul_rn((float)cs.z, p.cell)), pack_cell(cp, cs.x, cs.y, cs.z));
    }
    x_out[s] = xc;
    if (xs_next) {
        if (MIXED || p.frame)
            predict_one<true>(p, cp, g, xc, vc, s, xs_next, key, rank, count, cellk, tile_count);
        else
            predict_one<false>(p, cp, g, xc, vc, s, xs_next, key, rank, count, cellk, tile_count);
    }
}

template <int F, int U, int B>
__global__ void __launch_bounds__(B) k_xsph(StepParams p, CellPack cp, const float4* __restrict__ xs,
                                            const float4* __restrict__ v_in,
                                            const int* __restrict__ nbr, const int* __restrict__ cnt,
                                            const int* __restrict__ key_sorted,
                                            float4* __restrict__ x_out, float4* __restrict__ v_out,
                                            float4* __restrict__ xs_next, int* __restrict__ key,
                                            int* __restrict__ rank, int* __restrict__ count,
                                            int* __restrict__ cellk, int* __restrict__ tile_count) {
    xsph_commit<F, U>(p, cp, xs, v_in, nbr, cnt, key_sorted, x_out, v_out, xs_next, key, rank, count, cellk,
                      tile_count);
}

// Compact lists (F = 8, 24) with one gather in flight: registers capped at 32
// for every warp slot of the SM (at most 16 bytes spilled; config 3 XSPH 0.175 ->
// 0.141 ms at step 5, 0.239 -> 0.219 ms at step 100 against the best
// uncapped shape).  More gathers in flight keep k_xsph.
template <int F, int U, int B>
__global__ void __launch_bounds__(B, 2048 / B) k_xsph_compact(
    StepParams p, CellPack cp, const float4* __restrict__ xs, const float4* __restrict__ v_in,
    const int* __restrict__ nbr, const int* __restrict__ cnt, const int* __restrict__ key_sorted,
    float4* __restrict__ x_out, float4* __restrict__ v_out, float4* __restrict__ xs_next, int* __restrict__ key,
    int* __restrict__ rank, int* __restrict__ count, int* __restrict__ cellk, int* __restrict__ tile_count) {
    xsph_commit<F, U>(p, cp, xs, v_in, nbr, cnt, key_sorted, x_out, v_out, xs_next, key, rank, count, cellk,
                      tile_count);
}

// ------------------------------------------------------------- launch shape --

static inline int blocks_for(int n, int t) { return (n + t - 1) / t; }

// Kernels templated on (F, U, B) are instantiated for F in {0..3} (mixed,
// solids), U in {1, 2, 4, 8} and B in {64, 128, 256}; the tuning and the
// scene pick one (TUNE_DISPATCH expands the switch).
#define TUNE_LAUNCH(KERNEL, MIX, U_, B_, N, ST, ...)                                            \
    launch_k(KERNEL<MIX, U_, B_>, blocks_for(N, B_), B_, ST, pdl_enabled(), __VA_ARGS__)
// two particles per thread (the lambda and delta-p passes), U in {1, 2}
#define TUNE_LAUNCH_P2(KERNEL, MIX, U_, B_, N, ST, ...)                                         \
    launch_k(KERNEL<MIX, U_, B_, 2>, blocks_for(N, 2 * B_), B_, ST, pdl_enabled(), __VA_ARGS__)
#define TUNE_BLOCKS_P2(KERNEL, MIX, U_, tu, N, ST, ...)                                         \
    do {                                                                                        \
        if (tu.block <= 64)                                                                     \
            TUNE_LAUNCH_P2(KERNEL, MIX, U_, 64, N, ST, __VA_ARGS__);                            \
        else if (tu.block <= 128)                                                               \
            TUNE_LAUNCH_P2(KERNEL, MIX, U_, 128, N, ST, __VA_ARGS__);                           \
        else                                                                                    \
            TUNE_LAUNCH_P2(KERNEL, MIX, U_, 256, N, ST, __VA_ARGS__);                           \
    } while (0)
#define TUNE_CASE_P2(KERNEL, MIX, tu, N, ST, ...)                                               \
    do {                                                                                        \
        if (tu.unroll <= 1)                                                                     \
            TUNE_BLOCKS_P2(KERNEL, MIX, 1, tu, N, ST, __VA_ARGS__);                             \
        else                                                                                    \
            TUNE_BLOCKS_P2(KERNEL, MIX, 2, tu, N, ST, __VA_ARGS__);                             \
    } while (0)
#define TUNE_DISPATCH_PPT(KERNEL, fcode, tu, N, ST, ...)                                        \
    do {                                                                                        \
        if (tu.ppt != 2) {                                                                      \
            TUNE_DISPATCH(KERNEL, fcode, tu, N, ST, __VA_ARGS__);                               \
            break;                                                                              \
        }                                                                                       \
        switch (fcode) {                                                                        \
            case 0: TUNE_CASE_P2(KERNEL, 0, tu, N, ST, __VA_ARGS__); break;                     \
            case 1: TUNE_CASE_P2(KERNEL, 1, tu, N, ST, __VA_ARGS__); break;                     \
            case 2: TUNE_CASE_P2(KERNEL, 2, tu, N, ST, __VA_ARGS__); break;                     \
            default: TUNE_CASE_P2(KERNEL, 3, tu, N, ST, __VA_ARGS__); break;                    \
        }                                                                                       \
    } while (0)
#define TUNE_BLOCKS(KERNEL, MIX, U_, tu, N, ST, ...)                                            \
    do {                                                                                        \
        if (tu.block <= 64)                                                                     \
            TUNE_LAUNCH(KERNEL, MIX, U_, 64, N, ST, __VA_ARGS__);                               \
        else if (tu.block <= 128)                                                               \
            TUNE_LAUNCH(KERNEL, MIX, U_, 128, N, ST, __VA_ARGS__);                              \
        else                                                                                    \
            TUNE_LAUNCH(KERNEL, MIX, U_, 256, N, ST, __VA_ARGS__);                              \
    } while (0)
#define TUNE_CASE(KERNEL, MIX, tu, N, ST, ...)                                                  \
    do {                                                                                        \
        if (tu.unroll <= 1)                                                                     \
            TUNE_BLOCKS(KERNEL, MIX, 1, tu, N, ST, __VA_ARGS__);                                \
        else if (tu.unroll == 2)                                                                \
            TUNE_BLOCKS(KERNEL, MIX, 2, tu, N, ST, __VA_ARGS__);                                \
        else if (tu.unroll == 4)                                                                \
            TUNE_BLOCKS(KERNEL, MIX, 4, tu, N, ST, __VA_ARGS__);                                \
        else                                                                                    \
            TUNE_BLOCKS(KERNEL, MIX, 8, tu, N, ST, __VA_ARGS__);                                \
    } while (0)
// fcode: bit 0 mixed (cell-relative pair offsets), bit 1 static particles,
// bit 2 (the lambda pass only) the scene frame's compensated sums, bit 3
// compact lists (with bit 2 at most), bit 4 their wide records
#define TUNE_DISPATCH(KERNEL, fcode, tu, N, ST, ...)                                            \
    do {                                                                                        \
        switch (fcode) {                                                                        \
            case 0: TUNE_CASE(KERNEL, 0, tu, N, ST, __VA_ARGS__); break;                        \
            case 1: TUNE_CASE(KERNEL, 1, tu, N, ST, __VA_ARGS__); break;                        \
            case 2: TUNE_CASE(KERNEL, 2, tu, N, ST, __VA_ARGS__); break;                        \
            default: TUNE_CASE(KERNEL, 3, tu, N, ST, __VA_ARGS__); break;                       \
        }                                                                                       \
    } while (0)
#define TUNE_DISPATCH_FRAME(KERNEL, fcode, tu, N, ST, ...)                                      \
    do {                                                                                        \
        if (fcode == 4) TUNE_CASE(KERNEL, 4, tu, N, ST, __VA_ARGS__);                           \
        else if (fcode == 6) TUNE_CASE(KERNEL, 6, tu, N, ST, __VA_ARGS__);                      \
        else TUNE_DISPATCH(KERNEL, fcode, tu, N, ST, __VA_ARGS__);                              \
    } while (0)


}  // namespace lgb
