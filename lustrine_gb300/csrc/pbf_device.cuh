// pbf_device.cuh -- device helpers of the PBF step shared by the per-stage
// kernels (pbf_solver.cu) and the on-chip scene solve (pbf_scene_solve.cu):
// neighbour list entries, cell keys and buckets, the pair terms and the
// per-particle prediction.  Every kernel that includes them computes the same
// bits for the same inputs (explicit roundings, see the pair terms).
#pragma once

#include "pbf_common.cuh"

namespace lgb {

constexpr int SLOT_BITS = 25;
constexpr int SLOT_MASK = (1 << SLOT_BITS) - 1;

__device__ __forceinline__ int entry(int slot, int dx, int dy, int dz, bool solid) {
    return slot | ((dx + 1) << 25) | ((dy + 1) << 27) | ((dz + 1) << 29) | (solid ? (int)0x80000000u : 0);
}
__device__ __forceinline__ int entry_slot(int e) { return e & SLOT_MASK; }
__device__ __forceinline__ bool entry_solid(int e) { return e < 0; }
// Lists are padded to a multiple of StepParams::pad with entries of the
// sentinel slot n, a particle at (1e18, 1e18, 1e18) with zero velocity and
// lambda in every position and velocity array the passes gather from: every
// pair term with it is exactly zero (h^2 - r^2 and h - r clamp to 0), so the
// neighbour loops run whole chunks without per-entry checks.
__device__ __forceinline__ int sentinel_entry(const StepParams& p) { return entry(p.n, 0, 0, 0, false); }

// Bucket of a cell in a table of 2^bits buckets.  Cells are grouped in
// bricks of 4 (x) x 4 (y) x 8 (z); a brick starts at a hashed base
// (multiply-xorshift mix of its coordinates) and its 128 cells take the
// consecutive buckets after it (mod the table), so the sort keeps the
// particles of a brick together and a warp's particles stay neighbours.
__device__ __forceinline__ unsigned brick_base(int bx, int by, int bz, int bits) {
    unsigned h = ((unsigned)bx * 0x9E3779B1u) ^ ((unsigned)by * 0x85EBCA77u) ^ ((unsigned)bz * 0xC2B2AE3Du);
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 13;
    return h >> (32 - bits);
}
__device__ __forceinline__ int brick_bucket(unsigned base, int3 c, int bits) {
    const unsigned local = (unsigned)((((c.y & 3) << 2) | (c.x & 3)) << 3 | (c.z & 7));
    return (int)((base + local) & ((1u << bits) - 1u));
}
__device__ __forceinline__ int cell_bucket(int3 c, int bits) {
    return brick_bucket(brick_base(c.x >> 2, c.y >> 2, c.z >> 3, bits), c, bits);
}

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

// Grid and box of the scene a particle belongs to: the step's own for one
// scene, the batch table's entry otherwise.
struct Geo {
    int gx, gy, gz, off;
    float lox, loy, loz, hix, hiy, hiz;
    int slot0;  // first fluid slot of the scene
};

__device__ __forceinline__ Geo geo_single(const StepParams& p) {
    return Geo{p.gx, p.gy, p.gz, 0, p.lox, p.loy, p.loz, p.hix, p.hiy, p.hiz, 0};
}

__device__ __forceinline__ Geo geo_scene(const StepParams& p, int scene) {
    const SceneInfo si = p.scenes[scene];
    return Geo{si.gx, si.gy, si.gz, si.cell_off, si.lox, si.loy, si.loz, si.hix, si.hiy, si.hiz, si.slot0};
}

// Slot of a compact list's 16-bit entry v (record base: the scene's first slot).
__device__ __forceinline__ int compact_slot(const StepParams& p, int base, unsigned v) {
    return v == COMPACT_SENTINEL ? p.n : base + (int)v;
}

// geometry of fluid slot s (slots of a scene are a fixed range)
__device__ __forceinline__ Geo geo_slot(const StepParams& p, int s) {
    return p.scenes ? geo_scene(p, __ldg(&p.scene_of[s])) : geo_single(p);
}

// The scene of fluid slot s (0 for one scene), loaded ahead of its use, and
// the geometry from it.
__device__ __forceinline__ int scene_index(const StepParams& p, int s) {
    return p.scenes ? __ldg(&p.scene_of[s]) : 0;
}
// The scene of a slot whose 16-bit compact record starts with word rec_x
// (count | the scene's first slot << 8): scene_of at the scene's first slot,
// one address for all of a scene's particles (an L1 hit, where scene_of[s]
// streams 4 bytes a particle from DRAM).
__device__ __forceinline__ int scene_of_record(const StepParams& p, unsigned rec_x) {
    return p.scenes ? __ldg(&p.scene_of[rec_x >> 8]) : 0;
}
__device__ __forceinline__ Geo geo_of(const StepParams& p, int scene) {
    return p.scenes ? geo_scene(p, scene) : geo_single(p);
}

__device__ __forceinline__ int linear_cell(const Geo& g, int3 c) {
    return g.off + c.y * g.gx * g.gz + c.x * g.gz + c.z;
}

__device__ __forceinline__ int3 decode_cell(const Geo& g, int key) {
    const int slab = g.gx * g.gz;
    const int local = key - g.off;
    const int y = local / slab;
    const int r = local - y * slab;
    const int x = r / g.gz;
    return make_int3(x, y, r - x * g.gz);
}

__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }

__device__ __forceinline__ int3 plain_cell(const StepParams& p, const Geo& g, float x, float y, float z) {
    int cx = (int)floorf(__fmul_rn(x, p.inv_cell)), cy = (int)floorf(__fmul_rn(y, p.inv_cell)),
        cz = (int)floorf(__fmul_rn(z, p.inv_cell));
    return make_int3(min(max(cx, 0), g.gx - 1), min(max(cy, 0), g.gy - 1), min(max(cz, 0), g.gz - 1));
}

// One axis of the cell shift of an entry: the neighbour's cell is
// c_i + (bits - 1) on that axis, so (c_i - c_j) * cell = (1 - bits) * cell.
__device__ __forceinline__ float axis_shift(float cell, int e, int at) {
    const int b = (e >> at) & 3;
    return b == 1 ? 0.0f : (b == 0 ? cell : -cell);
}

// Mixed: the cell shift (c_i - c_j) * cell of every entry code (bits 25-30:
// the x, y, z codes d + 1), filled per block in shared memory so a pair
// reads its shift with one load.  All threads of the block call it.
__device__ __forceinline__ void fill_shift_table(const StepParams& p, float4* tab) {
    for (int k = threadIdx.x; k < 64; k += blockDim.x)
        tab[k] = make_float4(axis_shift(p.cell, k << 25, 25), axis_shift(p.cell, k << 25, 27),
                             axis_shift(p.cell, k << 25, 29), 0.0f);
    __syncthreads();
}

// x_i - x_j of a pair from the two stored positions and the list entry
// (mixed: plus the shift of its cell code from the block's table).
template <bool MIXED>
__device__ __forceinline__ float3 rel_t(float4 a, float4 b, int e, const float4* tab) {
    float3 d = make_float3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
    if (MIXED) {
        const float4 t = tab[(e >> 25) & 63];
        d.x = __fadd_rn(d.x, t.x);
        d.y = __fadd_rn(d.y, t.y);
        d.z = __fadd_rn(d.z, t.z);
    }
    return d;
}

// Pair terms.  Instruction issue takes much of the passes' time (61-73 % of
// the issue slots busy at config 3), so the pair loops keep only the
// r-dependent factors and the constants are applied once per particle:
//   poly6        W(r)  = K6 hd^3,            hd = max(h^2 - r^2, 0)
//   spiky        dW(d) = -Ks g d,            g  = max(h - r, 0)^2 / r
//   s_corr       -k (W(r) / W(dq))^n,        W(r) / W(dq) = (hd / (h^2 - dq^2))^3
// r and 1/r come from one reciprocal square root of max(r^2, 1e-30): at
// r = 0 the offset d is 0 and every pair term with it.
// The PBF arithmetic is written with explicit roundings (__fmaf_rn and
// friends): every instantiation of a kernel (precision, static particles,
// launch shape) and every kernel sharing a helper then computes the same
// bits, whatever multiply-adds the compiler would otherwise contract.
__device__ __forceinline__ float dot3e(float x, float y, float z) {
    return __fmaf_rn(z, z, __fmaf_rn(y, y, __fmul_rn(x, x)));
}

__device__ __forceinline__ float hdiff(const StepParams& p, float r2) { return fmaxf(__fsub_rn(p.h2, r2), 0.0f); }

__device__ __forceinline__ float inv_r_of(float r2) { return rsqrtf(fmaxf(r2, 1e-30f)); }

__device__ __forceinline__ float spiky_g(const StepParams& p, float r, float inv_r) {
    const float f = fmaxf(__fsub_rn(p.h, r), 0.0f);
    return __fmul_rn(__fmul_rn(f, f), inv_r);
}

// POW false: the exponent is an integer in [0, 32] (sn_int >= 0), and the
// powf branch is left out (inlined once per gather of an unrolled walk, its
// registers made the position pass over compact lists spill 100 bytes at 32
// registers although the default exponent, 4, never takes it).
template <bool POW = true>
__device__ __forceinline__ float scorr_hd(const StepParams& p, float hd) {
    const float x = __fmul_rn(hd, p.inv_hdq2);
    float pw;
    if (p.sn_int == 4) {  // (x^3)^4
        const float x2 = __fmul_rn(x, x), x4 = __fmul_rn(x2, x2);
        pw = __fmul_rn(__fmul_rn(x4, x4), x4);
    } else {
        const float t = __fmul_rn(__fmul_rn(x, x), x);
        if (!POW || p.sn_int >= 0) {
            pw = 1.0f;
            for (int e = 0; e < p.sn_int; e++) pw = __fmul_rn(pw, t);
        } else {
            pw = powf(t, p.sn);
        }
    }
    return __fmul_rn(-p.sk, pw);
}

__device__ __forceinline__ float4 load_entry(int e, const float4* __restrict__ xs,
                                             const float4* __restrict__ solid) {
    return entry_solid(e) ? __ldg(&solid[entry_slot(e)]) : xs[entry_slot(e)];
}

// Mixed: one axis of an (offset, cell) pair renormalised into [0, cell) and
// clamped to the box [lo, hi].
__device__ __forceinline__ void renorm_axis(const StepParams& p, float& o, int& c, float lo, float hi) {
    float k = floorf(__fmul_rn(o, p.inv_cell));
    if (k != 0.0f) {
        c += (int)k;
        o = __fmaf_rn(-k, p.cell, o);
        if (o >= p.cell) { o = __fsub_rn(o, p.cell); c += 1; }
        if (o < 0.0f) { o = __fadd_rn(o, p.cell); c -= 1; }
    }
    float a = __fmaf_rn((float)c, p.cell, o);
    if (a < lo || a > hi) {
        float t = clampf(a, lo, hi);
        int tc = (int)floorf(__fmul_rn(t, p.inv_cell));
        c = tc;
        o = __fmaf_rn(-(float)tc, p.cell, t);
    }
}

// Mixed: clamp an offset in a fixed cell so the absolute position is in [lo, hi].
__device__ __forceinline__ float clamp_offset(const StepParams& p, float o, int c, float lo, float hi) {
    const float base = __fmul_rn((float)c, p.cell);
    const float a = __fadd_rn(base, o);
    if (a < lo) return __fsub_rn(lo, base);
    if (a > hi) return __fsub_rn(hi, base);
    return o;
}

// ---------------------------------------------------------------- kernels --

__device__ __forceinline__ unsigned pack_bits(const CellPack& cp, int3 c) {
    return (unsigned)c.x | ((unsigned)c.y << cp.by_shift) | ((unsigned)c.z << cp.bz_shift);
}

// Sort key of a cell: its dense id, or its hash bucket.  The packed cell goes
// to cellk (when given): the hashed walk tells cells sharing a bucket apart by
// it, and mixed precision reads a slot's cell from it.
__device__ __forceinline__ int cell_key(const StepParams& p, const CellPack& cp, const Geo& g, int3 c,
                                        int* cellk, int i) {
    if (!p.hash_bits) {
        if (cellk) cellk[i] = (int)pack_bits(cp, c);
        return linear_cell(g, c);
    }
    // a static particle outside the box joins the last packable cell
    c = make_int3(min(c.x, (int)cp.mx), min(c.y, (int)cp.my), min(c.z, (int)cp.mz));
    cellk[i] = (int)pack_bits(cp, c);
    return cell_bucket(c, p.hash_bits);
}

// Prediction of one particle from its committed state: v' = v + g dt,
// x* = x + v' dt clamped to the box (mixed: renormalised into [0, cell) of a
// cell first), its cell key and its rank in the cell histogram.  Explicit
// fused multiply-adds keep the arithmetic identical wherever it is inlined:
// the prediction kernel and the commit kernel of the previous step (which
// predicts the next step when nothing changes in between) agree bit for bit.
// tile_count (may be null): the cell scan's per-tile totals, counted here
// with one atomic per tile a warp's particles fall in (slots are in cell
// order, so a warp's keys share a tile of CELL_TILE cells nearly always).
template <bool MIXED>
__device__ __forceinline__ void predict_one(const StepParams& p, const CellPack& cp, const Geo& g, float4 xi,
                                            float4 vi, int i, float4* __restrict__ xs, int* __restrict__ key,
                                            int* __restrict__ rank, int* __restrict__ count,
                                            int* __restrict__ cellk, int* __restrict__ tile_count) {
    vi.x = __fmaf_rn(p.gxv, p.dt, vi.x);
    vi.y = __fmaf_rn(p.gyv, p.dt, vi.y);
    vi.z = __fmaf_rn(p.gzv, p.dt, vi.z);
    int3 c;
    float4 s;
    if (!MIXED) {
        s = make_float4(clampf(__fmaf_rn(vi.x, p.dt, xi.x), g.lox, g.hix),
                        clampf(__fmaf_rn(vi.y, p.dt, xi.y), g.loy, g.hiy),
                        clampf(__fmaf_rn(vi.z, p.dt, xi.z), g.loz, g.hiz), 0.0f);
        c = plain_cell(p, g, s.x, s.y, s.z);
    } else {
        c = unpack_cell(cp, xi.w);
        float ox = __fmaf_rn(vi.x, p.dt, xi.x), oy = __fmaf_rn(vi.y, p.dt, xi.y), oz = __fmaf_rn(vi.z, p.dt, xi.z);
        renorm_axis(p, ox, c.x, g.lox, g.hix);
        renorm_axis(p, oy, c.y, g.loy, g.hiy);
        renorm_axis(p, oz, c.z, g.loz, g.hiz);
        // the scene frame: the position relative to the box corner
        s = p.frame ? make_float4(__fmaf_rn((float)c.x, p.cell, ox), __fmaf_rn((float)c.y, p.cell, oy),
                                  __fmaf_rn((float)c.z, p.cell, oz), 0.0f)
                    : make_float4(ox, oy, oz, 0.0f);
    }
    xs[i] = s;
    const int k = cell_key(p, cp, g, c, cellk, i);
    key[i] = k;
    rank[i] = atomicAdd(&count[k], 1);
    if (tile_count) {
        const int tile = k >> CELL_TILE_SHIFT;
        const unsigned peers = __match_any_sync(__activemask(), tile);
        if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&tile_count[tile], __popc(peers));
    }
}

// Neighbour search fused with the first lambda pass: walks the 27 cells
// around the particle's cell, writes the list and accumulates the density
// constraint over the accepted neighbours.  The particle itself is not in
// its list: its density term m W(0) starts the sum and it has no gradient.
struct LambdaAcc {
    float wsum, comp, S, gx, gy, gz;  // sum of hd^3 (compensated in mixed), sum g^2 r^2, sum g d
};

__device__ __forceinline__ LambdaAcc lambda_init(const StepParams&) {
    return LambdaAcc{0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
}

// KAHAN: compensated density sum (both mixed representations).  A term of
// exactly zero (a pair at r >= h, the sentinel entry that pads a chunk)
// leaves the compensated sum as it is: a compensation step with a zero
// addend would fold the carried error into the sum, so the result would
// depend on how many padding entries a walk visits.
template <bool KAHAN>
__device__ __forceinline__ void lambda_accumulate(const StepParams& p, LambdaAcc& a, float3 d,
                                                  bool solid) {
    const float r2 = dot3e(d.x, d.y, d.z);
    const float hd = hdiff(p, r2);
    const float w = __fmul_rn(__fmul_rn(hd, hd), hd);
    if (KAHAN) {
        const float y = __fsub_rn(w, a.comp);
        const float t = __fadd_rn(a.wsum, y);
        if (w != 0.0f) {
            a.comp = __fsub_rn(__fsub_rn(t, a.wsum), y);
            a.wsum = t;
        }
    } else {
        a.wsum = __fadd_rn(a.wsum, w);
    }
    const float inv_r = inv_r_of(r2);
    const float g = spiky_g(p, __fmul_rn(r2, inv_r), inv_r);
    if (!solid) a.S = __fmaf_rn(__fmul_rn(g, g), r2, a.S);
    a.gx = __fmaf_rn(g, d.x, a.gx);
    a.gy = __fmaf_rn(g, d.y, a.gy);
    a.gz = __fmaf_rn(g, d.z, a.gz);
}

// rho = m W(0) + m K6 sum hd^3
__device__ __forceinline__ float density_of(const StepParams& p, const LambdaAcc& a) {
    return __fmaf_rn(p.k6m, a.wsum, p.self_density);
}

// lambda = -(rho / rho0 - 1) / (S + eps), S = (Ks m / rho0)^2 (sum g^2 r^2 + |sum g d|^2),
// the two quotients as products by reciprocals (1 / rho0 from the host, one
// correctly rounded reciprocal): a rounding more each (~1e-7 relative) for
// a tenth fewer instructions in the lambda passes
__device__ __forceinline__ float lambda_of(const StepParams& p, const LambdaAcc& a) {
    const float S = __fmul_rn(p.lam_c2, __fadd_rn(a.S, dot3e(a.gx, a.gy, a.gz)));
    return __fmul_rn(-__fsub_rn(__fmul_rn(density_of(p, a), p.inv_rho0), 1.0f), __frcp_rn(__fadd_rn(S, p.eps)));
}

// Cell of fluid slot s in the current step: from its packed cell where the
// sort carried one (hashed grid, mixed precision), else from its dense key.
__device__ __forceinline__ int3 slot_cell(const StepParams& p, const CellPack& cp, const Geo& g,
                                          const int* __restrict__ key_sorted,
                                          const int* __restrict__ cell_sorted, int s) {
    if (cell_sorted) {
        const unsigned u = (unsigned)__ldg(&cell_sorted[s]);
        return make_int3((int)(u & cp.mx), (int)((u >> cp.by_shift) & cp.my), (int)((u >> cp.bz_shift) & cp.mz));
    }
    return decode_cell(g, __ldg(&key_sorted[s]));
}

}  // namespace lgb
