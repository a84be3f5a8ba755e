// pbf_common.cuh -- device-side types shared by the PBF kernels.
//
// Data layout in HBM (one scene, n fluid particles, ns static solids):
//   fluid state, structure of arrays in cell order (rebuilt every step):
//     x    float4[n]   committed positions  (w: packed cell in mixed precision)
//     xs   float4[n]   predicted positions, two copies for the Jacobi solve
//     v    float4[n]   velocities
//     id   int[n]      caller's particle id of each slot
//   cell table: count[C], start[C + 1] (exclusive scan of count)
//   solids: float4[ns] sorted by cell once at upload, sstart[C + 1]
//   neighbour lists: nbr[max_nbrs * n], column-major (entry k of slot i at
//     k * n + i) so a warp's loads of entry k are one coalesced line;
//     fluid neighbours are slot numbers >= 0, solids are -1 - solid slot.
//   compact lists (PBF mode, no static particles, no cell codes): rec
//     uint4[n], one 16-byte record per slot; rec2 uint4[n], a second record
//     for longer lists; the entries past both in the column-major rows of nbr
//     as plain slots.  Scenes of at most COMPACT_MAX_SCENE particles: the
//     count, the scene's first slot and 6 + 8 neighbours as 16-bit
//     scene-local slots; larger scenes (wide records): the count and 3 + 4
//     neighbours as 32-bit slots.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <utility>

namespace lgb {

// Device status bits, OR-ed into a status word instead of trapping.
enum : int {
    ST_NBR_OVERFLOW = 1,  // a neighbour list hit max_nbrs (list truncated)
    ST_CELL_RANGE = 2,    // compat mode: a cell id left the grid (clamped)
    ST_TIMEOUT = 4,       // a bounded wait gave up
    ST_BAD_VALUE = 8,     // a non-finite position was met
};

// One scene of a batch: its grid, the offset of its cells in the batch's
// cell numbering and its box.  The scenes' particles occupy fixed slot
// ranges (a scene's cells are contiguous in the global numbering, so the
// counting sort keeps every scene in its range).
struct SceneInfo {
    int gx, gy, gz, cell_off;
    float lox, loy, loz, hix, hiy, hiz;
    int slot0, spare;  // the scene's first fluid slot
};

// Compact neighbour lists (StepParams::rec, rec2): record.x = count | first
// slot of the particle's scene << 8; .y, .z, .w = entries 0-5 as 16-bit
// offsets from that slot, entry 2k in the low half, COMPACT_SENTINEL past the
// count (the sentinel slot n); the second record, entries 6-13 the same way.
constexpr int COMPACT_INLINE = 6;
constexpr int COMPACT_EXT = 8;
constexpr int COMPACT_RECORDS = COMPACT_INLINE + COMPACT_EXT;
// Wide records (StepParams::wide): record.x = count; .y, .z, .w = entries
// 0-2 as slots (the sentinel slot n past the count); the second record,
// entries 3-6.
constexpr int WIDE_INLINE = 3;
constexpr int WIDE_EXT = 4;
constexpr int WIDE_RECORDS = WIDE_INLINE + WIDE_EXT;
constexpr unsigned COMPACT_SENTINEL = 0xFFFFu;
constexpr int COMPACT_MAX_SCENE = 65535;   // scene-local offsets 0..65534
constexpr int COMPACT_MAX_N = 1 << 24;     // first slot in 24 bits
constexpr int COMPACT_MAX_NBRS = 255;      // count in 8 bits

// Everything a step kernel reads, passed by value (constant bank).
struct StepParams {
    // batches (nullptr for one scene): per-scene table, scene of each fluid
    // slot and of each solid slot
    const SceneInfo* scenes;
    const int* scene_of;
    const int* solid_scene_of;
    // hashed grid: packed cell of every sorted fluid slot (nullptr when dense)
    const int* cell_sorted;
    // per cell (bucket): whether a static particle lies in its 27-cell
    // neighbourhood (nullptr: no static particles)
    const unsigned char* solid_near;
    int n, ns;            // fluid, solid particle counts
    int gx, gy, gz;       // grid dims
    int num_cells;        // dense: cells; hashed: buckets (1 << hash_bits)
    int hash_bits;        // 0: dense cell grid; > 0: hashed grid of 2^hash_bits buckets
    int max_nbrs;
    int pad;              // PBF lists padded with sentinel entries to a multiple of pad (1, 2, 4, 8)
    int clamp_cells;      // compat mode: clamp cell coords per axis
    float cell, inv_cell;
    float h, h2;
    // reference (compat) cubic kernel, Kernels.cpp:6-41
    float kfac, cubic_k, cubic_l;
    // PBF kernels: poly6 K6 (h^2 - r^2)^3, spiky gradient -Ks (h - r)^2 d / r
    float k6, ks, inv_w_dq;
    float k6m;            // m K6
    float inv_hdq2;       // 1 / (h^2 - dq^2) (0 when dq >= h: no s_corr)
    float mass, rho0, eps;
    float mr;             // mass / rho0
    float lam_c2;         // (Ks mass / rho0)^2, the lambda denominator's factor
    float inv_rho0;       // 1 / rho0
    float self_density;   // m W(0) = m K6 h^6 (the particle's own density term)
    float inv_dt;
    float dq, sk, sn;     // s_corr distance, k and exponent
    int sn_int;           // exponent as an integer in [0, 32], or -1
    float c_xsph, contact;
    float gxv, gyv, gzv;  // gravity
    float lox, loy, loz, hix, hiy, hiz;  // box bounds for the position clamp
    float dt;
    int frame;            // mixed storage, iterations in the scene frame (LUSTRINE_PRECISION_MIXED_SCENE)
    uint4* rec;           // compact neighbour lists of this step (nullptr: column lists with counts)
    uint4* rec2;          // their second records
    int wide;             // compact lists in wide records (32-bit slots)
    const int* src;       // the previous slot of each sorted slot, whose committed position the last
                          // position pass reads from the unsorted state (nullptr: sorted with the step)
};

// Sand mode: simulate_sand's per-call inputs (Simulate.cpp:156-209).
struct SandParams {
    float px, py, pz;                       // player position
    int attract, blow, prev_attract;        // this call's flags and the previous call's attract flag
    float attract_radius, blow_radius;
    float attract_coeff, blow_coeff;
    float radius, diameter;                 // particleRadius, particleDiameter
    float w;                                // 1 / mass
};

// Launch shape of the PBF iteration kernels, chosen per scene by the autotuner.
struct Tuning {
    int block;        // threads per block of the lambda, delta and XSPH passes (64, 128, 256)
    int unroll;       // neighbour gathers in flight per thread of the lambda and delta passes (1, 2, 4, 8)
    int list_block;   // threads per block of the list build (64, 128, 256)
    int xsph_unroll;  // neighbour gathers in flight per thread of the XSPH pass (1, 2, 4, 8)
    int ppt;          // particles per thread of the lambda and delta passes (1, 2)
    int lists;        // 1: compact lists where the step allows them, 0: column lists
};

// Mixed precision: a cell's integer coordinates packed into 32 bits,
// x in the low bits, then y, then z.
struct CellPack {
    unsigned mx, my, mz;  // per-axis masks
    int by_shift, bz_shift;
};

__device__ __forceinline__ float dot3(float ax, float ay, float az) {
    return ax * ax + ay * ay + az * az;
}

// Programmatic dependent launch: a step kernel launched with programmatic
// stream serialisation may start while its predecessor drains; it waits
// here, before reading anything the predecessor wrote, until that grid has
// completed and its writes are visible.  It then lets its own successor
// launch: once every block of this grid has passed this point (all of them
// resident or done), the successor's blocks take the slots this grid's
// finished blocks free and wait in their own pdl_wait, so the successor's
// launch and ramp overlap this grid's tail.  Without the launch attribute
// both return at once.
__device__ __forceinline__ void pdl_wait() {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}

// Launch with programmatic stream serialisation allowed (when pdl is set).
template <typename... KArgs, typename... Args>
inline void launch_k(void (*kernel)(KArgs...), int grid, int block, cudaStream_t st, bool pdl,
                     Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// Whether the launchers of the calling thread use programmatic dependent
// launch (set by the context around a step's launches).
void set_pdl(bool on);
bool pdl_enabled();

// PBF neighbour lists: rows allocated = max_nbrs rounded up to LIST_PAD_MAX;
// the sentinel slot n sits at SENTINEL_POS on every axis.
constexpr int LIST_PAD_MAX = 8;
constexpr float SENTINEL_POS = 1e18f;

// Cell scan of the step: tiles of CELL_TILE cells, one block each.
constexpr int CELL_SCAN_THREADS = 256;
constexpr int CELL_SCAN_ITEMS = 16;
constexpr int CELL_TILE_SHIFT = 12;
constexpr int CELL_TILE = 1 << CELL_TILE_SHIFT;  // CELL_SCAN_THREADS * CELL_SCAN_ITEMS
constexpr int CELL_SCAN_MAX_TILES = 4096;         // 16.7 M cells

__device__ __forceinline__ void set_status(int* status, int bit) {
    if ((*(volatile int*)status & bit) == 0) atomicOr(status, bit);
}

// x^n for an integer n >= 0 evaluated in double and rounded once to float:
// the exact power of a float has at most 24 n significant bits, so for the
// small n used here the double product is within a few 2^-53 of it and the
// final rounding is the correctly rounded float (checked against a 113-bit
// evaluation over all floats in (1e-8, 1] for n = 3, 4).
__device__ __forceinline__ float ipow_rn(float x, int n) {
    double r = 1.0, b = (double)x;
    while (n) {
        if (n & 1) r *= b;
        b *= b;
        n >>= 1;
    }
    return (float)r;
}

}  // namespace lgb
