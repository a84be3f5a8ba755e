// pbf_compact.cu -- launchers of the PBF passes over compact neighbour lists
// (16-byte records of 16-bit scene-local entries, or wide records of 32-bit
// entries; see CompactLists and walk_compact in pbf_passes.cuh).  The
// kernels are the templates of pbf_passes.cuh with F bit 3 (compact) and bit
// 4 (wide records); this translation unit instantiates them, pbf_solver.cu
// the column-list ones.
#include "pbf_passes.cuh"

namespace lgb {

void launch_lists_compact(int B, const StepParams& p, const CellPack& cp, float4* xs, const int* key_sorted,
                          const int* cell_sorted, const int* fstart, const float4* solid, const int* solid_cell,
                          const int* sstart, int* nbr, int* cnt, float* rho, int* status, cudaStream_t st) {
    const bool pdl = pdl_enabled();
#define LGB_LISTS_C(H, FR, W, BB)                                                                     \
    launch_k(k_lists_compact<H, BB, FR, W>, blocks_for(p.n, BB), BB, st, pdl, p, cp, xs, key_sorted, \
             cell_sorted, fstart, solid, solid_cell, sstart, nbr, cnt, rho, status)
#define LGB_LISTS_CB(H, FR, W)                        \
    do {                                              \
        if (B == 64) LGB_LISTS_C(H, FR, W, 64);       \
        else if (B == 128) LGB_LISTS_C(H, FR, W, 128); \
        else LGB_LISTS_C(H, FR, W, 256);              \
    } while (0)
    if (p.frame && p.wide) LGB_LISTS_CB(false, true, true);
    else if (p.frame) LGB_LISTS_CB(false, true, false);
    else if (p.hash_bits && p.wide) LGB_LISTS_CB(true, false, true);
    else if (p.hash_bits) LGB_LISTS_CB(true, false, false);
    else if (p.wide) LGB_LISTS_CB(false, false, true);
    else LGB_LISTS_CB(false, false, false);
#undef LGB_LISTS_CB
#undef LGB_LISTS_C
}

// fcode of a compact pass: 8, | 16 for wide records; the lambda pass | 4 in
// the scene frame
static int compact_fcode(const StepParams& p) { return 8 | (p.wide ? 16 : 0); }

void launch_lambda_compact(const Tuning& tu, const StepParams& p, float4* xs, const int* nbr, const int* cnt,
                           const float4* solid, float* rho, cudaStream_t st) {
    switch (compact_fcode(p) | (p.frame ? 4 : 0)) {
        case 8: TUNE_CASE(k_lambda, 8, tu, p.n, st, p, xs, nbr, cnt, solid, rho); break;
        case 12: TUNE_CASE(k_lambda, 12, tu, p.n, st, p, xs, nbr, cnt, solid, rho); break;
        case 24: TUNE_CASE(k_lambda, 24, tu, p.n, st, p, xs, nbr, cnt, solid, rho); break;
        default: TUNE_CASE(k_lambda, 28, tu, p.n, st, p, xs, nbr, cnt, solid, rho); break;
    }
}

void launch_delta_compact(const Tuning& tu, const StepParams& p, const CellPack& cp, const float4* xs,
                          float4* xs_out, const int* nbr, const int* cnt, const float4* solid,
                          const int* key_sorted, const float4* x, float4* v_out, cudaStream_t st) {
    switch (compact_fcode(p)) {
        case 8: TUNE_CASE(k_delta, 8, tu, p.n, st, p, cp, xs, xs_out, nbr, cnt, solid, key_sorted, x, v_out); break;
        default: TUNE_CASE(k_delta, 24, tu, p.n, st, p, cp, xs, xs_out, nbr, cnt, solid, key_sorted, x, v_out); break;
    }
}

void launch_xsph_compact(const Tuning& tx, const StepParams& p, const CellPack& cp, const float4* xs,
                         const float4* v_in, const int* nbr, const int* cnt, const int* key_sorted, float4* x_out,
                         float4* v_out, float4* xs_next, int* key, int* rank, int* count, int* cellk,
                         int* tile_count, cudaStream_t st) {
    const int f = compact_fcode(p);
    if (tx.unroll <= 1) {  // the 32-register kernel, one gather in flight
        const int B = tx.block <= 64 ? 64 : (tx.block <= 128 ? 128 : 256);
#define LGB_XC(FF, BB)                                                                                  \
    launch_k(k_xsph_compact<FF, 1, BB>, blocks_for(p.n, BB), BB, st, pdl_enabled(), p, cp, xs, v_in, nbr, cnt, \
             key_sorted, x_out, v_out, xs_next, key, rank, count, cellk, tile_count)
#define LGB_XCB(FF)                        \
    do {                                   \
        if (B == 64) LGB_XC(FF, 64);       \
        else if (B == 128) LGB_XC(FF, 128); \
        else LGB_XC(FF, 256);              \
    } while (0)
        if (f == 8) LGB_XCB(8);
        else LGB_XCB(24);
#undef LGB_XCB
#undef LGB_XC
        return;
    }
    switch (f) {
        case 8: TUNE_CASE(k_xsph, 8, tx, p.n, st, p, cp, xs, v_in, nbr, cnt, key_sorted, x_out, v_out, xs_next, key,
                          rank, count, cellk, tile_count); break;
        default: TUNE_CASE(k_xsph, 24, tx, p.n, st, p, cp, xs, v_in, nbr, cnt, key_sorted, x_out, v_out, xs_next,
                           key, rank, count, cellk, tile_count); break;
    }
}

}  // namespace lgb
