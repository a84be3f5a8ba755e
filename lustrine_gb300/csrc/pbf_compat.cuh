// pbf_compat.cuh -- the reference's cell mapping, shared by the
// reference-semantics steps (fluid, pbf_compat.cu; sand, sand.cu).  Both are
// compiled with --fmad=false.
#pragma once

#include "pbf_common.cuh"

namespace lgb {

// get_cell_id (Utils.hpp:24-33): truncating division per axis; optional clamp.
__device__ __forceinline__ int cell_ref(const StepParams& p, float x, float y, float z, int* status) {
    int cx = (int)(x / p.cell);
    int cy = (int)(y / p.cell);
    int cz = (int)(z / p.cell);
    if (p.clamp_cells) {
        cx = min(max(cx, 0), p.gx - 1);
        cy = min(max(cy, 0), p.gy - 1);
        cz = min(max(cz, 0), p.gz - 1);
    }
    long long id = (long long)cy * p.gx * p.gz + (long long)cx * p.gz + cz;
    if (id < 0 || id >= p.num_cells) {
        // The reference writes past its cell table here; record it and clamp.
        cx = min(max(cx, 0), p.gx - 1);
        cy = min(max(cy, 0), p.gy - 1);
        cz = min(max(cz, 0), p.gz - 1);
        id = (long long)cy * p.gx * p.gz + (long long)cx * p.gz + cz;
        set_status(status, ST_CELL_RANGE);
    }
    return (int)id;
}

}  // namespace lgb
