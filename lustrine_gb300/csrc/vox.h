// vox.h -- reading the first model of a MagicaVoxel (.vox) file (vox.cpp).
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

#include "lustrine_gb300.h"

namespace lgb {

struct VoxModel {
    int sx = 0, sy = 0, sz = 0;
    std::vector<uint8_t> voxels;  // colour index of voxel (x, y, z) at x + y sx + z sx sy; 0: empty
    uint8_t rgba[256][4] = {};    // the file's RGBA chunk: colour index c names rgba[c - 1]
};

// LUSTRINE_OK, LUSTRINE_ERR_ARGS (not a .vox file, no model with a voxel),
// LUSTRINE_ERR_UNSUPPORTED (no RGBA chunk, or an index map); the model is
// filled in the last case too.
int vox_parse(const uint8_t* data, size_t size, VoxModel* out);
int vox_read_file(const char* path, VoxModel* out);

}  // namespace lgb
