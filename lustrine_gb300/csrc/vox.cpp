// vox.cpp -- MagicaVoxel (.vox) files as voxel grids: the first model of the
// file and its palette, the input of the wrapper's init_grid_magikavoxel and
// create_grid (LustrineWrapper.cpp:146-151, 537-624), which the reference
// reads through opengametools' ogt_vox (VoxelLoader.cpp:14-99).
//
// The format (MagicaVoxel's published file description): "VOX " and a
// version (150 or 200), then chunks, each an id of four characters, the byte sizes of its
// content and of its children, the content and the children.  MAIN holds all
// other chunks as children; SIZE (three int32: x, y, z) precedes each XYZI
// (int32 count, then count x, y, z, colour-index bytes); RGBA holds 256
// colours, colour index c (1..255) naming entry c - 1.  Chunks this reader
// does not use (PACK, the scene graph, materials, layers, ...) are skipped.
// As in the reference's reader, the model used is the first one with at
// least one voxel, a voxel listed twice keeps its last colour, and a file
// without an RGBA chunk uses MagicaVoxel's default palette -- which this
// reader does not carry: such a file, and one with an index map (IMAP),
// which reorders colour indices, is reported as unsupported.
#include "vox.h"

#include <cstdio>
#include <cstring>

namespace lgb {
namespace {

inline uint32_t le32(const uint8_t* p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

inline bool is_id(const uint8_t* p, const char* id) { return std::memcmp(p, id, 4) == 0; }

}  // namespace

int vox_parse(const uint8_t* b, size_t n, VoxModel* out) {
    *out = VoxModel();
    if (n < 8 || !is_id(b, "VOX ")) return LUSTRINE_ERR_ARGS;
    const uint32_t version = le32(b + 4);
    if (version != 150 && version != 200) return LUSTRINE_ERR_ARGS;  // the versions the reference reads
    size_t pos = 8;
    uint32_t sx = 0, sy = 0, sz = 0;
    bool have_model = false, have_palette = false, index_map = false;
    while (pos + 12 <= n) {
        const uint8_t* h = b + pos;
        const size_t content = le32(h + 4);
        pos += 12;
        if (is_id(h, "MAIN")) continue;  // its children are the chunks that follow
        const size_t end = content <= n - pos ? pos + content : n;
        const uint8_t* c = b + pos;
        const size_t len = end - pos;
        if (is_id(h, "SIZE")) {
            if (len < 12) return LUSTRINE_ERR_ARGS;
            sx = le32(c);
            sy = le32(c + 4);
            sz = le32(c + 8);
        } else if (is_id(h, "XYZI") && len >= 4 && !have_model) {
            const uint32_t count = le32(c);
            if (count > 0) {
                if (sx == 0 || sy == 0 || sz == 0 || (unsigned long long)sx * sy * sz > (1ull << 30))
                    return LUSTRINE_ERR_ARGS;
                out->sx = (int)sx;
                out->sy = (int)sy;
                out->sz = (int)sz;
                out->voxels.assign((size_t)sx * sy * sz, 0);
                const size_t avail = (len - 4) / 4;
                const size_t m = count < avail ? count : avail;
                for (size_t k = 0; k < m; k++) {
                    const uint8_t* v = c + 4 + 4 * k;
                    if (v[0] < sx && v[1] < sy && v[2] < sz)
                        out->voxels[(size_t)v[0] + (size_t)v[1] * sx + (size_t)v[2] * sx * sy] = v[3];
                }
                have_model = true;
            }
        } else if (is_id(h, "RGBA") && len >= 1024) {
            std::memcpy(out->rgba, c, 1024);
            have_palette = true;
        } else if (is_id(h, "IMAP")) {
            index_map = true;
        }
        pos = end;
    }
    if (!have_model) return LUSTRINE_ERR_ARGS;
    if (!have_palette || index_map) return LUSTRINE_ERR_UNSUPPORTED;
    return LUSTRINE_OK;
}

int vox_read_file(const char* path, VoxModel* out) {
    std::FILE* f = path ? std::fopen(path, "rb") : nullptr;
    if (!f) return LUSTRINE_ERR_ARGS;
    std::vector<uint8_t> buf;
    uint8_t chunk[1 << 16];
    size_t got;
    while ((got = std::fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + got);
    std::fclose(f);
    return vox_parse(buf.data(), buf.size(), out);
}

}  // namespace lgb
