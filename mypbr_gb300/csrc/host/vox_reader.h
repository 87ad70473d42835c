// MagicaVoxel .vox reading for the host scene layer.
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "host_math.h"

namespace mypbr_host {

struct VoxModel {
    int nx = 0, ny = 0, nz = 0;
    std::vector<uint8_t> cells;  // x fastest, then y, then z; 0 = empty
    uint8_t at(int x, int y, int z) const {
        if (x < 0 || y < 0 || z < 0 || x >= nx || y >= ny || z >= nz)
            return 0;
        return cells[(size_t(z) * ny + y) * nx + x];
    }
};

struct VoxInstance {
    int model;
    Xf xform;  // model cells -> the file's z-up world
};

struct VoxFile {
    std::vector<VoxModel> models;
    std::vector<VoxInstance> instances;
    V3 palette[256];                                     // sRGB-encoded colours in [0, 1]
    std::map<std::string, std::string> materials[256];   // MATL properties per index
};

bool read_vox(const std::string& path, VoxFile& out, std::string& error);

}  // namespace mypbr_host
