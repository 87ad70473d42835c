// MagicaVoxel .vox files (versions 150 and 200) for the `vox` scene keyword.
//
// The format: "VOX ", a version, then a MAIN chunk whose children are a flat
// sequence of chunks, each a 4-byte id, the byte sizes of its content and of
// its children, then both. Used here: SIZE + XYZI (one pair per model:
// dimensions, then (x, y, z, palette index) bytes), RGBA (colours of palette
// indices 1..255), MATL (a string dictionary per palette index), and the scene
// graph nTRN / nGRP / nSHP that places models. The reference reads the same
// chunks (include/vox_loader.h:154-327); a model's cells are placed relative
// to its centre rounded down, and a file without a scene graph stands each
// model on z = 0 (vox_loader.h:287-299).
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "vox_reader.h"

namespace mypbr_host {

namespace {

// MagicaVoxel's default palette, for files without an RGBA chunk: index 0
// empty, then the 6 x 6 x 6 cube of channel levels 0xff, 0xcc, .., 0x00
// (red slowest, blue fastest) without black, then ten-step ramps of red,
// green, blue and grey (0xee, 0xdd, 0xbb, 0xaa, 0x88, 0x77, 0x55, 0x44, 0x22, 0x11).
void default_palette(V3 palette[256]) {
    int k = 0;
    palette[k++] = V3(0, 0, 0);
    const int levels[6] = {0xff, 0xcc, 0x99, 0x66, 0x33, 0x00};
    for (int r = 0; r < 6; r++)
        for (int g = 0; g < 6; g++)
            for (int b = 0; b < 6; b++) {
                if (r == 5 && g == 5 && b == 5)
                    continue;
                palette[k++] = V3(levels[r] / 255.0, levels[g] / 255.0, levels[b] / 255.0);
            }
    const int ramp[10] = {0xee, 0xdd, 0xbb, 0xaa, 0x88, 0x77, 0x55, 0x44, 0x22, 0x11};
    for (int channel = 0; channel < 4; channel++)
        for (int s = 0; s < 10; s++) {
            double v = ramp[s] / 255.0;
            palette[k++] = channel == 3 ? V3(v, v, v) : V3(channel == 0 ? v : 0, channel == 1 ? v : 0, channel == 2 ? v : 0);
        }
}

struct Reader {
    const uint8_t* p;
    const uint8_t* end;
    bool good = true;
    size_t left() const { return size_t(end - p); }
    int32_t i32() {
        if (left() < 4) {
            good = false;
            p = end;
            return 0;
        }
        uint32_t v = uint32_t(p[0]) | uint32_t(p[1]) << 8 | uint32_t(p[2]) << 16 | uint32_t(p[3]) << 24;
        p += 4;
        return int32_t(v);
    }
    std::string str() {
        int32_t n = i32();
        if (n < 0 || size_t(n) > left()) {
            good = false;
            p = end;
            return "";
        }
        std::string s(reinterpret_cast<const char*>(p), size_t(n));
        p += n;
        return s;
    }
    std::map<std::string, std::string> dict() {
        std::map<std::string, std::string> d;
        int32_t n = i32();
        for (int32_t k = 0; k < n && good; k++) {
            std::string key = str();
            d[key] = str();
        }
        return d;
    }
};

// The signed permutation of a ROTATION byte: bits 0-1 and 2-3 give the
// columns of the non-zero entries of rows 0 and 1 (row 2 takes the remaining
// column), bits 4, 5, 6 their signs.
Xf rotation_byte(int r) {
    int c0 = r & 3, c1 = (r >> 2) & 3, c2 = 3 - c0 - c1;
    Xf x;
    double m[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    if (c0 < 3 && c1 < 3 && c2 >= 0 && c2 < 3) {
        m[0][c0] = (r & 16) ? -1 : 1;
        m[1][c1] = (r & 32) ? -1 : 1;
        m[2][c2] = (r & 64) ? -1 : 1;
    } else {
        m[0][0] = m[1][1] = m[2][2] = 1;
    }
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            x.m[i][j] = m[i][j];
            x.inv_m[j][i] = m[i][j];  // orthogonal: the inverse is the transpose
        }
    return x;
}

int to_int(const std::string& s, int fallback) {
    try {
        return std::stoi(s);
    } catch (...) {
        return fallback;
    }
}

struct Node {
    char type = 0;
    bool hidden = false;
    std::vector<int> children, models;
    Xf xform;
};

}  // namespace

bool read_vox(const std::string& path, VoxFile& out, std::string& error) {
    std::ifstream file(path, std::ios::binary);
    if (!file) {
        error = "cannot open '" + path + "'";
        return false;
    }
    std::vector<uint8_t> bytes((std::istreambuf_iterator<char>(file)), std::istreambuf_iterator<char>());
    if (bytes.size() < 20 || std::memcmp(bytes.data(), "VOX ", 4) != 0) {
        error = "'" + path + "' is not a MagicaVoxel .vox file";
        return false;
    }
    default_palette(out.palette);
    std::map<int, Node> nodes;
    const uint8_t* p = bytes.data() + 8;
    const uint8_t* end = bytes.data() + bytes.size();
    if (end - p < 12 || std::memcmp(p, "MAIN", 4) != 0) {
        error = "'" + path + "' has no MAIN chunk";
        return false;
    }
    {
        Reader head{p + 4, p + 12};
        int32_t content = head.i32();
        p += 12 + std::max(content, 0);
    }
    int sx = 0, sy = 0, sz = 0;
    while (end - p >= 12) {
        std::string id(reinterpret_cast<const char*>(p), 4);
        Reader head{p + 4, p + 12};
        int32_t content = head.i32(), children = head.i32();
        if (content < 0 || children < 0 || size_t(content) + size_t(children) > size_t(end - p - 12)) {
            error = "'" + path + "' is truncated or corrupt (chunk " + id + ")";
            return false;
        }
        const uint8_t* body = p + 12;
        Reader in{body, body + content};
        p += 12 + size_t(content) + size_t(children);
        if (id == "SIZE") {
            sx = in.i32();
            sy = in.i32();
            sz = in.i32();
            if (sx <= 0 || sy <= 0 || sz <= 0 || sx > 2048 || sy > 2048 || sz > 2048) {
                error = "'" + path + "' has a model of invalid size";
                return false;
            }
        } else if (id == "XYZI") {
            if (sx <= 0) {
                error = "'" + path + "' has voxels before their SIZE";
                return false;
            }
            VoxModel m;
            m.nx = sx;
            m.ny = sy;
            m.nz = sz;
            m.cells.assign(size_t(sx) * sy * sz, 0);
            int32_t n = in.i32();
            if (n < 0 || size_t(n) * 4 > in.left()) {
                error = "'" + path + "' has a truncated voxel list";
                return false;
            }
            const uint8_t* v = in.p;
            for (int32_t k = 0; k < n; k++, v += 4)
                if (v[0] < sx && v[1] < sy && v[2] < sz)
                    m.cells[(size_t(v[2]) * sy + v[1]) * sx + v[0]] = v[3];
            out.models.push_back(std::move(m));
            sx = sy = sz = 0;
        } else if (id == "RGBA") {
            if (content < 1024) {
                error = "'" + path + "' has a short palette";
                return false;
            }
            for (int k = 0; k < 255; k++)
                out.palette[k + 1] = V3(body[4 * k] / 255.0, body[4 * k + 1] / 255.0, body[4 * k + 2] / 255.0);
        } else if (id == "MATL") {
            int index = in.i32();
            auto props = in.dict();
            if (in.good && index >= 0 && index < 256)
                out.materials[index] = props;
        } else if (id == "nTRN") {
            int nid = in.i32();
            auto attributes = in.dict();
            Node& t = nodes[nid];
            t.type = 'T';
            t.hidden = attributes["_hidden"] == "1";
            t.children.push_back(in.i32());
            in.i32();  // reserved
            in.i32();  // layer
            int frames = in.i32();
            if (frames > 0) {
                auto frame = in.dict();  // the first animation frame
                Xf rotation;
                if (frame.count("_r"))
                    rotation = rotation_byte(to_int(frame["_r"], 4));
                V3 offset;
                if (frame.count("_t")) {
                    std::istringstream xyz(frame["_t"]);
                    xyz >> offset.x >> offset.y >> offset.z;
                }
                t.xform = Xf::translate(offset).then_after(rotation);
            }
        } else if (id == "nGRP") {
            int nid = in.i32();
            auto attributes = in.dict();
            Node& g = nodes[nid];
            g.type = 'G';
            g.hidden = attributes["_hidden"] == "1";
            int n = in.i32();
            for (int k = 0; k < n && in.good; k++)
                g.children.push_back(in.i32());
        } else if (id == "nSHP") {
            int nid = in.i32();
            in.dict();
            Node& s = nodes[nid];
            s.type = 'S';
            int n = in.i32();
            if (n > 0) {
                s.models.push_back(in.i32());  // the first frame's model
                in.dict();
            }
        }
        if (!in.good) {
            error = "'" + path + "' has a corrupt " + id + " chunk";
            return false;
        }
    }
    if (out.models.empty()) {
        error = "'" + path + "' has no voxels";
        return false;
    }
    auto centered = [&](int model) {
        const auto& m = out.models[size_t(model)];
        return Xf::translate(V3(-(m.nx / 2), -(m.ny / 2), -(m.nz / 2)));
    };
    if (nodes.empty() || !nodes.count(0)) {
        for (int k = 0; k < int(out.models.size()); k++)
            out.instances.push_back({k, Xf::translate(V3(0, 0, out.models[size_t(k)].nz / 2)).then_after(centered(k))});
        return true;
    }
    std::vector<std::pair<int, Xf>> stack = {{0, Xf()}};
    std::vector<int> depth = {0};
    while (!stack.empty()) {
        auto [nid, xform] = stack.back();
        int d = depth.back();
        stack.pop_back();
        depth.pop_back();
        auto it = nodes.find(nid);
        if (it == nodes.end() || it->second.hidden || d > 64)
            continue;
        const Node& n = it->second;
        Xf here = n.type == 'T' ? xform.then_after(n.xform) : xform;
        for (int child : n.children) {
            stack.push_back({child, here});
            depth.push_back(d + 1);
        }
        for (int model : n.models)
            if (model >= 0 && model < int(out.models.size()))
                out.instances.push_back({model, here.then_after(centered(model))});
    }
    return true;
}

}  // namespace mypbr_host
