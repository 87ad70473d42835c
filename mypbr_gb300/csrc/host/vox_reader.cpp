// MagicaVoxel .vox files (versions 150 and 200) for the `vox` scene keyword.
//
// A file is "VOX ", a version, then a MAIN chunk. Every chunk is a 4-byte id,
// the byte sizes of its content and of its children, then both; MAIN's
// children are read as one flat run of chunks (the children of those are
// skipped). This reader works in three steps:
//
//   1. index   split the run into (id, content span) records, checking that
//              every record fits in the file;
//   2. decode  hand each record to the handler its id names in a table
//              (SIZE + XYZI: a model's dimensions, then its (x, y, z, palette
//              index) bytes; RGBA: colours of palette indices 1..255; MATL: a
//              string dictionary per palette index; nTRN / nGRP / nSHP: the
//              scene graph). Unknown ids are skipped;
//   3. place   flatten the scene graph into model instances.
//
// What must agree with the reference's reader (vox_loader.h:154-327), since
// the same files have to give the same models, instances and light order: the
// error messages; a model's cells placed relative to its centre rounded down;
// a file without a scene graph (or without node 0) standing each model on
// z = 0; graph nodes keyed by id (a repeated id adds to the same node);
// hidden nodes and everything under them left out; placement depth-limited
// to 64 levels; instances listed in the order of a depth-first walk that
// takes a node's own models first and its children last to first.
//
// One deliberate difference: a ROTATION byte whose two packed column indices
// do not name a permutation (equal columns, or column 3) is read as no
// rotation; the reference then writes outside its 3 x 3 matrix.
#include <cstring>
#include <fstream>
#include <functional>
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

using Bytes = std::vector<uint8_t>;

// Little-endian 32-bit word at byte offset `at` (the caller checked the range).
int32_t word_at(const Bytes& b, size_t at) {
    uint32_t v = 0;
    for (int k = 3; k >= 0; k--)
        v = (v << 8) | b[at + size_t(k)];
    return int32_t(v);
}

// Reads the values of one chunk's content. A read past the content's end
// returns 0 or an empty string and marks the cursor failed, after which it
// stays at the end: the chunk is then reported corrupt.
class ContentCursor {
  public:
    ContentCursor(const Bytes& b, size_t begin, size_t size) : bytes_(b), at_(begin), stop_(begin + size) {}

    bool failed() const { return failed_; }
    size_t remaining() const { return stop_ - at_; }
    size_t offset() const { return at_; }

    int32_t word() {
        if (remaining() < 4)
            return fail(), 0;
        int32_t v = word_at(bytes_, at_);
        at_ += 4;
        return v;
    }

    std::string text() {
        int32_t length = word();
        if (length < 0 || size_t(length) > remaining())
            return fail(), std::string();
        std::string s(reinterpret_cast<const char*>(bytes_.data() + at_), size_t(length));
        at_ += size_t(length);
        return s;
    }

    // A DICT: a count, then that many (key, value) strings; a repeated key
    // keeps its last value.
    std::map<std::string, std::string> pairs() {
        std::map<std::string, std::string> out;
        int32_t count = word();
        for (int32_t k = 0; k < count && !failed_; k++) {
            std::string key = text();
            std::string value = text();
            out[key] = value;
        }
        return out;
    }

  private:
    void fail() {
        failed_ = true;
        at_ = stop_;
    }
    const Bytes& bytes_;
    size_t at_, stop_;
    bool failed_ = false;
};

struct ChunkRecord {
    std::string id;
    size_t content = 0, size = 0;  // offset and length of its own content
};

struct GraphNode {
    char kind = 0;  // 'T' transform, 'G' group, 'S' shape
    bool hidden = false;
    std::vector<int> children;
    std::vector<int> models;
    Xf local;  // transform nodes: the first animation frame
};

// A signed permutation from a ROTATION byte: bits 0-1 and 2-3 are the
// columns of rows 0 and 1, row 2 takes the column left over, bits 4, 5 and 6
// negate rows 0, 1 and 2.
Xf rotation_from(int packed) {
    int col[3] = {packed & 3, (packed >> 2) & 3, 0};
    col[2] = 3 - col[0] - col[1];
    bool permutation = col[0] < 3 && col[1] < 3 && col[0] != col[1];
    Xf x;
    if (!permutation)
        return x;
    for (int row = 0; row < 3; row++) {
        double sign = (packed >> (4 + row)) & 1 ? -1.0 : 1.0;
        for (int c = 0; c < 3; c++) {
            x.m[row][c] = c == col[row] ? sign : 0.0;
            x.inv_m[c][row] = x.m[row][c];  // orthogonal: the inverse is the transpose
        }
    }
    return x;
}

int leading_int(const std::string& s, int otherwise) {
    try {
        return std::stoi(s);
    } catch (...) {
        return otherwise;
    }
}

V3 three_numbers(const std::string& s) {
    V3 v;
    std::istringstream in(s);
    in >> v.x >> v.y >> v.z;
    return v;
}

// What the decode step builds up.
struct Decoder {
    VoxFile& out;
    std::map<int, GraphNode> graph;
    int pending[3] = {0, 0, 0};  // the last SIZE, until its XYZI comes
    std::string problem;         // the first error, without the file's name

    void on_size(ContentCursor& in) {
        for (int& n : pending)
            n = in.word();
        for (int n : pending)
            if (n <= 0 || n > 2048) {
                problem = "has a model of invalid size";
                return;
            }
    }

    void on_voxels(ContentCursor& in, const Bytes& bytes) {
        if (pending[0] <= 0) {
            problem = "has voxels before their SIZE";
            return;
        }
        VoxModel m;
        m.nx = pending[0];
        m.ny = pending[1];
        m.nz = pending[2];
        m.cells.assign(size_t(m.nx) * m.ny * m.nz, 0);
        int32_t count = in.word();
        if (count < 0 || size_t(count) * 4 > in.remaining()) {
            problem = "has a truncated voxel list";
            return;
        }
        for (size_t at = in.offset(), stop = at + size_t(count) * 4; at < stop; at += 4) {
            const uint8_t* v = bytes.data() + at;
            if (v[0] < m.nx && v[1] < m.ny && v[2] < m.nz)
                m.cells[(size_t(v[2]) * m.ny + v[1]) * m.nx + v[0]] = v[3];
        }
        out.models.push_back(std::move(m));
        pending[0] = pending[1] = pending[2] = 0;
    }

    void on_palette(const ChunkRecord& c, const Bytes& bytes) {
        if (c.size < 1024) {
            problem = "has a short palette";
            return;
        }
        for (int k = 1; k < 256; k++) {
            const uint8_t* rgba = bytes.data() + c.content + 4 * size_t(k - 1);
            out.palette[k] = V3(rgba[0] / 255.0, rgba[1] / 255.0, rgba[2] / 255.0);
        }
    }

    void on_material(ContentCursor& in) {
        int index = in.word();
        auto props = in.pairs();
        if (!in.failed() && index >= 0 && index < 256)
            out.materials[index] = std::move(props);
    }

    void on_transform(ContentCursor& in) {
        GraphNode& n = graph[in.word()];
        n.kind = 'T';
        n.hidden = in.pairs()["_hidden"] == "1";
        n.children.push_back(in.word());
        in.word();  // reserved
        in.word();  // layer
        if (in.word() <= 0)
            return;  // no frames
        auto frame = in.pairs();
        Xf turn = frame.count("_r") ? rotation_from(leading_int(frame["_r"], 4)) : Xf();
        V3 shift = frame.count("_t") ? three_numbers(frame["_t"]) : V3();
        n.local = Xf::translate(shift).then_after(turn);
    }

    void on_group(ContentCursor& in) {
        GraphNode& n = graph[in.word()];
        n.kind = 'G';
        n.hidden = in.pairs()["_hidden"] == "1";
        int32_t count = in.word();
        for (int32_t k = 0; k < count && !in.failed(); k++)
            n.children.push_back(in.word());
    }

    void on_shape(ContentCursor& in) {
        GraphNode& n = graph[in.word()];
        in.pairs();
        n.kind = 'S';
        if (in.word() > 0) {
            n.models.push_back(in.word());  // the first frame's model
            in.pairs();
        }
    }
};

// Step 1: the flat run of chunks under MAIN. A record that does not fit ends
// the run; its message goes to `tail` and is reported only if the records
// before it decode without an error of their own (the order a reader that
// decodes as it walks would report them in).
bool index_chunks(const Bytes& bytes, std::vector<ChunkRecord>& chunks, std::string& problem, std::string& tail) {
    const size_t total = bytes.size();
    size_t at = 8;  // past "VOX " and the version
    if (total - at < 12 || std::memcmp(bytes.data() + at, "MAIN", 4) != 0) {
        problem = "has no MAIN chunk";
        return false;
    }
    int32_t main_content = word_at(bytes, at + 4);
    at += 12 + size_t(main_content > 0 ? main_content : 0);
    while (at <= total && total - at >= 12) {
        ChunkRecord c;
        c.id.assign(reinterpret_cast<const char*>(bytes.data() + at), 4);
        int32_t content = word_at(bytes, at + 4), children = word_at(bytes, at + 8);
        if (content < 0 || children < 0 || size_t(content) + size_t(children) > total - at - 12) {
            tail = "is truncated or corrupt (chunk " + c.id + ")";
            break;
        }
        c.content = at + 12;
        c.size = size_t(content);
        chunks.push_back(c);
        at += 12 + size_t(content) + size_t(children);
    }
    return true;
}

// Step 3: instances from the scene graph (or one per model without one).
void place(const std::map<int, GraphNode>& graph, VoxFile& out) {
    auto about_centre = [&](int model) {
        const VoxModel& m = out.models[size_t(model)];
        return Xf::translate(V3(-(m.nx / 2), -(m.ny / 2), -(m.nz / 2)));
    };
    if (!graph.count(0)) {
        for (int k = 0; k < int(out.models.size()); k++) {
            V3 lift(0, 0, out.models[size_t(k)].nz / 2);
            out.instances.push_back({k, Xf::translate(lift).then_after(about_centre(k))});
        }
        return;
    }
    std::function<void(int, const Xf&, int)> visit = [&](int id, const Xf& parent, int level) {
        auto found = graph.find(id);
        if (found == graph.end() || found->second.hidden || level > 64)
            return;
        const GraphNode& n = found->second;
        Xf here = n.kind == 'T' ? parent.then_after(n.local) : parent;
        for (int model : n.models)
            if (model >= 0 && model < int(out.models.size()))
                out.instances.push_back({model, here.then_after(about_centre(model))});
        for (auto child = n.children.rbegin(); child != n.children.rend(); ++child)
            visit(*child, here, level + 1);
    };
    visit(0, Xf(), 0);
}

}  // namespace

bool read_vox(const std::string& path, VoxFile& out, std::string& error) {
    auto fail = [&](const std::string& what) {
        error = "'" + path + "' " + what;
        return false;
    };
    std::ifstream file(path, std::ios::binary);
    if (!file) {
        error = "cannot open '" + path + "'";
        return false;
    }
    Bytes bytes((std::istreambuf_iterator<char>(file)), std::istreambuf_iterator<char>());
    if (bytes.size() < 20 || std::memcmp(bytes.data(), "VOX ", 4) != 0)
        return fail("is not a MagicaVoxel .vox file");
    default_palette(out.palette);

    std::vector<ChunkRecord> chunks;
    std::string problem, tail;
    if (!index_chunks(bytes, chunks, problem, tail))
        return fail(problem);

    Decoder d{out, {}, {0, 0, 0}, {}};
    using Handler = std::function<void(const ChunkRecord&, ContentCursor&)>;
    const std::map<std::string, Handler> handlers = {
        {"SIZE", [&](const ChunkRecord&, ContentCursor& in) { d.on_size(in); }},
        {"XYZI", [&](const ChunkRecord&, ContentCursor& in) { d.on_voxels(in, bytes); }},
        {"RGBA", [&](const ChunkRecord& c, ContentCursor&) { d.on_palette(c, bytes); }},
        {"MATL", [&](const ChunkRecord&, ContentCursor& in) { d.on_material(in); }},
        {"nTRN", [&](const ChunkRecord&, ContentCursor& in) { d.on_transform(in); }},
        {"nGRP", [&](const ChunkRecord&, ContentCursor& in) { d.on_group(in); }},
        {"nSHP", [&](const ChunkRecord&, ContentCursor& in) { d.on_shape(in); }},
    };
    for (const ChunkRecord& c : chunks) {
        auto h = handlers.find(c.id);
        if (h == handlers.end())
            continue;  // layers, cameras, render settings, notes
        ContentCursor in(bytes, c.content, c.size);
        h->second(c, in);
        if (!d.problem.empty())
            return fail(d.problem);
        if (in.failed())
            return fail("has a corrupt " + c.id + " chunk");
    }
    if (!tail.empty())
        return fail(tail);
    if (out.models.empty())
        return fail("has no voxels");
    place(d.graph, out);
    return true;
}

}  // namespace mypbr_host
