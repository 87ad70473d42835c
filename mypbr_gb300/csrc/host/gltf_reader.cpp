// glTF 2.0 reading: JSON (or the GLB container's JSON chunk), buffers (files,
// base64 data URIs, the GLB binary chunk), accessors, the node tree and the
// metallic-roughness materials. Geometry is flattened the way the reference's
// loader does it (gltf_loader.h:254-363): every mesh instance is copied into
// the model's space with its node's world matrix (normals by the cofactor
// matrix, the winding flipped by mirroring matrices), TEXCOORD_0 with v
// flipped, non-indexed primitives read in order, out-of-range and degenerate
// triangles dropped.
#include "gltf_reader.h"

#include <cmath>
#include <cstring>
#include <fstream>
#include <map>

#include "json.h"

namespace mypbr_host {

namespace {

bool read_file(const std::string& path, std::vector<uint8_t>& out) {
    std::ifstream f(path, std::ios::binary);
    if (!f)
        return false;
    out.assign((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    return true;
}

// %XX escapes of a relative URI
std::string decode_uri(const std::string& uri) {
    std::string out;
    for (size_t k = 0; k < uri.size(); k++) {
        auto hex = [](char c) {
            return c >= '0' && c <= '9' ? c - '0' : c >= 'a' && c <= 'f' ? c - 'a' + 10 : c >= 'A' && c <= 'F' ? c - 'A' + 10 : -1;
        };
        if (uri[k] == '%' && k + 2 < uri.size() && hex(uri[k + 1]) >= 0 && hex(uri[k + 2]) >= 0) {
            out += char(hex(uri[k + 1]) * 16 + hex(uri[k + 2]));
            k += 2;
        } else {
            out += uri[k];
        }
    }
    return out;
}

bool base64(const std::string& text, size_t from, std::vector<uint8_t>& out) {
    out.clear();
    uint32_t acc = 0;
    int bits = 0;
    for (size_t k = from; k < text.size(); k++) {
        char c = text[k];
        int v;
        if (c >= 'A' && c <= 'Z')
            v = c - 'A';
        else if (c >= 'a' && c <= 'z')
            v = c - 'a' + 26;
        else if (c >= '0' && c <= '9')
            v = c - '0' + 52;
        else if (c == '+' || c == '-')
            v = 62;
        else if (c == '/' || c == '_')
            v = 63;
        else if (c == '=')
            break;
        else
            return false;
        acc = (acc << 6) | uint32_t(v);
        bits += 6;
        if (bits >= 8) {
            bits -= 8;
            out.push_back(uint8_t(acc >> bits));
        }
    }
    return true;
}

uint32_t le32(const uint8_t* p) { return uint32_t(p[0]) | uint32_t(p[1]) << 8 | uint32_t(p[2]) << 16 | uint32_t(p[3]) << 24; }

struct Doc {
    Json json;
    std::vector<std::vector<uint8_t>> buffers;
    std::string dir;
    std::string error;

    const Json* list(const char* name) const {
        const Json* v = json.find(name);
        return v && v->kind == Json::Array ? v : nullptr;
    }
    const Json* item(const char* name, long long k) const {
        const Json* l = list(name);
        return l && k >= 0 ? l->at(size_t(k)) : nullptr;
    }
};

// A buffer view's bytes, or nullptr if it or its buffer is missing / too short.
const uint8_t* view_bytes(const Doc& d, long long index, size_t& length, size_t& stride) {
    const Json* v = d.item("bufferViews", index);
    if (!v)
        return nullptr;
    long long b = v->integer("buffer", -1), off = v->integer("byteOffset", 0), len = v->integer("byteLength", -1);
    stride = size_t(std::max(0LL, v->integer("byteStride", 0)));
    if (b < 0 || size_t(b) >= d.buffers.size() || off < 0 || len < 0 ||
        size_t(off) + size_t(len) > d.buffers[size_t(b)].size())
        return nullptr;
    length = size_t(len);
    return d.buffers[size_t(b)].data() + off;
}

int component_count(const std::string& type) {
    if (type == "SCALAR") return 1;
    if (type == "VEC2") return 2;
    if (type == "VEC3") return 3;
    if (type == "VEC4" || type == "MAT2") return 4;
    if (type == "MAT3") return 9;
    if (type == "MAT4") return 16;
    return 0;
}

int component_size(long long type) {
    switch (type) {
        case 5120: case 5121: return 1;
        case 5122: case 5123: return 2;
        case 5125: case 5126: return 4;
        default: return 0;
    }
}

// An accessor read element by element: floats (normalized integers scaled as
// the glTF specification says) or integers.
struct Accessor {
    const uint8_t* base = nullptr;  // nullptr: no buffer view, every element reads 0
    size_t count = 0, stride = 0;
    int components = 0, ctype = 0, csize = 0;
    bool normalized = false, sparse = false;

    double component(const uint8_t* p) const {
        switch (ctype) {
            case 5126: {
                float f;
                std::memcpy(&f, p, 4);
                return f;
            }
            case 5120: {
                int8_t v = int8_t(p[0]);
                return normalized ? std::max(double(float(v) / 127.0f), -1.0) : double(v);
            }
            case 5121: return normalized ? double(float(p[0]) / 255.0f) : double(p[0]);
            case 5122: {
                int16_t v = int16_t(uint16_t(p[0] | p[1] << 8));
                return normalized ? std::max(double(float(v) / 32767.0f), -1.0) : double(v);
            }
            case 5123: {
                uint16_t v = uint16_t(p[0] | p[1] << 8);
                return normalized ? double(float(v) / 65535.0f) : double(v);
            }
            case 5125: return double(le32(p));
            default: return 0;
        }
    }
    // n components of element k as floats (as the file stores them: glTF
    // floats are single precision); missing components stay as given
    void floats(size_t k, float* out, int n) const {
        if (sparse)
            return;  // sparse accessors are not read
        if (!base) {
            for (int c = 0; c < n; c++)
                out[c] = 0;
            return;
        }
        const uint8_t* e = base + k * stride;
        for (int c = 0; c < n && c < components; c++)
            out[c] = float(component(e + size_t(c) * size_t(csize)));
    }
    long long index(size_t k) const {
        if (!base || sparse)
            return 0;
        const uint8_t* e = base + k * stride;
        switch (ctype) {
            case 5121: return e[0];
            case 5123: return e[0] | e[1] << 8;
            case 5125: return le32(e);
            default: return (long long)component(e);
        }
    }
};

bool make_accessor(Doc& d, long long index, Accessor& a) {
    const Json* j = d.item("accessors", index);
    if (!j) {
        d.error = "accessor " + std::to_string(index) + " does not exist";
        return false;
    }
    a = Accessor();
    long long count = j->integer("count", -1);
    a.components = component_count(j->str("type"));
    a.ctype = int(j->integer("componentType", 0));
    a.csize = component_size(a.ctype);
    a.normalized = j->flag("normalized", false);
    a.sparse = j->find("sparse") != nullptr;
    if (count < 0 || a.components == 0 || a.csize == 0) {
        d.error = "accessor " + std::to_string(index) + " is malformed";
        return false;
    }
    a.count = size_t(count);
    const Json* bv = j->find("bufferView");
    if (!bv || bv->kind != Json::Number) {
        // all zeros: sized by the count alone, which must stay sane
        if (a.count > (size_t(1) << 24)) {
            d.error = "accessor " + std::to_string(index) + " has no data for its " + std::to_string(count) + " elements";
            return false;
        }
        return true;
    }
    size_t length, stride;
    const uint8_t* bytes = view_bytes(d, (long long)bv->number, length, stride);
    long long off = j->integer("byteOffset", 0);
    size_t element = size_t(a.components) * size_t(a.csize);
    a.stride = stride ? stride : element;
    if (!bytes || off < 0 || (a.count > 0 && size_t(off) + (a.count - 1) * a.stride + element > length)) {
        d.error = "accessor " + std::to_string(index) + " runs past its buffer";
        return false;
    }
    a.base = bytes + off;
    return true;
}

bool load_buffers(Doc& d, const std::vector<uint8_t>* glb_bin) {
    const Json* list = d.list("buffers");
    size_t n = list ? list->size() : 0;
    d.buffers.resize(n);
    for (size_t k = 0; k < n; k++) {
        const Json& b = list->items[k];
        long long len = b.integer("byteLength", -1);
        std::string uri = b.str("uri");
        std::vector<uint8_t>& out = d.buffers[k];
        if (uri.empty()) {
            if (k != 0 || !glb_bin)
                return false;
            out = *glb_bin;
        } else if (uri.compare(0, 5, "data:") == 0) {
            size_t comma = uri.find(";base64,");
            if (comma == std::string::npos || !base64(uri, comma + 8, out))
                return false;
        } else {
            std::string file = decode_uri(uri);
            if (!read_file(file[0] == '/' ? file : d.dir + file, out))
                return false;
        }
        if (len < 0 || out.size() < size_t(len))
            return false;
        out.resize(size_t(len));
    }
    return true;
}

GltfTextureRef texture_ref(const Json* info) {
    GltfTextureRef r;
    if (!info || info->kind != Json::Object)
        return r;
    r.texture = int(info->integer("index", -1));
    r.texcoord = int(info->integer("texCoord", 0));
    r.strength = info->num("scale", 1.0);
    if (const Json* ext = info->find("extensions"))
        if (const Json* t = ext->find("KHR_texture_transform")) {
            r.has_transform = true;
            if (const Json* o = t->find("offset"); o && o->size() >= 2)
                r.offset[0] = o->items[0].number, r.offset[1] = o->items[1].number;
            if (const Json* s = t->find("scale"); s && s->size() >= 2)
                r.scale[0] = s->items[0].number, r.scale[1] = s->items[1].number;
            r.rotation = t->num("rotation", 0.0);
            if (t->find("texCoord"))
                r.texcoord = int(t->integer("texCoord", 0));
        }
    return r;
}

GltfMaterial material(const Json& m) {
    GltfMaterial g;
    g.name = m.str("name");
    if (const Json* pbr = m.find("pbrMetallicRoughness")) {
        if (const Json* c = pbr->find("baseColorFactor"); c && c->size() >= 4)
            for (int k = 0; k < 4; k++)
                g.base_color[k] = c->items[size_t(k)].number;
        g.metallic = pbr->num("metallicFactor", 1.0);
        g.roughness = pbr->num("roughnessFactor", 1.0);
        g.base_texture = texture_ref(pbr->find("baseColorTexture"));
        g.metal_rough_texture = texture_ref(pbr->find("metallicRoughnessTexture"));
    }
    g.normal_texture = texture_ref(m.find("normalTexture"));
    g.emissive_texture = texture_ref(m.find("emissiveTexture"));
    if (const Json* e = m.find("emissiveFactor"); e && e->size() >= 3)
        for (int k = 0; k < 3; k++)
            g.emissive[k] = e->items[size_t(k)].number;
    std::string mode = m.str("alphaMode", "OPAQUE");
    g.alpha_mode = mode == "MASK" ? 1 : mode == "BLEND" ? 2 : 0;
    g.alpha_cutoff = m.num("alphaCutoff", 0.5);
    if (const Json* ext = m.find("extensions")) {
        if (const Json* e = ext->find("KHR_materials_emissive_strength"))
            g.emissive_strength = e->num("emissiveStrength", 1.0);
        if (const Json* e = ext->find("KHR_materials_ior"))
            g.ior = e->num("ior", 1.5);
        if (const Json* e = ext->find("KHR_materials_transmission")) {
            g.has_transmission = true;
            g.transmission = e->num("transmissionFactor", 0.0);
        }
        if (const Json* e = ext->find("KHR_materials_clearcoat")) {
            g.has_clearcoat = true;
            g.clearcoat = e->num("clearcoatFactor", 0.0);
            g.clearcoat_roughness = e->num("clearcoatRoughnessFactor", 0.0);
            g.clearcoat_texture = texture_ref(e->find("clearcoatTexture"));
            g.clearcoat_roughness_texture = texture_ref(e->find("clearcoatRoughnessTexture"));
            g.clearcoat_normal_texture = texture_ref(e->find("clearcoatNormalTexture"));
        }
        const std::pair<const char*, const char*> left_out[] = {
            {"KHR_materials_sheen", "sheen"},       {"KHR_materials_iridescence", "iridescence"},
            {"KHR_materials_volume", "volume"},     {"KHR_materials_specular", "specular"},
            {"KHR_materials_anisotropy", "anisotropy"}, {"KHR_materials_unlit", "unlit"}};
        for (const auto& [key, what] : left_out)
            if (ext->find(key))
                g.unsupported.push_back(what);
    }
    return g;
}

// A node's local matrix, column-major, in single precision: its matrix, or
// translation * rotation (unit quaternion x, y, z, w) * scale.
void local_matrix(const Json& node, float* m) {
    if (const Json* mat = node.find("matrix"); mat && mat->size() == 16) {
        for (int k = 0; k < 16; k++)
            m[k] = float(mat->items[size_t(k)].number);
        return;
    }
    float t[3] = {0, 0, 0}, q[4] = {0, 0, 0, 1}, s[3] = {1, 1, 1};
    if (const Json* v = node.find("translation"); v && v->size() == 3)
        for (int k = 0; k < 3; k++)
            t[k] = float(v->items[size_t(k)].number);
    if (const Json* v = node.find("rotation"); v && v->size() == 4)
        for (int k = 0; k < 4; k++)
            q[k] = float(v->items[size_t(k)].number);
    if (const Json* v = node.find("scale"); v && v->size() == 3)
        for (int k = 0; k < 3; k++)
            s[k] = float(v->items[size_t(k)].number);
    float x = q[0], y = q[1], z = q[2], w = q[3];
    // the rotation matrix of a unit quaternion, columns scaled
    m[0] = (1 - 2 * (y * y + z * z)) * s[0];
    m[1] = (2 * (x * y + z * w)) * s[0];
    m[2] = (2 * (x * z - y * w)) * s[0];
    m[3] = 0;
    m[4] = (2 * (x * y - z * w)) * s[1];
    m[5] = (1 - 2 * (x * x + z * z)) * s[1];
    m[6] = (2 * (y * z + x * w)) * s[1];
    m[7] = 0;
    m[8] = (2 * (x * z + y * w)) * s[2];
    m[9] = (2 * (y * z - x * w)) * s[2];
    m[10] = (1 - 2 * (x * x + y * y)) * s[2];
    m[11] = 0;
    m[12] = t[0];
    m[13] = t[1];
    m[14] = t[2];
    m[15] = 1;
}

// out = a * b, column-major 4 x 4, single precision
void mul(const float* a, const float* b, float* out) {
    float r[16];
    for (int c = 0; c < 4; c++)
        for (int row = 0; row < 4; row++) {
            float v = 0;
            for (int k = 0; k < 4; k++)
                v += a[k * 4 + row] * b[c * 4 + k];
            r[c * 4 + row] = v;
        }
    std::memcpy(out, r, sizeof r);
}

bool add_primitive(Doc& d, const Json& prim, const float* m, GltfModel& model) {
    if (prim.integer("mode", 4) != 4) {
        model.ignored.insert("non-triangle primitives");
        return true;
    }
    if (const Json* ext = prim.find("extensions"); ext && ext->find("KHR_draco_mesh_compression")) {
        model.ignored.insert("Draco-compressed meshes");
        return true;
    }
    const Json* attrs = prim.find("attributes");
    if (!attrs)
        return true;
    long long pos_i = attrs->integer("POSITION", -1), nrm_i = attrs->integer("NORMAL", -1),
              uv_i = attrs->integer("TEXCOORD_0", -1);
    if (pos_i < 0)
        return true;
    Accessor pos, nrm, uv;
    if (!make_accessor(d, pos_i, pos))
        return false;
    bool has_n = nrm_i >= 0, has_t = uv_i >= 0;
    if (has_n && !make_accessor(d, nrm_i, nrm))
        return false;
    if (has_t && !make_accessor(d, uv_i, uv))
        return false;

    // rows of the 3 x 3 part, and its cofactors: the inverse transpose up to
    // the determinant, whose sign alone is kept (normals are normalized later)
    double a00 = m[0], a01 = m[4], a02 = m[8], a10 = m[1], a11 = m[5], a12 = m[9], a20 = m[2], a21 = m[6],
           a22 = m[10];
    double c00 = a11 * a22 - a12 * a21, c01 = a12 * a20 - a10 * a22, c02 = a10 * a21 - a11 * a20;
    double c10 = a02 * a21 - a01 * a22, c11 = a00 * a22 - a02 * a20, c12 = a01 * a20 - a00 * a21;
    double c20 = a01 * a12 - a02 * a11, c21 = a02 * a10 - a00 * a12, c22 = a00 * a11 - a01 * a10;
    double det = a00 * c00 + a01 * c01 + a02 * c02;
    double sign = det < 0 ? -1 : 1;

    size_t count = pos.count;
    int v_base = int(model.positions.size() / 3), n_base = int(model.normals.size() / 3),
        t_base = int(model.uvs.size() / 2);
    for (size_t k = 0; k < count; k++) {
        float p[3] = {0, 0, 0};
        pos.floats(k, p, 3);
        model.positions.push_back(a00 * p[0] + a01 * p[1] + a02 * p[2] + m[12]);
        model.positions.push_back(a10 * p[0] + a11 * p[1] + a12 * p[2] + m[13]);
        model.positions.push_back(a20 * p[0] + a21 * p[1] + a22 * p[2] + m[14]);
    }
    has_n = has_n && nrm.count == count;
    if (has_n)
        for (size_t k = 0; k < count; k++) {
            float n[3] = {0, 0, 1};
            nrm.floats(k, n, 3);
            model.normals.push_back(sign * (c00 * n[0] + c01 * n[1] + c02 * n[2]));
            model.normals.push_back(sign * (c10 * n[0] + c11 * n[1] + c12 * n[2]));
            model.normals.push_back(sign * (c20 * n[0] + c21 * n[1] + c22 * n[2]));
        }
    has_t = has_t && uv.count == count;
    if (has_t)
        for (size_t k = 0; k < count; k++) {
            float t[2] = {0, 0};
            uv.floats(k, t, 2);
            model.uvs.push_back(t[0]);
            model.uvs.push_back(1.0 - double(t[1]));  // glTF's v runs down the image
        }

    int mat = int(prim.integer("material", -1));
    if (mat >= int(model.materials.size()))
        mat = -1;
    Accessor idx;
    long long idx_i = prim.integer("indices", -1);
    if (idx_i >= 0 && !make_accessor(d, idx_i, idx))
        return false;
    size_t index_count = idx_i >= 0 ? idx.count : count;
    const double* P = model.positions.data();
    for (size_t k = 0; k + 2 < index_count; k += 3) {
        long long id[3];
        for (int c = 0; c < 3; c++)
            id[c] = idx_i >= 0 ? idx.index(k + size_t(c)) : (long long)(k + size_t(c));
        if (det < 0)
            std::swap(id[1], id[2]);  // a mirroring matrix flips the winding
        if (id[0] >= (long long)count || id[1] >= (long long)count || id[2] >= (long long)count)
            continue;
        GltfFace f;
        for (int c = 0; c < 3; c++) {
            f.v[c] = v_base + int(id[c]);
            f.n[c] = has_n ? n_base + int(id[c]) : -1;
            f.t[c] = has_t ? t_base + int(id[c]) : -1;
        }
        const double* p0 = P + 3 * f.v[0];
        const double* p1 = P + 3 * f.v[1];
        const double* p2 = P + 3 * f.v[2];
        double e1[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
        double e2[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
        double cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2],
               cz = e1[0] * e2[1] - e1[1] * e2[0];
        const double s = 1e-8;  // vec3::near_zero (vec3.h)
        if (std::fabs(cx) < s && std::fabs(cy) < s && std::fabs(cz) < s)
            continue;
        f.material = mat;
        model.faces.push_back(f);
    }
    return true;
}

}  // namespace

bool read_gltf(const std::string& path, GltfModel& model, std::string& error) {
    model = GltfModel();
    Doc d;
    auto slash = path.find_last_of('/');
    d.dir = slash == std::string::npos ? "" : path.substr(0, slash + 1);
    std::vector<uint8_t> file;
    const std::string unreadable = "cannot read glTF file '" + path + "'";
    if (!read_file(path, file)) {
        error = unreadable;
        return false;
    }
    // GLB: "glTF", version 2, length; a JSON chunk, then an optional binary chunk
    std::vector<uint8_t> bin;
    bool glb = file.size() >= 12 && std::memcmp(file.data(), "glTF", 4) == 0;
    const char* json_text = reinterpret_cast<const char*>(file.data());
    size_t json_size = file.size();
    if (glb) {
        if (le32(&file[4]) != 2 || file.size() < 20) {
            error = unreadable;
            return false;
        }
        size_t pos = 12;
        bool have_json = false;
        while (pos + 8 <= file.size()) {
            uint32_t len = le32(&file[pos]), type = le32(&file[pos + 4]);
            if (size_t(len) > file.size() - pos - 8) {
                error = unreadable;
                return false;
            }
            if (type == 0x4E4F534Au && !have_json) {
                json_text = reinterpret_cast<const char*>(&file[pos + 8]);
                json_size = len;
                have_json = true;
            } else if (type == 0x004E4942u && bin.empty()) {
                bin.assign(file.begin() + long(pos + 8), file.begin() + long(pos + 8 + len));
            }
            pos += 8 + ((size_t(len) + 3) & ~size_t(3));
        }
        if (!have_json) {
            error = unreadable;
            return false;
        }
    }
    std::string jerr;
    if (!parse_json(json_text, json_size, d.json, jerr) || d.json.kind != Json::Object) {
        error = unreadable;
        return false;
    }
    const Json* asset = d.json.find("asset");
    std::string version = asset ? asset->str("version") : "";
    if (version.empty() || version[0] != '2') {
        error = unreadable;
        return false;
    }
    if (!load_buffers(d, glb ? &bin : nullptr)) {
        error = "cannot load the buffers of '" + path + "'";
        return false;
    }

    if (const Json* mats = d.list("materials"))
        for (const Json& m : mats->items)
            model.materials.push_back(material(m));
    if (const Json* texs = d.list("textures"))
        for (const Json& t : texs->items) {
            GltfTexture g;
            g.image = int(t.integer("source", -1));
            if (const Json* s = d.item("samplers", t.integer("sampler", -1)))
                g.repeat = !(s->integer("wrapS", 10497) == 33071 && s->integer("wrapT", 10497) == 33071);
            model.textures.push_back(g);
        }
    if (const Json* imgs = d.list("images"))
        for (const Json& im : imgs->items) {
            GltfImage g;
            std::string uri = im.str("uri");
            g.label = !uri.empty() ? uri : !im.str("name").empty() ? im.str("name") : "embedded";
            const Json* bv = im.find("bufferView");
            if (bv && bv->kind == Json::Number) {
                size_t length, stride;
                if (const uint8_t* b = view_bytes(d, (long long)bv->number, length, stride))
                    g.bytes.assign(b, b + length);
            } else if (!uri.empty() && uri.compare(0, 5, "data:") != 0) {
                std::string file_name = decode_uri(uri);
                g.path = file_name[0] == '/' ? file_name : d.dir + file_name;
            }
            model.images.push_back(std::move(g));
        }

    // the default scene's root nodes, else every node without a parent
    const Json* nodes = d.list("nodes");
    size_t node_count = nodes ? nodes->size() : 0;
    std::vector<int> parent(node_count, -1);
    for (size_t k = 0; k < node_count; k++)
        if (const Json* ch = nodes->items[k].find("children"))
            for (const Json& c : ch->items)
                if (c.kind == Json::Number && c.number >= 0 && size_t(c.number) < node_count)
                    parent[size_t(c.number)] = int(k);
    std::vector<long long> stack;
    const Json* scene = d.item("scenes", d.json.integer("scene", 0));
    if (scene) {
        if (const Json* roots = scene->find("nodes"))
            for (const Json& r : roots->items)
                stack.push_back((long long)r.number);
    } else {
        for (size_t k = 0; k < node_count; k++)
            if (parent[k] < 0)
                stack.push_back((long long)k);
    }
    std::vector<float> world(node_count * 16);
    std::vector<char> done(node_count, 0);
    auto world_of = [&](size_t k) {
        // parent chain, innermost first: world = parent_world * local
        float m[16], pm[16];
        local_matrix(nodes->items[k], m);
        int guard = 0;
        for (int p = parent[k]; p >= 0 && guard < int(node_count); p = parent[size_t(p)], guard++) {
            local_matrix(nodes->items[size_t(p)], pm);
            mul(pm, m, m);
        }
        std::memcpy(&world[k * 16], m, sizeof m);
    };
    while (!stack.empty()) {
        long long k = stack.back();
        stack.pop_back();
        if (k < 0 || size_t(k) >= node_count || done[size_t(k)])
            continue;  // a node met twice (a malformed tree) is walked once
        done[size_t(k)] = 1;
        const Json& node = nodes->items[size_t(k)];
        if (const Json* ch = node.find("children"))
            for (const Json& c : ch->items)
                stack.push_back((long long)c.number);
        long long mesh_i = node.integer("mesh", -1);
        const Json* mesh = d.item("meshes", mesh_i);
        if (!mesh)
            continue;
        if (node.find("skin") || mesh->find("weights"))
            model.ignored.insert("skins and morph targets (the rest pose is used)");
        world_of(size_t(k));
        if (const Json* prims = mesh->find("primitives"))
            for (const Json& prim : prims->items)
                if (!add_primitive(d, prim, &world[size_t(k) * 16], model)) {
                    error = "'" + path + "': " + d.error;
                    return false;
                }
    }
    return true;
}

}  // namespace mypbr_host
