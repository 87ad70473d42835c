// The host scene layer: parses mypbr's .scene language into a mypbr_flat_scene.
//
// It accepts the reference's grammar (include/scene.h:44-243, parsed at
// scene.h:244-551) and keeps its meaning: the same defaults, the same order in
// which lights enter the light list (emissive objects as they appear, the
// environment at its line, then "sky uniform" and the sun at the end of the
// file), the same bounding boxes for the scene radius that env/sun power uses
// (light_list.h:45-96), and "path:line: message" errors. What changes is the
// result: instead of a graph of virtual objects, transforms are baked into
// world-space quads and triangles (spheres and media keep their transform,
// as instance::hit does), and one BVH is built over every primitive.
//
// MagicaVoxel models (`vox`) become voxel blocks walked by a grid DDA, or
// with `quads` their visible faces; `sky atmosphere` is baked into a 256 x 128
// environment (sky_model.h). Not handled here (MYPBR_ERR_UNSUPPORTED with a
// message): glTF meshes, cyclorama, softbox, MTL files and 8-bit image
// textures (PNG/JPEG); .hdr images are read.
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <memory>
#include <set>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

#include "../../../include/mypbr_gpu.h"
#include "bvh_build.h"
#include "host_math.h"
#include "host_scene.h"
#include "gltf_reader.h"
#include "image_reader.h"
#include "scene_words.h"
#include "sky_model.h"
#include "vox_reader.h"

#include <algorithm>
#include <array>

using namespace mypbr_host;

namespace {

thread_local std::string g_last_error;

}  // namespace

namespace mypbr_host {

void set_error(const std::string& message) { g_last_error = message; }
void clear_error() { g_last_error.clear(); }

// ------------------------------------------------------------ .hdr reading

// Reads a Radiance RGBE (.hdr) image as linear RGB floats, row 0 at the top.
// Each pixel is mantissa * 2^(exponent - 136) per channel (exponent 0 is
// black); scanlines may be flat or use the newer per-channel run-length code.
bool decode_hdr(std::istream& f, const std::string& path, int& width, int& height, std::vector<float>& rgb,
                std::string& error) {
    std::string line;
    if (!std::getline(f, line) || (line.rfind("#?RADIANCE", 0) != 0 && line.rfind("#?RGBE", 0) != 0)) {
        error = "'" + path + "' is not a Radiance .hdr file";
        return false;
    }
    bool rgbe = false;
    while (std::getline(f, line)) {
        if (line.empty())
            break;
        if (line.find("FORMAT=32-bit_rle_rgbe") != std::string::npos)
            rgbe = true;
    }
    if (!rgbe) {
        error = "'" + path + "': unsupported .hdr pixel format";
        return false;
    }
    if (!std::getline(f, line)) {
        error = "'" + path + "': missing resolution line";
        return false;
    }
    char ya[3] = {}, xa[3] = {};
    int h = 0, w = 0;
    if (std::sscanf(line.c_str(), "%2s %d %2s %d", ya, &h, xa, &w) != 4 || std::strcmp(ya, "-Y") != 0 ||
        std::strcmp(xa, "+X") != 0 || w <= 0 || h <= 0) {
        error = "'" + path + "': unsupported .hdr orientation '" + line + "'";
        return false;
    }
    std::vector<uint8_t> data((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    size_t pos = 0;
    auto get = [&](uint8_t& b) {
        if (pos >= data.size())
            return false;
        b = data[pos++];
        return true;
    };
    width = w;
    height = h;
    rgb.assign(size_t(w) * h * 3, 0.0f);
    std::vector<uint8_t> scan(size_t(w) * 4);
    for (int j = 0; j < h; j++) {
        uint8_t b0, b1, b2, b3;
        size_t start = pos;
        if (!get(b0) || !get(b1) || !get(b2) || !get(b3)) {
            error = "'" + path + "': truncated";
            return false;
        }
        if (w >= 8 && w < 32768 && b0 == 2 && b1 == 2 && ((b2 << 8) | b3) == w && !(b2 & 0x80)) {
            for (int c = 0; c < 4; c++) {
                int i = 0;
                while (i < w) {
                    uint8_t n;
                    if (!get(n)) {
                        error = "'" + path + "': truncated";
                        return false;
                    }
                    if (n > 128) {
                        int run = n - 128;
                        uint8_t v;
                        if (!get(v) || i + run > w) {
                            error = "'" + path + "': bad run";
                            return false;
                        }
                        for (int k = 0; k < run; k++)
                            scan[size_t(i++) * 4 + c] = v;
                    } else {
                        if (n == 0 || i + n > w) {
                            error = "'" + path + "': bad run";
                            return false;
                        }
                        for (int k = 0; k < n; k++) {
                            uint8_t v;
                            if (!get(v)) {
                                error = "'" + path + "': truncated";
                                return false;
                            }
                            scan[size_t(i++) * 4 + c] = v;
                        }
                    }
                }
            }
        } else {
            pos = start;
            for (int i = 0; i < w; i++)
                for (int c = 0; c < 4; c++)
                    if (!get(scan[size_t(i) * 4 + c])) {
                        error = "'" + path + "': truncated";
                        return false;
                    }
        }
        for (int i = 0; i < w; i++) {
            const uint8_t* p = &scan[size_t(i) * 4];
            float* o = &rgb[(size_t(j) * w + i) * 3];
            if (p[3] == 0) {
                o[0] = o[1] = o[2] = 0.0f;
            } else {
                float s = std::ldexp(1.0f, int(p[3]) - 136);
                o[0] = p[0] * s;
                o[1] = p[1] * s;
                o[2] = p[2] * s;
            }
        }
    }
    return true;
}

bool read_hdr(const std::string& path, int& width, int& height, std::vector<float>& rgb, std::string& error) {
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        error = "cannot open '" + path + "'";
        return false;
    }
    return decode_hdr(f, path, width, height, rgb, error);
}

// --------------------------------------------------------- Fresnel helpers

double fresnel_conductor(double cos_i, double eta, double k) {
    cos_i = std::clamp(cos_i, 0.0, 1.0);
    std::complex<double> n(eta, k);
    std::complex<double> sin2_t = (1 - cos_i * cos_i) / (n * n);
    std::complex<double> cos_t = std::sqrt(1.0 - sin2_t);
    std::complex<double> rp = (n * cos_i - cos_t) / (n * cos_i + cos_t);
    std::complex<double> rs = (cos_i - n * cos_t) / (cos_i + n * cos_t);
    return (std::norm(rp) + std::norm(rs)) / 2;
}

// The named conductors' RGB complex indices (include/microfacet.h:76-93).
bool find_conductor(const std::string& name, V3& eta, V3& k) {
    struct Entry {
        const char* names[3];
        double eta[3], k[3];
    };
    static const Entry table[] = {
        {{"Al", "aluminium", "aluminum"}, {1.6575, 0.880405, 0.521244}, {9.22381, 6.2695, 4.837}},
        {{"Ti", "titanium", "titanium"}, {3.2754, 2.37975, 2.02469}, {4.57233, 3.22453, 2.72781}},
        {{"Cu", "copper", "copper"}, {0.201005, 0.92375, 1.10222}, {3.91326, 2.45305, 2.14209}},
        {{"Au", "gold", "gold"}, {0.143036, 0.375307, 1.44205}, {3.983, 2.38556, 1.60336}},
        {{"Ag", "silver", "silver"}, {0.155276, 0.116728, 0.138388}, {4.82835, 3.12222, 2.1469}},
        {{"Cr", "chromium", "chrome"}, {4.36967, 2.91651, 1.6549}, {5.20655, 4.23131, 3.7547}},
    };
    for (const auto& e : table)
        for (const char* n : e.names)
            if (name == n) {
                eta = V3(e.eta[0], e.eta[1], e.eta[2]);
                k = V3(e.k[0], e.k[1], e.k[2]);
                return true;
            }
    return false;
}

// f0 and the cosine-weighted hemispherical average F_avg of a measured metal:
// 2 * int F(mu) mu dmu by the 512-point midpoint rule (microfacet.h:109-123).
void measured_fresnel(const V3& eta, const V3& k, V3& f0, V3& f_avg) {
    for (int c = 0; c < 3; c++) {
        f0[c] = fresnel_conductor(1.0, eta[c], k[c]);
        const int n = 512;
        double sum = 0;
        for (int i = 0; i < n; i++) {
            double mu = (i + 0.5) / n;
            sum += fresnel_conductor(mu, eta[c], k[c]) * mu;
        }
        f_avg[c] = 2 * sum / n;
    }
}

}  // namespace mypbr_host

// ------------------------------------------------------------------ parser

namespace {

struct PendingLight {
    int kind;  // MYPBR_LIGHT_*
    int first_member, member_count;
    double power;  // < 0: computed at the end (environment / sun need the radius)
};

class Loader {
  public:
    mypbr_host_scene& S;
    std::string path_for_errors;
    std::string scene_dir;
    int line_number = 0;
    std::string error;

    std::map<std::string, int> materials;
    std::map<std::string, int> textures;
    int default_material = -1;
    bool use_normal_maps = true;

    Box world_box;
    std::vector<BuildItem> items;
    std::vector<PendingLight> pending_lights;

    // End-of-file settings (scene.h:421-451)
    bool sun_on = false;
    double sun_elevation = 45, sun_azimuth = 45, sun_intensity = 3, sun_angle = 4;
    V3 sun_tint{1, 1, 1};
    bool sun_disk = true;
    bool sky_uniform = false, sky_atmosphere = false;
    mypbr_sky::Settings air;
    std::vector<double> env_fp64;  // a baked sky's pixels as the reference keeps them (FP64), for its power
    V3 sky_radiance;
    bool ground = false;
    double ground_height = 0;
    int ground_material = -1;
    double fog_density = 0;
    int fog_material = -1;
    bool has_environment = false;
    bool uniform_sky_env = false;  // the environment is the 8 x 4 "sky uniform" image
    bool power_selection = true;

    explicit Loader(mypbr_host_scene& s) : S(s) {}

    bool fail(const std::string& message) {
        error = path_for_errors + ":" + std::to_string(line_number) + ": " + message;
        return false;
    }

    // ------------------------------------------------------ tables

    int add_texture_solid(const V3& c) {
        mypbr_texture t{};
        t.type = MYPBR_TEX_SOLID;
        t.a = t.b = -1;
        t.p[0] = c.x;
        t.p[1] = c.y;
        t.p[2] = c.z;
        S.textures.push_back(t);
        return int(S.textures.size()) - 1;
    }

    int add_material(const mypbr_material& m) {
        S.materials.push_back(m);
        return int(S.materials.size()) - 1;
    }

    static mypbr_material blank_material(int type) {
        mypbr_material m{};
        m.type = type;
        for (int& t : m.tex)
            t = -1;
        m.normal_map = -1;
        m.emission_tex = -1;
        return m;
    }

    int lambertian(const V3& albedo) {
        auto m = blank_material(MYPBR_MAT_LAMBERTIAN);
        m.tex[0] = add_texture_solid(albedo);
        return add_material(m);
    }

    // principled(base, metallic, roughness, ior) without a coat (material.h:346-387)
    static mypbr_material principled_desc(int base, int metallic, int roughness, double ior) {
        auto m = blank_material(MYPBR_MAT_PRINCIPLED);
        double r0 = (ior - 1) / (ior + 1);
        m.p[0] = r0 * r0;
        m.tex[0] = base;
        m.tex[1] = metallic;
        m.tex[2] = roughness;
        m.p[13] = m.p[14] = m.p[15] = 1;
        return m;
    }

    // ------------------------------------------------------ images

    // What image_texture knows of an 8-bit image beyond its pixels
    // (texture.h:110-117, 161-179).
    struct ImageInfo {
        bool alpha_channel = false, opaque = true, grey = false;
    };
    std::map<std::tuple<std::string, bool, bool>, int> image_cache;  // (path, repeat, linear) -> texture
    std::map<int, ImageInfo> image_info;                              // texture -> 8-bit image facts

    // An image texture from a file, loaded once per (path, repeat, linear):
    // Radiance HDR as linear floats, the 8-bit formats as RGBA bytes
    // (texture.h:67-98). Returns the texture index, or -1 with err empty if the
    // file is missing, else err saying why it did not decode, and
    // image_unsupported set when that is a variant this backend does not read
    // (rather than a damaged file).
    bool image_unsupported = false;
    int load_image(const std::string& file, bool repeat, bool linear, std::string& err) {
        err.clear();
        image_unsupported = false;
        auto key = std::make_tuple(file, repeat, linear);
        auto hit = image_cache.find(key);
        if (hit != image_cache.end())
            return hit->second;
        std::vector<uint8_t> bytes;
        if (!mypbr_host::read_file_bytes(file, bytes))
            return -1;
        int index = add_image(bytes, repeat, linear, err);
        if (index >= 0)
            image_cache[key] = index;
        return index;
    }

    // An image texture from an image file's bytes (a file, or one held in a
    // glTF buffer); -1 as load_image says.
    int add_image(const std::vector<uint8_t>& bytes, bool repeat, bool linear, std::string& err) {
        err.clear();
        mypbr_texture t{};
        t.type = MYPBR_TEX_IMAGE;
        t.a = t.b = -1;
        int flags = (linear ? MYPBR_TEXF_LINEAR : 0) | (repeat ? MYPBR_TEXF_REPEAT : 0);
        mypbr_host::ImageKind kind = mypbr_host::sniff_image(bytes.data(), bytes.size());
        ImageInfo info;
        if (kind == mypbr_host::ImageKind::Hdr) {
            int w, h;
            std::vector<float> rgb;
            std::string e;
            std::istringstream in(std::string(bytes.begin(), bytes.end()));
            if (!decode_hdr(in, "image", w, h, rgb, e))
                return -1;
            t.width = w;
            t.height = h;
            t.flags = flags | MYPBR_TEXF_HDR;
            t.offset = int64_t(S.texels_hdr.size() / 3);
            S.texels_hdr.insert(S.texels_hdr.end(), rgb.begin(), rgb.end());
        } else {
            mypbr_host::LdrImage img;
            std::string e;
            if (!mypbr_host::decode_ldr_image(bytes.data(), bytes.size(), img, e)) {
                err = e;
                image_unsupported = img.unsupported;
                return -1;
            }
            // take_ldr (texture.h:161-181): the mask reads the alpha channel,
            // or the grey level of an image without one
            info.alpha_channel = img.channels == 2 || img.channels == 4;
            size_t mask_offset = info.alpha_channel ? 3 : 0;
            for (size_t k = mask_offset; k < img.rgba.size(); k += 4)
                if (img.rgba[k] < 255) {
                    info.opaque = false;
                    break;
                }
            info.grey = img.channels <= 2;
            for (size_t k = 0; info.grey && k < img.rgba.size(); k += 4)
                info.grey = img.rgba[k] == img.rgba[k + 1] && img.rgba[k] == img.rgba[k + 2];
            t.width = img.width;
            t.height = img.height;
            t.flags = flags | (info.alpha_channel ? 0 : MYPBR_TEXF_GREY_MASK);
            t.offset = int64_t(S.texels_ldr.size() / 4);
            S.texels_ldr.insert(S.texels_ldr.end(), img.rgba.begin(), img.rgba.end());
        }
        S.textures.push_back(t);
        int index = int(S.textures.size()) - 1;
        image_info[index] = info;
        return index;
    }

    // A 1 x 1 white image whose alpha is the coverage: a constant mask
    // (texture.h:100-106, glTF's baseColorFactor alpha without a texture).
    int coverage_image(double coverage) {
        uint8_t a = uint8_t(std::lround(255 * std::clamp(coverage, 0.0, 1.0)));
        mypbr_texture t{};
        t.type = MYPBR_TEX_IMAGE;
        t.a = t.b = -1;
        t.width = t.height = 1;
        t.offset = int64_t(S.texels_ldr.size() / 4);
        for (uint8_t b : {uint8_t(255), uint8_t(255), uint8_t(255), a})
            S.texels_ldr.push_back(b);
        S.textures.push_back(t);
        int index = int(S.textures.size()) - 1;
        ImageInfo info;
        info.alpha_channel = true;
        info.opaque = a == 255;
        image_info[index] = info;
        return index;
    }

    // A wrapper texture around inner (MYPBR_TEX_SCALED ... NORMAL_SCALE).
    int wrap_texture(int type, int inner, std::initializer_list<double> p, int b = -1) {
        mypbr_texture t{};
        t.type = type;
        t.a = inner;
        t.b = b;
        int k = 0;
        for (double x : p)
            t.p[k++] = x;
        S.textures.push_back(t);
        return int(S.textures.size()) - 1;
    }

    bool is_emissive(int mat) const { return S.materials[mat].type == MYPBR_MAT_DIFFUSE_LIGHT; }

    // luminance of diffuse_light::average_emission (material.h:588)
    double average_emission_luminance(int mat) const {
        const auto& m = S.materials[mat];
        if (m.type != MYPBR_MAT_DIFFUSE_LIGHT)
            return 0;
        return luminance(V3(m.p[0], m.p[1], m.p[2]) * m.p[5]);
    }

    // ------------------------------------------------------ values of a line

    // "<name>" of a texture defined on an earlier line.
    bool named_texture(Words& w, int& tex) {
        std::string name;
        if (!w.word(name)) {
            error = "expected a texture name";
            return false;
        }
        auto found = textures.find(name);
        if (found == textures.end()) {
            error = "unknown texture '" + name + "'";
            return false;
        }
        tex = found->second;
        return true;
    }

    // A color: "<r> <g> <b>" (a new solid texture) or "texture <name>". A
    // missing name leaves `error` empty, so the line's usage is reported.
    bool color_source(Words& w, int& tex) {
        if (w.peek() == "texture") {
            w.skip();
            if (!w.more())
                return false;
            return named_texture(w, tex);
        }
        V3 c;
        if (!w.triple(c))
            return false;
        tex = add_texture_solid(c);
        return true;
    }

    // A principled weight: a number in [0, 1] (a new grey solid texture) or
    // "texture <name>" (its red channel is read at every hit).
    bool unit_source(Words& w, int& tex) {
        if (w.peek() == "texture") {
            w.skip();
            return named_texture(w, tex);
        }
        double x;
        if (!w.number(x, between(0, 1, false, false)))
            return false;
        tex = add_texture_solid(V3(x, x, x));
        return true;
    }

    // The transforms an object line may end with, applied in the order
    // written. `count` numbers follow the name; scale takes one (uniform) or,
    // when a second number follows, three.
    struct TransformForm {
        const char* name;
        int count;
        Xf (*step)(const double* v);
        bool (*valid)(const double* v);
    };
    static const TransformForm* transform_form(const std::string& name) {
        static const TransformForm forms[] = {
            {"translate", 3, [](const double* v) { return Xf::translate(V3(v[0], v[1], v[2])); }, nullptr},
            {"scale", 1, [](const double* v) { return Xf::scale(V3(v[0], v[1], v[2])); },
             [](const double* v) { return v[0] != 0 && v[1] != 0 && v[2] != 0; }},
            {"rotate", 4, [](const double* v) { return Xf::rotate(v[0], V3(v[1], v[2], v[3])); },
             [](const double* v) { return V3(v[1], v[2], v[3]).length_squared() > 0; }},
            {"rotate_x", 1, [](const double* v) { return Xf::rotate(v[0], V3(1, 0, 0)); }, nullptr},
            {"rotate_y", 1, [](const double* v) { return Xf::rotate(v[0], V3(0, 1, 0)); }, nullptr},
            {"rotate_z", 1, [](const double* v) { return Xf::rotate(v[0], V3(0, 0, 1)); }, nullptr},
        };
        for (const auto& f : forms)
            if (name == f.name)
                return &f;
        return nullptr;
    }

    // Where an object goes: the material named after its geometry (else the
    // default grey), and the transforms after that (scene.h's grammar,
    // scene.h:44-243: "Any object can be followed by transforms").
    struct Placement {
        int material = -1;
        Xf xform;            // object space to world space
        bool moved = false;  // any transform was given
    };

    bool read_placement(Words& w, Placement& out) {
        out = Placement();
        out.material = default_material;
        if (w.more() && !transform_form(w.peek())) {
            std::string name;
            w.word(name);
            auto found = materials.find(name);
            if (found == materials.end()) {
                error = "unknown material '" + name + "'";
                return false;
            }
            out.material = found->second;
        }
        std::string name;
        while (w.word(name)) {
            const TransformForm* form = transform_form(name);
            if (!form) {
                error = "unexpected value '" + name +
                        "' (expected a transform: translate, scale, rotate, rotate_x, rotate_y or rotate_z)";
                return false;
            }
            double v[4] = {0, 0, 0, 0};
            bool ok = true;
            for (int k = 0; k < form->count && ok; k++)
                ok = w.number(v[k]);
            if (ok && form->count == 1 && std::string(form->name) == "scale") {
                if (w.next_is_number())
                    ok = w.number(v[1]) && w.number(v[2]);
                else
                    v[1] = v[2] = v[0];
            }
            if (ok && form->valid)
                ok = form->valid(v);
            if (!ok) {
                error = "bad values for '" + name + "'";
                return false;
            }
            out.xform = form->step(v).then_after(out.xform);
            out.moved = true;
        }
        return true;
    }

    // ------------------------------------------------------ geometry

    int add_xform(const Xf& x) {
        mypbr_xform o{};
        for (int i = 0; i < 3; i++) {
            for (int j = 0; j < 3; j++) {
                o.m[i][j] = x.m[i][j];
                o.inv_m[i][j] = x.inv_m[i][j];
            }
            o.t[i] = x.t[i];
            o.inv_t[i] = x.inv_t[i];
        }
        S.xforms.push_back(o);
        return int(S.xforms.size()) - 1;
    }

    void add_item(int kind, int index, const Box& box) {
        BuildItem it;
        it.box = box;
        it.centroid = box.centroid();
        it.ref.kind = kind;
        it.ref.index = index;
        items.push_back(it);
    }

    void add_light(int first_member, int count, double power) {
        pending_lights.push_back({MYPBR_LIGHT_GROUP, first_member, count, power});
    }

    void add_member(int kind, int index, double weight) {
        mypbr_light_member m{};
        m.prim_kind = kind;
        m.prim_index = index;
        m.weight = weight;
        S.light_members.push_back(m);
    }

    bool check_light_xform(int mat, const Xf& xform, bool transformed) {
        if (transformed && is_emissive(mat) && !xform.is_similarity()) {
            error = "lights can only be moved, rotated and scaled uniformly";
            return false;
        }
        return true;
    }

    bool add_sphere(const V3& c, double r, int mat, const Xf& xform, bool transformed) {
        if (!check_light_xform(mat, xform, transformed))
            return false;
        mypbr_sphere s{};
        s.center[0] = c.x;
        s.center[1] = c.y;
        s.center[2] = c.z;
        s.radius = r;
        s.material = mat;
        s.xform = transformed ? add_xform(xform) : -1;
        S.spheres.push_back(s);
        int index = int(S.spheres.size()) - 1;
        V3 rv(std::fabs(r), std::fabs(r), std::fabs(r));
        Box box = Box::from_points(c - rv, c + rv);
        if (transformed)
            box = xform.box(box);
        world_box.grow(box);
        add_item(MYPBR_PRIM_SPHERE, index, box);
        if (is_emissive(mat)) {
            double power = kPi * 4 * kPi * r * r * average_emission_luminance(mat);
            if (transformed)
                power *= xform.area_scale();
            int first = int(S.light_members.size());
            add_member(MYPBR_PRIM_SPHERE, index, 1.0);
            add_light(first, 1, power);
        }
        return true;
    }

    static Box quad_box(const V3& q, const V3& u, const V3& v) {
        Box b = Box::from_points(q, q + u + v);
        b.grow(Box::from_points(q + u, q + v));
        return b;
    }

    // Adds one world-space quad (object-space q, u, v moved by xform); returns
    // its index. in_bvh = false keeps it out of the BVH (a light-only face).
    int push_quad(const V3& q, const V3& u, const V3& v, int mat, const Xf& xform, bool transformed,
                  bool in_bvh = true) {
        mypbr_quad o{};
        V3 n = unit(cross(u, v));
        V3 wq = q, wu = u, wv = v, wn = n;
        if (transformed) {
            wq = xform.point(q);
            wu = xform.vec(u);
            wv = xform.vec(v);
            wn = unit(xform.normal(n));
        }
        for (int k = 0; k < 3; k++) {
            o.q[k] = wq[k];
            o.u[k] = wu[k];
            o.v[k] = wv[k];
            o.normal[k] = wn[k];
        }
        o.material = mat;
        S.quads.push_back(o);
        int index = int(S.quads.size()) - 1;
        Box box = transformed ? xform.box(quad_box(q, u, v)) : quad_box(q, u, v);
        if (in_bvh)
            add_item(MYPBR_PRIM_QUAD, index, box);
        return index;
    }

    bool add_quad(const V3& q, const V3& u, const V3& v, int mat, const Xf& xform, bool transformed) {
        if (!check_light_xform(mat, xform, transformed))
            return false;
        int index = push_quad(q, u, v, mat, xform, transformed);
        Box box = quad_box(q, u, v);
        world_box.grow(transformed ? xform.box(box) : box);
        if (is_emissive(mat)) {
            double power = kPi * cross(u, v).length() * average_emission_luminance(mat);
            if (transformed)
                power *= xform.area_scale();
            int first = int(S.light_members.size());
            add_member(MYPBR_PRIM_QUAD, index, 1.0);
            add_light(first, 1, power);
        }
        return true;
    }

    // The six sides of the box with opposite corners a, b (quad.h:95-113).
    static void box_sides(const V3& a, const V3& b, V3 q[6], V3 u[6], V3 v[6]) {
        V3 mn(std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z));
        V3 mx(std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z));
        V3 dx(mx.x - mn.x, 0, 0), dy(0, mx.y - mn.y, 0), dz(0, 0, mx.z - mn.z);
        q[0] = V3(mn.x, mn.y, mx.z); u[0] = dx;  v[0] = dy;   // front
        q[1] = V3(mx.x, mn.y, mx.z); u[1] = -dz; v[1] = dy;   // right
        q[2] = V3(mx.x, mn.y, mn.z); u[2] = -dx; v[2] = dy;   // back
        q[3] = V3(mn.x, mn.y, mn.z); u[3] = dz;  v[3] = dy;   // left
        q[4] = V3(mn.x, mx.y, mx.z); u[4] = dx;  v[4] = -dz;  // top
        q[5] = V3(mn.x, mn.y, mn.z); u[5] = dx;  v[5] = dz;   // bottom
    }

    static Box box_bounds(const V3& a, const V3& b) {
        V3 q[6], u[6], v[6];
        box_sides(a, b, q, u, v);
        Box box;
        for (int s = 0; s < 6; s++)
            box.grow(quad_box(q[s], u[s], v[s]));
        return box;
    }

    bool add_box(const V3& a, const V3& b, int mat, const Xf& xform, bool transformed) {
        if (!check_light_xform(mat, xform, transformed))
            return false;
        V3 q[6], u[6], v[6];
        box_sides(a, b, q, u, v);
        int idx[6];
        double power = 0;
        for (int s = 0; s < 6; s++) {
            idx[s] = push_quad(q[s], u[s], v[s], mat, xform, transformed);
            power += kPi * cross(u[s], v[s]).length() * average_emission_luminance(mat);
        }
        Box box = box_bounds(a, b);
        world_box.grow(transformed ? xform.box(box) : box);
        if (is_emissive(mat)) {
            if (transformed)
                power *= xform.area_scale();
            int first = int(S.light_members.size());
            for (int s = 0; s < 6; s++)
                add_member(MYPBR_PRIM_QUAD, idx[s], 1.0 / 6);
            add_light(first, 6, power);
        }
        return true;
    }

    bool add_medium(double density, bool sphere, const V3& a, const V3& b, int mat, const Xf& xform,
                    bool transformed) {
        mypbr_medium m{};
        m.shape = sphere ? 0 : 1;
        m.xform = transformed ? add_xform(xform) : -1;
        m.material = mat;
        m.density = density;
        for (int k = 0; k < 3; k++) {
            m.a[k] = a[k];
            m.b[k] = b[k];
        }
        Box box;
        if (sphere) {
            double r = b.x;
            V3 rv(r, r, r);
            box = Box::from_points(a - rv, a + rv);
        } else {
            box = box_bounds(a, b);
        }
        if (transformed)
            box = xform.box(box);
        S.media.push_back(m);
        int index = int(S.media.size()) - 1;
        world_box.grow(box);
        add_item(MYPBR_PRIM_MEDIUM, index, box);
        return true;
    }

    // A material of an MTL file with the mask that cuts holes in the
    // surfaces using it (-1 when they are opaque), obj_loader.h:25-31.
    struct MtlMaterial {
        int material = -1, alpha_mask = -1;
    };

    // The directory part of a path, with its slash ("" for a bare name).
    static std::string directory_of(const std::string& path) {
        auto slash = path.find_last_of('/');
        return slash == std::string::npos ? "" : path.substr(0, slash + 1);
    }

    // One MTL material as its statements leave it (obj_loader.h:33-177 says
    // what each means and the defaults: Kd 0.8 grey, no Ks or Ke, Ns 0, Ni 1.5).
    struct MtlEntry {
        V3 kd{0.8, 0.8, 0.8}, ks{0, 0, 0}, ke{0, 0, 0};
        double ns = 0, ni = 1.5;
        int map_kd = -1, map_d = -1, normal_map = -1;
    };

    // Reads an MTL file into result. Each statement has an entry in a table
    // that says how it changes the material being defined: Kd / Ks / Ke a
    // color (one value is grey), Ns / Ni a number, map_Kd / map_d an image
    // (the last word of the line: options before the file name are skipped),
    // norm and the bump / displacement names a tangent-space normal map (a
    // grey image under the bump and disp names is a height map, skipped).
    // Textures repeat and are relative to the MTL file; one that cannot be
    // loaded gives a warning and the plain color. Then each material becomes
    // a lambertian, a principled material (a non-black Ks: roughness
    // sqrt(sqrt(2 / (Ns + 2))), ior Ni unless it is not above 1) or an
    // emissive one (a non-black Ke), with map_d, else an alpha channel of
    // map_Kd, as its coverage mask. False only if the file cannot be opened.
    bool load_mtl(const std::string& path, std::map<std::string, MtlMaterial>& result, std::string& err) {
        std::ifstream file(path);
        if (!file) {
            err = "cannot open '" + path + "'";
            return false;
        }
        const std::string dir = directory_of(path);
        auto image = [&](const std::string& name, bool linear) {
            std::string full = name[0] == '/' ? name : dir + name;
            std::string e;
            int t = load_image(full, true, linear, e);
            if (t < 0)
                std::fprintf(stderr, "Warning: %s: cannot load texture '%s'\n", path.c_str(), full.c_str());
            return t;
        };
        auto last_word = [](Words& w) {
            std::string word, last;
            while (w.word(word))
                last = word;
            return last;
        };
        using Statement = std::function<void(MtlEntry&, Words&)>;
        auto color = [](V3 MtlEntry::*field) -> Statement {
            return [field](MtlEntry& e, Words& w) {
                double grey;
                if (!w.number(grey))
                    return;
                V3 rgb(grey, grey, grey);
                double g, b;
                if (w.number(g) && w.number(b))
                    rgb = V3(grey, g, b);
                e.*field = rgb;
            };
        };
        auto scalar = [](double MtlEntry::*field) -> Statement {
            return [field](MtlEntry& e, Words& w) {
                if (!w.more())
                    return;
                double x = 0;
                e.*field = w.number(x) ? x : 0.0;
            };
        };
        auto picture = [&](int MtlEntry::*field) -> Statement {
            return [&, field](MtlEntry& e, Words& w) {
                std::string f = last_word(w);
                if (!f.empty())
                    e.*field = image(f, false);
            };
        };
        auto normals = [&](bool named_norm) -> Statement {
            return [&, named_norm](MtlEntry& e, Words& w) {
                std::string f = last_word(w);
                if (f.empty() || !use_normal_maps)
                    return;
                int t = image(f, true);
                if (t >= 0 && !named_norm && image_info[t].grey) {
                    std::fprintf(stderr, "Warning: %s: '%s' is a height map; only normal maps are supported\n",
                                 path.c_str(), f.c_str());
                    return;
                }
                if (t >= 0)
                    e.normal_map = t;
            };
        };
        const std::map<std::string, Statement> statements = {
            {"Kd", color(&MtlEntry::kd)},         {"Ks", color(&MtlEntry::ks)},
            {"Ke", color(&MtlEntry::ke)},         {"Ns", scalar(&MtlEntry::ns)},
            {"Ni", scalar(&MtlEntry::ni)},        {"map_Kd", picture(&MtlEntry::map_kd)},
            {"map_d", picture(&MtlEntry::map_d)}, {"norm", normals(true)},
            {"map_Bump", normals(false)},         {"map_bump", normals(false)},
            {"bump", normals(false)},             {"map_Disp", normals(false)},
            {"disp", normals(false)},
        };
        std::vector<std::pair<std::string, MtlEntry>> defined;
        std::string line;
        while (std::getline(file, line)) {
            Words w(line);
            std::string keyword;
            if (!w.word(keyword) || keyword[0] == '#')
                continue;
            if (keyword == "newmtl") {
                std::string name;
                w.word(name);
                defined.emplace_back(name, MtlEntry());
                continue;
            }
            auto st = statements.find(keyword);
            if (st != statements.end() && !defined.empty())
                st->second(defined.back().second, w);
        }
        for (const auto& [name, e] : defined)
            result[name] = mtl_material(e);
        return true;
    }

    // The material and coverage mask an MTL entry stands for.
    MtlMaterial mtl_material(const MtlEntry& e) {
        MtlMaterial out;
        auto albedo = [&]() { return e.map_kd >= 0 ? e.map_kd : add_texture_solid(e.kd); };
        const bool emits = e.ke.length_squared() > 0;
        mypbr_material m;
        if (emits) {
            m = blank_material(MYPBR_MAT_DIFFUSE_LIGHT);
            m.p[0] = e.ke.x;
            m.p[1] = e.ke.y;
            m.p[2] = e.ke.z;
            m.p[3] = 180;
            m.p[4] = kInf;
            m.p[5] = 1;
        } else if (e.ks.length_squared() > 0) {
            // a Phong exponent n spreads like a microfacet alpha of
            // sqrt(2 / (n + 2)), and roughness is sqrt(alpha)
            double alpha = std::sqrt(2 / (std::max(e.ns, 0.0) + 2));
            double roughness = std::sqrt(alpha);
            int color = albedo();
            int metallic = add_texture_solid(V3(0, 0, 0));
            int rough = add_texture_solid(V3(roughness, roughness, roughness));
            m = principled_desc(color, metallic, rough, e.ni > 1 ? e.ni : 1.5);
        } else {
            m = blank_material(MYPBR_MAT_LAMBERTIAN);
            m.tex[0] = albedo();
        }
        // a normal map bends surfaces, not lights (obj_loader.h:166-167)
        if (e.normal_map >= 0 && !emits)
            m.normal_map = e.normal_map;
        out.material = add_material(m);
        auto masks = [&](int t) { return t >= 0 && !image_info[t].opaque; };
        if (e.map_d >= 0)
            out.alpha_mask = masks(e.map_d) ? e.map_d : -1;
        else if (e.map_kd >= 0 && image_info[e.map_kd].alpha_channel && masks(e.map_kd))
            out.alpha_mask = e.map_kd;
        return out;
    }

    // A Wavefront OBJ file (include/obj_loader.h:191-340): faces triangulated
    // as fans, degenerate triangles dropped, one part per usemtl surface: the
    // scene material of that name, else the MTL material of that name (from
    // the mtllib files read so far, with its alpha mask), else the line's
    // material.
    struct Face {
        int v[3], n[3], t[3];
    };
    using Surface = std::pair<int, int>;  // (material, alpha mask texture or -1)

    // An OBJ index (1-based, or negative: counted back from the end of the
    // list so far) as a 0-based one; -1 when it is 0 (absent) or outside.
    static int obj_index(long index, size_t count) {
        long n = long(count);
        long k = index > 0 ? index - 1 : n + index;
        return index != 0 && k >= 0 && k < n ? int(k) : -1;
    }

    // Up to `n` leading numbers of the words left (fewer present: zeros).
    static V3 leading_numbers(Words& w, int n) {
        double x[3] = {0, 0, 0};
        for (int k = 0; k < n && w.number(x[k]); k++) {
        }
        return V3(x[0], x[1], x[2]);
    }

    // One corner of a face: "v", "v/t", "v//n" or "v/t/n" (each an OBJ
    // index; an empty or unreadable t or n is absent). False when v is not
    // an integer.
    static bool face_corner(const std::string& word, long& v, long& t, long& n) {
        long parts[3] = {0, 0, 0};
        size_t field = 0, begin = 0;
        for (size_t i = 0; i <= word.size() && field < 3; i++) {
            if (i < word.size() && word[i] != '/')
                continue;
            int value;
            if (word_is_integer(word.substr(begin, i - begin), value))
                parts[field] = value;
            else if (field == 0)
                return false;
            field++;
            begin = i + 1;
        }
        v = parts[0];
        t = parts[1];
        n = parts[2];
        return true;
    }

    // Reads an OBJ file line by line: v / vn / vt lists, f polygons (each
    // cut into a fan of triangles around its first corner as the corners
    // arrive; degenerate ones dropped), usemtl (the rest of the line names a
    // surface: the scene material of that name, else the MTL material of
    // that name with its mask, else the mesh line's material) and mtllib
    // (MTL files relative to the OBJ; one that is missing gives a warning).
    // Other statements are ignored. With `smooth`, a file without normals
    // gets at each vertex the sum of the (area-weighted) normals of the
    // faces around it.
    bool add_obj(const std::string& file, bool smooth, int line_mat, const Xf& xform, bool transformed) {
        std::ifstream in(file);
        if (!in) {
            error = "cannot open '" + file + "'";
            return false;
        }
        const std::string obj_dir = directory_of(file);
        std::vector<V3> pos, nrm, uv;
        std::vector<Surface> part_order;
        std::map<Surface, std::vector<Face>> faces;
        Surface current{line_mat, -1};
        std::map<std::string, MtlMaterial> file_materials;
        auto where = [&](int ln) { return file + ":" + std::to_string(ln) + ": "; };
        auto emit = [&](const int (&c)[3][3]) {
            const V3& p0 = pos[size_t(c[0][0])];
            if (cross(pos[size_t(c[1][0])] - p0, pos[size_t(c[2][0])] - p0).near_zero())
                return;
            Face f;
            for (int k = 0; k < 3; k++) {
                f.v[k] = c[k][0];
                f.t[k] = c[k][1];
                f.n[k] = c[k][2];
            }
            auto& list = faces[current];
            if (list.empty())
                part_order.push_back(current);
            list.push_back(f);
        };
        std::string line;
        for (int ln = 1; std::getline(in, line); ln++) {
            Words w(line);
            std::string key;
            if (!w.word(key))
                continue;
            if (key == "v") {
                pos.push_back(leading_numbers(w, 3));
            } else if (key == "vn") {
                nrm.push_back(leading_numbers(w, 3));
            } else if (key == "vt") {
                uv.push_back(leading_numbers(w, 2));
            } else if (key == "f") {
                int fan[3][3];  // first corner, previous corner, this corner: (v, t, n)
                int corners = 0;
                std::string word;
                while (w.word(word)) {
                    long v, t, n;
                    if (!face_corner(word, v, t, n)) {
                        error = where(ln) + "bad face";
                        return false;
                    }
                    int vi = obj_index(v, pos.size());
                    if (vi < 0) {
                        error = where(ln) + "vertex index out of range";
                        return false;
                    }
                    int slot = std::min(corners, 2);
                    if (corners >= 3)
                        std::copy(std::begin(fan[2]), std::end(fan[2]), std::begin(fan[1]));
                    fan[slot][0] = vi;
                    fan[slot][1] = obj_index(t, uv.size());
                    fan[slot][2] = obj_index(n, nrm.size());
                    if (++corners >= 3)
                        emit(fan);
                }
            } else if (key == "usemtl") {
                std::string name = line.substr(line.find("usemtl") + 6);
                name.erase(0, name.find_first_not_of(" \t"));
                name.erase(name.find_last_not_of(" \t\r") + 1);
                if (auto scene_mat = materials.find(name); scene_mat != materials.end())
                    current = {scene_mat->second, -1};
                else if (auto own = file_materials.find(name); own != file_materials.end())
                    current = {own->second.material, own->second.alpha_mask};
                else
                    current = {line_mat, -1};
            } else if (key == "mtllib") {
                std::string name, why;
                while (w.word(name))
                    if (!load_mtl(name[0] == '/' ? name : obj_dir + name, file_materials, why))
                        std::fprintf(stderr, "Warning: %s: %s\n", file.c_str(), why.c_str());
            }
        }
        if (smooth && nrm.empty()) {
            nrm.assign(pos.size(), V3());
            for (const Surface& surface : part_order)
                for (Face& f : faces[surface]) {
                    V3 area_normal = cross(pos[size_t(f.v[1])] - pos[size_t(f.v[0])], pos[size_t(f.v[2])] - pos[size_t(f.v[0])]);
                    for (int k = 0; k < 3; k++) {
                        nrm[size_t(f.v[k])] = nrm[size_t(f.v[k])] + area_normal;
                        f.n[k] = f.v[k];
                    }
                }
        }
        if (part_order.empty()) {
            error = "'" + file + "' has no faces";
            return false;
        }
        return add_mesh_parts(pos, nrm, uv, part_order, faces, xform, transformed);
    }

    // A glTF 2.0 model (gltf_loader.h:59-363): its metallic-roughness
    // materials mapped onto principled / thin glass / emissive ones, base
    // color alpha as a coverage mask, one part per surface. override_mat >= 0
    // replaces every material (a clay render); replace swaps materials by
    // name. Warnings and the list of features left out go to stderr.
    bool add_gltf(const std::string& file, int override_mat, const std::map<std::string, int>& replace,
                  const Xf& xform, bool transformed) {
        mypbr_host::GltfModel g;
        if (!mypbr_host::read_gltf(file, g, error))
            return false;
        for (const auto& r : replace) {
            bool found = false;
            for (const auto& m : g.materials)
                found = found || m.name == r.first;
            if (!found) {
                error = "'" + file + "' has no material named '" + r.first + "'";
                return false;
            }
        }
        std::set<std::string>& ignored = g.ignored;
        // images once per (image, linear): colors as sRGB, data linear
        std::map<std::pair<int, bool>, int> images;
        auto image_of = [&](int texture, bool linear) -> int {
            if (texture < 0 || texture >= int(g.textures.size()))
                return -1;
            int im = g.textures[size_t(texture)].image;
            if (im < 0 || im >= int(g.images.size()))
                return -1;
            auto key = std::make_pair(im, linear);
            auto it = images.find(key);
            if (it != images.end())
                return it->second;
            const auto& src = g.images[size_t(im)];
            bool repeat = g.textures[size_t(texture)].repeat;
            std::string e;
            int t = -1;
            if (!src.bytes.empty())
                t = add_image(src.bytes, repeat, linear, e);
            else if (!src.path.empty())
                t = load_image(src.path, repeat, linear, e);
            if (t < 0)
                std::fprintf(stderr, "Warning: %s: cannot load image '%s'\n", file.c_str(), src.label.c_str());
            images[key] = t;
            return t;
        };
        // a texture view: the image, moved by KHR_texture_transform
        auto view = [&](const mypbr_host::GltfTextureRef& r, bool linear) -> int {
            if (r.texcoord != 0) {
                ignored.insert("second texture coordinates");
                return -1;
            }
            int t = image_of(r.texture, linear);
            if (t >= 0 && r.has_transform)
                t = wrap_texture(MYPBR_TEX_UV_TRANSFORM, t,
                                 {r.offset[0], r.offset[1], r.rotation, r.scale[0], r.scale[1]});
            return t;
        };
        auto normal_view = [&](const mypbr_host::GltfTextureRef& r) -> int {
            if (!use_normal_maps)
                return -1;
            int t = view(r, true);
            if (t >= 0 && r.strength != 1)
                t = wrap_texture(MYPBR_TEX_NORMAL_SCALE, t, {r.strength});
            return t;
        };
        std::map<int, Surface> converted;
        auto convert = [&](int index) -> Surface {
            auto it = converted.find(index);
            if (it != converted.end())
                return it->second;
            Surface result{-1, -1};
            if (index < 0) {
                // the specification's default material: white, metallic 1, roughness 1
                result.first = override_mat >= 0
                                   ? override_mat
                                   : add_material(principled_desc(add_texture_solid(V3(1, 1, 1)),
                                                                  add_texture_solid(V3(1, 1, 1)),
                                                                  add_texture_solid(V3(1, 1, 1)), 1.5));
                return converted[index] = result;
            }
            const auto& m = g.materials[size_t(index)];
            if (auto r = replace.find(m.name); !m.name.empty() && r != replace.end()) {
                result.first = r->second;
                return converted[index] = result;
            }
            V3 base_factor(m.base_color[0], m.base_color[1], m.base_color[2]);
            int base_image = view(m.base_texture, false);
            if (m.alpha_mode != 0 && !m.base_texture.has_transform) {
                int image = image_of(m.base_texture.texture, false);
                double alpha = m.base_color[3];
                if (image >= 0 && image_info[image].alpha_channel && !image_info[image].opaque) {
                    result.second = image;
                    if (alpha < 1)
                        ignored.insert("alpha factor times an alpha texture (the texture is used alone)");
                } else if (image < 0 && alpha < 1) {
                    // a constant coverage: MASK cuts it at alphaCutoff, BLEND keeps it
                    if (m.alpha_mode == 1)
                        alpha = alpha >= m.alpha_cutoff ? 1 : 0;
                    if (alpha < 1)
                        result.second = coverage_image(alpha);
                }
            }
            if (override_mat >= 0) {
                result.first = override_mat;
                return converted[index] = result;
            }
            for (const auto& u : m.unsupported)
                ignored.insert(u);
            int base = base_image >= 0
                           ? wrap_texture(MYPBR_TEX_SCALED, base_image, {base_factor.x, base_factor.y, base_factor.z})
                           : add_texture_solid(base_factor);
            mypbr_material mat;
            if (m.has_transmission && m.transmission > 0) {
                if (m.transmission < 1 || m.roughness > 0)
                    ignored.insert("partial or rough transmission");
                mat = blank_material(MYPBR_MAT_THIN_DIELECTRIC);
                mat.p[0] = m.ior;
                mat.p[2] = base_factor.x;
                mat.p[3] = base_factor.y;
                mat.p[4] = base_factor.z;
            } else {
                int metallic, roughness;
                int mr = view(m.metal_rough_texture, true);
                if (mr >= 0) {
                    metallic = wrap_texture(MYPBR_TEX_CHANNEL, mr, {m.metallic}, 2);
                    roughness = wrap_texture(MYPBR_TEX_CHANNEL, mr, {m.roughness}, 1);
                } else {
                    metallic = add_texture_solid(V3(m.metallic, m.metallic, m.metallic));
                    roughness = add_texture_solid(V3(m.roughness, m.roughness, m.roughness));
                }
                mat = principled_desc(base, metallic, roughness, m.ior);
                mat.tex[3] = normal_view(m.normal_texture);
                if (m.has_clearcoat && m.clearcoat > 0) {
                    // weight in red, roughness in green, each times its factor; without
                    // a clearcoatNormalTexture the coat is not bent
                    int t = view(m.clearcoat_texture, true);
                    int weight = t >= 0 ? wrap_texture(MYPBR_TEX_CHANNEL, t, {m.clearcoat}, 0)
                                        : add_texture_solid(V3(m.clearcoat, m.clearcoat, m.clearcoat));
                    t = view(m.clearcoat_roughness_texture, true);
                    double cr = m.clearcoat_roughness;
                    int coat_rough = t >= 0 ? wrap_texture(MYPBR_TEX_CHANNEL, t, {cr}, 1)
                                            : add_texture_solid(V3(cr, cr, cr));
                    mat.flags |= MYPBR_MATF_COAT;
                    mat.tex[4] = weight;
                    mat.tex[5] = coat_rough;
                    mat.tex[6] = normal_view(m.clearcoat_normal_texture);
                }
            }
            V3 emission = V3(m.emissive[0], m.emissive[1], m.emissive[2]) * m.emissive_strength;
            if (emission.length_squared() > 0) {
                if (m.emissive_texture.texture >= 0) {
                    // emissive_surface: glows, but is not sampled as a light
                    int image = view(m.emissive_texture, false);
                    if (image >= 0)
                        mat.emission_tex = wrap_texture(MYPBR_TEX_SCALED, image, {emission.x, emission.y, emission.z});
                } else {
                    mat = blank_material(MYPBR_MAT_DIFFUSE_LIGHT);  // a light of the scene
                    mat.p[0] = emission.x;
                    mat.p[1] = emission.y;
                    mat.p[2] = emission.z;
                    mat.p[3] = 180;
                    mat.p[4] = kInf;
                    mat.p[5] = 1;
                }
            }
            result.first = add_material(mat);
            return converted[index] = result;
        };

        std::vector<V3> pos, nrm, uv;
        for (size_t k = 0; k + 2 < g.positions.size(); k += 3)
            pos.emplace_back(g.positions[k], g.positions[k + 1], g.positions[k + 2]);
        for (size_t k = 0; k + 2 < g.normals.size(); k += 3)
            nrm.emplace_back(g.normals[k], g.normals[k + 1], g.normals[k + 2]);
        for (size_t k = 0; k + 1 < g.uvs.size(); k += 2)
            uv.emplace_back(g.uvs[k], g.uvs[k + 1], 0);
        std::vector<Surface> part_order;
        std::map<Surface, std::vector<Face>> faces;
        for (const auto& f : g.faces) {
            Surface sf = convert(f.material);
            Face face;
            for (int c = 0; c < 3; c++) {
                face.v[c] = f.v[c];
                face.n[c] = f.n[c];
                face.t[c] = f.t[c];
            }
            if (!faces.count(sf))
                part_order.push_back(sf);
            faces[sf].push_back(face);
        }
        if (!ignored.empty()) {
            std::string list;
            for (const auto& what : ignored)
                list += (list.empty() ? " " : ", ") + what;
            std::fprintf(stderr, "Note: %s: not supported, left out:%s\n", file.c_str(), list.c_str());
        }
        if (part_order.empty()) {
            error = "'" + file + "' has no triangles";
            return false;
        }
        return add_mesh_parts(pos, nrm, uv, part_order, faces, xform, transformed);
    }

    // The parts of a mesh file: its vertex data (in the file's space) and its
    // faces grouped by surface, in the order the surfaces were first used.
    // Each part is a mesh (mesh.h:175-216); an emissive part is a light.
    bool add_mesh_parts(const std::vector<V3>& pos, const std::vector<V3>& nrm, const std::vector<V3>& uv,
                        const std::vector<Surface>& part_order, std::map<Surface, std::vector<Face>>& faces,
                        const Xf& xform, bool transformed) {
        for (const Surface& pm : part_order)
            if (!check_light_xform(pm.first, xform, transformed))
                return false;

        // Vertex data in world space; normals by the inverse transpose, kept
        // unnormalized so that interpolation commutes with the transform.
        int64_t vbase = S.position_count(), nbase = S.normal_count(), tbase = S.uv_count();
        for (const V3& p : pos) {
            V3 w = transformed ? xform.point(p) : p;
            S.positions.push_back(w.x);
            S.positions.push_back(w.y);
            S.positions.push_back(w.z);
        }
        for (const V3& n : nrm) {
            V3 w = transformed ? xform.normal(n) : n;
            S.normals.push_back(w.x);
            S.normals.push_back(w.y);
            S.normals.push_back(w.z);
        }
        for (const V3& t : uv) {
            S.uvs.push_back(t.x);
            S.uvs.push_back(t.y);
        }
        bool flip = transformed && xform.det() < 0;
        double area_scale = transformed ? xform.area_scale() : 1.0;
        for (const Surface& surface : part_order) {
            const auto& fs = faces[surface];
            const int pm = surface.first, mask = surface.second;
            mypbr_mesh mesh{};
            mesh.first_triangle = int64_t(S.triangles.size());
            mesh.triangle_count = int64_t(fs.size());
            mesh.material = pm;
            mesh.alpha_mask = mask;
            S.meshes.push_back(mesh);
            int mesh_index = int(S.meshes.size()) - 1;
            Box part_box;
            double total_area = 0;
            std::vector<double> areas;
            areas.reserve(fs.size());
            for (const auto& f : fs) {
                mypbr_triangle t{};
                for (int c = 0; c < 3; c++) {
                    t.v[c] = int(vbase + f.v[c]);
                    t.n[c] = f.n[c] >= 0 ? int(nbase + f.n[c]) : -1;
                    t.t[c] = f.t[c] >= 0 ? int(tbase + f.t[c]) : -1;
                }
                // A vertex-normal index counts only if all three are present (mesh.h:100)
                if (t.n[0] < 0 || t.n[1] < 0 || t.n[2] < 0)
                    t.n[0] = t.n[1] = t.n[2] = -1;
                if (t.t[0] < 0 || t.t[1] < 0 || t.t[2] < 0)
                    t.t[0] = t.t[1] = t.t[2] = -1;
                t.material = pm;
                t.flags = (flip ? MYPBR_TRI_FLIP_NORMAL : 0) | (mask >= 0 ? MYPBR_TRI_ALPHA_MASK : 0);
                t.mesh = mesh_index;
                S.triangles.push_back(t);
                int ti = int(S.triangles.size()) - 1;
                const V3 &p0 = pos[f.v[0]], &p1 = pos[f.v[1]], &p2 = pos[f.v[2]];
                Box obox = Box::from_points(p0, p1);
                obox.grow(Box::from_points(p2, p2));
                part_box.grow(obox);
                // World-space box for the BVH item
                V3 w0 = transformed ? xform.point(p0) : p0, w1 = transformed ? xform.point(p1) : p1,
                   w2 = transformed ? xform.point(p2) : p2;
                Box wbox = Box::from_points(w0, w1);
                wbox.grow(Box::from_points(w2, w2));
                add_item(MYPBR_PRIM_TRIANGLE, ti, wbox);
                double a = 0.5 * cross(p1 - p0, p2 - p0).length();
                areas.push_back(a);
                total_area += a;
            }
            world_box.grow(transformed ? xform.box(part_box) : part_box);
            if (is_emissive(pm)) {
                double lum = average_emission_luminance(pm), power = 0;
                int first = int(S.light_members.size());
                for (size_t k = 0; k < fs.size(); k++) {
                    power += kPi * areas[k] * lum;
                    add_member(MYPBR_PRIM_TRIANGLE, int(mesh.first_triangle + int64_t(k)),
                               total_area > 0 ? areas[k] / total_area : 0.0);
                }
                add_light(first, int(fs.size()), power * area_scale);
            }
        }
        return true;
    }

    // ------------------------------------------------------ lines

    // An optional "normal_map <texture>" closing a lambertian or metal line.
    bool optional_normal_map(Words& w, int& normal_map) {
        if (!w.more())
            return true;
        if (w.peek() != "normal_map") {
            error = "unexpected value '" + w.peek() + "' (expected 'normal_map <texture>')";
            return false;
        }
        w.skip();
        return named_texture(w, normal_map);
    }

    // "key value..." settings in any order: `read` has a reader per key. A
    // key that is not in it, or whose values are missing or out of range, is
    // reported with the message `unknown(key)` or `bad(key)` (a reader may
    // put its own message in `error` instead).
    using SettingReader = std::function<bool(Words&)>;
    bool settings(Words& w, const std::map<std::string, SettingReader>& read,
                  const std::function<std::string(const std::string&)>& unknown,
                  const std::function<std::string(const std::string&)>& bad) {
        std::string key;
        while (w.word(key)) {
            auto reader = read.find(key);
            if (reader == read.end())
                return fail(unknown(key));
            error.clear();
            if (!reader->second(w))
                return fail(error.empty() ? bad(key) : error);
        }
        return true;
    }

    // The material types of a "material <name> <type> ..." line
    // (scene.h:44-243 documents each; the checks on their values follow it).
    using MaterialReader = bool (Loader::*)(Words&, mypbr_material&, int&);
    static const std::map<std::string, MaterialReader>& material_readers() {
        static const std::map<std::string, MaterialReader> table = {
            {"lambertian", &Loader::lambertian_line}, {"metal", &Loader::metal_line},
            {"dielectric", &Loader::dielectric_line}, {"thin_glass", &Loader::thin_glass_line},
            {"principled", &Loader::principled_line}, {"volume", &Loader::volume_line},
            {"emissive", &Loader::emissive_line},
        };
        return table;
    }

    bool lambertian_line(Words& w, mypbr_material& m, int& normal_map) {
        m.type = MYPBR_MAT_LAMBERTIAN;
        error.clear();
        if (!color_source(w, m.tex[0]))
            return fail(error.empty() ? "expected 'material <name> lambertian <r> <g> <b>' or '... lambertian texture <name>'"
                                      : error);
        return optional_normal_map(w, normal_map) || fail(error);
    }

    bool metal_line(Words& w, mypbr_material& m, int& normal_map) {
        const char* usage = "expected 'material <name> metal <r> <g> <b> <roughness>' or "
                            "'... metal <Al|Ti|Cu|Au|Ag|Cr> <roughness>'";
        m.type = MYPBR_MAT_METAL;
        V3 eta, k, albedo;
        double roughness = 0;
        const bool measured = find_conductor(w.peek(), eta, k);
        if (measured)
            w.skip();
        else if (!w.triple(albedo))
            return fail(usage);
        if (!w.number(roughness, non_negative()))
            return fail(usage);
        if (!optional_normal_map(w, normal_map))
            return fail(error);
        m.p[3] = std::clamp(roughness, 0.0, 1.0);
        if (measured) {
            V3 f0, f_avg;
            measured_fresnel(eta, k, f0, f_avg);
            m.flags |= MYPBR_MATF_MEASURED;
            for (int c = 0; c < 3; c++) {
                m.p[c] = f0[c];
                m.p[4 + c] = eta[c];
                m.p[7 + c] = k[c];
                m.p[10 + c] = f_avg[c];
            }
        } else {
            for (int c = 0; c < 3; c++) {
                m.p[c] = albedo[c];
                m.p[10 + c] = albedo[c] + (1 - albedo[c]) / 21;  // Schlick's hemispherical average
            }
        }
        return true;
    }

    bool dielectric_line(Words& w, mypbr_material& m, int&) {
        const std::string usage = "expected 'material <name> dielectric <index of refraction> [roughness <r>] "
                                  "[color <r> <g> <b> [distance <d>]]'";
        double ior, roughness = 0, distance = 1;
        V3 tint(1, 1, 1);
        if (!w.number(ior, positive()))
            return fail(usage);
        auto says = [&](const std::string&) { return usage; };
        if (!settings(w,
                      {{"roughness", [&](Words& v) { return v.number(roughness, non_negative()); }},
                       {"color", [&](Words& v) { return v.triple(tint, between(0, 1, true, false)); }},
                       {"distance", [&](Words& v) { return v.number(distance, positive()); }}},
                      says, says))
            return false;
        m.type = MYPBR_MAT_DIELECTRIC;
        m.p[0] = ior;
        m.p[1] = std::clamp(roughness, 0.0, 1.0);
        for (int c = 0; c < 3; c++)
            m.p[2 + c] = -std::log(tint[c]) / distance;  // Beer-Lambert absorption per unit length
        return true;
    }

    bool thin_glass_line(Words& w, mypbr_material& m, int&) {
        const char* usage = "expected 'material <name> thin_glass <index of refraction> [color <r> <g> <b>]'";
        double ior;
        V3 tint(1, 1, 1);
        if (!w.number(ior, positive()))
            return fail(usage);
        if (w.more()) {  // one optional setting
            std::string key;
            w.word(key);
            if (key != "color" || !w.triple(tint, between(0, 1, false, false)))
                return fail(usage);
        }
        m.type = MYPBR_MAT_THIN_DIELECTRIC;
        m.p[0] = ior;
        for (int c = 0; c < 3; c++)
            m.p[2 + c] = tint[c];
        return true;
    }

    bool principled_line(Words& w, mypbr_material& m, int&) {
        m.type = MYPBR_MAT_PRINCIPLED;
        int base = add_texture_solid(V3(0.8, 0.8, 0.8));
        int metallic = add_texture_solid(V3(0, 0, 0));
        int rough = add_texture_solid(V3(0.5, 0.5, 0.5));
        int coat = -1, coat_rough = -1, coat_normals = -1, base_normals = -1;
        V3 coat_tint(1, 1, 1), eta, k;
        bool coat_tinted = false, measured = false;
        double ior = 1.5;
        const std::map<std::string, SettingReader> read = {
            {"texture", [&](Words& v) { return v.more() && named_texture(v, base); }},
            {"color", [&](Words& v) { return color_source(v, base); }},
            {"metallic", [&](Words& v) { return unit_source(v, metallic); }},
            {"roughness", [&](Words& v) { return unit_source(v, rough); }},
            {"ior", [&](Words& v) { return v.number(ior, positive()); }},
            {"normal_map", [&](Words& v) { return named_texture(v, base_normals); }},
            {"clearcoat", [&](Words& v) { return unit_source(v, coat); }},
            {"clearcoat_roughness", [&](Words& v) { return unit_source(v, coat_rough); }},
            {"clearcoat_normal_map", [&](Words& v) { return named_texture(v, coat_normals); }},
            {"conductor",
             [&](Words& v) {
                 std::string metal;
                 v.word(metal);
                 measured = find_conductor(metal, eta, k);
                 if (!measured)
                     error = "unknown conductor '" + metal + "' (known: Al Ti Cu Au Ag Cr)";
                 return measured;
             }},
            {"clearcoat_color",
             [&](Words& v) { return coat_tinted = v.triple(coat_tint, between(0, 1, true, false)); }},
        };
        if (!settings(w, read, [](const std::string& key) { return "unknown principled setting '" + key + "'"; },
                      [](const std::string& key) { return "bad value for principled setting '" + key + "'"; }))
            return false;
        if (coat < 0 && (coat_rough >= 0 || coat_normals >= 0 || coat_tinted))
            return fail("clearcoat_roughness, clearcoat_normal_map and clearcoat_color need 'clearcoat <weight>'");
        double r0 = (ior - 1) / (ior + 1);
        m.p[0] = r0 * r0;
        m.tex[0] = base;
        m.tex[1] = metallic;
        m.tex[2] = rough;
        m.tex[3] = use_normal_maps ? base_normals : -1;
        if (measured) {
            V3 f0, f_avg;
            measured_fresnel(eta, k, f0, f_avg);
            m.flags |= MYPBR_MATF_MEASURED;
            for (int c = 0; c < 3; c++) {
                m.p[4 + c] = eta[c];
                m.p[7 + c] = k[c];
                m.p[10 + c] = f_avg[c];
            }
        }
        m.p[13] = m.p[14] = m.p[15] = 1;
        if (coat >= 0) {
            m.flags |= MYPBR_MATF_COAT;
            m.tex[4] = coat;
            m.tex[5] = coat_rough >= 0 ? coat_rough : add_texture_solid(V3(0, 0, 0));
            m.tex[6] = use_normal_maps ? coat_normals : -1;
            for (int c = 0; c < 3; c++)
                m.p[13 + c] = coat_tint[c];
            if (coat_tint.x != 1 || coat_tint.y != 1 || coat_tint.z != 1)
                m.flags |= MYPBR_MATF_COAT_TINT;
        }
        return true;
    }

    bool volume_line(Words& w, mypbr_material& m, int&) {
        V3 albedo;
        double g = 0;
        if (!w.triple(albedo))
            return fail("expected 'material <name> volume <r> <g> <b> [g <anisotropy>]'");
        if (w.more()) {  // one optional setting
            std::string key;
            w.word(key);
            if (key != "g" || !w.number(g, between(-1, 1, true, true)))
                return fail("expected 'material <name> volume <r> <g> <b> [g <anisotropy between -1 and 1>]'");
        }
        m.type = MYPBR_MAT_PHASE;
        m.p[0] = albedo.x;
        m.p[1] = albedo.y;
        m.p[2] = albedo.z;
        m.p[3] = g;
        return true;
    }

    bool emissive_line(Words& w, mypbr_material& m, int&) {
        const char* usage = "expected 'material <name> emissive <r> <g> <b> [spread <degrees, 0 to 180>]'";
        V3 radiance;
        double spread = 180;
        if (!w.triple(radiance))
            return fail(usage);
        if (w.more()) {  // one optional setting
            std::string key;
            w.word(key);
            if (key != "spread" || !w.number(spread, between(0, 180, true, false)))
                return fail(usage);
        }
        m.type = MYPBR_MAT_DIFFUSE_LIGHT;
        m.p[0] = radiance.x;
        m.p[1] = radiance.y;
        m.p[2] = radiance.z;
        m.p[3] = spread;
        double half = radians(spread) / 2;
        m.p[4] = spread >= 180 ? kInf : std::tan(half);
        // the cosine-weighted share a honeycomb of that spread lets through
        // (material.h:600-608): 1 for a bare diffuser
        if (half >= kPi / 2 - 1e-9) {
            m.p[5] = 1;
        } else {
            double sn = std::sin(half), cs = std::cos(half);
            m.p[5] = sn * sn - (half - sn * cs) * cs / sn;
        }
        return true;
    }

    bool material_line(Words& w) {
        std::string name, type;
        if (!w.word(name) || !w.word(type))
            return fail("expected 'material <name> <type> <parameters...>'");
        auto reader = material_readers().find(type);
        if (reader == material_readers().end())
            return fail("unknown material type '" + type + "'");
        mypbr_material m = blank_material(0);
        int normal_map = -1;
        if (!(this->*(reader->second))(w, m, normal_map))
            return false;
        if (normal_map >= 0 && use_normal_maps)
            m.normal_map = normal_map;
        materials[name] = add_material(m);
        return true;
    }

    bool texture_line(Words& w) {
        std::string name, type;
        if (!w.word(name) || !w.word(type))
            return fail("expected 'texture <name> <type> <parameters...>'");
        if (type == "solid") {
            V3 c;
            if (!w.triple(c))
                return fail("expected 'texture <name> solid <r> <g> <b>'");
            textures[name] = add_texture_solid(c);
            return true;
        }
        if (type == "checker") {
            double scale;
            V3 even, odd;
            if (!w.number(scale, positive()) || !w.triple(even) || !w.triple(odd))
                return fail("expected 'texture <name> checker <scale> <r g b> <r g b>'");
            mypbr_texture t{};
            t.type = MYPBR_TEX_CHECKER;
            t.a = add_texture_solid(even);
            t.b = add_texture_solid(odd);
            t.p[0] = 1.0 / scale;
            S.textures.push_back(t);
            textures[name] = int(S.textures.size()) - 1;
            return true;
        }
        if (type == "image") {
            const char* usage = "expected 'texture <name> image <path> [linear]'";
            std::string file;
            if (!w.word(file))
                return fail(usage);
            bool linear = w.peek() == "linear";
            if (linear)
                w.skip();
            else if (w.more())
                return fail(usage);
            if (file[0] != '/')
                file = scene_dir + file;
            std::string why;
            int index = load_image(file, false, linear, why);
            if (index < 0) {
                if (image_unsupported) {
                    unsupported = true;
                    return fail("image texture '" + file + "': " + why);
                }
                return fail("cannot load image '" + file + "'" + (why.empty() ? "" : ": " + why));
            }
            textures[name] = index;
            return true;
        }
        return fail("unknown texture type '" + type + "'");
    }

    bool unsupported = false;

    // A MagicaVoxel palette as materials and voxel kinds (voxel.h:48-97):
    // sRGB colours decoded to linear albedo; MATL _metal -> principled,
    // _glass -> absorbing dielectric of kind transparent, _emit -> light,
    // anything else -> lambertian. Returns the first of the 256 entries.
    int add_vox_palette(const VoxFile& vox, double emission_scale, std::vector<bool>& emissive) {
        auto number = [](const std::map<std::string, std::string>& props, const char* key, double fallback) {
            auto it = props.find(key);
            if (it == props.end())
                return fallback;
            try {
                return std::stod(it->second);
            } catch (...) {
                return fallback;
            }
        };
        auto srgb = [](double e) { return e <= 0.04045 ? e / 12.92 : std::pow((e + 0.055) / 1.055, 2.4); };
        int base = int(S.voxel_palettes.size());
        emissive.assign(256, false);
        for (int k = 0; k < 256; k++) {
            const V3& c = vox.palette[k];
            V3 albedo(srgb(c.x), srgb(c.y), srgb(c.z));
            const auto& props = vox.materials[k];
            auto type_it = props.find("_type");
            std::string type = type_it == props.end() ? "_diffuse" : type_it->second;
            double roughness = std::clamp(number(props, "_rough", 0.1), 0.0, 1.0);
            double ior = number(props, "_ri", 1 + number(props, "_ior", 0.5));
            if (ior <= 1)
                ior = 1.5;
            mypbr_voxel_entry e{};
            e.kind = k == 0 ? MYPBR_VOXEL_EMPTY : MYPBR_VOXEL_OPAQUE;
            mypbr_material m = blank_material(MYPBR_MAT_LAMBERTIAN);
            if (type == "_metal") {
                double metallic =
                    number(props, "_plastic", 0) > 0 ? 0 : std::clamp(number(props, "_metal", 1), 0.0, 1.0);
                m.type = MYPBR_MAT_PRINCIPLED;
                m.tex[0] = add_texture_solid(albedo);
                m.tex[1] = add_texture_solid(V3(metallic, metallic, metallic));
                m.tex[2] = add_texture_solid(V3(roughness, roughness, roughness));
                double r0 = (ior - 1) / (ior + 1);
                m.p[0] = r0 * r0;
                m.p[13] = m.p[14] = m.p[15] = 1;
            } else if (type == "_glass") {
                double att = std::clamp(number(props, "_att", 0.5), 0.0, 1.0);
                m.type = MYPBR_MAT_DIELECTRIC;
                m.p[0] = ior;
                m.p[1] = roughness <= 0.05 ? 0 : roughness;
                for (int ch = 0; ch < 3; ch++) {
                    double tint = std::clamp((1 - att) + att * albedo[ch], 1e-3, 1.0);
                    m.p[2 + ch] = -std::log(tint) / 1.0;
                }
                e.kind = MYPBR_VOXEL_TRANSPARENT;
            } else if (type == "_emit") {
                double strength = number(props, "_emit", 1) * std::pow(10.0, number(props, "_flux", 0)) * emission_scale;
                m.type = MYPBR_MAT_DIFFUSE_LIGHT;
                for (int ch = 0; ch < 3; ch++)
                    m.p[ch] = strength * albedo[ch];
                m.p[3] = 180;
                m.p[4] = kInf;
                m.p[5] = 1;
                emissive[size_t(k)] = strength > 0;
            } else {
                m.tex[0] = add_texture_solid(albedo);
            }
            e.material = add_material(m);
            S.voxel_palettes.push_back(e);
        }
        return base;
    }

    static bool face_visible(int k, int n) {  // voxel.h:100-106
        if (k == MYPBR_VOXEL_EMPTY)
            return false;
        if (n == MYPBR_VOXEL_EMPTY)
            return true;
        return k == MYPBR_VOXEL_OPAQUE && n == MYPBR_VOXEL_TRANSPARENT;
    }

    struct VoxFace {
        V3 q, u, v;
        int material;
        bool emissive;
    };

    // The visible faces of a model in model space, wound so that cross(u, v)
    // points out of the cell (voxel.h:112-147).
    std::vector<VoxFace> vox_faces(const VoxModel& m, int palette, const std::vector<bool>& emissive) {
        static const int off[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
        static const double corner[6][3] = {{1, 0, 0}, {0, 0, 0}, {0, 1, 0}, {0, 0, 0}, {0, 0, 1}, {0, 0, 0}};
        static const double us[6][3] = {{0, 1, 0}, {0, 0, 1}, {0, 0, 1}, {1, 0, 0}, {1, 0, 0}, {0, 1, 0}};
        static const double vs[6][3] = {{0, 0, 1}, {0, 1, 0}, {1, 0, 0}, {0, 0, 1}, {0, 1, 0}, {1, 0, 0}};
        std::vector<VoxFace> faces;
        auto kind = [&](int idx) { return S.voxel_palettes[size_t(palette + idx)].kind; };
        for (int z = 0; z < m.nz; z++)
            for (int y = 0; y < m.ny; y++)
                for (int x = 0; x < m.nx; x++) {
                    int idx = m.at(x, y, z);
                    int k = kind(idx);
                    if (k == MYPBR_VOXEL_EMPTY)
                        continue;
                    for (int f = 0; f < 6; f++) {
                        int n = kind(m.at(x + off[f][0], y + off[f][1], z + off[f][2]));
                        if (!face_visible(k, n))
                            continue;
                        VoxFace face;
                        face.q = V3(x + corner[f][0], y + corner[f][1], z + corner[f][2]);
                        face.u = V3(us[f][0], us[f][1], us[f][2]);
                        face.v = V3(vs[f][0], vs[f][1], vs[f][2]);
                        face.material = S.voxel_palettes[size_t(palette + idx)].material;
                        face.emissive = emissive[size_t(idx)];
                        faces.push_back(face);
                    }
                }
        return faces;
    }

    // vox <file> [quads] [emission <s>] [edges <w> [<r g b>]] [transforms] (scene.h:341-429)
    bool vox_line(Words& w) {
        const char* usage = "expected 'vox <file.vox> [quads] [emission <scale>] [edges <width> [<r g b>]] [transforms]'";
        std::string file;
        if (!w.word(file))
            return fail(usage);
        if (file[0] != '/')
            file = scene_dir + file;
        bool quads = false;
        double emission = 1, edge_width = 0;
        V3 edge_color(0, 0, 0);
        // options, until a word that is none (a keyword with no value after it
        // ends them too, and is then read as a material name)
        for (bool options = true; options && w.more();) {
            const std::string& key = w.peek();
            if (key == "quads") {
                quads = true;
                w.skip();
            } else if ((key == "emission" || key == "edges") && w.left() >= 2) {
                bool edges = key == "edges";
                w.skip();
                double x;
                bool ok = word_is_number(w.peek(), x) &&
                          (edges ? x > 0 && x < 0.5 : x >= 0);
                if (!ok)
                    return fail(usage);
                w.skip();
                (edges ? edge_width : emission) = x;
                if (edges && w.left() >= 3)
                    w.triple(edge_color);  // an optional color; left for the tail if it is not one
            } else {
                options = false;
            }
        }
        Placement at;
        error.clear();
        if (!read_placement(w, at))
            return fail(error);
        if (at.material != default_material)
            return fail("vox models take their materials from the file's palette");
        const Xf& xform = at.xform;
        VoxFile vox;
        std::string err;
        if (!read_vox(file, vox, err))
            return fail(err);
        std::vector<bool> emissive;
        int palette = add_vox_palette(vox, emission, emissive);
        int edge_material = (!quads && edge_width > 0) ? lambertian(edge_color) : -1;
        struct ModelData {
            int64_t cells;
            std::vector<VoxFace> faces;
            std::vector<std::array<int, 6>> blocks;  // lo, hi
            Box box;                                 // model-space box of the geometry
        };
        std::vector<ModelData> models(vox.models.size());
        for (size_t mi = 0; mi < vox.models.size(); mi++) {
            const VoxModel& m = vox.models[mi];
            ModelData& md = models[mi];
            md.faces = vox_faces(m, palette, emissive);
            if (quads) {
                for (const auto& f : md.faces)
                    md.box.grow(quad_box(f.q, f.u, f.v));
                continue;
            }
            md.cells = int64_t(S.voxel_cells.size());
            S.voxel_cells.insert(S.voxel_cells.end(), m.cells.begin(), m.cells.end());
            const int block = 8;  // voxel.h:356
            for (int z0 = 0; z0 < m.nz; z0 += block)
                for (int y0 = 0; y0 < m.ny; y0 += block)
                    for (int x0 = 0; x0 < m.nx; x0 += block) {
                        int lo[3] = {x0 + block, y0 + block, z0 + block}, hi[3] = {x0, y0, z0};
                        for (int z = z0; z < std::min(z0 + block, m.nz); z++)
                            for (int y = y0; y < std::min(y0 + block, m.ny); y++)
                                for (int x = x0; x < std::min(x0 + block, m.nx); x++)
                                    if (S.voxel_palettes[size_t(palette + m.at(x, y, z))].kind != MYPBR_VOXEL_EMPTY) {
                                        int c[3] = {x, y, z};
                                        for (int a = 0; a < 3; a++) {
                                            lo[a] = std::min(lo[a], c[a]);
                                            hi[a] = std::max(hi[a], c[a] + 1);
                                        }
                                    }
                        if (hi[0] > lo[0]) {
                            md.blocks.push_back({lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]});
                            md.box.grow(Box::from_points(V3(lo[0], lo[1], lo[2]), V3(hi[0], hi[1], hi[2])));
                        }
                    }
        }
        // MagicaVoxel is z-up: +z becomes +y (and +y becomes -z)
        Xf z_up = Xf::rotate(-90, V3(1, 0, 0));
        for (const auto& placed : vox.instances) {
            const ModelData& md = models[size_t(placed.model)];
            Xf to_world = xform.then_after(z_up.then_after(placed.xform));
            bool has_emitters = false;
            for (const auto& f : md.faces)
                has_emitters = has_emitters || f.emissive;
            if (has_emitters && !to_world.is_similarity())
                return fail("a vox model with emissive voxels can only be scaled uniformly");
            if (!md.box.empty())
                world_box.grow(to_world.box(md.box));
            std::vector<int> emitter_quads;
            if (quads) {
                for (const auto& f : md.faces) {
                    int qi = push_quad(f.q, f.u, f.v, f.material, to_world, true);
                    if (f.emissive)
                        emitter_quads.push_back(qi);
                }
            } else {
                mypbr_voxel_model vm{};
                const VoxModel& m = vox.models[size_t(placed.model)];
                vm.nx = m.nx;
                vm.ny = m.ny;
                vm.nz = m.nz;
                vm.xform = add_xform(to_world);
                vm.cells = md.cells;
                vm.palette = palette;
                vm.edge_material = edge_material;
                vm.edge_width = edge_width;
                S.voxel_models.push_back(vm);
                int model_index = int(S.voxel_models.size()) - 1;
                for (const auto& b : md.blocks) {
                    mypbr_voxel_block vb{};
                    vb.model = model_index;
                    for (int a = 0; a < 3; a++) {
                        vb.lo[a] = b[size_t(a)];
                        vb.hi[a] = b[size_t(3 + a)];
                    }
                    S.voxel_blocks.push_back(vb);
                    Box box = Box::from_points(V3(b[0], b[1], b[2]), V3(b[3], b[4], b[5]));
                    add_item(MYPBR_PRIM_VOXEL_BLOCK, int(S.voxel_blocks.size()) - 1, to_world.box(box));
                }
                // emissive faces are sampled as lights; the grid itself is hit
                for (const auto& f : md.faces)
                    if (f.emissive)
                        emitter_quads.push_back(push_quad(f.q, f.u, f.v, f.material, to_world, true, false));
            }
            if (!emitter_quads.empty()) {
                double power = 0;
                int first = int(S.light_members.size());
                for (int qi : emitter_quads) {
                    power += kPi * 1.0 * average_emission_luminance(S.quads[size_t(qi)].material);
                    add_member(MYPBR_PRIM_QUAD, qi, 1.0 / double(emitter_quads.size()));
                }
                add_light(first, int(emitter_quads.size()), power * to_world.area_scale());
            }
        }
        return true;
    }

    // ------------------------------------------------------ keywords
    //
    // Every keyword of the .scene language (scene.h:44-243) has a handler in
    // one table; a handler reads its words and says false (with the message
    // in `error`) when they are wrong. Whatever a handler leaves unread is an
    // error too ("unexpected value").

    using LineHandler = bool (Loader::*)(Words&);
    static const std::map<std::string, LineHandler>& keywords() {
        static const std::map<std::string, LineHandler> table = {
            {"image_width", &Loader::image_width_line},
            {"aspect_ratio", &Loader::aspect_ratio_line},
            {"samples_per_pixel", &Loader::samples_line},
            {"max_depth", &Loader::max_depth_line},
            {"camera", &Loader::camera_line},
            {"vfov", &Loader::vfov_line},
            {"aperture", &Loader::aperture_line},
            {"focus", &Loader::focus_line},
            {"background", &Loader::background_line},
            {"light_selection", &Loader::light_selection_line},
            {"environment", &Loader::environment_line},
            {"sun", &Loader::sun_line},
            {"sky", &Loader::sky_line},
            {"ground", &Loader::ground_line},
            {"style", &Loader::style_line},
            {"bounces", &Loader::bounces_line},
            {"transparent_shadows", &Loader::transparent_shadows_line},
            {"height_fog", &Loader::height_fog_line},
            {"bloom", &Loader::bloom_line},
            {"vignette", &Loader::vignette_line},
            {"exposure", &Loader::exposure_line},
            {"tonemap", &Loader::tonemap_line},
            {"normal_maps", &Loader::normal_maps_line},
            {"texture", &Loader::texture_line},
            {"material", &Loader::material_line},
            {"sphere", &Loader::sphere_line},
            {"quad", &Loader::quad_line},
            {"box", &Loader::box_line},
            {"medium", &Loader::medium_line},
            {"fog", &Loader::fog_line},
            {"mesh", &Loader::mesh_line},
            {"vox", &Loader::vox_line},
            {"cyclorama", &Loader::studio_line},
            {"softbox", &Loader::studio_line},
        };
        return table;
    }

    bool parse_line(Words& w, const std::string& keyword) {
        auto handler = keywords().find(keyword);
        if (handler == keywords().end())
            return fail("unknown keyword '" + keyword + "'");
        current_keyword = keyword;
        if (!(this->*(handler->second))(w))
            return false;
        if (w.more())
            return fail("unexpected value '" + w.peek() + "'");
        return true;
    }
    std::string current_keyword;

    // One word that must be one of `choices`.
    static bool one_of(Words& w, std::initializer_list<const char*> choices, std::string& out) {
        if (!w.more())
            return false;
        for (const char* c : choices)
            if (w.peek() == c) {
                w.word(out);
                return true;
            }
        return false;
    }
    static bool on_off(Words& w, bool& state) {
        std::string v;
        if (!one_of(w, {"on", "off"}, v))
            return false;
        state = v == "on";
        return true;
    }
    static bool positive_integer(Words& w, int& x) {
        int v;
        if (!w.integer(v) || v < 1)
            return false;
        x = v;
        return true;
    }

    bool image_width_line(Words& w) {
        return positive_integer(w, S.camera.image_width) || fail("expected 'image_width <positive integer>'");
    }
    bool samples_line(Words& w) {
        return positive_integer(w, S.opts.samples_per_pixel) || fail("expected 'samples_per_pixel <positive integer>'");
    }
    bool max_depth_line(Words& w) {
        return positive_integer(w, S.opts.max_depth) || fail("expected 'max_depth <positive integer>'");
    }

    // "16/9" or a plain number
    bool aspect_ratio_line(Words& w) {
        std::string word;
        if (!w.word(word))
            return fail("expected 'aspect_ratio <w>/<h>' or 'aspect_ratio <number>'");
        size_t slash = word.find('/');
        double num, den = 1;
        if (!word_is_number(word.substr(0, slash), num))
            return fail("expected 'aspect_ratio <w>/<h>' or 'aspect_ratio <number>'");
        if (slash != std::string::npos && !word_is_number(word.substr(slash + 1), den))
            return fail("expected 'aspect_ratio <w>/<h>'");
        if (num <= 0 || den <= 0)
            return fail("aspect_ratio must be positive");
        S.camera.aspect_ratio = num / den;
        return true;
    }

    bool camera_line(Words& w) {
        auto& cam = S.camera;
        return settings(
            w,
            {{"lookfrom", [&](Words& v) { return v.triple(cam.lookfrom); }},
             {"lookat", [&](Words& v) { return v.triple(cam.lookat); }},
             {"vup", [&](Words& v) { return v.triple(cam.vup); }},
             {"vfov", [&](Words& v) { return v.number(cam.vfov, between(0, 180, true, true)); }},
             {"aperture", [&](Words& v) { return v.number(cam.defocus_angle, non_negative()); }},
             {"focus", [&](Words& v) { return v.number(cam.focus_dist, positive()); }},
             {"ortho", [&](Words& v) { return v.number(cam.ortho_height, non_negative()); }},
             {"blades",
              [&](Words& v) {
                  int n;
                  if (!v.integer(n) || (n != 0 && n < 3))
                      return false;
                  cam.blades = n;
                  return true;
              }},
             {"blade_rotation", [&](Words& v) { return v.number(cam.blade_rotation); }}},
            [](const std::string& key) { return "unknown camera setting '" + key + "'"; },
            [](const std::string& key) { return "bad value for camera setting '" + key + "'"; });
    }

    bool vfov_line(Words& w) {
        return w.number(S.camera.vfov, between(0, 180, true, true)) ||
               fail("expected 'vfov <degrees between 0 and 180>'");
    }
    bool aperture_line(Words& w) {
        return w.number(S.camera.defocus_angle, non_negative()) ||
               fail("expected 'aperture <defocus angle in degrees>'");
    }
    bool focus_line(Words& w) {
        return w.number(S.camera.focus_dist, positive()) || fail("expected 'focus <positive distance>'");
    }
    bool background_line(Words& w) {
        V3 c;
        if (!w.triple(c))
            return fail("expected 'background <r> <g> <b>'");
        S.use_sky = false;
        S.background = c;
        return true;
    }
    bool light_selection_line(Words& w) {
        std::string mode;
        if (!one_of(w, {"power", "uniform"}, mode))
            return fail("expected 'light_selection power|uniform'");
        power_selection = mode == "power";
        return true;
    }

    bool environment_line(Words& w) {
        const std::string usage = "expected 'environment <file.hdr> [intensity <s>] [rotate <degrees>]'";
        std::string file;
        double intensity = 1, rotation = 0;
        if (!w.word(file))
            return fail(usage);
        auto says = [&](const std::string&) { return usage; };
        if (!settings(w,
                      {{"intensity", [&](Words& v) { return v.number(intensity, non_negative()); }},
                       {"rotate", [&](Words& v) { return v.number(rotation); }}},
                      says, says))
            return false;
        if (file[0] != '/')
            file = scene_dir + file;
        int width, height;
        std::vector<float> rgb;
        std::string why;
        if (!read_hdr(file, width, height, rgb, why))
            return fail("cannot load environment map '" + file + "'");
        if (has_environment)
            return fail("only one environment is allowed");
        set_environment(width, height, std::move(rgb), intensity, rotation / 360);
        return true;
    }

    bool sun_line(Words& w) {
        const std::string usage = "expected 'sun elevation <deg> azimuth <deg> [intensity <E>] [color <r g b>] "
                                  "[angle <deg>] [disk on|off]' or 'sun off'";
        auto says = [&](const std::string&) { return usage; };
        sun_on = true;
        return settings(w,
                        {{"off", [&](Words&) { return !(sun_on = false); }},
                         {"elevation", [&](Words& v) { return v.number(sun_elevation, between(-90, 90, false, false)); }},
                         {"azimuth", [&](Words& v) { return v.number(sun_azimuth); }},
                         {"intensity", [&](Words& v) { return v.number(sun_intensity, non_negative()); }},
                         {"color", [&](Words& v) { return v.triple(sun_tint); }},
                         {"angle", [&](Words& v) { return v.number(sun_angle, between(0, 90, true, true)); }},
                         {"disk", [&](Words& v) { return on_off(v, sun_disk); }}},
                        says, says);
    }

    bool sky_line(Words& w) {
        std::string type;
        if (!w.word(type))
            return fail("expected 'sky uniform <r g b>', 'sky atmosphere [...]' or 'sky gradient'");
        if (type == "uniform") {
            if (!w.triple(sky_radiance))
                return fail("expected 'sky uniform <r g b>'");
            sky_uniform = true;
            sky_atmosphere = false;
        } else if (type == "atmosphere") {  // scene.h:574-586
            const std::string usage =
                "expected 'sky atmosphere [rayleigh <x>] [mie <x>] [mie_g <g>] [ozone <x>] [intensity <s>]'";
            auto says = [&](const std::string&) { return usage; };
            if (!settings(w,
                          {{"rayleigh", [&](Words& v) { return v.number(air.rayleigh, non_negative()); }},
                           {"mie", [&](Words& v) { return v.number(air.mie, non_negative()); }},
                           {"mie_g", [&](Words& v) { return v.number(air.mie_g, between(-1, 1, true, true)); }},
                           {"ozone", [&](Words& v) { return v.number(air.ozone, non_negative()); }},
                           {"intensity", [&](Words& v) { return v.number(air.intensity, non_negative()); }}},
                          says, says))
                return false;
            sky_atmosphere = true;
            sky_uniform = false;
        } else if (type == "gradient") {
            sky_uniform = false;
            sky_atmosphere = false;
        } else {
            return fail("unknown sky type '" + type + "' (expected uniform, atmosphere or gradient)");
        }
        S.use_sky = true;
        return true;
    }

    // "ground [off] [height <y>] [material]", in any order
    bool ground_line(Words& w) {
        ground = true;
        std::string key;
        while (w.word(key)) {
            if (key == "off") {
                ground = false;
            } else if (key == "height") {
                if (!w.number(ground_height))
                    return fail("expected 'ground [height <y>] [material]'");
            } else {
                auto found = materials.find(key);
                if (found == materials.end())
                    return fail("unknown material '" + key + "'");
                ground_material = found->second;
            }
        }
        return true;
    }

    // A preset of the lines it stands for (scene.h:612-640)
    bool style_line(Words& w) {
        std::string name;
        if (!one_of(w, {"voxel", "classic"}, name))
            return fail("expected 'style voxel' or 'style classic'");
        const bool voxel = name == "voxel";
        sun_on = voxel;
        sun_elevation = voxel ? 50 : 45;
        sun_azimuth = voxel ? 50 : 45;
        sun_intensity = voxel ? 4 : 3;
        sun_angle = voxel ? 3 : 4;
        sun_tint = V3(1, 1, 1);
        sun_disk = true;
        sky_uniform = false;
        sky_atmosphere = voxel;
        air = mypbr_sky::Settings();
        S.use_sky = true;
        ground = voxel;
        ground_material = voxel ? lambertian(V3(0.3, 0.3, 0.3)) : default_material;
        S.opts.max_diffuse = voxel ? 2 : 0;
        S.opts.max_specular = voxel ? 5 : 0;
        S.opts.max_scatter = voxel ? 5 : 0;
        S.opts.transparent_shadows = voxel;
        return true;
    }

    bool bounces_line(Words& w) {
        const std::string usage = "expected 'bounces [diffuse <n>] [specular <n>] [scatter <n>]'";
        auto says = [&](const std::string&) { return usage; };
        auto cap = [](int& field) {
            return [&field](Words& v) {
                int n;
                if (!v.integer(n) || n < 0)
                    return false;
                field = n;
                return true;
            };
        };
        return settings(w,
                        {{"diffuse", cap(S.opts.max_diffuse)},
                         {"specular", cap(S.opts.max_specular)},
                         {"scatter", cap(S.opts.max_scatter)}},
                        says, says);
    }

    bool transparent_shadows_line(Words& w) {
        bool on;
        if (!on_off(w, on))
            return fail("expected 'transparent_shadows on|off'");
        S.opts.transparent_shadows = on;
        return true;
    }
    bool normal_maps_line(Words& w) {
        return on_off(w, use_normal_maps) || fail("expected 'normal_maps on|off'");
    }

    // A volume material by name, for fog lines
    bool volume_material(const std::string& name, int& mat) {
        auto found = materials.find(name);
        if (found == materials.end() || S.materials[found->second].type != MYPBR_MAT_PHASE)
            return fail("expected a volume material, got '" + name + "'");
        mat = found->second;
        return true;
    }

    bool height_fog_line(Words& w) {
        const char* usage = "expected 'height_fog <density> <scale height> <volume material> [base <y>]'";
        double density, scale, base = 0;
        std::string name;
        if (!w.number(density, positive()) || !w.number(scale, positive()) || !w.word(name))
            return fail(usage);
        if (w.more()) {  // one optional setting
            std::string key;
            w.word(key);
            if (key != "base" || !w.number(base))
                return fail(usage);
        }
        mypbr_unbounded u{};
        if (!volume_material(name, u.material))
            return false;
        u.kind = MYPBR_UNBOUNDED_HEIGHT_FOG;
        u.height = base;
        u.density = density;
        u.scale_height = scale;
        S.unbounded.push_back(u);
        return true;
    }

    bool fog_line(Words& w) {
        std::string name;
        if (!w.number(fog_density, positive()) || !w.word(name))
            return fail("expected 'fog <positive density> <volume material>'");
        return volume_material(name, fog_material);
    }

    // Display settings: they change written images, not the radiance
    // frame, so they are checked and not kept.
    bool bloom_line(Words& w) {
        const std::string usage = "expected 'bloom <strength> [threshold <radiance>] [radius <fraction of width>]'";
        double x;
        if (!w.number(x, non_negative()))
            return fail(usage);
        auto says = [&](const std::string&) { return usage; };
        return settings(w,
                        {{"threshold", [&](Words& v) { return v.number(x, non_negative()); }},
                         {"radius", [&](Words& v) { return v.number(x, positive()); }}},
                        says, says);
    }
    bool vignette_line(Words& w) {
        double v;
        return w.number(v, non_negative()) || fail("expected 'vignette <strength>'");
    }
    bool exposure_line(Words& w) {
        double v;
        return w.number(v) || fail("expected 'exposure <stops>'");
    }
    bool tonemap_line(Words& w) {
        std::string op;
        return one_of(w, {"none", "reinhard", "aces"}, op) || fail("expected 'tonemap none|reinhard|aces'");
    }

    bool studio_line(Words&) {
        unsupported = true;
        return fail("'" + current_keyword + "' is not supported by this backend");
    }

    // ------------------------------------------------------ objects

    bool sphere_line(Words& w) {
        V3 c;
        double r;
        if (!w.triple(c) || !w.number(r) || r == 0)
            return fail("expected 'sphere <x> <y> <z> <non-zero radius> [material] [transforms]'");
        Placement at;
        error.clear();
        return (read_placement(w, at) && add_sphere(c, r, at.material, at.xform, at.moved)) || fail(error);
    }

    bool quad_line(Words& w) {
        V3 q, u, v;
        if (!w.triple(q) || !w.triple(u) || !w.triple(v))
            return fail("expected 'quad <Qx Qy Qz> <ux uy uz> <vx vy vz> [material] [transforms]'");
        if (cross(u, v).near_zero())
            return fail("quad edges must not be parallel");
        Placement at;
        error.clear();
        return (read_placement(w, at) && add_quad(q, u, v, at.material, at.xform, at.moved)) || fail(error);
    }

    bool box_line(Words& w) {
        V3 a, b;
        if (!w.triple(a) || !w.triple(b))
            return fail("expected 'box <x0 y0 z0> <x1 y1 z1> [material] [transforms]'");
        Placement at;
        error.clear();
        return (read_placement(w, at) && add_box(a, b, at.material, at.xform, at.moved)) || fail(error);
    }

    bool medium_line(Words& w) {
        double density;
        std::string shape;
        if (!w.number(density, positive()) || !w.word(shape))
            return fail("expected 'medium <positive density> sphere|box <...> <material> [transforms]'");
        V3 a, b;
        const bool sphere = shape == "sphere";
        if (sphere) {
            double r;
            if (!w.triple(a) || !w.number(r, positive()))
                return fail("expected 'medium <density> sphere <x> <y> <z> <positive radius> <material>'");
            b = V3(r, 0, 0);
        } else if (shape == "box") {
            if (!w.triple(a) || !w.triple(b))
                return fail("expected 'medium <density> box <x0 y0 z0> <x1 y1 z1> <material>'");
        } else {
            return fail("a medium's boundary must be 'sphere' or 'box'");
        }
        Placement at;
        error.clear();
        if (!read_placement(w, at))
            return fail(error);
        if (S.materials[at.material].type != MYPBR_MAT_PHASE)
            return fail("a medium needs a volume material");
        add_medium(density, sphere, a, b, at.material, at.xform, at.moved);
        return true;
    }

    // "mesh <file> [smooth] [replace <file material> <scene material>]...
    // [material] [transforms]": OBJ, or glTF (.gltf / .glb) with its own
    // materials, which one named on the line replaces all of.
    bool mesh_line(Words& w) {
        std::string file;
        if (!w.word(file))
            return fail("expected 'mesh <file.obj> [material] [transforms]'");
        if (file[0] != '/')
            file = scene_dir + file;
        const bool smooth = w.peek() == "smooth";
        if (smooth)
            w.skip();
        std::map<std::string, int> replace;
        while (w.peek() == "replace") {
            w.skip();
            std::string from, to;
            if (!w.word(from) || !w.word(to))
                return fail("expected 'replace <material in the file> <scene material>'");
            auto found = materials.find(to);
            if (found == materials.end())
                return fail("unknown material '" + to + "'");
            replace[from] = found->second;
        }
        Placement at;
        error.clear();
        if (!read_placement(w, at))
            return fail(error);
        if (!replace.empty() && at.material != default_material)
            return fail("'replace' and a material for the whole mesh can't be used together");
        auto has_suffix = [&](const std::string& suffix) {
            return file.size() >= suffix.size() && file.compare(file.size() - suffix.size(), suffix.size(), suffix) == 0;
        };
        const bool gltf = has_suffix(".gltf") || has_suffix(".glb");
        if (!gltf && !replace.empty())
            return fail("'replace' is for glTF files (OBJ files take scene materials by usemtl name)");
        bool ok = gltf ? add_gltf(file, at.material == default_material ? -1 : at.material, replace, at.xform, at.moved)
                       : add_obj(file, smooth, at.material, at.xform, at.moved);
        return ok || fail(error);
    }

    void set_environment(int w, int h, std::vector<float> rgb, double intensity, double rotation_turns) {
        S.env_pixels = std::move(rgb);
        S.env_width = w;
        S.env_height = h;
        S.env_intensity = intensity;
        S.env_rotation = rotation_turns;
        has_environment = true;
        pending_lights.push_back({MYPBR_LIGHT_ENVIRONMENT, 0, 0, -1});
    }

    // env power: pi R^2 times the integral of luminance over the sphere (environment.h:252-263)
    double environment_power(double radius) const {
        double sum = 0;
        int w = S.env_width, h = S.env_height;
        for (int j = 0; j < h; j++) {
            double s = std::sin(kPi * (j + 0.5) / h);
            for (int i = 0; i < w; i++) {
                // "sky uniform" keeps its FP64 radiance, as the reference's in-memory sky does
                size_t k = (size_t(j) * w + i) * 3;
                const float* p = &S.env_pixels[k];
                V3 c = uniform_sky_env     ? sky_radiance
                       : !env_fp64.empty() ? V3(env_fp64[k], env_fp64[k + 1], env_fp64[k + 2])
                                           : V3(p[0], p[1], p[2]);
                double wgt = luminance(c) * s;
                sum += std::fmax(wgt, 0.0);
            }
        }
        double integral = S.env_intensity * sum * (2 * kPi / w) * (kPi / h);
        return kPi * radius * radius * integral;
    }

    bool finish() {
        if (items.empty() && S.media.empty())
            return fail("the scene has no objects");
        if (sky_uniform) {
            if (has_environment)
                return fail("'sky uniform' and 'environment' can't be used together");
            std::vector<float> rgb(8 * 4 * 3);
            for (int k = 0; k < 32; k++) {
                rgb[3 * k] = float(sky_radiance.x);
                rgb[3 * k + 1] = float(sky_radiance.y);
                rgb[3 * k + 2] = float(sky_radiance.z);
            }
            set_environment(8, 4, std::move(rgb), 1.0, 0.0);
            uniform_sky_env = true;
        }
        double el = radians(sun_elevation), az = radians(sun_azimuth);
        V3 sun_dir(std::cos(el) * std::sin(az), std::sin(el), -std::cos(el) * std::cos(az));
        V3 sun_irr = sun_intensity * sun_tint;
        if (sky_atmosphere) {  // scene.h:1220-1230: a 256 x 128 bake, the sun reddened by the air
            if (has_environment)
                return fail("'sky atmosphere' and 'environment' can't be used together");
            const int w = 256, h = 128;
            double sd[3] = {sun_dir.x, sun_dir.y, sun_dir.z};
            mypbr_sky::C3 irr{sun_irr.x, sun_irr.y, sun_irr.z};
            std::vector<float> rgb(size_t(w) * h * 3);
            env_fp64.assign(rgb.size(), 0.0);
            for (int j = 0; j < h; j++)
                for (int i = 0; i < w; i++) {
                    mypbr_sky::C3 c = mypbr_sky::bake_pixel(air, i, j, w, h, sd, irr);
                    size_t k = (size_t(j) * w + i) * 3;
                    env_fp64[k] = c.r;
                    env_fp64[k + 1] = c.g;
                    env_fp64[k + 2] = c.b;
                    rgb[k] = float(c.r);
                    rgb[k + 1] = float(c.g);
                    rgb[k + 2] = float(c.b);
                }
            set_environment(w, h, std::move(rgb), 1.0, 0.0);
            mypbr_sky::C3 t = mypbr_sky::sun_transmittance(air, sd);
            sun_irr = V3(sun_irr.x * t.r, sun_irr.y * t.g, sun_irr.z * t.b);
        }
        if (sun_on) {
            S.sun.enabled = 1;
            S.sun.disk_visible = sun_disk;
            V3 d = unit(sun_dir);
            for (int k = 0; k < 3; k++) {
                S.sun.direction[k] = d[k];
                S.sun.irradiance[k] = sun_irr[k];
            }
            S.sun.angular_diameter = sun_angle;
            pending_lights.push_back({MYPBR_LIGHT_SUN, 0, 0, -1});
        }
        if (ground) {
            mypbr_unbounded u{};
            u.kind = MYPBR_UNBOUNDED_GROUND;
            u.material = ground_material;
            u.height = ground_height;
            S.unbounded.push_back(u);
        }
        if (fog_material >= 0) {
            Box e = world_box;
            add_medium(fog_density, false, e.lo, e.hi, fog_material, Xf(), false);
        }
        V3 lf(S.camera.lookfrom[0], S.camera.lookfrom[1], S.camera.lookfrom[2]);
        V3 la(S.camera.lookat[0], S.camera.lookat[1], S.camera.lookat[2]);
        V3 vu(S.camera.vup[0], S.camera.vup[1], S.camera.vup[2]);
        if ((lf - la).near_zero() || cross(vu, lf - la).near_zero())
            return fail("camera lookfrom must differ from lookat, and vup must not point along the view");

        // Light selection probabilities (light_list.h:45-96)
        size_t n = pending_lights.size();
        std::vector<double> prob(n, n > 0 ? 1.0 / n : 0.0);
        if (n > 0 && power_selection) {
            double radius = 0;
            if (world_box.size(0) > 0 && world_box.size(1) > 0 && world_box.size(2) > 0)
                radius = 0.5 * std::sqrt(world_box.size(0) * world_box.size(0) +
                                         world_box.size(1) * world_box.size(1) +
                                         world_box.size(2) * world_box.size(2));
            if (!std::isfinite(radius) || radius <= 0)
                radius = 1;
            std::vector<double> power(n);
            double known_sum = 0;
            int known = 0;
            for (size_t k = 0; k < n; k++) {
                const auto& L = pending_lights[k];
                if (L.kind == MYPBR_LIGHT_ENVIRONMENT)
                    power[k] = environment_power(radius);
                else if (L.kind == MYPBR_LIGHT_SUN)
                    power[k] = kPi * radius * radius * luminance(sun_irr);
                else
                    power[k] = L.power;
                if (std::isfinite(power[k]) && power[k] > 0) {
                    known_sum += power[k];
                    known++;
                }
            }
            double fallback = known > 0 ? known_sum / known : 1.0;
            double total = 0;
            for (auto& p : power) {
                if (!std::isfinite(p) || p <= 0)
                    p = fallback;
                total += p;
            }
            const double uniform_fraction = 0.2;
            for (size_t k = 0; k < n; k++)
                prob[k] = (1 - uniform_fraction) * power[k] / total + uniform_fraction / n;
        }
        for (size_t k = 0; k < n; k++) {
            mypbr_light l{};
            l.kind = pending_lights[k].kind;
            l.first_member = pending_lights[k].first_member;
            l.member_count = pending_lights[k].member_count;
            l.probability = prob[k];
            S.lights.push_back(l);
        }
        build_bvh(items, S.bvh_nodes, S.bvh_prims);
        return true;
    }

    int run(std::istream& file) {
        default_material = lambertian(V3(0.5, 0.5, 0.5));
        ground_material = default_material;
        std::string line;
        while (std::getline(file, line)) {
            line_number++;
            auto comment = line.find('#');
            if (comment != std::string::npos)
                line.erase(comment);
            Words w(line);
            std::string keyword;
            if (!w.word(keyword))
                continue;
            if (!parse_line(w, keyword)) {
                set_error(error);
                return unsupported ? MYPBR_ERR_UNSUPPORTED : MYPBR_ERR_BAD_SCENE;
            }
        }
        if (!finish()) {
            set_error(error);
            return unsupported ? MYPBR_ERR_UNSUPPORTED : MYPBR_ERR_BAD_SCENE;
        }
        S.finalize();
        return MYPBR_OK;
    }
};

}  // namespace

// ----------------------------------------------------------- host scene

void mypbr_host_scene::finalize() {
    flat = mypbr_flat_scene{};
    flat.abi_version = MYPBR_ABI_VERSION;
    flat.spheres = spheres.data();
    flat.sphere_count = int64_t(spheres.size());
    flat.quads = quads.data();
    flat.quad_count = int64_t(quads.size());
    flat.positions = positions.data();
    flat.position_count = position_count();
    flat.normals = normals.data();
    flat.normal_count = normal_count();
    flat.uvs = uvs.data();
    flat.uv_count = uv_count();
    flat.triangles = triangles.data();
    flat.triangle_count = int64_t(triangles.size());
    flat.meshes = meshes.data();
    flat.mesh_count = int64_t(meshes.size());
    flat.media = media.data();
    flat.medium_count = int64_t(media.size());
    flat.xforms = xforms.data();
    flat.xform_count = int64_t(xforms.size());
    flat.unbounded = unbounded.data();
    flat.unbounded_count = int64_t(unbounded.size());
    flat.bvh_nodes = bvh_nodes.data();
    flat.bvh_node_count = int64_t(bvh_nodes.size());
    flat.bvh_prims = bvh_prims.data();
    flat.bvh_prim_count = int64_t(bvh_prims.size());
    flat.materials = materials.data();
    flat.material_count = int64_t(materials.size());
    flat.textures = textures.data();
    flat.texture_count = int64_t(textures.size());
    flat.texels_ldr = texels_ldr.data();
    flat.texels_ldr_bytes = int64_t(texels_ldr.size());
    flat.texels_hdr = texels_hdr.data();
    flat.texels_hdr_count = int64_t(texels_hdr.size());
    flat.lights = lights.data();
    flat.light_count = int64_t(lights.size());
    flat.light_members = light_members.data();
    flat.light_member_count = int64_t(light_members.size());
    flat.environment.width = env_pixels.empty() ? 0 : env_width;
    flat.environment.height = env_pixels.empty() ? 0 : env_height;
    flat.environment.pixels = env_pixels.data();
    flat.environment.intensity = env_intensity;
    flat.environment.rotation = env_rotation;
    flat.sun = sun;
    flat.use_sky = use_sky ? 1 : 0;
    flat.background[0] = background.x;
    flat.background[1] = background.y;
    flat.background[2] = background.z;
    flat.voxel_models = voxel_models.data();
    flat.voxel_model_count = int64_t(voxel_models.size());
    flat.voxel_blocks = voxel_blocks.data();
    flat.voxel_block_count = int64_t(voxel_blocks.size());
    flat.voxel_palettes = voxel_palettes.data();
    flat.voxel_palette_count = int64_t(voxel_palettes.size());
    flat.voxel_cells = voxel_cells.data();
    flat.voxel_cell_bytes = int64_t(voxel_cells.size());
    // Camera height as camera::initialize computes it (camera.h:143-144)
    int h = int(camera.image_width / camera.aspect_ratio);
    camera.image_height = h < 1 ? 1 : h;
}

extern "C" {

void mypbr_camera_init(mypbr_camera* cam) {
    if (!cam)
        return;
    *cam = mypbr_camera{};
    cam->image_width = 100;
    cam->aspect_ratio = 1.0;
    cam->image_height = 100;
    cam->vfov = 90;
    cam->lookat[2] = -1;
    cam->vup[1] = 1;
    cam->focus_dist = 10;
}

void mypbr_render_opts_init(mypbr_render_opts* opts) {
    if (!opts)
        return;
    *opts = mypbr_render_opts{};
    opts->samples_per_pixel = 10;
    opts->max_depth = 10;
    opts->seed = 0x6d797062725f6762ull;
}

const char* mypbr_last_error(void) { return g_last_error.c_str(); }

const char* mypbr_gpu_status_string(int status) {
    switch (status) {
        case MYPBR_OK: return "ok";
        case MYPBR_ERR_CUDA: return "CUDA error";
        case MYPBR_ERR_UNSUPPORTED: return "unsupported feature";
        case MYPBR_ERR_QUEUE_OVERFLOW: return "device queue overflow";
        case MYPBR_ERR_DEVICE_TIMEOUT: return "device wait timed out";
        case MYPBR_ERR_INVALID_ARGUMENT: return "invalid argument";
        case MYPBR_ERR_OUT_OF_MEMORY: return "out of memory";
        case MYPBR_ERR_BAD_SCENE: return "bad scene";
        case MYPBR_ERR_IO: return "I/O error";
        case MYPBR_ERR_NO_DEVICE: return "no CUDA device";
        case MYPBR_ERR_DEVICE_CHECK: return "device bounds check failed";
        default: return "unknown status";
    }
}

static int load_from_stream(std::istream& in, const std::string& name, const std::string& dir,
                            mypbr_host_scene** out) {
    auto s = std::make_unique<mypbr_host_scene>();
    mypbr_camera_init(&s->camera);
    mypbr_render_opts_init(&s->opts);
    Loader loader(*s);
    loader.path_for_errors = name;
    loader.scene_dir = dir;
    int status;
    try {
        status = loader.run(in);
    } catch (const std::bad_alloc&) {
        set_error(name + ": out of host memory");
        return MYPBR_ERR_OUT_OF_MEMORY;
    }
    if (status != MYPBR_OK)
        return status;
    *out = s.release();
    return MYPBR_OK;
}

int mypbr_scene_load(const char* path, mypbr_host_scene** out) {
    if (!path || !out) {
        set_error("mypbr_scene_load: null argument");
        return MYPBR_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    clear_error();
    std::string p(path);
    std::ifstream file(p);
    if (!file) {
        set_error("Error: cannot open scene file '" + p + "'");
        return MYPBR_ERR_IO;
    }
    auto slash = p.find_last_of('/');
    std::string dir = slash == std::string::npos ? "" : p.substr(0, slash + 1);
    return load_from_stream(file, p, dir, out);
}

int mypbr_scene_parse(const char* text, const char* base_dir, mypbr_host_scene** out) {
    if (!text || !out) {
        set_error("mypbr_scene_parse: null argument");
        return MYPBR_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    clear_error();
    std::string dir = base_dir ? base_dir : "";
    if (!dir.empty() && dir.back() != '/')
        dir += '/';
    std::istringstream in{std::string(text)};
    return load_from_stream(in, "<scene text>", dir, out);
}

const mypbr_flat_scene* mypbr_scene_flat(const mypbr_host_scene* s) { return s ? &s->flat : nullptr; }
const mypbr_camera* mypbr_scene_camera(const mypbr_host_scene* s) { return s ? &s->camera : nullptr; }
const mypbr_render_opts* mypbr_scene_render_opts(const mypbr_host_scene* s) { return s ? &s->opts : nullptr; }
void mypbr_scene_free(mypbr_host_scene* s) { delete s; }

int mypbr_ggx_albedo_table(double* out) {
    if (!out) {
        set_error("mypbr_ggx_albedo_table: null argument");
        return MYPBR_ERR_INVALID_ARGUMENT;
    }
    ggx_albedo_table(out);
    return MYPBR_OK;
}

int mypbr_image_read(const char* path, int32_t* width, int32_t* height, int32_t* channels, uint8_t* rgba,
                     int64_t capacity) {
    if (!path || !width || !height || !channels) {
        set_error("mypbr_image_read: null argument");
        return MYPBR_ERR_INVALID_ARGUMENT;
    }
    clear_error();
    mypbr_host::LdrImage img;
    std::string err;
    if (!mypbr_host::read_ldr_image(path, img, err)) {
        std::vector<uint8_t> probe;
        bool readable = mypbr_host::read_file_bytes(path, probe);
        set_error("cannot load image '" + std::string(path) + "': " + err);
        if (!readable)
            return MYPBR_ERR_IO;
        auto kind = mypbr_host::sniff_image(probe.data(), probe.size());
        return img.unsupported || kind == mypbr_host::ImageKind::Hdr ? MYPBR_ERR_UNSUPPORTED : MYPBR_ERR_BAD_SCENE;
    }
    *width = img.width;
    *height = img.height;
    *channels = img.channels;
    if (rgba) {
        if (capacity < int64_t(img.rgba.size())) {
            set_error("mypbr_image_read: the buffer holds fewer than width * height * 4 bytes");
            return MYPBR_ERR_INVALID_ARGUMENT;
        }
        std::memcpy(rgba, img.rgba.data(), img.rgba.size());
    }
    return MYPBR_OK;
}

}  // extern "C"
