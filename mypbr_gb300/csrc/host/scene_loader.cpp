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

    // ------------------------------------------------------ number reading

    bool read_color_or_texture(std::istringstream& in, const std::string& first, int& tex) {
        if (first == "texture") {
            std::string name;
            if (!(in >> name))
                return false;
            auto it = textures.find(name);
            if (it == textures.end()) {
                error = "unknown texture '" + name + "'";
                return false;
            }
            tex = it->second;
            return true;
        }
        std::istringstream rgb(first);
        double r, g, b;
        if (!(rgb >> r) || !(in >> g >> b))
            return false;
        tex = add_texture_solid(V3(r, g, b));
        return true;
    }

    bool read_texture_name(std::istringstream& in, int& tex) {
        std::string name;
        if (!(in >> name)) {
            error = "expected a texture name";
            return false;
        }
        auto it = textures.find(name);
        if (it == textures.end()) {
            error = "unknown texture '" + name + "'";
            return false;
        }
        tex = it->second;
        return true;
    }

    bool read_value_or_texture(std::istringstream& in, int& tex) {
        std::string first;
        if (!(in >> first))
            return false;
        if (first == "texture")
            return read_texture_name(in, tex);
        std::istringstream number(first);
        double x;
        if (!(number >> x) || x < 0 || x > 1)
            return false;
        tex = add_texture_solid(V3(x, x, x));
        return true;
    }

    // Optional material name, then transforms in order (scene.h:330-403).
    bool read_tail(std::istringstream& in, int& mat, Xf& xform, bool& transformed) {
        mat = default_material;
        xform = Xf();
        transformed = false;
        auto is_transform = [](const std::string& t) {
            return t == "translate" || t == "scale" || t == "rotate" || t == "rotate_x" || t == "rotate_y" ||
                   t == "rotate_z";
        };
        std::string token;
        if (!(in >> token))
            return true;
        if (!is_transform(token)) {
            auto it = materials.find(token);
            if (it == materials.end()) {
                error = "unknown material '" + token + "'";
                return false;
            }
            mat = it->second;
            if (!(in >> token))
                return true;
        }
        do {
            Xf step;
            bool ok = true;
            if (token == "translate") {
                V3 d;
                ok = bool(in >> d.x >> d.y >> d.z);
                step = Xf::translate(d);
            } else if (token == "rotate_x" || token == "rotate_y" || token == "rotate_z") {
                double deg;
                ok = bool(in >> deg);
                V3 axis(token == "rotate_x", token == "rotate_y", token == "rotate_z");
                step = Xf::rotate(deg, axis);
            } else if (token == "rotate") {
                double deg;
                V3 axis;
                ok = bool(in >> deg >> axis.x >> axis.y >> axis.z) && axis.length_squared() > 0;
                if (ok)
                    step = Xf::rotate(deg, axis);
            } else if (token == "scale") {
                V3 f;
                ok = bool(in >> f.x);
                if (ok) {
                    std::streampos mark = in.tellg();
                    if (in >> f.y) {
                        ok = bool(in >> f.z);
                    } else {
                        in.clear();
                        in.seekg(mark);
                        f = V3(f.x, f.x, f.x);
                    }
                }
                ok = ok && f.x != 0 && f.y != 0 && f.z != 0;
                step = Xf::scale(f);
            } else {
                error = "unexpected value '" + token +
                        "' (expected a transform: translate, scale, rotate, rotate_x, rotate_y or rotate_z)";
                return false;
            }
            if (!ok) {
                error = "bad values for '" + token + "'";
                return false;
            }
            xform = step.then_after(xform);
            transformed = true;
        } while (in >> token);
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

    // Reads an MTL file into result (include/obj_loader.h:33-177): Kd / map_Kd
    // give a lambertian, a non-black Ks a principled material with roughness
    // sqrt(sqrt(2 / (Ns + 2))) and ior Ni (1.5 unless above 1), Ke an emissive
    // one; norm / map_Bump / bump / map_Disp / disp a tangent-space normal map
    // (grey images under the bump and disp names are height maps, skipped);
    // map_d, else an alpha channel in map_Kd, the alpha mask. Textures repeat
    // and are relative to the MTL file; options before a file name are skipped
    // by taking the last word. An image that cannot be loaded gives a warning
    // and the plain color. False only if the file cannot be opened.
    bool load_mtl(const std::string& path, std::map<std::string, MtlMaterial>& result, std::string& err) {
        std::ifstream file(path);
        if (!file) {
            err = "cannot open '" + path + "'";
            return false;
        }
        auto slash = path.find_last_of('/');
        std::string dir = slash == std::string::npos ? "" : path.substr(0, slash + 1);
        auto image = [&](const std::string& name, bool linear) {
            std::string full = name[0] == '/' ? name : dir + name;
            std::string e;
            int t = load_image(full, true, linear, e);
            if (t < 0)
                std::fprintf(stderr, "Warning: %s: cannot load texture '%s'\n", path.c_str(), full.c_str());
            return t;
        };
        struct Entry {
            V3 kd{0.8, 0.8, 0.8}, ks{0, 0, 0}, ke{0, 0, 0};
            double ns = 0, ni = 1.5;
            int map_kd = -1, map_d = -1, normal_map = -1;
        };
        std::vector<std::pair<std::string, Entry>> entries;
        std::string line;
        while (std::getline(file, line)) {
            std::istringstream in(line);
            std::string keyword;
            if (!(in >> keyword) || keyword[0] == '#')
                continue;
            if (keyword == "newmtl") {
                std::string name;
                in >> name;
                entries.push_back({name, Entry()});
                continue;
            }
            if (entries.empty())
                continue;
            Entry& e = entries.back().second;
            auto read_color = [&](V3& c) {
                double r, g, b;
                if (in >> r) {
                    c = V3(r, r, r);  // one value is grey
                    if (in >> g >> b)
                        c = V3(r, g, b);
                }
            };
            auto last_word = [&]() {
                std::string word, last;
                while (in >> word)
                    last = word;
                return last;
            };
            if (keyword == "Kd") {
                read_color(e.kd);
            } else if (keyword == "Ks") {
                read_color(e.ks);
            } else if (keyword == "Ke") {
                read_color(e.ke);
            } else if (keyword == "Ns") {
                in >> e.ns;
            } else if (keyword == "Ni") {
                in >> e.ni;
            } else if (keyword == "map_Kd") {
                std::string f = last_word();
                if (!f.empty())
                    e.map_kd = image(f, false);
            } else if (keyword == "map_d") {
                std::string f = last_word();
                if (!f.empty())
                    e.map_d = image(f, false);
            } else if (keyword == "norm" || keyword == "map_Bump" || keyword == "map_bump" || keyword == "bump" ||
                       keyword == "map_Disp" || keyword == "disp") {
                std::string f = last_word();
                if (f.empty() || !use_normal_maps)
                    continue;
                int t = image(f, true);
                if (t >= 0 && keyword != "norm" && image_info[t].grey) {
                    std::fprintf(stderr, "Warning: %s: '%s' is a height map; only normal maps are supported\n",
                                 path.c_str(), f.c_str());
                    continue;
                }
                if (t >= 0)
                    e.normal_map = t;
            }
        }
        for (auto& [name, e] : entries) {
            MtlMaterial out;
            int base = e.map_kd >= 0 ? e.map_kd : -1;
            bool emits = e.ke.length_squared() > 0;
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
                double roughness = std::sqrt(std::sqrt(2 / (std::fmax(e.ns, 0.0) + 2)));
                double ior = e.ni > 1 ? e.ni : 1.5;
                int color = base >= 0 ? base : add_texture_solid(e.kd);
                int metallic = add_texture_solid(V3(0, 0, 0));
                m = principled_desc(color, metallic, add_texture_solid(V3(roughness, roughness, roughness)), ior);
            } else {
                m = blank_material(MYPBR_MAT_LAMBERTIAN);
                m.tex[0] = base >= 0 ? base : add_texture_solid(e.kd);
            }
            // normal_mapped wraps the surface materials, not lights (obj_loader.h:166-167)
            if (e.normal_map >= 0 && !emits)
                m.normal_map = e.normal_map;
            out.material = add_material(m);
            if (e.map_d >= 0 && !image_info[e.map_d].opaque)
                out.alpha_mask = e.map_d;
            else if (e.map_d < 0 && e.map_kd >= 0 && image_info[e.map_kd].alpha_channel && !image_info[e.map_kd].opaque)
                out.alpha_mask = e.map_kd;
            result[name] = out;
        }
        return true;
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

    bool add_obj(const std::string& file, bool smooth, int line_mat, const Xf& xform, bool transformed) {
        std::ifstream in(file);
        if (!in) {
            error = "cannot open '" + file + "'";
            return false;
        }
        std::vector<V3> pos, nrm, uv;
        std::vector<Surface> part_order;
        std::map<Surface, std::vector<Face>> faces;
        Surface current{line_mat, -1};
        std::map<std::string, MtlMaterial> file_materials;
        auto slash = file.find_last_of('/');
        std::string obj_dir = slash == std::string::npos ? "" : file.substr(0, slash + 1);
        auto resolve = [](long index, size_t count) -> int {
            if (index > 0 && size_t(index) <= count)
                return int(index - 1);
            if (index < 0 && size_t(-index) <= count)
                return int(long(count) + index);
            return -1;
        };
        std::string line;
        int ln = 0;
        while (std::getline(in, line)) {
            ln++;
            const char* s = line.c_str();
            while (*s == ' ' || *s == '\t')
                s++;
            auto read_vec = [&](const char* p, int n) {
                double x[3] = {0, 0, 0};
                char* end;
                for (int k = 0; k < n; k++) {
                    x[k] = std::strtod(p, &end);
                    p = end;
                }
                return V3(x[0], x[1], x[2]);
            };
            if (s[0] == 'v' && (s[1] == ' ' || s[1] == '\t')) {
                pos.push_back(read_vec(s + 2, 3));
            } else if (s[0] == 'v' && s[1] == 'n') {
                nrm.push_back(read_vec(s + 2, 3));
            } else if (s[0] == 'v' && s[1] == 't') {
                uv.push_back(read_vec(s + 2, 2));
            } else if (s[0] == 'f' && (s[1] == ' ' || s[1] == '\t')) {
                std::vector<int> vs, ns, ts;
                const char* p = s + 2;
                while (true) {
                    while (*p == ' ' || *p == '\t' || *p == '\r')
                        p++;
                    if (*p == '\0')
                        break;
                    char* end;
                    long v = std::strtol(p, &end, 10), t = 0, n = 0;
                    if (end == p) {
                        error = file + ":" + std::to_string(ln) + ": bad face";
                        return false;
                    }
                    p = end;
                    if (*p == '/') {
                        p++;
                        if (*p != '/') {
                            t = std::strtol(p, &end, 10);
                            p = end;
                        }
                        if (*p == '/') {
                            p++;
                            n = std::strtol(p, &end, 10);
                            p = end;
                        }
                    }
                    int vi = resolve(v, pos.size());
                    if (vi < 0) {
                        error = file + ":" + std::to_string(ln) + ": vertex index out of range";
                        return false;
                    }
                    vs.push_back(vi);
                    ts.push_back(resolve(t, uv.size()));
                    ns.push_back(resolve(n, nrm.size()));
                }
                for (size_t k = 1; k + 1 < vs.size(); k++) {
                    Face f;
                    size_t id[3] = {0, k, k + 1};
                    for (int c = 0; c < 3; c++) {
                        f.v[c] = vs[id[c]];
                        f.n[c] = ns[id[c]];
                        f.t[c] = ts[id[c]];
                    }
                    const V3& p0 = pos[f.v[0]];
                    if (cross(pos[f.v[1]] - p0, pos[f.v[2]] - p0).near_zero())
                        continue;
                    if (!faces.count(current))
                        part_order.push_back(current);
                    faces[current].push_back(f);
                }
            } else if (line.compare(size_t(s - line.c_str()), 6, "usemtl") == 0) {
                std::string name(s + 6);
                name.erase(0, name.find_first_not_of(" \t"));
                name.erase(name.find_last_not_of(" \t\r") + 1);
                auto it = materials.find(name);
                auto mtl = file_materials.find(name);
                if (it != materials.end())
                    current = {it->second, -1};
                else if (mtl != file_materials.end())
                    current = {mtl->second.material, mtl->second.alpha_mask};
                else
                    current = {line_mat, -1};
            } else if (line.compare(size_t(s - line.c_str()), 6, "mtllib") == 0) {
                // usually one file name; several are allowed
                std::string names(s + 6);
                std::istringstream list(names);
                std::string name, mtl_error;
                while (list >> name)
                    if (!load_mtl(name[0] == '/' ? name : obj_dir + name, file_materials, mtl_error))
                        std::fprintf(stderr, "Warning: %s: %s\n", file.c_str(), mtl_error.c_str());
            }
        }
        if (smooth && nrm.empty()) {
            nrm.assign(pos.size(), V3());
            for (const Surface& pm : part_order)
                for (auto& f : faces[pm]) {
                    const V3& p0 = pos[f.v[0]];
                    V3 n = cross(pos[f.v[1]] - p0, pos[f.v[2]] - p0);
                    for (int c = 0; c < 3; c++) {
                        nrm[f.v[c]] = nrm[f.v[c]] + n;
                        f.n[c] = f.v[c];
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

    bool parse_material(std::istringstream& in) {
        std::string name, type;
        if (!(in >> name >> type))
            return fail("expected 'material <name> <type> <parameters...>'");
        int normal_map = -1;
        auto read_normal_map = [&]() {
            std::string key;
            if (!(in >> key))
                return true;
            if (key != "normal_map") {
                error = "unexpected value '" + key + "' (expected 'normal_map <texture>')";
                return false;
            }
            return read_texture_name(in, normal_map);
        };
        mypbr_material m = blank_material(0);
        if (type == "lambertian") {
            m.type = MYPBR_MAT_LAMBERTIAN;
            std::string first;
            error.clear();
            if (!(in >> first) || !read_color_or_texture(in, first, m.tex[0]))
                return fail(error.empty()
                                ? "expected 'material <name> lambertian <r> <g> <b>' or '... lambertian texture <name>'"
                                : error);
            if (!read_normal_map())
                return fail(error);
        } else if (type == "metal") {
            const char* usage = "expected 'material <name> metal <r> <g> <b> <roughness>' or "
                                "'... metal <Al|Ti|Cu|Au|Ag|Cr> <roughness>'";
            m.type = MYPBR_MAT_METAL;
            std::string first;
            double r = 0, g = 0, b = 0, roughness = 0;
            V3 eta, k;
            if (!(in >> first))
                return fail(usage);
            bool measured = find_conductor(first, eta, k);
            if (measured) {
                if (!(in >> roughness) || roughness < 0)
                    return fail(usage);
            } else {
                std::istringstream number(first);
                if (!(number >> r) || !(in >> g >> b >> roughness) || roughness < 0)
                    return fail(usage);
            }
            error.clear();
            if (!read_normal_map())
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
                V3 f0(r, g, b);
                for (int c = 0; c < 3; c++) {
                    m.p[c] = f0[c];
                    m.p[10 + c] = f0[c] + (1 - f0[c]) / 21;
                }
            }
        } else if (type == "dielectric") {
            const char* usage = "expected 'material <name> dielectric <index of refraction> [roughness <r>] "
                                "[color <r> <g> <b> [distance <d>]]'";
            double ior, roughness = 0, distance = 1;
            V3 tint(1, 1, 1);
            std::string key;
            if (!(in >> ior) || ior <= 0)
                return fail(usage);
            while (in >> key) {
                bool ok = true;
                if (key == "roughness") {
                    ok = bool(in >> roughness) && roughness >= 0;
                } else if (key == "color") {
                    double r, g, b;
                    ok = bool(in >> r >> g >> b) && r > 0 && g > 0 && b > 0 && r <= 1 && g <= 1 && b <= 1;
                    tint = V3(r, g, b);
                } else if (key == "distance") {
                    ok = bool(in >> distance) && distance > 0;
                } else {
                    ok = false;
                }
                if (!ok)
                    return fail(usage);
            }
            m.type = MYPBR_MAT_DIELECTRIC;
            m.p[0] = ior;
            m.p[1] = std::clamp(roughness, 0.0, 1.0);
            for (int c = 0; c < 3; c++)
                m.p[2 + c] = -std::log(tint[c]) / distance;
        } else if (type == "thin_glass") {
            const char* usage = "expected 'material <name> thin_glass <index of refraction> [color <r> <g> <b>]'";
            double ior;
            V3 tint(1, 1, 1);
            std::string key;
            if (!(in >> ior) || ior <= 0)
                return fail(usage);
            if (in >> key) {
                double r, g, b;
                if (key != "color" || !(in >> r >> g >> b) || r < 0 || g < 0 || b < 0 || r > 1 || g > 1 || b > 1)
                    return fail(usage);
                tint = V3(r, g, b);
            }
            m.type = MYPBR_MAT_THIN_DIELECTRIC;
            m.p[0] = ior;
            for (int c = 0; c < 3; c++)
                m.p[2 + c] = tint[c];
        } else if (type == "principled") {
            m.type = MYPBR_MAT_PRINCIPLED;
            int base = add_texture_solid(V3(0.8, 0.8, 0.8));
            int metallic = add_texture_solid(V3(0, 0, 0));
            int rough = add_texture_solid(V3(0.5, 0.5, 0.5));
            int coat = -1, coat_rough = -1, coat_normals = -1, base_normals = -1;
            V3 coat_tint(1, 1, 1), eta, k;
            bool coat_tinted = false, measured = false;
            double ior = 1.5;
            std::string key;
            error.clear();
            while (in >> key) {
                bool ok = true;
                if (key == "texture") {
                    ok = read_color_or_texture(in, key, base);
                } else if (key == "color") {
                    std::string first;
                    ok = bool(in >> first) && read_color_or_texture(in, first, base);
                } else if (key == "metallic") {
                    ok = read_value_or_texture(in, metallic);
                } else if (key == "roughness") {
                    ok = read_value_or_texture(in, rough);
                } else if (key == "ior") {
                    ok = bool(in >> ior) && ior > 0;
                } else if (key == "normal_map") {
                    ok = read_texture_name(in, base_normals);
                } else if (key == "clearcoat") {
                    ok = read_value_or_texture(in, coat);
                } else if (key == "clearcoat_roughness") {
                    ok = read_value_or_texture(in, coat_rough);
                } else if (key == "clearcoat_normal_map") {
                    ok = read_texture_name(in, coat_normals);
                } else if (key == "conductor") {
                    std::string metal_name;
                    ok = bool(in >> metal_name) && (measured = find_conductor(metal_name, eta, k));
                    if (!ok)
                        error = "unknown conductor '" + metal_name + "' (known: Al Ti Cu Au Ag Cr)";
                } else if (key == "clearcoat_color") {
                    double r, g, b;
                    ok = bool(in >> r >> g >> b) && r > 0 && g > 0 && b > 0 && r <= 1 && g <= 1 && b <= 1;
                    coat_tint = V3(r, g, b);
                    coat_tinted = true;
                } else {
                    return fail("unknown principled setting '" + key + "'");
                }
                if (!ok)
                    return fail(error.empty() ? "bad value for principled setting '" + key + "'" : error);
            }
            if ((coat_rough >= 0 || coat_normals >= 0 || coat_tinted) && coat < 0)
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
                if (!(coat_tint.x == 1 && coat_tint.y == 1 && coat_tint.z == 1))
                    m.flags |= MYPBR_MATF_COAT_TINT;
            }
        } else if (type == "volume") {
            double r, g, b, aniso = 0;
            std::string key;
            if (!(in >> r >> g >> b))
                return fail("expected 'material <name> volume <r> <g> <b> [g <anisotropy>]'");
            if (in >> key) {
                if (key != "g" || !(in >> aniso) || aniso <= -1 || aniso >= 1)
                    return fail(
                        "expected 'material <name> volume <r> <g> <b> [g <anisotropy between -1 and 1>]'");
            }
            m.type = MYPBR_MAT_PHASE;
            m.p[0] = r;
            m.p[1] = g;
            m.p[2] = b;
            m.p[3] = aniso;
        } else if (type == "emissive") {
            const char* usage = "expected 'material <name> emissive <r> <g> <b> [spread <degrees, 0 to 180>]'";
            double r, g, b, spread = 180;
            std::string key;
            if (!(in >> r >> g >> b))
                return fail(usage);
            if (in >> key && (key != "spread" || !(in >> spread) || spread <= 0 || spread > 180))
                return fail(usage);
            m.type = MYPBR_MAT_DIFFUSE_LIGHT;
            m.p[0] = r;
            m.p[1] = g;
            m.p[2] = b;
            m.p[3] = spread;
            double half = radians(spread) / 2;
            m.p[4] = spread >= 180 ? kInf : std::tan(half);
            // Cosine-weighted share of the gridded emission (material.h:600-608)
            if (half >= kPi / 2 - 1e-9) {
                m.p[5] = 1;
            } else {
                double s = std::sin(half), c = std::cos(half);
                m.p[5] = s * s - (half - s * c) * c / s;
            }
        } else {
            return fail("unknown material type '" + type + "'");
        }
        if (normal_map >= 0 && use_normal_maps)
            m.normal_map = normal_map;
        materials[name] = add_material(m);
        return true;
    }

    bool parse_texture(std::istringstream& in) {
        std::string name, type;
        if (!(in >> name >> type))
            return fail("expected 'texture <name> <type> <parameters...>'");
        if (type == "solid") {
            double r, g, b;
            if (!(in >> r >> g >> b))
                return fail("expected 'texture <name> solid <r> <g> <b>'");
            textures[name] = add_texture_solid(V3(r, g, b));
        } else if (type == "checker") {
            double scale, r0, g0, b0, r1, g1, b1;
            if (!(in >> scale >> r0 >> g0 >> b0 >> r1 >> g1 >> b1) || scale <= 0)
                return fail("expected 'texture <name> checker <scale> <r g b> <r g b>'");
            int even = add_texture_solid(V3(r0, g0, b0));
            int odd = add_texture_solid(V3(r1, g1, b1));
            mypbr_texture t{};
            t.type = MYPBR_TEX_CHECKER;
            t.a = even;
            t.b = odd;
            t.p[0] = 1.0 / scale;
            S.textures.push_back(t);
            textures[name] = int(S.textures.size()) - 1;
        } else if (type == "image") {
            std::string file, option;
            if (!(in >> file))
                return fail("expected 'texture <name> image <path> [linear]'");
            bool linear = false;
            if (in >> option) {
                if (option != "linear")
                    return fail("expected 'texture <name> image <path> [linear]'");
                linear = true;
            }
            if (file[0] != '/')
                file = scene_dir + file;
            std::string err;
            int index = load_image(file, false, linear, err);
            if (index < 0) {
                if (image_unsupported) {
                    unsupported = true;
                    return fail("image texture '" + file + "': " + err);
                }
                return fail("cannot load image '" + file + "'" + (err.empty() ? "" : ": " + err));
            }
            textures[name] = index;
        } else {
            return fail("unknown texture type '" + type + "'");
        }
        return true;
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
    bool parse_vox(std::istringstream& in) {
        const char* usage = "expected 'vox <file.vox> [quads] [emission <scale>] [edges <width> [<r g b>]] [transforms]'";
        std::string file, token;
        if (!(in >> file))
            return fail(usage);
        if (file[0] != '/')
            file = scene_dir + file;
        bool quads = false;
        double emission = 1, edge_width = 0;
        V3 edge_color(0, 0, 0);
        std::vector<std::string> rest;
        while (in >> token)
            rest.push_back(token);
        size_t k = 0;
        for (; k < rest.size(); k++) {
            if (rest[k] == "quads") {
                quads = true;
            } else if (rest[k] == "emission" && k + 1 < rest.size()) {
                std::istringstream number(rest[++k]);
                if (!(number >> emission) || emission < 0)
                    return fail(usage);
            } else if (rest[k] == "edges" && k + 1 < rest.size()) {
                std::istringstream number(rest[++k]);
                if (!(number >> edge_width) || edge_width <= 0 || edge_width >= 0.5)
                    return fail(usage);
                if (k + 3 < rest.size()) {
                    std::istringstream rgb(rest[k + 1] + ' ' + rest[k + 2] + ' ' + rest[k + 3]);
                    V3 c;
                    if (rgb >> c.x >> c.y >> c.z) {
                        edge_color = c;
                        k += 3;
                    }
                }
            } else {
                break;
            }
        }
        std::string tail_text;
        for (; k < rest.size(); k++)
            tail_text += rest[k] + ' ';
        std::istringstream tail(tail_text);
        int mat;
        Xf xform;
        bool transformed;
        error.clear();
        if (!read_tail(tail, mat, xform, transformed))
            return fail(error);
        if (mat != default_material)
            return fail("vox models take their materials from the file's palette");
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

    bool parse_line(std::istringstream& in, const std::string& keyword) {
        auto& cam = S.camera;
        auto& opts = S.opts;
        if (keyword == "image_width") {
            if (!(in >> cam.image_width) || cam.image_width < 1)
                return fail("expected 'image_width <positive integer>'");
        } else if (keyword == "aspect_ratio") {
            double num, den = 1.0;
            if (!(in >> num))
                return fail("expected 'aspect_ratio <w>/<h>' or 'aspect_ratio <number>'");
            if (in.peek() == '/') {
                in.get();
                if (!(in >> den))
                    return fail("expected 'aspect_ratio <w>/<h>'");
            }
            if (num <= 0 || den <= 0)
                return fail("aspect_ratio must be positive");
            cam.aspect_ratio = num / den;
        } else if (keyword == "samples_per_pixel") {
            if (!(in >> opts.samples_per_pixel) || opts.samples_per_pixel < 1)
                return fail("expected 'samples_per_pixel <positive integer>'");
        } else if (keyword == "max_depth") {
            if (!(in >> opts.max_depth) || opts.max_depth < 1)
                return fail("expected 'max_depth <positive integer>'");
        } else if (keyword == "camera") {
            std::string key;
            while (in >> key) {
                bool ok = true;
                if (key == "lookfrom")
                    ok = bool(in >> cam.lookfrom[0] >> cam.lookfrom[1] >> cam.lookfrom[2]);
                else if (key == "lookat")
                    ok = bool(in >> cam.lookat[0] >> cam.lookat[1] >> cam.lookat[2]);
                else if (key == "vup")
                    ok = bool(in >> cam.vup[0] >> cam.vup[1] >> cam.vup[2]);
                else if (key == "vfov")
                    ok = bool(in >> cam.vfov) && cam.vfov > 0 && cam.vfov < 180;
                else if (key == "aperture")
                    ok = bool(in >> cam.defocus_angle) && cam.defocus_angle >= 0;
                else if (key == "focus")
                    ok = bool(in >> cam.focus_dist) && cam.focus_dist > 0;
                else if (key == "ortho")
                    ok = bool(in >> cam.ortho_height) && cam.ortho_height >= 0;
                else if (key == "blades")
                    ok = bool(in >> cam.blades) && (cam.blades == 0 || cam.blades >= 3);
                else if (key == "blade_rotation")
                    ok = bool(in >> cam.blade_rotation);
                else
                    return fail("unknown camera setting '" + key + "'");
                if (!ok)
                    return fail("bad value for camera setting '" + key + "'");
            }
        } else if (keyword == "vfov") {
            if (!(in >> cam.vfov) || cam.vfov <= 0 || cam.vfov >= 180)
                return fail("expected 'vfov <degrees between 0 and 180>'");
        } else if (keyword == "aperture") {
            if (!(in >> cam.defocus_angle) || cam.defocus_angle < 0)
                return fail("expected 'aperture <defocus angle in degrees>'");
        } else if (keyword == "focus") {
            if (!(in >> cam.focus_dist) || cam.focus_dist <= 0)
                return fail("expected 'focus <positive distance>'");
        } else if (keyword == "background") {
            double r, g, b;
            if (!(in >> r >> g >> b))
                return fail("expected 'background <r> <g> <b>'");
            S.use_sky = false;
            S.background = V3(r, g, b);
        } else if (keyword == "light_selection") {
            std::string mode;
            if (!(in >> mode) || (mode != "power" && mode != "uniform"))
                return fail("expected 'light_selection power|uniform'");
            power_selection = mode == "power";
        } else if (keyword == "environment") {
            std::string file, key;
            double intensity = 1, rotation = 0;
            const char* usage = "expected 'environment <file.hdr> [intensity <s>] [rotate <degrees>]'";
            if (!(in >> file))
                return fail(usage);
            while (in >> key) {
                bool ok = (key == "intensity" && in >> intensity && intensity >= 0) ||
                          (key == "rotate" && in >> rotation);
                if (!ok)
                    return fail(usage);
            }
            if (file[0] != '/')
                file = scene_dir + file;
            int w, h;
            std::vector<float> rgb;
            std::string err;
            if (!read_hdr(file, w, h, rgb, err))
                return fail("cannot load environment map '" + file + "'");
            if (has_environment)
                return fail("only one environment is allowed");
            set_environment(w, h, std::move(rgb), intensity, rotation / 360);
        } else if (keyword == "sun") {
            const char* usage = "expected 'sun elevation <deg> azimuth <deg> [intensity <E>] [color <r g b>] "
                                "[angle <deg>] [disk on|off]' or 'sun off'";
            std::string key;
            sun_on = true;
            while (in >> key) {
                bool ok = true;
                if (key == "off")
                    sun_on = false;
                else if (key == "elevation")
                    ok = bool(in >> sun_elevation) && sun_elevation >= -90 && sun_elevation <= 90;
                else if (key == "azimuth")
                    ok = bool(in >> sun_azimuth);
                else if (key == "intensity")
                    ok = bool(in >> sun_intensity) && sun_intensity >= 0;
                else if (key == "color")
                    ok = bool(in >> sun_tint.x >> sun_tint.y >> sun_tint.z);
                else if (key == "angle")
                    ok = bool(in >> sun_angle) && sun_angle > 0 && sun_angle < 90;
                else if (key == "disk") {
                    std::string value;
                    ok = bool(in >> value) && (value == "on" || value == "off");
                    sun_disk = value == "on";
                } else
                    ok = false;
                if (!ok)
                    return fail(usage);
            }
        } else if (keyword == "sky") {
            std::string type;
            if (!(in >> type))
                return fail("expected 'sky uniform <r g b>', 'sky atmosphere [...]' or 'sky gradient'");
            if (type == "uniform") {
                if (!(in >> sky_radiance.x >> sky_radiance.y >> sky_radiance.z))
                    return fail("expected 'sky uniform <r g b>'");
                sky_uniform = true;
                S.use_sky = true;
                sky_atmosphere = false;
            } else if (type == "atmosphere") {  // scene.h:574-586
                const char* usage =
                    "expected 'sky atmosphere [rayleigh <x>] [mie <x>] [mie_g <g>] [ozone <x>] [intensity <s>]'";
                std::string key;
                while (in >> key) {
                    bool ok = (key == "rayleigh" && in >> air.rayleigh && air.rayleigh >= 0) ||
                              (key == "mie" && in >> air.mie && air.mie >= 0) ||
                              (key == "mie_g" && in >> air.mie_g && air.mie_g > -1 && air.mie_g < 1) ||
                              (key == "ozone" && in >> air.ozone && air.ozone >= 0) ||
                              (key == "intensity" && in >> air.intensity && air.intensity >= 0);
                    if (!ok)
                        return fail(usage);
                }
                sky_atmosphere = true;
                sky_uniform = false;
                S.use_sky = true;
            } else if (type == "gradient") {
                sky_uniform = false;
                sky_atmosphere = false;
                S.use_sky = true;
            } else {
                return fail("unknown sky type '" + type + "' (expected uniform, atmosphere or gradient)");
            }
        } else if (keyword == "ground") {
            std::string key;
            ground = true;
            while (in >> key) {
                if (key == "off") {
                    ground = false;
                } else if (key == "height") {
                    if (!(in >> ground_height))
                        return fail("expected 'ground [height <y>] [material]'");
                } else {
                    auto it = materials.find(key);
                    if (it == materials.end())
                        return fail("unknown material '" + key + "'");
                    ground_material = it->second;
                }
            }
        } else if (keyword == "style") {
            std::string name;
            if (!(in >> name) || (name != "voxel" && name != "classic"))
                return fail("expected 'style voxel' or 'style classic'");
            bool voxel = name == "voxel";
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
            opts.max_diffuse = voxel ? 2 : 0;
            opts.max_specular = voxel ? 5 : 0;
            opts.max_scatter = voxel ? 5 : 0;
            opts.transparent_shadows = voxel;
        } else if (keyword == "bounces") {
            const char* usage = "expected 'bounces [diffuse <n>] [specular <n>] [scatter <n>]'";
            std::string key;
            while (in >> key) {
                bool ok = (key == "diffuse" && in >> opts.max_diffuse && opts.max_diffuse >= 0) ||
                          (key == "specular" && in >> opts.max_specular && opts.max_specular >= 0) ||
                          (key == "scatter" && in >> opts.max_scatter && opts.max_scatter >= 0);
                if (!ok)
                    return fail(usage);
            }
        } else if (keyword == "transparent_shadows") {
            std::string value;
            if (!(in >> value) || (value != "on" && value != "off"))
                return fail("expected 'transparent_shadows on|off'");
            opts.transparent_shadows = value == "on";
        } else if (keyword == "height_fog") {
            double density, scale, base = 0;
            std::string name, key;
            const char* usage = "expected 'height_fog <density> <scale height> <volume material> [base <y>]'";
            if (!(in >> density >> scale >> name) || density <= 0 || scale <= 0)
                return fail(usage);
            if (in >> key && (key != "base" || !(in >> base)))
                return fail(usage);
            auto it = materials.find(name);
            if (it == materials.end() || S.materials[it->second].type != MYPBR_MAT_PHASE)
                return fail("expected a volume material, got '" + name + "'");
            mypbr_unbounded u{};
            u.kind = MYPBR_UNBOUNDED_HEIGHT_FOG;
            u.material = it->second;
            u.height = base;
            u.density = density;
            u.scale_height = scale;
            S.unbounded.push_back(u);
        } else if (keyword == "bloom") {
            // Display settings: they change written images, not the radiance frame
            double strength;
            if (!(in >> strength) || strength < 0)
                return fail("expected 'bloom <strength> [threshold <radiance>] [radius <fraction of width>]'");
            std::string key;
            double x;
            while (in >> key) {
                if (!((key == "threshold" && in >> x && x >= 0) || (key == "radius" && in >> x && x > 0)))
                    return fail("expected 'bloom <strength> [threshold <radiance>] [radius <fraction of width>]'");
            }
        } else if (keyword == "vignette") {
            double v;
            if (!(in >> v) || v < 0)
                return fail("expected 'vignette <strength>'");
        } else if (keyword == "exposure") {
            double v;
            if (!(in >> v))
                return fail("expected 'exposure <stops>'");
        } else if (keyword == "tonemap") {
            std::string name;
            if (!(in >> name) || (name != "none" && name != "reinhard" && name != "aces"))
                return fail("expected 'tonemap none|reinhard|aces'");
        } else if (keyword == "normal_maps") {
            std::string state;
            if (!(in >> state) || (state != "on" && state != "off"))
                return fail("expected 'normal_maps on|off'");
            use_normal_maps = state == "on";
        } else if (keyword == "texture") {
            return parse_texture(in);
        } else if (keyword == "material") {
            return parse_material(in);
        } else if (keyword == "sphere" || keyword == "quad" || keyword == "box") {
            int mat;
            Xf xform;
            bool transformed;
            error.clear();
            if (keyword == "sphere") {
                double x, y, z, r;
                if (!(in >> x >> y >> z >> r) || r == 0)
                    return fail("expected 'sphere <x> <y> <z> <non-zero radius> [material] [transforms]'");
                if (!read_tail(in, mat, xform, transformed))
                    return fail(error);
                if (!add_sphere(V3(x, y, z), r, mat, xform, transformed))
                    return fail(error);
            } else if (keyword == "quad") {
                V3 q, u, v;
                if (!(in >> q.x >> q.y >> q.z >> u.x >> u.y >> u.z >> v.x >> v.y >> v.z))
                    return fail("expected 'quad <Qx Qy Qz> <ux uy uz> <vx vy vz> [material] [transforms]'");
                if (cross(u, v).near_zero())
                    return fail("quad edges must not be parallel");
                if (!read_tail(in, mat, xform, transformed))
                    return fail(error);
                if (!add_quad(q, u, v, mat, xform, transformed))
                    return fail(error);
            } else {
                V3 a, b;
                if (!(in >> a.x >> a.y >> a.z >> b.x >> b.y >> b.z))
                    return fail("expected 'box <x0 y0 z0> <x1 y1 z1> [material] [transforms]'");
                if (!read_tail(in, mat, xform, transformed))
                    return fail(error);
                if (!add_box(a, b, mat, xform, transformed))
                    return fail(error);
            }
        } else if (keyword == "medium") {
            double density;
            std::string shape;
            if (!(in >> density >> shape) || density <= 0)
                return fail("expected 'medium <positive density> sphere|box <...> <material> [transforms]'");
            V3 a, b;
            bool sphere = shape == "sphere";
            if (sphere) {
                double r;
                if (!(in >> a.x >> a.y >> a.z >> r) || r <= 0)
                    return fail("expected 'medium <density> sphere <x> <y> <z> <positive radius> <material>'");
                b = V3(r, 0, 0);
            } else if (shape == "box") {
                if (!(in >> a.x >> a.y >> a.z >> b.x >> b.y >> b.z))
                    return fail("expected 'medium <density> box <x0 y0 z0> <x1 y1 z1> <material>'");
            } else {
                return fail("a medium's boundary must be 'sphere' or 'box'");
            }
            int mat;
            Xf xform;
            bool transformed;
            error.clear();
            if (!read_tail(in, mat, xform, transformed))
                return fail(error);
            if (S.materials[mat].type != MYPBR_MAT_PHASE)
                return fail("a medium needs a volume material");
            add_medium(density, sphere, a, b, mat, xform, transformed);
        } else if (keyword == "fog") {
            std::string name;
            if (!(in >> fog_density >> name) || fog_density <= 0)
                return fail("expected 'fog <positive density> <volume material>'");
            auto it = materials.find(name);
            if (it == materials.end() || S.materials[it->second].type != MYPBR_MAT_PHASE)
                return fail("expected a volume material, got '" + name + "'");
            fog_material = it->second;
        } else if (keyword == "mesh") {
            std::string file;
            if (!(in >> file))
                return fail("expected 'mesh <file.obj> [material] [transforms]'");
            if (file[0] != '/')
                file = scene_dir + file;
            std::string rest, first;
            std::getline(in, rest);
            std::istringstream peek(rest);
            bool smooth = (peek >> first) && first == "smooth";
            std::istringstream tail(smooth ? rest.substr(rest.find("smooth") + 6) : rest);
            auto ends_with = [&](const char* suf) {
                size_t n = std::strlen(suf);
                return file.size() >= n && file.compare(file.size() - n, n, suf) == 0;
            };
            // then any number of "replace <file material> <scene material>" (glTF)
            std::map<std::string, int> replace;
            std::streampos mark = tail.tellg();
            std::string token;
            while (tail >> token && token == "replace") {
                std::string from, to;
                if (!(tail >> from >> to))
                    return fail("expected 'replace <material in the file> <scene material>'");
                auto it = materials.find(to);
                if (it == materials.end())
                    return fail("unknown material '" + to + "'");
                replace[from] = it->second;
                mark = tail.tellg();
            }
            tail.clear();
            tail.seekg(mark);
            int mat;
            Xf xform;
            bool transformed;
            error.clear();
            if (!read_tail(tail, mat, xform, transformed))
                return fail(error);
            if (!replace.empty() && mat != default_material)
                return fail("'replace' and a material for the whole mesh can't be used together");
            bool gltf = ends_with(".gltf") || ends_with(".glb");
            if (!gltf && !replace.empty())
                return fail("'replace' is for glTF files (OBJ files take scene materials by usemtl name)");
            // glTF files bring their own materials: one named on the line replaces them all
            if (gltf ? !add_gltf(file, mat == default_material ? -1 : mat, replace, xform, transformed)
                     : !add_obj(file, smooth, mat, xform, transformed))
                return fail(error);
            std::string extra;
            if (tail >> extra)
                return fail("unexpected value '" + extra + "'");
        } else if (keyword == "vox") {
            return parse_vox(in);
        } else if (keyword == "cyclorama" || keyword == "softbox") {
            unsupported = true;
            return fail("'" + keyword + "' is not supported by this backend");
        } else {
            return fail("unknown keyword '" + keyword + "'");
        }
        std::string extra;
        if (in >> extra)
            return fail("unexpected value '" + extra + "'");
        return true;
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
            std::istringstream in(line);
            std::string keyword;
            if (!(in >> keyword))
                continue;
            if (!parse_line(in, keyword)) {
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
