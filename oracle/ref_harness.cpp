// ORACLE PIN — test infrastructure only.
//
// Compiled (by oracle/Makefile, target `ref`) against the reference's own
// headers where they lie (include/*.h, external/ of adriendjn/mypbr) into
// oracle/_ref/ref_harness. It never ships and never runs on the product path:
// tests/golden/gen_golden.py runs it once, in the container that has the
// reference, to write the golden vectors that pin the FP64 oracle
// (oracle/pt_oracle.cpp) and, through it, the CUDA kernels.
//
// Sub-commands (all write little-endian float64 records to <out>):
//   hits   <scene> <n> <seed> <out>   world.hit of n seeded rays (bvh.h:45-86 + scene::unbounded)
//   bsdf   <scene> <out>              eval / scatter pdf of each probe sphere's material on a grid
//   lights <scene> <n> <seed> <out>   light probabilities, pdf_value of light-sampled and uniform directions
//   env    <scene> <n> <seed> <out>   environment radiance() and pdf_value()
//   ggx    <out>                      ggx_albedo_table E(mu, alpha) / E_avg and ggx_ms_* on a grid
//   render <scene> <width> <spp> <batches> <threads> <out>
//                                      batch means of camera::render (mean and variance of the mean)
//   features <scene> <width> <spp> <batches> <threads> <out>
//                                      the same with collect_features: radiance, albedo, normal, variance
//   denoise <w> <h> <seed> <out>      denoiser::run on a seeded frame
//   post   <w> <h> <seed> <out>       postprocess + display_settings::apply + to_byte on a seeded image
//   sky    <w> <h> <out>              atmosphere::bake and sun_transmittance for four suns and settings
//   image  <file> <out>               image_texture's decoding of an 8-bit file (stb_image)
//   load   <scene> <out>              load_scene's result: "ok", or the message it prints (text)
#include <bvh.h>
#include <denoiser.h>
#include <scene.h>
#include <atmosphere.h>
#include <tonemap.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

namespace {

struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next_u64() {
        uint64_t z = (s += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    double next() { return double(next_u64() >> 11) * (1.0 / 9007199254740992.0); }
};

struct Out {
    std::ofstream f;
    explicit Out(const char* path) : f(path, std::ios::binary) {}
    void put(double x) { f.write(reinterpret_cast<const char*>(&x), sizeof x); }
    void put(const vec3& v) {
        put(v.x());
        put(v.y());
        put(v.z());
    }
};

bool load(const char* path, scene& sc) {
    std::clog.setstate(std::ios::failbit);
    bool ok = load_scene(path, sc);
    std::clog.clear();
    if (!ok)
        std::cerr << "cannot load " << path << "\n";
    return ok;
}

// The world as main.cpp:70-74 assembles it.
struct World {
    std::shared_ptr<bvh> tree;
    hittable_list everything;
    const hittable* world;
    explicit World(scene& sc) {
        tree = std::make_shared<bvh>(sc.world);
        everything.add(tree);
        for (const auto& o : sc.unbounded.objects)
            everything.add(o);
        world = sc.unbounded.empty() ? static_cast<const hittable*>(tree.get()) : &everything;
    }
};

// Material identity of a hit: the probe scenes give every object its own
// lambertian whose red albedo is (id + 1) / 1024, read back here.
double material_id(const hit_record& rec) {
    scatter_record srec;
    ray r(rec.p + rec.normal, -rec.normal);
    if (!rec.mat->scatter(r, rec, srec))
        return -2;
    return std::round(srec.attenuation.x() * 1024) - 1;
}

vec3 uniform_dir(Rng& g) {
    while (true) {
        vec3 p(2 * g.next() - 1, 2 * g.next() - 1, 2 * g.next() - 1);
        double l = p.length_squared();
        if (l > 1e-6 && l <= 1)
            return p / std::sqrt(l);
    }
}

int cmd_hits(int argc, char** argv) {
    if (argc < 6)
        return 2;
    scene sc;
    if (!load(argv[2], sc))
        return 1;
    long n = std::atol(argv[3]);
    Rng g(std::strtoull(argv[4], nullptr, 10));
    World w(sc);
    aabb b = sc.world.bounding_box();
    Out out(argv[5]);
    vec3 lo(b.x.min, b.y.min, b.z.min), hi(b.x.max, b.y.max, b.z.max), ext = hi - lo;
    lo = lo - 0.1 * ext;
    ext = 1.2 * ext;
    for (long k = 0; k < n; k++) {
        vec3 o(lo.x() + ext.x() * g.next(), lo.y() + ext.y() * g.next(), lo.z() + ext.z() * g.next());
        vec3 d;
        if (k % 2 == 0) {
            vec3 t(lo.x() + ext.x() * g.next(), lo.y() + ext.y() * g.next(), lo.z() + ext.z() * g.next());
            d = t - o;
            if (k % 4 == 0)
                d = unit_vector(d);
        } else {
            d = uniform_dir(g);
        }
        hit_record rec;
        bool h = w.world->hit(ray(o, d), interval(0.001, infinity), rec);
        out.put(o);
        out.put(d);
        out.put(h ? 1.0 : 0.0);
        if (h) {
            out.put(rec.t);
            out.put(rec.normal);
            out.put(rec.u);
            out.put(rec.v);
            out.put(rec.front_face ? 1.0 : 0.0);
            out.put(material_id(rec));
            out.put(rec.p);
        } else {
            for (int c = 0; c < 11; c++)
                out.put(0.0);
        }
    }
    return 0;
}

// The grid of pdf_test.cpp:232-245 (wo) plus a spread of wi, as fixed data.
std::vector<vec3> wo_grid() {
    return {vec3(0, 0, 1), unit_vector(vec3(1, 0, 1)), unit_vector(vec3(1, 0.2, 0.15)),
            unit_vector(vec3(-0.3, 0.5, 0.2)), unit_vector(vec3(0.1, -0.9, 0.05))};
}
std::vector<vec3> wi_grid() {
    std::vector<vec3> v;
    const int n = 48;
    for (int k = 0; k < n; k++) {  // a Fibonacci sphere
        double z = 1 - 2 * (k + 0.5) / n;
        double r = std::sqrt(std::fmax(0.0, 1 - z * z));
        double phi = k * 2.399963229728653;
        v.push_back(vec3(r * std::cos(phi), r * std::sin(phi), z));
    }
    return v;
}

int cmd_bsdf(int argc, char** argv) {
    if (argc < 4)
        return 2;
    scene sc;
    if (!load(argv[2], sc))
        return 1;
    Out out(argv[3]);
    // Probe sphere k sits at (10 k, 0, 0), radius 1: a ray straight down finds its material
    int count = int(sc.world.objects.size());
    for (int k = 0; k < count; k++) {
        hit_record probe;
        if (!sc.world.objects[k]->hit(ray(point3(10.0 * k, 5, 0), vec3(0, -1, 0)), interval(0.001, infinity), probe)) {
            std::cerr << "probe " << k << " missed\n";
            return 1;
        }
        const material* m = probe.mat;
        for (int face = 0; face < 2; face++) {
            for (const vec3& wo : wo_grid()) {
                for (const vec3& wi : wi_grid()) {
                    hit_record rec{};
                    rec.p = point3(0, 0, 0);
                    rec.normal = vec3(0, 0, 1);
                    rec.front_face = face == 0;
                    rec.u = 0.25;
                    rec.v = 0.75;
                    rec.dpdu = vec3(2, 0, 0);
                    rec.dpdv = vec3(0, 3, 0);
                    rec.t = 1;
                    ray r_in(wo, -wo);
                    color e = m->eval(r_in, rec, wi);
                    scatter_record srec;
                    bool sc_ok = m->scatter(r_in, rec, srec);
                    double pdf = (sc_ok && !srec.skip_pdf) ? srec.pdf_ptr->value(wi) : 0;
                    out.put(double(k));
                    out.put(double(face));
                    out.put(wo);
                    out.put(wi);
                    out.put(e);
                    out.put(pdf);
                    out.put(sc_ok && srec.skip_pdf ? 1.0 : 0.0);
                    out.put(sc_ok ? 1.0 : 0.0);
                }
            }
        }
    }
    return 0;
}

int cmd_lights(int argc, char** argv) {
    if (argc < 6)
        return 2;
    scene sc;
    if (!load(argv[2], sc))
        return 1;
    long n = std::atol(argv[3]);
    Rng g(std::strtoull(argv[4], nullptr, 10));
    Out out(argv[5]);
    out.put(double(sc.lights.objects.size()));
    for (size_t k = 0; k < sc.lights.objects.size(); k++)
        out.put(sc.lights.probability(k));
    aabb b = sc.world.bounding_box();
    vec3 lo(b.x.min, b.y.min, b.z.min), hi(b.x.max, b.y.max, b.z.max), ext = hi - lo;
    for (long k = 0; k < n; k++) {
        point3 o(lo.x() + ext.x() * g.next(), lo.y() + ext.y() * g.next(), lo.z() + ext.z() * g.next());
        vec3 d = (k % 2 == 0) ? sc.lights.random(o) : uniform_dir(g);
        out.put(o);
        out.put(d);
        out.put(sc.lights.pdf_value(o, d));
    }
    return 0;
}

int cmd_env(int argc, char** argv) {
    if (argc < 6)
        return 2;
    scene sc;
    if (!load(argv[2], sc))
        return 1;
    if (!sc.cam.environment) {
        std::cerr << "no environment\n";
        return 1;
    }
    long n = std::atol(argv[3]);
    Rng g(std::strtoull(argv[4], nullptr, 10));
    Out out(argv[5]);
    for (long k = 0; k < n; k++) {
        vec3 d = (k % 2 == 0) ? sc.cam.environment->random(point3(0, 0, 0)) : uniform_dir(g);
        out.put(d);
        out.put(sc.cam.environment->radiance(d));
        out.put(sc.cam.environment->pdf_value(point3(0, 0, 0), d));
    }
    return 0;
}

int cmd_ggx(int argc, char** argv) {
    if (argc < 3)
        return 2;
    Out out(argv[2]);
    const auto& t = ggx_albedo_table::get();
    for (int j = 0; j <= 40; j++) {
        double roughness = j / 40.0;
        double alpha = roughness_to_alpha(roughness);
        for (int i = 0; i <= 40; i++) {
            double mu = i / 40.0;
            out.put(alpha);
            out.put(mu);
            out.put(t.E(mu, alpha));
            out.put(t.E_avg(alpha));
            out.put(ggx_ms_albedo(mu, alpha));
            out.put(ggx_ms_eval(mu, 0.37, alpha));
        }
    }
    return 0;
}

int cmd_render(int argc, char** argv) {
    if (argc < 8)
        return 2;
    scene sc;
    if (!load(argv[2], sc))
        return 1;
    int width = std::atoi(argv[3]), spp = std::atoi(argv[4]), batches = std::atoi(argv[5]);
    int threads = std::atoi(argv[6]);
    auto& cam = sc.cam;
    if (width > 0)
        cam.image_width = width;
    cam.samples_per_pixel = spp;
    cam.threads = threads;
    World w(sc);
    std::vector<double> sum, sum2;
    int W = 0, H = 0;
    std::clog.setstate(std::ios::failbit);
    auto t0 = std::chrono::steady_clock::now();
    for (int b = 0; b < batches; b++) {
        frame f = cam.render(*w.world, sc.lights);
        W = cam.image_width;
        H = cam.height();
        if (sum.empty()) {
            sum.assign(f.radiance.size() * 3, 0.0);
            sum2.assign(f.radiance.size() * 3, 0.0);
        }
        for (size_t k = 0; k < f.radiance.size(); k++)
            for (int c = 0; c < 3; c++) {
                double x = f.radiance[k][c];
                sum[3 * k + c] += x;
                sum2[3 * k + c] += x * x;
            }
    }
    double seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::clog.clear();
    Out out(argv[7]);
    out.put(double(W));
    out.put(double(H));
    out.put(double(spp));
    out.put(double(batches));
    out.put(seconds);
    for (size_t k = 0; k < sum.size(); k++) {
        double m = sum[k] / batches;
        double var_of_mean = batches > 1 ? std::fmax(sum2[k] / batches - m * m, 0.0) / (batches - 1) : 0;
        out.put(m);
        out.put(var_of_mean);
    }
    return 0;
}

// features <scene> <width> <spp> <batches> <threads> <out>: camera::render
// with collect_features (camera.h:207-221, first_surface :253-277); per pixel
// the batch mean and variance of the mean of radiance, albedo and normal
// (3 x 2 each), then the mean over batches of frame.variance.
int cmd_features(int argc, char** argv) {
    if (argc < 8)
        return 2;
    scene sc;
    if (!load(argv[2], sc))
        return 1;
    int width = std::atoi(argv[3]), spp = std::atoi(argv[4]), batches = std::atoi(argv[5]);
    auto& cam = sc.cam;
    if (width > 0)
        cam.image_width = width;
    cam.samples_per_pixel = spp;
    cam.threads = std::atoi(argv[6]);
    cam.collect_features = true;
    World w(sc);
    std::vector<double> sum, sum2, var;
    int W = 0, H = 0;
    std::clog.setstate(std::ios::failbit);
    for (int b = 0; b < batches; b++) {
        frame f = cam.render(*w.world, sc.lights);
        W = cam.image_width;
        H = cam.height();
        size_t n = f.radiance.size();
        if (sum.empty()) {
            sum.assign(n * 9, 0.0);
            sum2.assign(n * 9, 0.0);
            var.assign(n, 0.0);
        }
        for (size_t k = 0; k < n; k++) {
            const color* src[3] = {&f.radiance[k], &f.albedo[k], &f.normal[k]};
            for (int q = 0; q < 3; q++)
                for (int c = 0; c < 3; c++) {
                    double x = (*src[q])[c];
                    sum[9 * k + 3 * q + c] += x;
                    sum2[9 * k + 3 * q + c] += x * x;
                }
            var[k] += f.variance[k] / batches;
        }
    }
    std::clog.clear();
    Out out(argv[7]);
    out.put(double(W));
    out.put(double(H));
    out.put(double(spp));
    out.put(double(batches));
    for (size_t k = 0; k < var.size(); k++) {
        for (int q = 0; q < 9; q++) {
            double m = sum[9 * k + q] / batches;
            out.put(m);
            out.put(batches > 1 ? std::fmax(sum2[9 * k + q] / batches - m * m, 0.0) / (batches - 1) : 0.0);
        }
        out.put(var[k]);
    }
    return 0;
}

// denoise <w> <h> <seed> <out>: a seeded synthetic frame (noisy radiance over
// an albedo edge, a normal edge, a few fireflies, per-pixel variance) and
// denoiser::run's output with the default settings (denoiser.h:39-43).
int cmd_denoise(int argc, char** argv) {
    if (argc < 6)
        return 2;
    int w = std::atoi(argv[2]), h = std::atoi(argv[3]);
    Rng g(std::strtoull(argv[4], nullptr, 10));
    frame f;
    size_t n = size_t(w) * h;
    f.radiance.resize(n);
    f.albedo.resize(n);
    f.normal.resize(n);
    f.variance.resize(n);
    for (int j = 0; j < h; j++)
        for (int i = 0; i < w; i++) {
            size_t k = size_t(j) * w + i;
            color a = i < w / 2 ? color(0.8, 0.7, 0.6) : color(0.2, 0.5, 0.3);
            vec3 nn = j < h / 3 ? vec3(0, 1, 0) : unit_vector(vec3(0.3, 0.2, 1));
            double light = 0.5 + 0.3 * std::sin(0.2 * i) * std::cos(0.15 * j);
            double noise = 1 + 0.6 * (g.next() - 0.5);
            if (g.next() < 0.01)
                noise = 40;  // a firefly
            f.radiance[k] = a * (light * noise);
            f.albedo[k] = a;
            f.normal[k] = nn;
            double l = luminance(f.radiance[k]);
            f.variance[k] = 0.02 * l * l + 1e-4 + (noise > 10 ? l * l : 0.0);
        }
    denoiser dn;
    dn.threads = 1;
    auto out = dn.run(f, w, h);
    Out o(argv[5]);
    o.put(double(w));
    o.put(double(h));
    for (size_t k = 0; k < n; k++) {
        o.put(f.radiance[k]);
        o.put(f.albedo[k]);
        o.put(f.normal[k]);
        o.put(f.variance[k]);
        o.put(out[k]);
    }
    return 0;
}

// A seeded HDR image: a gradient, noise and a few very bright spots. Then for
// each of four display settings: the post-processed radiance and the bytes
// of display_settings::apply + to_byte.
int cmd_post(int argc, char** argv) {
    if (argc < 6)
        return 2;
    int w = std::atoi(argv[2]), h = std::atoi(argv[3]);
    Rng g(std::strtoull(argv[4], nullptr, 10));
    size_t n = size_t(w) * h;
    std::vector<color> px(n);
    for (int j = 0; j < h; j++)
        for (int i = 0; i < w; i++) {
            double base = 0.05 + 0.9 * double(i) / w * (0.3 + 0.7 * double(j) / h);
            px[size_t(j) * w + i] = color(base * (0.8 + 0.4 * g.next()), base * (0.6 + 0.4 * g.next()),
                                          base * (0.3 + 0.6 * g.next()));
            if (g.next() < 0.004)
                px[size_t(j) * w + i] = color(40 * g.next(), 30 * g.next(), 20 * g.next());
        }
    Out o(argv[5]);
    o.put(double(w));
    o.put(double(h));
    for (const auto& c : px)
        o.put(c);
    struct Setting {
        double exposure, bloom, threshold, radius, vignette;
        tonemapper op;
    } settings[4] = {{0, 0, 1, 0.04, 0, tonemapper::none},
                     {0.5, 0.3, 1, 0.08, 0.4, tonemapper::reinhard},
                     {-0.7, 0.8, 0.5, 0.2, 0, tonemapper::aces},
                     {1.3, 0.15, 2, 0.01, 1.5, tonemapper::none}};
    for (const auto& st : settings) {
        display_settings d;
        d.exposure = st.exposure;
        d.op = st.op;
        d.post.bloom = st.bloom;
        d.post.bloom_threshold = st.threshold;
        d.post.bloom_radius = st.radius;
        d.post.vignette = st.vignette;
        std::vector<color> post = d.post.active() ? postprocess(px, w, h, d.post) : px;
        for (const auto& c : post)
            o.put(c);
        for (const auto& c : post) {
            color a = d.apply(c);
            o.put(double(to_byte(a.x())));
            o.put(double(to_byte(a.y())));
            o.put(double(to_byte(a.z())));
        }
    }
    return 0;
}

// Four (settings, sun) cases: the default air at a high, a low and a set sun,
// and a hazier, ozone-free air; per case the bake then the transmittance.
int cmd_sky(int argc, char** argv) {
    if (argc < 5)
        return 2;
    int w = std::atoi(argv[2]), h = std::atoi(argv[3]);
    Out o(argv[4]);
    struct Case {
        double el, az, e, rayleigh, mie, g, ozone, intensity;
    } cases[4] = {{40, 160, 1000, 1, 1, 0.8, 1, 3}, {5, 60, 4, 1, 1, 0.8, 1, 3}, {-2, 250, 10, 1, 1, 0.8, 1, 3},
                  {25, 300, 3, 1.5, 4, 0.9, 0, 2}};
    for (const auto& c : cases) {
        atmosphere_settings s;
        s.rayleigh = c.rayleigh;
        s.mie = c.mie;
        s.mie_g = c.g;
        s.ozone = c.ozone;
        s.intensity = c.intensity;
        atmosphere air(s);
        double el = degrees_to_radians(c.el), az = degrees_to_radians(c.az);
        vec3 dir(std::cos(el) * std::sin(az), std::sin(el), -std::cos(el) * std::cos(az));
        color irr(c.e, 0.9 * c.e, 0.8 * c.e);
        for (const auto& p : air.bake(w, h, dir, irr))
            o.put(p);
        o.put(air.sun_transmittance(dir));
    }
    return 0;
}

// image <file> <out>: how image_texture reads an 8-bit file (texture.h:67-98,
// 161-181): stb_image's width, height and channel count, the texture's
// has_alpha_channel / fully_opaque / greyscale, then the RGBA bytes (as
// doubles) — or a single -1 if stb_image cannot decode the file.
int cmd_image(int argc, char** argv) {
    if (argc < 4)
        return 2;
    Out out(argv[3]);
    int w, h, channels;
    unsigned char* data = stbi_load(argv[2], &w, &h, &channels, 4);
    if (!data) {
        out.put(-1.0);
        return 0;
    }
    image_texture tex(argv[2], false, false);
    out.put(double(w));
    out.put(double(h));
    out.put(double(channels));
    out.put(tex.has_alpha_channel() ? 1.0 : 0.0);
    out.put(tex.fully_opaque() ? 1.0 : 0.0);
    out.put(tex.greyscale() ? 1.0 : 0.0);
    for (size_t k = 0; k < size_t(w) * h * 4; k++)
        out.put(double(data[k]));
    stbi_image_free(data);
    return 0;
}

// load <scene> <out>: load_scene on a file; writes "ok" or what it printed
// on std::cerr ("path:line: message"), as text.
int cmd_load(int argc, char** argv) {
    if (argc < 4)
        return 2;
    std::ostringstream captured;
    std::streambuf* old = std::cerr.rdbuf(captured.rdbuf());
    std::clog.setstate(std::ios::failbit);
    scene sc;
    bool ok = load_scene(argv[2], sc);
    std::clog.clear();
    std::cerr.rdbuf(old);
    std::ofstream out(argv[3], std::ios::binary);
    out << (ok ? std::string("ok") : captured.str());
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        std::cerr << "usage: ref_harness hits|bsdf|lights|env|ggx|render ...\n";
        return 2;
    }
    std::string c = argv[1];
    int rc = 2;
    if (c == "hits") rc = cmd_hits(argc, argv);
    else if (c == "bsdf") rc = cmd_bsdf(argc, argv);
    else if (c == "lights") rc = cmd_lights(argc, argv);
    else if (c == "env") rc = cmd_env(argc, argv);
    else if (c == "ggx") rc = cmd_ggx(argc, argv);
    else if (c == "render") rc = cmd_render(argc, argv);
    else if (c == "features") rc = cmd_features(argc, argv);
    else if (c == "denoise") rc = cmd_denoise(argc, argv);
    else if (c == "post") rc = cmd_post(argc, argv);
    else if (c == "sky") rc = cmd_sky(argc, argv);
    else if (c == "image") rc = cmd_image(argc, argv);
    else if (c == "load") rc = cmd_load(argc, argv);
    if (rc == 2)
        std::cerr << "bad arguments for '" << c << "'\n";
    return rc;
}
