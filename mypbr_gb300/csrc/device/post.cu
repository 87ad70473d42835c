// Display post-processing on the device and the image writers.
//
// postprocess (include/postprocess.h:104-151): bloom from a pyramid of
// half-size, Gaussian-blurred copies of the image's bright part, and
// vignetting; then display_settings::apply (tonemap.h:28-37): exposure and
// the none / Reinhard / ACES-fit tonemappers; then the sRGB curve and 8-bit
// quantisation of to_byte (color3.h:17-36). All in FP64 with the reference's
// order of operations, and compiled without FMA contraction (build.py), so
// that the bytes of a display image are the reference's.
//
// Writers (image_io.h:16-106): .png (8-bit RGB, zlib stored blocks), .ppm
// (P3 text), .hdr (Radiance RGBE, flat scanlines), .pfm (little-endian
// floats, bottom row first). Display formats get the post-processing,
// .hdr / .pfm keep the raw radiance.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

#include "gpu_scene.h"

namespace mypbr_dev {

namespace {

constexpr int kBlurTaps = 11;  // sigma 1.5: r = ceil(3 sigma) = 5
__constant__ double c_blur[kBlurTaps];

struct Img {
    int w, h;
    double* px;  // rgb
};

__device__ __forceinline__ void at(const Img& m, int i, int j, double& r, double& g, double& b) {
    i = min(max(i, 0), m.w - 1);
    j = min(max(j, 0), m.h - 1);
    const double* p = m.px + 3 * (size_t(j) * m.w + i);
    r = p[0];
    g = p[1];
    b = p[2];
}

__global__ void k_bright(const double* in, int n, double threshold, double* out) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        double r = in[3 * k], g = in[3 * k + 1], b = in[3 * k + 2];
        double l = 0.2126 * r + 0.7152 * g + 0.0722 * b;
        bool keep = isfinite(l) && l > threshold;
        double s = keep ? (l - threshold) / l : 0.0;
        out[3 * k] = keep ? r * s : 0.0;
        out[3 * k + 1] = keep ? g * s : 0.0;
        out[3 * k + 2] = keep ? b * s : 0.0;
    }
}

// postprocess.h:50-59
__global__ void k_down(Img in, Img out) {
    int n = out.w * out.h;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        int i = k % out.w, j = k / out.w;
        double a[3], b[3], c[3], d[3];
        at(in, 2 * i, 2 * j, a[0], a[1], a[2]);
        at(in, 2 * i + 1, 2 * j, b[0], b[1], b[2]);
        at(in, 2 * i, 2 * j + 1, c[0], c[1], c[2]);
        at(in, 2 * i + 1, 2 * j + 1, d[0], d[1], d[2]);
        for (int ch = 0; ch < 3; ch++)
            out.px[3 * size_t(k) + ch] = 0.25 * (((a[ch] + b[ch]) + c[ch]) + d[ch]);
    }
}

// postprocess.h:62-84, one direction per launch
__global__ void k_blur(Img in, Img out, int horizontal) {
    int n = in.w * in.h;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        int i = k % in.w, j = k / in.w;
        double c[3] = {0.0, 0.0, 0.0};
        for (int t = -5; t <= 5; t++) {
            double r, g, b;
            if (horizontal)
                at(in, i + t, j, r, g, b);
            else
                at(in, i, j + t, r, g, b);
            double wgt = c_blur[t + 5];
            c[0] = c[0] + wgt * r;
            c[1] = c[1] + wgt * g;
            c[2] = c[2] + wgt * b;
        }
        for (int ch = 0; ch < 3; ch++)
            out.px[3 * size_t(k) + ch] = c[ch];
    }
}

struct Levels {
    Img lv[10];
    int n;
};

// postprocess.h:36-44
__device__ void sample(const Img& m, double x, double y, double* c) {
    x -= 0.5;
    y -= 0.5;
    int i = int(floor(x)), j = int(floor(y));
    double fx = x - i, fy = y - j;
    double p00[3], p10[3], p01[3], p11[3];
    at(m, i, j, p00[0], p00[1], p00[2]);
    at(m, i + 1, j, p10[0], p10[1], p10[2]);
    at(m, i, j + 1, p01[0], p01[1], p01[2]);
    at(m, i + 1, j + 1, p11[0], p11[1], p11[2]);
    for (int ch = 0; ch < 3; ch++)
        c[ch] = (1 - fy) * ((1 - fx) * p00[ch] + fx * p10[ch]) + fy * ((1 - fx) * p01[ch] + fx * p11[ch]);
}

struct Display {
    double scale;  // 2^exposure
    int op;        // MYPBR_TONEMAP_*
    int bytes;     // 1: quantise to 8-bit sRGB; 0: keep linear (postprocess only)
    double bloom, vignette;
};

__device__ double rrt_odt_fit(double x) {  // tonemap.h:63-67
    double a = x * (x + 0.0245786) - 0.000090537;
    double b = x * (0.983729 * x + 0.4329510) + 0.238081;
    return a / b;
}
__device__ double clamp01(double x) { return x < 0 ? 0 : (x > 1 ? 1 : x); }

__device__ void apply(const Display& D, double* c) {
    double r = D.scale * c[0], g = D.scale * c[1], b = D.scale * c[2];
    if (D.op == MYPBR_TONEMAP_REINHARD) {
        r = r / (1 + r);
        g = g / (1 + g);
        b = b / (1 + b);
    } else if (D.op == MYPBR_TONEMAP_ACES) {  // tonemap.h:46-60 (Hill's fit of the ACES RRT + ODT)
        double vr = 0.59719 * r + 0.35458 * g + 0.04823 * b;
        double vg = 0.07600 * r + 0.90834 * g + 0.01566 * b;
        double vb = 0.02840 * r + 0.13383 * g + 0.83777 * b;
        vr = rrt_odt_fit(vr);
        vg = rrt_odt_fit(vg);
        vb = rrt_odt_fit(vb);
        r = clamp01(1.60475 * vr + -0.53108 * vg + -0.07367 * vb);
        g = clamp01(-0.10208 * vr + 1.10813 * vg + -0.00605 * vb);
        b = clamp01(-0.00327 * vr + -0.07276 * vg + 1.07602 * vb);
    }
    c[0] = r;
    c[1] = g;
    c[2] = b;
}

__device__ unsigned char to_byte(double x) {  // color3.h:17-36
    double s;
    if (x <= 0)
        s = 0;
    else if (x <= 0.0031308)
        s = 12.92 * x;
    else
        s = 1.055 * pow(x, 1.0 / 2.4) - 0.055;
    s = s < 0.0 ? 0.0 : (s > 0.999 ? 0.999 : s);
    return (unsigned char)(256 * s);
}

__global__ void k_compose(const double* in, int w, int h, Levels L, Display D, double* lin, unsigned char* rgb8) {
    int n = w * h;
    double cx = 0.5 * w, cy = 0.5 * h;
    double corner2 = cx * cx + cy * cy;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        int i = k % w, j = k / w;
        double c[3] = {in[3 * size_t(k)], in[3 * size_t(k) + 1], in[3 * size_t(k) + 2]};
        if (L.n > 0) {
            double glow[3] = {0.0, 0.0, 0.0};
            for (int b = 0; b < L.n; b++) {
                double sx = double(L.lv[b].w) / w, sy = double(L.lv[b].h) / h;
                double s[3];
                sample(L.lv[b], (i + 0.5) * sx, (j + 0.5) * sy, s);
                glow[0] = glow[0] + s[0];
                glow[1] = glow[1] + s[1];
                glow[2] = glow[2] + s[2];
            }
            double f = D.bloom / L.n;
            c[0] = c[0] + f * glow[0];
            c[1] = c[1] + f * glow[1];
            c[2] = c[2] + f * glow[2];
        }
        if (D.vignette > 0) {  // postprocess.h:142-150
            double dx = i + 0.5 - cx, dy = j + 0.5 - cy;
            double f = 1 + D.vignette * (dx * dx + dy * dy) / corner2;
            double inv = 1 / (f * f);  // vec3 / t is (1 / t) * v (vec3.h:95-97)
            c[0] = inv * c[0];
            c[1] = inv * c[1];
            c[2] = inv * c[2];
        }
        if (D.bytes) {
            apply(D, c);
            rgb8[3 * size_t(k)] = to_byte(c[0]);
            rgb8[3 * size_t(k) + 1] = to_byte(c[1]);
            rgb8[3 * size_t(k) + 2] = to_byte(c[2]);
        } else {
            lin[3 * size_t(k)] = c[0];
            lin[3 * size_t(k) + 1] = c[1];
            lin[3 * size_t(k) + 2] = c[2];
        }
    }
}

struct DevMem {
    std::vector<void*> ptrs;
    ~DevMem() {
        for (void* p : ptrs)
            cudaFree(p);
    }
    template <typename T>
    int get(T*& p, size_t n) {
        void* q = nullptr;
        MYPBR_CUDA(cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)));
        ptrs.push_back(q);
        p = static_cast<T*>(q);
        return MYPBR_OK;
    }
};

int grid_for(size_t n) { return int(std::min<size_t>((n + 255) / 256, 152 * 16)); }

// Bloom, vignette and (bytes) the display transform of a device image.
int run_post(const double* d_in, int w, int h, const mypbr_display_opts& o, bool bytes, double* d_lin,
             unsigned char* d_rgb8) {
    DevMem mem;
    Levels L{};
    size_t n = size_t(w) * h;
    if (o.bloom > 0) {
        // blur weights as postprocess.h:63-69 forms them
        double kernel[kBlurTaps], sum = 0;
        for (int k = -5; k <= 5; k++)
            sum += kernel[k + 5] = std::exp(-0.5 * k * k / (1.5 * 1.5));
        for (double& k : kernel)
            k /= sum;
        MYPBR_CUDA(cudaMemcpyToSymbol(c_blur, kernel, sizeof kernel));
        Img bright{w, h, nullptr};
        int s = mem.get(bright.px, 3 * n);
        if (s != MYPBR_OK)
            return s;
        k_bright<<<grid_for(n), 256>>>(d_in, int(n), o.bloom_threshold, bright.px);
        double reach = std::fmax(o.bloom_radius * w, 1.0);
        int levels = std::clamp(int(std::ceil(std::log2(reach))), 1, 10);
        Img level = bright;
        for (int k = 0; k < levels && level.w > 1 && level.h > 1; k++) {
            Img down{std::max(1, level.w / 2), std::max(1, level.h / 2), nullptr};
            Img tmp = down, blurred = down;
            size_t m = size_t(down.w) * down.h;
            if ((s = mem.get(down.px, 3 * m)) || (s = mem.get(tmp.px, 3 * m)) || (s = mem.get(blurred.px, 3 * m)))
                return s;
            k_down<<<grid_for(m), 256>>>(level, down);
            k_blur<<<grid_for(m), 256>>>(down, tmp, 1);
            k_blur<<<grid_for(m), 256>>>(tmp, blurred, 0);
            L.lv[L.n++] = blurred;
            level = down;
        }
    }
    Display D{std::pow(2.0, o.exposure), o.tonemap, bytes ? 1 : 0, o.bloom, o.vignette};
    k_compose<<<grid_for(n), 256>>>(d_in, w, h, L, D, d_lin, d_rgb8);
    MYPBR_CUDA(cudaGetLastError());
    MYPBR_CUDA(cudaDeviceSynchronize());
    return MYPBR_OK;
}

int check_opts(const double* radiance, int w, int h, const mypbr_display_opts* o) {
    if (!radiance || w < 1 || h < 1) {
        set_error_message("display: radiance and a positive size are required");
        return MYPBR_ERR_INVALID_ARGUMENT;
    }
    if (o && (o->tonemap < MYPBR_TONEMAP_NONE || o->tonemap > MYPBR_TONEMAP_ACES)) {
        set_error_message("display: unknown tonemapper");
        return MYPBR_ERR_INVALID_ARGUMENT;
    }
    return MYPBR_OK;
}

// ------------------------------------------------------------ writers

uint32_t crc32(const unsigned char* p, size_t n, uint32_t c = 0xffffffffu) {
    static uint32_t table[256];
    static bool ready = false;
    if (!ready) {
        for (uint32_t k = 0; k < 256; k++) {
            uint32_t v = k;
            for (int b = 0; b < 8; b++)
                v = (v & 1) ? 0xedb88320u ^ (v >> 1) : v >> 1;
            table[k] = v;
        }
        ready = true;
    }
    for (size_t k = 0; k < n; k++)
        c = table[(c ^ p[k]) & 0xff] ^ (c >> 8);
    return c;
}

void put32(std::string& s, uint32_t v) {
    s.push_back(char(v >> 24));
    s.push_back(char(v >> 16));
    s.push_back(char(v >> 8));
    s.push_back(char(v));
}

void png_chunk(std::string& out, const char* type, const std::string& data) {
    put32(out, uint32_t(data.size()));
    std::string td = std::string(type, 4) + data;
    out += td;
    put32(out, crc32(reinterpret_cast<const unsigned char*>(td.data()), td.size()) ^ 0xffffffffu);
}

// An 8-bit RGB PNG whose zlib stream holds stored (uncompressed) deflate
// blocks: filter byte 0 before each row, Adler-32 at the end (RFC 1950/1951).
bool write_png(const std::string& path, int w, int h, const unsigned char* rgb) {
    std::string raw;
    raw.reserve(size_t(h) * (3 * size_t(w) + 1));
    for (int j = 0; j < h; j++) {
        raw.push_back('\0');
        raw.append(reinterpret_cast<const char*>(rgb + 3 * size_t(j) * w), 3 * size_t(w));
    }
    std::string z;
    z.push_back(char(0x78));
    z.push_back(char(0x01));
    size_t pos = 0;
    do {
        size_t len = std::min<size_t>(65535, raw.size() - pos);
        bool last = pos + len == raw.size();
        z.push_back(char(last ? 1 : 0));
        z.push_back(char(len & 0xff));
        z.push_back(char(len >> 8));
        z.push_back(char(~len & 0xff));
        z.push_back(char((~len >> 8) & 0xff));
        z.append(raw, pos, len);
        pos += len;
    } while (pos < raw.size());
    uint32_t a = 1, b = 0;
    for (unsigned char c : raw) {
        a = (a + c) % 65521;
        b = (b + a) % 65521;
    }
    put32(z, (b << 16) | a);
    std::string ihdr;
    put32(ihdr, uint32_t(w));
    put32(ihdr, uint32_t(h));
    ihdr += std::string("\x08\x02\x00\x00\x00", 5);
    std::string out("\x89PNG\r\n\x1a\n", 8);
    png_chunk(out, "IHDR", ihdr);
    png_chunk(out, "IDAT", z);
    png_chunk(out, "IEND", "");
    std::ofstream f(path, std::ios::binary);
    f.write(out.data(), std::streamsize(out.size()));
    return bool(f);
}

bool write_ppm(std::FILE* f, int w, int h, const unsigned char* rgb) {
    std::fprintf(f, "P3\n%d %d\n255\n", w, h);
    for (size_t k = 0; k < size_t(w) * h; k++)
        std::fprintf(f, "%d %d %d\n", rgb[3 * k], rgb[3 * k + 1], rgb[3 * k + 2]);
    return std::ferror(f) == 0;
}

// Radiance RGBE after Ward ("Real Pixels", Graphics Gems II, 1991): the
// largest channel's binary exponent is shared, each channel keeps 8 bits.
bool write_hdr(const std::string& path, int w, int h, const double* rad) {
    std::ofstream f(path, std::ios::binary);
    f << "#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y " << h << " +X " << w << "\n";
    std::vector<unsigned char> row(4 * size_t(w));
    for (int j = 0; j < h; j++) {
        for (int i = 0; i < w; i++) {
            const double* p = rad + 3 * (size_t(j) * w + i);
            float r = float(p[0]), g = float(p[1]), b = float(p[2]);
            float v = std::max(r, std::max(g, b));
            unsigned char* o = &row[4 * size_t(i)];
            if (v < 1e-32f) {
                o[0] = o[1] = o[2] = o[3] = 0;
            } else {
                int e;
                float m = std::frexp(v, &e);
                float scale = m * 256.0f / v;
                o[0] = (unsigned char)(r * scale);
                o[1] = (unsigned char)(g * scale);
                o[2] = (unsigned char)(b * scale);
                o[3] = (unsigned char)(e + 128);
            }
        }
        f.write(reinterpret_cast<const char*>(row.data()), std::streamsize(row.size()));
    }
    return bool(f);
}

bool write_pfm(const std::string& path, int w, int h, const double* rad) {
    std::ofstream f(path, std::ios::binary);
    f << "PF\n" << w << ' ' << h << "\n-1.0\n";
    std::vector<float> row(3 * size_t(w));
    for (int j = h - 1; j >= 0; j--) {
        for (size_t k = 0; k < row.size(); k++)
            row[k] = float(rad[3 * size_t(j) * w + k]);
        f.write(reinterpret_cast<const char*>(row.data()), std::streamsize(row.size() * sizeof(float)));
    }
    return bool(f);
}

bool ends_with(const std::string& s, const char* suffix) {
    size_t n = std::strlen(suffix);
    return s.size() >= n && s.compare(s.size() - n, n, suffix) == 0;
}

}  // namespace

}  // namespace mypbr_dev

using namespace mypbr_dev;

extern "C" {

void mypbr_display_opts_init(mypbr_display_opts* o) {
    if (!o)
        return;
    *o = mypbr_display_opts{};
    o->exposure = 0;  // tonemap.h:16-18, postprocess.h:14-18
    o->tonemap = MYPBR_TONEMAP_NONE;
    o->bloom = 0;
    o->bloom_threshold = 1;
    o->bloom_radius = 0.04;
    o->vignette = 0;
}

int mypbr_gpu_display(const double* radiance, int32_t w, int32_t h, const mypbr_display_opts* opts,
                      double* linear, uint8_t* rgb8, int on_device) {
    int s = check_opts(radiance, w, h, opts);
    if (s != MYPBR_OK)
        return s;
    if (!linear && !rgb8) {
        set_error_message("mypbr_gpu_display: give linear or rgb8 (or both)");
        return MYPBR_ERR_INVALID_ARGUMENT;
    }
    mypbr_display_opts o;
    mypbr_display_opts_init(&o);
    if (opts)
        o = *opts;
    size_t n = size_t(w) * h;
    DevMem mem;
    const double* d_in = radiance;
    if (!on_device) {
        double* p;
        if ((s = mem.get(p, 3 * n)) != MYPBR_OK)
            return s;
        MYPBR_CUDA(cudaMemcpy(p, radiance, 3 * n * sizeof(double), cudaMemcpyHostToDevice));
        d_in = p;
    }
    if (linear) {
        double* d_lin = linear;
        if (!on_device && (s = mem.get(d_lin, 3 * n)) != MYPBR_OK)
            return s;
        if ((s = run_post(d_in, w, h, o, false, d_lin, nullptr)) != MYPBR_OK)
            return s;
        if (!on_device)
            MYPBR_CUDA(cudaMemcpy(linear, d_lin, 3 * n * sizeof(double), cudaMemcpyDeviceToHost));
    }
    if (rgb8) {
        unsigned char* d_b = rgb8;
        if (!on_device && (s = mem.get(d_b, 3 * n)) != MYPBR_OK)
            return s;
        if ((s = run_post(d_in, w, h, o, true, nullptr, d_b)) != MYPBR_OK)
            return s;
        if (!on_device)
            MYPBR_CUDA(cudaMemcpy(rgb8, d_b, 3 * n, cudaMemcpyDeviceToHost));
    }
    return MYPBR_OK;
}

int mypbr_write_image(const char* path, const double* radiance, int32_t w, int32_t h, const mypbr_display_opts* opts,
                      int on_device) {
    int s = check_opts(radiance, w, h, opts);
    if (s != MYPBR_OK)
        return s;
    std::string p = path ? path : "";
    bool shown = p.empty() || ends_with(p, ".png") || ends_with(p, ".ppm");
    size_t n = size_t(w) * h;
    bool ok = false;
    if (shown) {
        std::vector<uint8_t> rgb(3 * n);
        if ((s = mypbr_gpu_display(radiance, w, h, opts, nullptr, rgb.data(), on_device)) != MYPBR_OK)
            return s;
        if (p.empty()) {
            ok = write_ppm(stdout, w, h, rgb.data());
        } else if (ends_with(p, ".png")) {
            ok = write_png(p, w, h, rgb.data());
        } else {
            std::FILE* f = std::fopen(p.c_str(), "w");
            ok = f && write_ppm(f, w, h, rgb.data());
            if (f)
                std::fclose(f);
        }
    } else if (ends_with(p, ".hdr") || ends_with(p, ".pfm")) {
        std::vector<double> host;
        const double* rad = radiance;
        if (on_device) {
            host.resize(3 * n);
            MYPBR_CUDA(cudaMemcpy(host.data(), radiance, 3 * n * sizeof(double), cudaMemcpyDeviceToHost));
            rad = host.data();
        }
        ok = ends_with(p, ".hdr") ? write_hdr(p, w, h, rad) : write_pfm(p, w, h, rad);
    } else {
        set_error_message("unsupported output format '" + p + "' (use .png, .ppm, .hdr or .pfm)");
        return MYPBR_ERR_INVALID_ARGUMENT;
    }
    if (!ok) {
        set_error_message("cannot write '" + p + "'");
        return MYPBR_ERR_IO;
    }
    return MYPBR_OK;
}

}  // extern "C"
