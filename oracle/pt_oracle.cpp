// ORACLE — test infrastructure only, never part of the product path.
//
// A CPU restatement, in FP64, of mypbr's per-pixel path tracer
// (include/camera.h:79-529 of the reference) over the flat scene arrays of
// include/mypbr_gpu.h. Only the tests, the smoke check and the benchmark's
// CPU-baseline leg load it, as the checker and as the CPU timing; the product
// (mypbr_gb300/) never links or calls it.
//
// Each function follows the reference function cited beside it. Parity of this
// restatement is pinned against the reference itself: tests/golden/ holds
// vectors produced by oracle/ref_harness.cpp, which compiles the reference's
// own headers (intersection results, BSDF eval/pdf, light probabilities and
// pdfs, environment radiance and pdf, the GGX albedo table, and batch-mean
// images of full renders).
//
// Randomness: the reference draws from an unseeded thread-local mt19937
// (include/rtweekend.h:21-25); here every (pixel, pass) gets its own
// splitmix64-seeded xoshiro256+ stream, so renders are reproducible.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

#include "../include/mypbr_gpu.h"

namespace {

constexpr double PI = 3.1415926535897932385;
constexpr double INF = std::numeric_limits<double>::infinity();

// ------------------------------------------------------------------ vectors

struct V {
    double x = 0, y = 0, z = 0;
    V() = default;
    V(double a, double b, double c) : x(a), y(b), z(c) {}
    explicit V(const double* p) : x(p[0]), y(p[1]), z(p[2]) {}
    double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    double& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    V operator-() const { return {-x, -y, -z}; }
    V& operator+=(const V& o) {
        x += o.x;
        y += o.y;
        z += o.z;
        return *this;
    }
    double len2() const { return x * x + y * y + z * z; }
    double len() const { return std::sqrt(len2()); }
};
V operator+(const V& a, const V& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V operator-(const V& a, const V& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V operator*(const V& a, const V& b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
V operator*(double s, const V& a) { return {s * a.x, s * a.y, s * a.z}; }
V operator*(const V& a, double s) { return {s * a.x, s * a.y, s * a.z}; }
V operator/(const V& a, double s) { return (1 / s) * a; }
double dot(const V& a, const V& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V cross(const V& a, const V& b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
V unit(const V& a) { return a / a.len(); }
double lum(const V& c) { return 0.2126 * c.x + 0.7152 * c.y + 0.0722 * c.z; }
double avg3(const V& c) { return (c.x + c.y + c.z) / 3; }
V reflect(const V& v, const V& n) { return v - 2 * dot(v, n) * n; }
// vec3.h:324-329
V refract(const V& uv, const V& n, double ratio) {
    double c = std::fmin(dot(-uv, n), 1.0);
    V perp = ratio * (uv + c * n);
    V par = -std::sqrt(std::fabs(1.0 - perp.len2())) * n;
    return perp + par;
}

// -------------------------------------------------------------------- RNG

struct Rng {
    uint64_t s[4];
    static uint64_t splitmix(uint64_t& x) {
        uint64_t z = (x += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    }
    explicit Rng(uint64_t seed) {
        for (auto& w : s)
            w = splitmix(seed);
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    double next() {  // [0, 1)
        uint64_t r = s[0] + s[3];
        uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return double(r >> 11) * (1.0 / 9007199254740992.0);
    }
};

// vec3.h:286-293
V random_unit_vector(Rng& g) {
    while (true) {
        V p(2 * g.next() - 1, 2 * g.next() - 1, 2 * g.next() - 1);
        double l2 = p.len2();
        if (1e-160 < l2 && l2 <= 1)
            return p / std::sqrt(l2);
    }
}
// vec3.h:296-306
V random_cosine_direction(Rng& g) {
    double r1 = g.next(), r2 = g.next();
    double phi = 2 * PI * r1;
    return {std::cos(phi) * std::sqrt(r2), std::sin(phi) * std::sqrt(r2), std::sqrt(1 - r2)};
}
// vec3.h:309-315
V random_in_unit_disk(Rng& g) {
    while (true) {
        V p(2 * g.next() - 1, 2 * g.next() - 1, 0);
        if (p.len2() < 1)
            return p;
    }
}

// -------------------------------------------------------------------- ONB

// onb.h:9-28
struct Onb {
    V a[3];
    Onb() = default;
    explicit Onb(const V& n) {
        a[2] = unit(n);
        V t = std::fabs(a[2].x) > 0.9 ? V(0, 1, 0) : V(1, 0, 0);
        a[1] = unit(cross(a[2], t));
        a[0] = cross(a[2], a[1]);
    }
    V to_world(const V& v) const { return v.x * a[0] + v.y * a[1] + v.z * a[2]; }
    V to_local(const V& v) const { return {dot(v, a[0]), dot(v, a[1]), dot(v, a[2])}; }
};

// ------------------------------------------------------------ the scene

struct Xform {
    double m[3][3], t[3], im[3][3], it[3];
    static V mul(const double a[3][3], const V& v) {
        return {a[0][0] * v.x + a[0][1] * v.y + a[0][2] * v.z, a[1][0] * v.x + a[1][1] * v.y + a[1][2] * v.z,
                a[2][0] * v.x + a[2][1] * v.y + a[2][2] * v.z};
    }
    V point(const V& p) const { return mul(m, p) + V(t); }
    V vec(const V& v) const { return mul(m, v); }
    V ipoint(const V& p) const { return mul(im, p) + V(it); }
    V ivec(const V& v) const { return mul(im, v); }
    V normal(const V& n) const {
        return {im[0][0] * n.x + im[1][0] * n.y + im[2][0] * n.z, im[0][1] * n.x + im[1][1] * n.y + im[2][1] * n.z,
                im[0][2] * n.x + im[1][2] * n.y + im[2][2] * n.z};
    }
};

struct Hit {
    V p, normal, dpdu, dpdv;
    double t = 0, u = 0, v = 0;
    bool front = true;
    int mat = -1;
    int kind = -1, index = -1;
    void set_face(const V& d, const V& outward) {
        front = dot(d, outward) < 0;
        normal = front ? outward : -outward;
    }
};

struct EnvDist {
    int w = 0, h = 0;
    std::vector<double> cond, marg, roww;
    double total = 0;
};

struct Scene {
    const mypbr_flat_scene* f;
    std::vector<Xform> xf;
    std::vector<double> light_cdf;
    std::vector<std::vector<double>> member_cdf;
    EnvDist env;
    double E[32][32], Eavg[32];
    // sun (sun.h:23-43)
    Onb sun_frame;
    double sun_cos_max = 1, sun_solid_angle = 0;
    V sun_radiance;
};

// ------------------------------------------------------- primitive hits

bool in_open(double t, double a, double b) { return a < t && t < b; }
bool in_closed(double t, double a, double b) { return a <= t && t <= b; }

// sphere.h:536-560
void sphere_uv(const V& p, double& u, double& v) {
    double theta = std::acos(std::clamp(-p.y, -1.0, 1.0));
    double phi = std::atan2(-p.z, p.x) + PI;
    u = phi / (2 * PI);
    v = theta / PI;
}
void sphere_tangents(const V& p, double r, V& dpdu, V& dpdv) {
    double st = std::sqrt(p.x * p.x + p.z * p.z);
    if (st < 1e-8) {
        dpdu = dpdv = V();
        return;
    }
    dpdu = (2 * PI * r) * V(p.z, 0, -p.x);
    dpdv = (PI * r / st) * V(-p.x * p.y, st * st, -p.y * p.z);
}

// sphere.h:23-52 (object space)
bool hit_sphere_local(const V& c, double radius, const V& o, const V& d, double tmin, double tmax, Hit& rec) {
    V oc = c - o;
    double a = d.len2(), h = dot(d, oc), cc = oc.len2() - radius * radius;
    double disc = h * h - a * cc;
    if (disc < 0)
        return false;
    double sq = std::sqrt(disc);
    double root = (h - sq) / a;
    if (!in_open(root, tmin, tmax)) {
        root = (h + sq) / a;
        if (!in_open(root, tmin, tmax))
            return false;
    }
    rec.t = root;
    rec.p = o + root * d;
    V outward = (rec.p - c) / radius;
    rec.set_face(d, outward);
    V un = outward * (radius < 0 ? -1.0 : 1.0);
    sphere_uv(un, rec.u, rec.v);
    sphere_tangents(un, std::fabs(radius), rec.dpdu, rec.dpdv);
    return true;
}

// sphere.h:23-52, moved by instance::hit (instance.h:29-41) when transformed
bool hit_sphere(const Scene& S, int i, const V& o, const V& d, double tmin, double tmax, Hit& rec) {
    const auto& s = S.f->spheres[i];
    V c(s.center);
    if (s.xform < 0) {
        if (!hit_sphere_local(c, s.radius, o, d, tmin, tmax, rec))
            return false;
    } else {
        const Xform& x = S.xf[s.xform];
        if (!hit_sphere_local(c, s.radius, x.ipoint(o), x.ivec(d), tmin, tmax, rec))
            return false;
        rec.p = x.point(rec.p);
        rec.normal = unit(x.normal(rec.normal));
        rec.dpdu = x.vec(rec.dpdu);
        rec.dpdv = x.vec(rec.dpdv);
    }
    rec.mat = s.material;
    return true;
}

// quad.h:30-62
bool hit_quad(const Scene& S, int i, const V& o, const V& d, double tmin, double tmax, Hit& rec) {
    const auto& q = S.f->quads[i];
    V Q(q.q), u(q.u), v(q.v), n(q.normal);
    V nn = cross(u, v);
    V w = nn / dot(nn, nn);
    double denom = dot(n, d);
    if (std::fabs(denom) < 1e-8)
        return false;
    double t = (dot(n, Q) - dot(n, o)) / denom;
    if (!in_closed(t, tmin, tmax))
        return false;
    V p = o + t * d;
    V hp = p - Q;
    double alpha = dot(w, cross(hp, v)), beta = dot(w, cross(u, hp));
    if (alpha < 0 || alpha > 1 || beta < 0 || beta > 1)
        return false;
    rec.t = t;
    rec.p = p;
    rec.u = alpha;
    rec.v = beta;
    rec.dpdu = u;
    rec.dpdv = v;
    rec.mat = q.material;
    rec.set_face(d, n);
    return true;
}

V pos(const Scene& S, int k) { return V(S.f->positions + 3 * int64_t(k)); }

// image_texture::alpha_value (texture.h:132-136) of the mask of a triangle
// flagged MYPBR_TRI_ALPHA_MASK: the alpha byte, or the grey level of an image
// without an alpha channel, at the nearest pixel (texture.h:181-194), / 255.
// An HDR image is opaque.
double alpha_coverage(const Scene& S, const mypbr_triangle& tr, double u, double v) {
    const mypbr_texture& tx = S.f->textures[S.f->meshes[tr.mesh].alpha_mask];
    if (tx.flags & MYPBR_TEXF_HDR)
        return 1;
    if (tx.flags & MYPBR_TEXF_REPEAT) {
        u -= std::floor(u);
        v -= std::floor(v);
    } else {
        u = std::fmin(std::fmax(u, 0.0), 1.0);
        v = std::fmin(std::fmax(v, 0.0), 1.0);
    }
    v = 1.0 - v;
    int x = std::clamp(int(u * tx.width), 0, tx.width - 1);
    int y = std::clamp(int(v * tx.height), 0, tx.height - 1);
    int64_t k = tx.offset + int64_t(y) * tx.width + x;
    return S.f->texels_ldr[4 * k + ((tx.flags & MYPBR_TEXF_GREY_MASK) ? 0 : 3)] / 255.0;
}

// mesh.h:47-108 (Moller-Trumbore). An alpha-masked triangle is met with
// probability equal to its coverage (mesh.h:81-86), decided with g; without
// g (queries that draw no random numbers) it is there wherever the coverage
// is above 0, and with masked false it is solid (light sampling densities,
// whose holes are ignored like the power estimate's, mesh.h:138).
bool hit_triangle(const Scene& S, int i, const V& o, const V& d, double tmin, double tmax, Hit& rec,
                  Rng* rng = nullptr, bool masked = true) {
    const auto& tr = S.f->triangles[i];
    V p0 = pos(S, tr.v[0]);
    V e1 = pos(S, tr.v[1]) - p0, e2 = pos(S, tr.v[2]) - p0;
    V pv = cross(d, e2);
    double det = dot(e1, pv);
    if (std::fabs(det) < 1e-12)
        return false;
    double inv = 1 / det;
    V tv = o - p0;
    double b1 = dot(tv, pv) * inv;
    if (b1 < 0 || b1 > 1)
        return false;
    V qv = cross(tv, e1);
    double b2 = dot(d, qv) * inv;
    if (b2 < 0 || b1 + b2 > 1)
        return false;
    double t = dot(e2, qv) * inv;
    if (!in_open(t, tmin, tmax))
        return false;
    double b0 = 1 - b1 - b2, u = b1, v = b2;
    bool has_uv = tr.t[0] >= 0;
    V uv0, uv1, uv2;
    if (has_uv) {
        auto uvat = [&](int k) { return V(S.f->uvs[2 * int64_t(k)], S.f->uvs[2 * int64_t(k) + 1], 0); };
        uv0 = uvat(tr.t[0]);
        uv1 = uvat(tr.t[1]);
        uv2 = uvat(tr.t[2]);
        V uv = b0 * uv0 + b1 * uv1 + b2 * uv2;
        u = uv.x;
        v = uv.y;
    }
    // checked before rec changes: a miss keeps the closest hit so far
    if (masked && (tr.flags & MYPBR_TRI_ALPHA_MASK)) {
        double coverage = alpha_coverage(S, tr, u, v);
        if (coverage < 1 && (rng ? rng->next() >= coverage : coverage <= 0))
            return false;
    }
    rec.t = t;
    rec.u = u;
    rec.v = v;
    rec.p = o + t * d;
    rec.mat = tr.material;
    if (!has_uv) {
        rec.dpdu = e1;
        rec.dpdv = e2;
    } else {
        V d1 = uv1 - uv0, d2 = uv2 - uv0;
        double dt = d1.x * d2.y - d2.x * d1.y;
        if (std::fabs(dt) < 1e-12) {
            rec.dpdu = rec.dpdv = V();
        } else {
            double iv = 1 / dt;
            rec.dpdu = (d2.y * e1 - d1.y * e2) * iv;
            rec.dpdv = (d1.x * e2 - d2.x * e1) * iv;
        }
    }
    V g = unit(cross(e1, e2));
    if (tr.flags & MYPBR_TRI_FLIP_NORMAL)
        g = -g;
    rec.set_face(d, g);
    if (tr.n[0] >= 0) {
        auto nat = [&](int k) { return V(S.f->normals + 3 * int64_t(k)); };
        V sh = b0 * nat(tr.n[0]) + b1 * nat(tr.n[1]) + b2 * nat(tr.n[2]);
        if (sh.len2() > 0) {
            sh = unit(sh);
            rec.normal = dot(sh, rec.normal) < 0 ? -sh : sh;
        }
    }
    return true;
}

// Where a line enters and leaves a convex boundary, the two hits that
// constant_medium::hit asks its boundary for (medium.h:298-302).
bool medium_span(const Scene& S, const mypbr_medium& m, const V& o, const V& d, double& t_in, double& t_out) {
    V lo = o, ld = d;
    if (m.xform >= 0) {
        lo = S.xf[m.xform].ipoint(o);
        ld = S.xf[m.xform].ivec(d);
    }
    if (m.shape == 0) {
        V c(m.a);
        double r = m.b[0];
        V oc = c - lo;
        double a = ld.len2(), h = dot(ld, oc), cc = oc.len2() - r * r;
        double disc = h * h - a * cc;
        if (disc < 0)
            return false;
        double sq = std::sqrt(disc);
        double r1 = (h - sq) / a, r2 = (h + sq) / a;
        // first hit over (-inf, inf), then the next one after it + 1e-4
        t_in = r1;
        if (!(r2 > r1 + 0.0001))
            return false;
        t_out = r2;
        return true;
    }
    // box: the slab interval of the six faces
    double t0 = -INF, t1 = INF;
    for (int k = 0; k < 3; k++) {
        double mn = std::fmin(m.a[k], m.b[k]), mx = std::fmax(m.a[k], m.b[k]);
        if (ld[k] == 0) {
            if (lo[k] < mn || lo[k] > mx)
                return false;
            continue;
        }
        double ta = (mn - lo[k]) / ld[k], tb = (mx - lo[k]) / ld[k];
        if (ta > tb)
            std::swap(ta, tb);
        t0 = std::fmax(t0, ta);
        t1 = std::fmin(t1, tb);
    }
    if (!(t1 > t0 + 0.0001))
        return false;
    t_in = t0;
    t_out = t1;
    return true;
}

// medium.h:295-323
bool hit_medium(const Scene& S, int i, const V& o, const V& d, double tmin, double tmax, Hit& rec, Rng& g) {
    const auto& m = S.f->media[i];
    double a, b;
    if (!medium_span(S, m, o, d, a, b))
        return false;
    double t0 = std::fmax(a, tmin), t1 = std::fmin(b, tmax);
    if (t0 >= t1)
        return false;
    double len = d.len();
    double inside = (t1 - t0) * len;
    double dist = -std::log(1 - g.next()) / m.density;
    if (dist > inside)
        return false;
    rec.t = t0 + dist / len;
    rec.p = o + rec.t * d;
    rec.normal = V(1, 0, 0);
    rec.front = true;
    rec.u = rec.v = 0;
    rec.dpdu = rec.dpdv = V();
    rec.mat = m.material;
    return true;
}

// plane.h:17-34
bool hit_ground(const mypbr_unbounded& gp, const V& o, const V& d, double tmin, double tmax, Hit& rec) {
    double dy = d.y;
    if (std::fabs(dy) < 1e-12)
        return false;
    double t = (gp.height - o.y) / dy;
    if (!in_open(t, tmin, tmax))
        return false;
    rec.t = t;
    rec.p = o + t * d;
    rec.p.y = gp.height;
    rec.u = rec.p.x;
    rec.v = -rec.p.z;
    rec.dpdu = V(1, 0, 0);
    rec.dpdv = V(0, 0, -1);
    rec.mat = gp.material;
    rec.set_face(d, V(0, 1, 0));
    return true;
}

// medium.h:352-381
bool hit_height_fog(const mypbr_unbounded& hf, const V& o, const V& d, double tmin, double tmax, Hit& rec, Rng& g) {
    double length = d.len();
    double k = d.y / hf.scale_height;
    double t0 = tmin;
    double start = hf.density * length * std::exp(-(o.y + t0 * d.y - hf.height) / hf.scale_height);
    if (!(start > 0))
        return false;
    double tau = -std::log(1 - g.next());
    double t;
    if (std::fabs(k) < 1e-12) {
        t = t0 + tau / start;
    } else {
        double x = 1 - tau * k / start;
        if (x <= 0)
            return false;
        t = t0 - std::log(x) / k;
    }
    if (!(t < tmax) || !std::isfinite(t))
        return false;
    rec.t = t;
    rec.p = o + t * d;
    rec.normal = V(1, 0, 0);
    rec.front = true;
    rec.u = rec.v = 0;
    rec.dpdu = rec.dpdv = V();
    rec.mat = hf.material;
    return true;
}

// ---------------------------------------------------------------- voxels

// A block of a placed voxel model: voxel_grid::hit (voxel.h:193-268) in the
// model's space, a 3D DDA (Amanatides and Woo 1987) whose surfaces are the
// crossings between cells of different kind (voxel.h:294-305), placed in the
// world as instance::hit does (instance.h:29-40).
struct VoxelWalk {
    const Scene& S;
    const mypbr_voxel_model& m;
    const uint8_t* cells;
    int kind_of(int idx) const { return S.f->voxel_palettes[m.palette + idx].kind; }
    int at(const int c[3]) const {  // voxel.h:284-288
        if (unsigned(c[0]) >= unsigned(m.nx) || unsigned(c[1]) >= unsigned(m.ny) || unsigned(c[2]) >= unsigned(m.nz))
            return 0;
        return cells[(size_t(c[2]) * m.ny + c[1]) * m.nx + c[0]];
    }
    static bool face_visible(int k, int n) {  // voxel.h:100-106
        if (k == MYPBR_VOXEL_EMPTY)
            return false;
        if (n == MYPBR_VOXEL_EMPTY)
            return true;
        return k == MYPBR_VOXEL_OPAQUE && n == MYPBR_VOXEL_TRANSPARENT;
    }
    bool on_edge(const V& p, int axis, int sign, const int cell[3]) const {  // voxel.h:313-331
        int k = kind_of(at(cell));
        for (int side = 1; side <= 2; side++) {
            int tangent = (axis + side) % 3;
            double f = p[tangent] - cell[tangent];
            for (int dir = -1; dir <= 1; dir += 2) {
                if ((dir > 0 ? 1 - f : f) >= m.edge_width)
                    continue;
                int beside[3] = {cell[0], cell[1], cell[2]};
                beside[tangent] += dir;
                int above[3] = {beside[0], beside[1], beside[2]};
                above[axis] += sign;
                if (face_visible(k, kind_of(at(beside))) || kind_of(at(above)) != MYPBR_VOXEL_EMPTY)
                    return true;
            }
        }
        return false;
    }
    // voxel.h:333-350, in model space
    bool record(const V& o, const V& d, double t, int axis, int sign, int index, const int cell[3], Hit& rec) const {
        rec.t = t;
        rec.p = o + t * d;
        V outward, tb, tc;
        outward[axis] = sign;
        tb[(axis + 1) % 3] = 1;
        tc[(axis + 2) % 3] = 1;
        rec.dpdu = sign > 0 ? tb : tc;
        rec.dpdv = sign > 0 ? tc : tb;
        rec.u = dot(rec.p, rec.dpdu) - std::floor(dot(rec.p, rec.dpdu));
        rec.v = dot(rec.p, rec.dpdv) - std::floor(dot(rec.p, rec.dpdv));
        rec.mat = m.edge_width > 0 && on_edge(rec.p, axis, sign, cell) ? m.edge_material
                                                                        : S.f->voxel_palettes[m.palette + index].material;
        rec.set_face(d, outward);
        return true;
    }
    bool crossing(const V& o, const V& d, double t, int axis, int step, int from, int to, const int to_cell[3],
                  Hit& rec) const {  // voxel.h:294-305
        int k_from = kind_of(from), k_to = kind_of(to);
        if (k_to != MYPBR_VOXEL_EMPTY && face_visible(k_to, k_from))
            return record(o, d, t, axis, -step, to, to_cell, rec);
        if (face_visible(k_from, k_to)) {
            int from_cell[3] = {to_cell[0], to_cell[1], to_cell[2]};
            from_cell[axis] -= step;
            return record(o, d, t, axis, step, from, from_cell, rec);
        }
        return false;
    }
    bool hit(const int lo[3], const int hi[3], const V& o, const V& d, double tmin, double tmax, Hit& rec) const {
        double t_enter = -INF, t_exit = INF;
        int enter_axis = 0;
        for (int a = 0; a < 3; a++) {
            if (d[a] == 0) {
                if (o[a] < lo[a] || o[a] > hi[a])
                    return false;
                continue;
            }
            double t0 = (lo[a] - o[a]) / d[a], t1 = (hi[a] - o[a]) / d[a];
            if (t0 > t1)
                std::swap(t0, t1);
            if (t0 > t_enter) {
                t_enter = t0;
                enter_axis = a;
            }
            t_exit = std::fmin(t_exit, t1);
        }
        bool from_outside = t_enter >= tmin;
        double t_start = from_outside ? t_enter : tmin;
        if (t_start > std::fmin(t_exit, tmax))
            return false;
        V start = o + t_start * d;
        int c[3], step[3];
        double t_next[3], t_delta[3];
        for (int a = 0; a < 3; a++) {
            c[a] = std::clamp(int(std::floor(start[a])), lo[a], hi[a] - 1);
            if (from_outside && a == enter_axis)
                c[a] = d[a] > 0 ? lo[a] : hi[a] - 1;
            if (d[a] > 0) {
                step[a] = 1;
                t_next[a] = (c[a] + 1 - o[a]) / d[a];
                t_delta[a] = 1 / d[a];
            } else if (d[a] < 0) {
                step[a] = -1;
                t_next[a] = (c[a] - o[a]) / d[a];
                t_delta[a] = -1 / d[a];
            } else {
                step[a] = 0;
                t_next[a] = t_delta[a] = INF;
            }
        }
        int index = at(c);
        if (from_outside) {
            int behind[3] = {c[0], c[1], c[2]};
            behind[enter_axis] -= step[enter_axis];
            if (crossing(o, d, t_enter, enter_axis, step[enter_axis], at(behind), index, c, rec))
                return true;
        }
        while (true) {
            int a = t_next[0] < t_next[1] ? (t_next[0] < t_next[2] ? 0 : 2) : (t_next[1] < t_next[2] ? 1 : 2);
            double t = t_next[a];
            if (t > tmax)
                return false;
            c[a] += step[a];
            t_next[a] += t_delta[a];
            int next = at(c);
            if (crossing(o, d, t, a, step[a], index, next, c, rec))
                return true;
            if (c[a] < lo[a] || c[a] >= hi[a])
                return false;
            index = next;
        }
    }
};

bool hit_voxel_block(const Scene& S, int i, const V& o, const V& d, double tmin, double tmax, Hit& rec) {
    const auto& b = S.f->voxel_blocks[i];
    const auto& m = S.f->voxel_models[b.model];
    const Xform& X = S.xf[m.xform];
    VoxelWalk w{S, m, S.f->voxel_cells + m.cells};
    V lo = X.ipoint(o), ld = X.ivec(d);
    if (!w.hit(b.lo, b.hi, lo, ld, tmin, tmax, rec))
        return false;
    rec.p = X.point(rec.p);
    rec.normal = unit(X.normal(rec.normal));
    rec.dpdu = X.vec(rec.dpdu);
    rec.dpdv = X.vec(rec.dpdv);
    return true;
}

bool hit_prim(const Scene& S, int kind, int index, const V& o, const V& d, double tmin, double tmax, Hit& rec,
              Rng* g) {
    bool h = false;
    switch (kind) {
        case MYPBR_PRIM_SPHERE: h = hit_sphere(S, index, o, d, tmin, tmax, rec); break;
        case MYPBR_PRIM_QUAD: h = hit_quad(S, index, o, d, tmin, tmax, rec); break;
        case MYPBR_PRIM_TRIANGLE: h = hit_triangle(S, index, o, d, tmin, tmax, rec, g); break;
        case MYPBR_PRIM_MEDIUM: h = g ? hit_medium(S, index, o, d, tmin, tmax, rec, *g) : false; break;
        case MYPBR_PRIM_VOXEL_BLOCK: h = hit_voxel_block(S, index, o, d, tmin, tmax, rec); break;
        default: break;
    }
    if (h) {
        rec.kind = kind;
        rec.index = index;
    }
    return h;
}

// bvh.h:45-86 slab test (aabb.h:40-54)
bool box_hit(const mypbr_bvh_node& n, const V& o, const V& inv, double tmin, double tmax) {
    for (int a = 0; a < 3; a++) {
        double t0 = (n.bmin[a] - o[a]) * inv[a], t1 = (n.bmax[a] - o[a]) * inv[a];
        if (t0 > t1)
            std::swap(t0, t1);
        if (t0 > tmin)
            tmin = t0;
        if (t1 < tmax)
            tmax = t1;
        if (tmax <= tmin)
            return false;
    }
    return true;
}

// The world's closest hit: the BVH (bvh.h:45-86), then scene::unbounded beside
// it (main.cpp:70-74, hittable_list.h:25-37). brute_force tests every
// primitive instead of walking the BVH (a check of the BVH itself).
bool world_hit(const Scene& S, const V& o, const V& d, double tmin, double tmax, Hit& rec, Rng* g,
               bool brute_force = false) {
    const mypbr_flat_scene& F = *S.f;
    bool any = false;
    double closest = tmax;
    Hit tmp;
    if (brute_force) {
        for (int64_t k = 0; k < F.bvh_prim_count; k++) {
            const auto& r = F.bvh_prims[k];
            if (hit_prim(S, r.kind, r.index, o, d, tmin, closest, tmp, g)) {
                any = true;
                closest = tmp.t;
                rec = tmp;
            }
        }
    } else if (F.bvh_prim_count > 0) {
        V inv(1 / d.x, 1 / d.y, 1 / d.z);
        bool neg[3] = {inv.x < 0, inv.y < 0, inv.z < 0};
        int stack[128];
        int sp = 0, cur = 0;
        while (true) {
            const auto& n = F.bvh_nodes[cur];
            if (box_hit(n, o, inv, tmin, closest)) {
                if (n.count > 0) {
                    for (int k = 0; k < n.count; k++) {
                        const auto& r = F.bvh_prims[n.offset + k];
                        if (hit_prim(S, r.kind, r.index, o, d, tmin, closest, tmp, g)) {
                            any = true;
                            closest = tmp.t;
                            rec = tmp;
                        }
                    }
                    if (sp == 0)
                        break;
                    cur = stack[--sp];
                } else if (neg[n.axis]) {
                    stack[sp++] = cur + 1;
                    cur = n.offset;
                } else {
                    stack[sp++] = n.offset;
                    cur = cur + 1;
                }
            } else {
                if (sp == 0)
                    break;
                cur = stack[--sp];
            }
        }
    }
    for (int64_t k = 0; k < F.unbounded_count; k++) {
        const auto& ub = F.unbounded[k];
        bool h = false;
        if (ub.kind == MYPBR_UNBOUNDED_GROUND)
            h = hit_ground(ub, o, d, tmin, closest, tmp);
        else if (g)
            h = hit_height_fog(ub, o, d, tmin, closest, tmp, *g);
        if (h) {
            tmp.kind = 5 + ub.kind;  // after the MYPBR_PRIM_* kinds
            tmp.index = int(k);
            any = true;
            closest = tmp.t;
            rec = tmp;
        }
    }
    return any;
}

// ------------------------------------------------------------- textures

V tex_value(const Scene& S, int t, double u, double v, const V& p) {
    if (t < 0)
        return V(0, 0, 0);
    const auto& tx = S.f->textures[t];
    switch (tx.type) {
        case MYPBR_TEX_SOLID: return V(tx.p[0], tx.p[1], tx.p[2]);
        case MYPBR_TEX_CHECKER: {  // texture.h:43-50
            int x = int(std::floor(tx.p[0] * p.x)), y = int(std::floor(tx.p[0] * p.y)),
                z = int(std::floor(tx.p[0] * p.z));
            return (x + y + z) % 2 == 0 ? tex_value(S, tx.a, u, v, p) : tex_value(S, tx.b, u, v, p);
        }
        case MYPBR_TEX_IMAGE: {  // texture.h:119-127, 181-194
            if (tx.flags & MYPBR_TEXF_REPEAT) {
                u -= std::floor(u);
                v -= std::floor(v);
            } else {
                u = std::fmin(std::fmax(u, 0.0), 1.0);
                v = std::fmin(std::fmax(v, 0.0), 1.0);
            }
            v = 1.0 - v;
            int i = std::clamp(int(u * tx.width), 0, tx.width - 1);
            int j = std::clamp(int(v * tx.height), 0, tx.height - 1);
            int64_t k = tx.offset + int64_t(j) * tx.width + i;
            if (tx.flags & MYPBR_TEXF_HDR) {
                const float* px = S.f->texels_hdr + 3 * k;
                return V(px[0], px[1], px[2]);
            }
            const uint8_t* px = S.f->texels_ldr + 4 * k;
            if (tx.flags & MYPBR_TEXF_LINEAR)
                return V(px[0], px[1], px[2]) / 255.0;
            auto dec = [](int c) {
                double e = c / 255.0;
                return e <= 0.04045 ? e / 12.92 : std::pow((e + 0.055) / 1.055, 2.4);
            };
            return V(dec(px[0]), dec(px[1]), dec(px[2]));
        }
        case MYPBR_TEX_SCALED:  // texture.h:216-218
            return V(tx.p[0], tx.p[1], tx.p[2]) * tex_value(S, tx.a, u, v, p);
        case MYPBR_TEX_CHANNEL: {  // texture.h:233-236
            double x = tx.p[0] * tex_value(S, tx.a, u, v, p)[tx.b];
            return V(x, x, x);
        }
        case MYPBR_TEX_UV_TRANSFORM: {  // texture.h:255-259
            double c = std::cos(tx.p[2]), s = std::sin(tx.p[2]);
            double su = tx.p[3] * u, sv = tx.p[4] * (1 - v);
            double tu = c * su + s * sv + tx.p[0];
            double tv = -s * su + c * sv + tx.p[1];
            return tex_value(S, tx.a, tu, 1 - tv, p);
        }
        case MYPBR_TEX_NORMAL_SCALE: {  // texture.h:274-277
            V c = tex_value(S, tx.a, u, v, p);
            return V(0.5 + tx.p[0] * (c.x - 0.5), 0.5 + tx.p[0] * (c.y - 0.5), c.z);
        }
    }
    return V(0, 0, 0);
}

// ------------------------------------------------------- microfacet model

double rough_to_alpha(double r) { return std::max(r * r, 1e-3); }  // microfacet.h:17-19
double schlick(double c, double f0) { return f0 + (1 - f0) * std::pow(1 - std::clamp(c, 0.0, 1.0), 5); }
V schlick3(double c, const V& f0) { return {schlick(c, f0.x), schlick(c, f0.y), schlick(c, f0.z)}; }

// microfacet.h:34-48
double fresnel_dielectric(double ci, double eta) {
    ci = std::clamp(ci, -1.0, 1.0);
    if (ci < 0) {
        eta = 1 / eta;
        ci = -ci;
    }
    double s2i = 1 - ci * ci, s2t = s2i / (eta * eta);
    if (s2t >= 1)
        return 1;
    double ct = std::sqrt(1 - s2t);
    double rp = (eta * ci - ct) / (eta * ci + ct), rs = (ci - eta * ct) / (ci + eta * ct);
    return (rp * rp + rs * rs) / 2;
}

// microfacet.h:57-65
double fresnel_conductor(double ci, double eta, double k) {
    ci = std::clamp(ci, 0.0, 1.0);
    std::complex<double> n(eta, k);
    std::complex<double> s2t = (1 - ci * ci) / (n * n);
    std::complex<double> ct = std::sqrt(1.0 - s2t);
    std::complex<double> rp = (n * ci - ct) / (n * ci + ct), rs = (ci - n * ct) / (ci + n * ct);
    return (std::norm(rp) + std::norm(rs)) / 2;
}

// microfacet.h:145-212
struct Ggx {
    double a;
    double D(const V& h) const {
        if (h.z <= 0)
            return 0;
        double a2 = a * a, d = h.z * h.z * (a2 - 1) + 1;
        return a2 / (PI * d * d);
    }
    double lambda(const V& w) const {
        double c2 = w.z * w.z;
        if (c2 <= 0)
            return INF;
        double t2 = std::fmax(0.0, 1 - c2) / c2;
        return (-1 + std::sqrt(1 + a * a * t2)) / 2;
    }
    double G1(const V& w) const { return 1 / (1 + lambda(w)); }
    double G(const V& wo, const V& wi) const { return 1 / (1 + lambda(wo) + lambda(wi)); }
    double visible_pdf(const V& wo, const V& h) const {
        if (wo.z <= 0)
            return 0;
        return G1(wo) / wo.z * D(h) * std::fabs(dot(wo, h));
    }
    V sample_visible(const V& wo, double u1, double u2) const {
        V vh = unit(V(a * wo.x, a * wo.y, wo.z));
        double l2 = vh.x * vh.x + vh.y * vh.y;
        V t1 = l2 > 0 ? V(-vh.y, vh.x, 0) / std::sqrt(l2) : V(1, 0, 0);
        V t2 = cross(vh, t1);
        double r = std::sqrt(u1), phi = 2 * PI * u2;
        double p1 = r * std::cos(phi), p2 = r * std::sin(phi);
        double s = 0.5 * (1 + vh.z);
        p2 = (1 - s) * std::sqrt(std::fmax(0.0, 1 - p1 * p1)) + s * p2;
        V nh = p1 * t1 + p2 * t2 + std::sqrt(std::fmax(0.0, 1 - p1 * p1 - p2 * p2)) * vh;
        return unit(V(a * nh.x, a * nh.y, std::fmax(1e-6, nh.z)));
    }
};

// ggx_albedo_table (microfacet.h:276-293), ggx_ms_* (microfacet.h:341-373)
double table_E(const Scene& S, double c, double alpha) {
    double x = std::clamp(c, 0.0, 1.0) * 31, y = std::clamp(std::sqrt(alpha), 0.0, 1.0) * 31;
    int i = std::min(int(x), 30), j = std::min(int(y), 30);
    double tx = x - i, ty = y - j;
    double lo = (1 - tx) * S.E[j][i] + tx * S.E[j][i + 1];
    double hi = (1 - tx) * S.E[j + 1][i] + tx * S.E[j + 1][i + 1];
    return (1 - ty) * lo + ty * hi;
}
double table_Eavg(const Scene& S, double alpha) {
    double y = std::clamp(std::sqrt(alpha), 0.0, 1.0) * 31;
    int j = std::min(int(y), 30);
    double ty = y - j;
    return (1 - ty) * S.Eavg[j] + ty * S.Eavg[j + 1];
}
double ms_eval(const Scene& S, double co, double ci, double alpha) {
    if (co <= 0 || ci <= 0)
        return 0;
    double miss = 1 - table_Eavg(S, alpha);
    if (miss < 1e-6)
        return 0;
    return (1 - table_E(S, co, alpha)) * (1 - table_E(S, ci, alpha)) / (PI * miss) * ci;
}
double ms_albedo(const Scene& S, double co, double alpha) {
    if (co <= 0 || 1 - table_Eavg(S, alpha) < 1e-6)
        return 0;
    return 1 - table_E(S, co, alpha);
}
V ms_fresnel_avg(const Scene& S, const V& favg, double alpha) {
    double e = table_Eavg(S, alpha);
    V r;
    for (int k = 0; k < 3; k++)
        r[k] = favg[k] * favg[k] * e / (1 - favg[k] * (1 - e));
    return r;
}
V ms_fresnel(const Scene& S, const V& f0, double alpha) {
    return ms_fresnel_avg(S, f0 + (V(1, 1, 1) - f0) / 21, alpha);
}

// rough_dielectric_bsdf (microfacet.h:384-470)
struct RoughGlass {
    Onb frame;
    V wo;
    double eta;
    Ggx d;
    bool half_vector(const V& wiw, V& wi, V& wm, bool& refl) const {
        if (wiw.len2() == 0 || wo.z <= 0)
            return false;
        wi = unit(frame.to_local(wiw));
        if (wi.z == 0)
            return false;
        refl = wi.z > 0;
        wm = refl ? wo + wi : wi * eta + wo;
        if (wm.len2() == 0)
            return false;
        wm = unit(wm);
        if (wm.z < 0)
            wm = -wm;
        if (dot(wm, wi) * wi.z < 0 || dot(wm, wo) * wo.z < 0)
            return false;
        return true;
    }
    double eval(const V& wiw) const {
        V wi, wm;
        bool refl;
        if (!half_vector(wiw, wi, wm, refl))
            return 0;
        double F = fresnel_dielectric(dot(wo, wm), eta);
        if (refl)
            return F * d.D(wm) * d.G(wo, wi) / (4 * wo.z);
        double den = dot(wi, wm) + dot(wo, wm) / eta;
        den *= den;
        double ft = (1 - F) * d.D(wm) * d.G(wo, wi) * std::fabs(dot(wi, wm) * dot(wo, wm) / (wi.z * wo.z * den));
        ft /= eta * eta;
        return ft * std::fabs(wi.z);
    }
    double pdf(const V& wiw) const {
        V wi, wm;
        bool refl;
        if (!half_vector(wiw, wi, wm, refl))
            return 0;
        double F = fresnel_dielectric(dot(wo, wm), eta);
        if (refl)
            return F * d.visible_pdf(wo, wm) / (4 * std::fabs(dot(wo, wm)));
        double den = dot(wi, wm) + dot(wo, wm) / eta;
        den *= den;
        return (1 - F) * d.visible_pdf(wo, wm) * std::fabs(dot(wi, wm)) / den;
    }
    V sample(Rng& g) const {
        if (wo.z <= 0)
            return V();
        V wm = d.sample_visible(wo, g.next(), g.next());
        double F = fresnel_dielectric(dot(wo, wm), eta);
        V wi;
        if (g.next() < F) {
            wi = -wo + 2 * dot(wo, wm) * wm;
            if (wi.z <= 0)
                return V();
        } else {
            wi = refract(-wo, wm, 1 / eta);
            if (wi.z >= 0)
                return V();
        }
        return frame.to_world(wi);
    }
};

// ------------------------------------------------------ direction pdfs

enum LobeKind { L_COSINE, L_GGX, L_GLASS, L_HG };

struct Lobe {
    int kind = L_COSINE;
    Onb frame;
    V wo;        // GGX: local wo
    Ggx d{1};
    RoughGlass glass;
    double g = 0;  // HG
    // pdf.h:40-43, microfacet.h:220-228, :477, pdf.h:61-63
    double value(const V& dir) const {
        switch (kind) {
            case L_COSINE: return std::fmax(0.0, dot(unit(dir), frame.a[2]) / PI);
            case L_GGX: {
                if (dir.len2() == 0)
                    return 0;
                V wi = unit(frame.to_local(dir));
                if (wi.z <= 0 || wo.z <= 0)
                    return 0;
                V h = unit(wo + wi);
                return d.visible_pdf(wo, h) / (4 * std::fabs(dot(wo, h)));
            }
            case L_GLASS: return glass.pdf(dir);
            case L_HG: {
                double c = dot(unit(dir), frame.a[2]);
                double den = 1 + g * g - 2 * g * c;
                return (1 - g * g) / (4 * PI * den * std::sqrt(den));
            }
        }
        return 0;
    }
    V generate(Rng& rng) const {
        switch (kind) {
            case L_COSINE: return frame.to_world(random_cosine_direction(rng));
            case L_GGX: {
                if (wo.z <= 0)
                    return V();
                V h = d.sample_visible(wo, rng.next(), rng.next());
                V wi = -wo + 2 * dot(wo, h) * h;
                if (wi.z <= 0)
                    return V();
                return frame.to_world(wi);
            }
            case L_GLASS: return glass.sample(rng);
            case L_HG: {  // pdf.h:66-79
                double xi = rng.next(), ct;
                if (std::fabs(g) < 1e-3) {
                    ct = 1 - 2 * xi;
                } else {
                    double s = (1 - g * g) / (1 - g + 2 * g * xi);
                    ct = (1 + g * g - s * s) / (2 * g);
                }
                ct = std::clamp(ct, -1.0, 1.0);
                double st = std::sqrt(1 - ct * ct), phi = 2 * PI * rng.next();
                return frame.to_world(V(std::cos(phi) * st, std::sin(phi) * st, ct));
            }
        }
        return V();
    }
};

Lobe cosine_lobe(const V& n) {
    Lobe l;
    l.kind = L_COSINE;
    l.frame = Onb(n);
    return l;
}
Lobe ggx_lobe(const V& n, const V& wo_world, double alpha) {
    Lobe l;
    l.kind = L_GGX;
    l.frame = Onb(n);
    l.wo = unit(l.frame.to_local(wo_world));
    l.d = Ggx{alpha};
    return l;
}

// A mixture of up to three lobes (mixture_pdf, pdf.h:111-134, nested).
struct Pdf {
    int n = 0;
    Lobe lobe[3];
    double prob[3] = {0, 0, 0};
    double value(const V& dir) const {
        double s = 0;
        for (int k = 0; k < n; k++)
            if (prob[k] > 0)
                s += prob[k] * lobe[k].value(dir);
        return s;
    }
    V generate(Rng& g) const {
        double xi = g.next(), acc = 0;
        for (int k = 0; k < n - 1; k++) {
            acc += prob[k];
            if (xi < acc)
                return lobe[k].generate(g);
        }
        return lobe[n - 1].generate(g);
    }
};

// --------------------------------------------------------------- materials

struct Scatter {
    V attenuation;
    bool skip_pdf = false;
    V skip_dir;
    Pdf pdf;
};

const mypbr_material& M(const Scene& S, int m) { return S.f->materials[m]; }

// normal_from_map (material.h:282-308)
V normal_from_map(const Scene& S, const V& r_dir, const Hit& rec, int map) {
    const double min_cos_o = 0.01;
    V n = rec.front ? rec.normal : -rec.normal;
    V t = rec.dpdu - dot(rec.dpdu, n) * n;
    if (t.len2() <= 1e-12 * rec.dpdu.len2())
        return rec.normal;
    t = unit(t);
    V b = cross(n, t);
    if (dot(b, rec.dpdv) < 0)
        b = -b;
    V c = tex_value(S, map, rec.u, rec.v, rec.p);
    double nz = std::fmax(2 * c.z - 1, 1e-3);
    V m = unit((2 * c.x - 1) * t + (2 * c.y - 1) * b + nz * n);
    if (!rec.front)
        m = -m;
    V wo = unit(-r_dir);
    double co = dot(m, wo);
    if (co < min_cos_o)
        m = unit(m + (min_cos_o - co) * wo);
    return m;
}

struct Principled {
    const Scene& S;
    const mypbr_material& m;
    const Hit& rec;
    double metallic() const { return std::clamp(tex_value(S, m.tex[1], rec.u, rec.v, rec.p).x, 0.0, 1.0); }
    double alpha() const {
        return rough_to_alpha(std::clamp(tex_value(S, m.tex[2], rec.u, rec.v, rec.p).x, 0.0, 1.0));
    }
    double coat() const {
        if (!(m.flags & MYPBR_MATF_COAT))
            return 0;
        return std::clamp(tex_value(S, m.tex[4], rec.u, rec.v, rec.p).x, 0.0, 1.0);
    }
    double coat_alpha() const {
        return rough_to_alpha(std::clamp(tex_value(S, m.tex[5], rec.u, rec.v, rec.p).x, 0.0, 1.0));
    }
    V base() const { return tex_value(S, m.tex[0], rec.u, rec.v, rec.p); }
    bool measured() const { return m.flags & MYPBR_MATF_MEASURED; }
    V conductor_at(double c) const {
        return {fresnel_conductor(c, m.p[4], m.p[7]), fresnel_conductor(c, m.p[5], m.p[8]),
                fresnel_conductor(c, m.p[6], m.p[9])};
    }
    V spec_f0(const V& b, double mt) const {
        double f0 = m.p[0];
        return (1 - mt) * V(f0, f0, f0) + mt * b;
    }
    // material.h:536-549
    V spec_fresnel(double c, const V& b, double mt) const {
        if (!measured())
            return schlick3(c, spec_f0(b, mt));
        double fd = schlick(c, m.p[0]);
        return (1 - mt) * V(fd, fd, fd) + mt * conductor_at(c);
    }
    V ms_fres(const V& b, double mt, double alpha) const {
        if (!measured())
            return ms_fresnel(S, spec_f0(b, mt), alpha);
        double fd = m.p[0] + (1 - m.p[0]) / 21;
        return ms_fresnel_avg(S, (1 - mt) * V(fd, fd, fd) + mt * V(m.p[10], m.p[11], m.p[12]), alpha);
    }
    V coat_trans(double w, double co, double ci) const {  // material.h:471-482
        if (!(m.flags & MYPBR_MATF_COAT_TINT))
            return V(1, 1, 1);
        auto ct = [](double c) {
            c = std::clamp(c, 0.0, 1.0);
            return std::sqrt(1 - (1 - c * c) / (1.5 * 1.5));
        };
        double e = (1 / ct(co) + 1 / ct(ci)) / 2;
        V t(std::pow(m.p[13], e), std::pow(m.p[14], e), std::pow(m.p[15], e));
        return (1 - w) * V(1, 1, 1) + w * t;
    }
    // material.h:486-506
    V base_eval(const V& n, const V& wow, const V& wiw) const {
        Onb fr(n);
        V wo = unit(fr.to_local(wow)), wi = unit(fr.to_local(wiw));
        if (wo.z <= 0 || wi.z <= 0)
            return V();
        double mt = metallic(), a = alpha();
        V b = base();
        V h = unit(wo + wi);
        Ggx d{a};
        V spec = spec_fresnel(dot(wi, h), b, mt) * (d.D(h) * d.G(wo, wi) / (4 * wo.z)) +
                 ms_fres(b, mt, a) * ms_eval(S, wo.z, wi.z, a);
        double tr = (1 - schlick(wi.z, m.p[0])) * (1 - schlick(wo.z, m.p[0]));
        V diff = ((1 - mt) * tr * wi.z / PI) * b;
        return spec + diff;
    }
};

V coat_normal(const Scene& S, const mypbr_material& m, const V& r_dir, const Hit& rec) {
    return m.tex[6] >= 0 ? normal_from_map(S, r_dir, rec, m.tex[6]) : rec.normal;
}

// The metal's Fresnel curve (microfacet.h:125-131)
V metal_fresnel_at(const mypbr_material& m, double c) {
    if (!(m.flags & MYPBR_MATF_MEASURED))
        return schlick3(c, V(m.p[0], m.p[1], m.p[2]));
    return {fresnel_conductor(c, m.p[4], m.p[7]), fresnel_conductor(c, m.p[5], m.p[8]),
            fresnel_conductor(c, m.p[6], m.p[9])};
}

bool scatter_inner(const Scene& S, int mi, const V& r_dir, const Hit& rec, Scatter& sr, Rng& g);
V eval_inner(const Scene& S, int mi, const V& r_dir, const Hit& rec, const V& dir);

// The wrappers: normal_mapped (material.h:631-674); emissive_surface only adds emission.
bool scatter(const Scene& S, int mi, const V& r_dir, const Hit& rec, Scatter& sr, Rng& g) {
    const auto& m = M(S, mi);
    if (m.normal_map < 0 || m.type == MYPBR_MAT_PRINCIPLED)
        return scatter_inner(S, mi, r_dir, rec, sr, g);
    Hit sh = rec;
    sh.normal = normal_from_map(S, r_dir, rec, m.normal_map);
    if (!scatter_inner(S, mi, r_dir, sh, sr, g))
        return false;
    if (sr.skip_pdf) {
        V d = sr.skip_dir;
        if (dot(d, sh.normal) > 0 && dot(d, rec.normal) < 0)
            sr.skip_dir = d - 2 * dot(d, rec.normal) * rec.normal;
    }
    return true;
}

V eval(const Scene& S, int mi, const V& r_dir, const Hit& rec, const V& dir) {
    const auto& m = M(S, mi);
    if (m.normal_map < 0 || m.type == MYPBR_MAT_PRINCIPLED)
        return eval_inner(S, mi, r_dir, rec, dir);
    if (dot(dir, rec.normal) <= 0)
        return V();
    Hit sh = rec;
    sh.normal = normal_from_map(S, r_dir, rec, m.normal_map);
    return eval_inner(S, mi, r_dir, sh, dir);
}

bool scatter_inner(const Scene& S, int mi, const V& r_dir, const Hit& rec, Scatter& sr, Rng& g) {
    const auto& m = M(S, mi);
    sr.skip_pdf = false;
    sr.pdf.n = 0;
    switch (m.type) {
        case MYPBR_MAT_LAMBERTIAN:  // material.h:79-85
            sr.attenuation = tex_value(S, m.tex[0], rec.u, rec.v, rec.p);
            sr.pdf.n = 1;
            sr.pdf.lobe[0] = cosine_lobe(rec.normal);
            sr.pdf.prob[0] = 1;
            return true;
        case MYPBR_MAT_METAL: {  // material.h:123-150
            double roughness = m.p[3], alpha = rough_to_alpha(roughness);
            V albedo(m.p[0], m.p[1], m.p[2]);
            if (roughness == 0) {
                sr.attenuation = (m.flags & MYPBR_MATF_MEASURED)
                                     ? metal_fresnel_at(m, dot(rec.normal, unit(-r_dir)))
                                     : albedo;
                sr.skip_pdf = true;
                sr.skip_dir = reflect(unit(r_dir), rec.normal);
                return true;
            }
            sr.attenuation = albedo;
            Lobe spec = ggx_lobe(rec.normal, -r_dir, alpha);
            double co = std::fmax(0.0, dot(rec.normal, unit(-r_dir)));
            double msw = ms_albedo(S, co, alpha) * avg3(ms_fresnel_avg(S, V(m.p[10], m.p[11], m.p[12]), alpha));
            double ssw = table_E(S, co, alpha) * avg3(metal_fresnel_at(m, co));
            if (msw <= 0) {
                sr.pdf.n = 1;
                sr.pdf.lobe[0] = spec;
                sr.pdf.prob[0] = 1;
                return true;
            }
            double ps = std::clamp(ssw / (ssw + msw), 0.1, 1.0);
            sr.pdf.n = 2;
            sr.pdf.lobe[0] = spec;
            sr.pdf.lobe[1] = cosine_lobe(rec.normal);
            sr.pdf.prob[0] = ps;
            sr.pdf.prob[1] = 1 - ps;
            return true;
        }
        case MYPBR_MAT_DIELECTRIC: {  // material.h:210-242
            double ior = m.p[0], roughness = m.p[1];
            sr.attenuation = V(1, 1, 1);
            if (roughness > 0) {
                Lobe l;
                l.kind = L_GLASS;
                l.glass.frame = Onb(rec.normal);
                l.glass.wo = unit(l.glass.frame.to_local(-r_dir));
                l.glass.eta = rec.front ? ior : 1.0 / ior;
                l.glass.d = Ggx{rough_to_alpha(roughness)};
                sr.pdf.n = 1;
                sr.pdf.lobe[0] = l;
                sr.pdf.prob[0] = 1;
                return true;
            }
            sr.skip_pdf = true;
            double ri = rec.front ? 1.0 / ior : ior;
            V ud = unit(r_dir);
            double ct = std::fmin(dot(-ud, rec.normal), 1.0), st = std::sqrt(1.0 - ct * ct);
            bool cannot = ri * st > 1.0;
            if (cannot || fresnel_dielectric(ct, 1.0 / ri) > g.next())
                sr.skip_dir = reflect(ud, rec.normal);
            else
                sr.skip_dir = refract(ud, rec.normal, ri);
            return true;
        }
        case MYPBR_MAT_THIN_DIELECTRIC: {  // material.h:687-702
            V ud = unit(r_dir);
            double ct = std::fmin(dot(-ud, rec.normal), 1.0);
            double r = fresnel_dielectric(ct, m.p[0]);
            double refl = 2 * r / (1 + r);
            sr.skip_pdf = true;
            if (g.next() < refl) {
                sr.attenuation = V(1, 1, 1);
                sr.skip_dir = reflect(ud, rec.normal);
            } else {
                sr.attenuation = V(m.p[2], m.p[3], m.p[4]);
                sr.skip_dir = ud;
            }
            return true;
        }
        case MYPBR_MAT_PRINCIPLED: {  // material.h:387-421
            Principled P{S, m, rec};
            V wo = unit(-r_dir);
            V nb = m.tex[3] >= 0 ? normal_from_map(S, r_dir, rec, m.tex[3]) : rec.normal;
            double mt = P.metallic(), a = P.alpha();
            V b = P.base();
            double co = std::fmax(0.0, dot(nb, wo));
            double sw = avg3(P.spec_fresnel(co, b, mt));
            double dw = (1 - mt) * avg3(b) * (1 - schlick(co, m.p[0]));
            dw += ms_albedo(S, co, a) * avg3(P.ms_fres(b, mt, a));
            double ps = sw + dw > 0 ? sw / (sw + dw) : 1;
            ps = std::clamp(ps, 0.1, 1.0);
            sr.attenuation = b;
            double w = P.coat();
            if (w > 0) {
                V nc = coat_normal(S, m, r_dir, rec);
                double cw = w * schlick(dot(nc, wo), 0.04);
                double below = (1 - cw) * (sw + dw) * avg3(P.coat_trans(w, 1, 1));
                double pc = std::clamp(cw / (cw + below), 0.1, 0.9);
                sr.pdf.n = 3;
                sr.pdf.lobe[0] = ggx_lobe(nc, wo, P.coat_alpha());
                sr.pdf.lobe[1] = ggx_lobe(nb, wo, a);
                sr.pdf.lobe[2] = cosine_lobe(nb);
                sr.pdf.prob[0] = pc;
                sr.pdf.prob[1] = (1 - pc) * ps;
                sr.pdf.prob[2] = (1 - pc) * (1 - ps);
            } else {
                sr.pdf.n = 2;
                sr.pdf.lobe[0] = ggx_lobe(nb, wo, a);
                sr.pdf.lobe[1] = cosine_lobe(nb);
                sr.pdf.prob[0] = ps;
                sr.pdf.prob[1] = 1 - ps;
            }
            return true;
        }
        case MYPBR_MAT_PHASE: {  // medium.h:254-260
            sr.attenuation = V(m.p[0], m.p[1], m.p[2]);
            Lobe l;
            l.kind = L_HG;
            l.frame = Onb(r_dir);
            l.g = m.p[3];
            sr.pdf.n = 1;
            sr.pdf.lobe[0] = l;
            sr.pdf.prob[0] = 1;
            return true;
        }
        default: return false;  // diffuse_light scatters nothing
    }
}

V eval_inner(const Scene& S, int mi, const V& r_dir, const Hit& rec, const V& dir) {
    const auto& m = M(S, mi);
    switch (m.type) {
        case MYPBR_MAT_LAMBERTIAN: {  // material.h:88-97
            double c = dot(rec.normal, unit(dir));
            return tex_value(S, m.tex[0], rec.u, rec.v, rec.p) * (c < 0 ? 0 : c / PI);
        }
        case MYPBR_MAT_METAL: {  // material.h:154-164
            double alpha = rough_to_alpha(m.p[3]);
            Onb fr(rec.normal);
            V wo = unit(fr.to_local(-r_dir)), wi = unit(fr.to_local(dir));
            if (wo.z <= 0 || wi.z <= 0)
                return V();
            V h = unit(wo + wi);
            Ggx d{alpha};
            return metal_fresnel_at(m, dot(wi, h)) * (d.D(h) * d.G(wo, wi) / (4 * wo.z)) +
                   ms_fresnel_avg(S, V(m.p[10], m.p[11], m.p[12]), alpha) * ms_eval(S, wo.z, wi.z, alpha);
        }
        case MYPBR_MAT_DIELECTRIC: {  // material.h:244-249
            if (m.p[1] == 0)
                return V();
            RoughGlass rg;
            rg.frame = Onb(rec.normal);
            rg.wo = unit(rg.frame.to_local(-r_dir));
            rg.eta = rec.front ? m.p[0] : 1.0 / m.p[0];
            rg.d = Ggx{rough_to_alpha(m.p[1])};
            double f = rg.eval(dir);
            return V(f, f, f);
        }
        case MYPBR_MAT_PRINCIPLED: {  // material.h:423-453
            if (dot(dir, rec.normal) <= 0)
                return V();
            Principled P{S, m, rec};
            V wo = unit(-r_dir), wi = unit(dir);
            V nb = m.tex[3] >= 0 ? normal_from_map(S, r_dir, rec, m.tex[3]) : rec.normal;
            V below = P.base_eval(nb, wo, wi);
            double w = P.coat();
            if (w <= 0)
                return below;
            V nc = coat_normal(S, m, r_dir, rec);
            double co = dot(nc, wo), ci = dot(nc, wi);
            double through = (1 - w * schlick(co, 0.04)) * (1 - w * schlick(ci, 0.04));
            V result = through * P.coat_trans(w, co, ci) * below;
            if (co > 0 && ci > 0) {
                Onb fr(nc);
                V lo = unit(fr.to_local(wo)), li = unit(fr.to_local(wi));
                V h = unit(lo + li);
                double a = P.coat_alpha();
                Ggx d{a};
                double c = schlick(dot(li, h), 0.04) * d.D(h) * d.G(lo, li) / (4 * lo.z);
                c += (ms_fresnel(S, V(0.04, 0.04, 0.04), a) * ms_eval(S, lo.z, li.z, a)).x;
                result += V(w * c, w * c, w * c);
            }
            return result;
        }
        case MYPBR_MAT_PHASE: {  // medium.h:265-269
            double c = dot(unit(r_dir), unit(dir)), gg = m.p[3];
            double den = 1 + gg * gg - 2 * gg * c;
            double ph = (1 - gg * gg) / (4 * PI * den * std::sqrt(den));
            return V(m.p[0], m.p[1], m.p[2]) * ph;
        }
        default: return V();
    }
}

// material.h:578-598 and :731-736
V emitted(const Scene& S, int mi, const V& r_dir, const Hit& rec) {
    const auto& m = M(S, mi);
    if (m.emission_tex >= 0)
        return rec.front ? tex_value(S, m.emission_tex, rec.u, rec.v, rec.p) : V();
    if (m.type != MYPBR_MAT_DIFFUSE_LIGHT || !rec.front)
        return V();
    V e(m.p[0], m.p[1], m.p[2]);
    if (m.p[3] >= 180)
        return e;
    double c = -dot(unit(r_dir), rec.normal);
    if (c <= 0)
        return V();
    double tt = std::sqrt(std::fmax(0.0, 1 - c * c)) / c;
    return e * std::fmax(0.0, 1 - tt / m.p[4]);
}

// material.h:201-206
V interior_transmittance(const Scene& S, int mi, const V& r_dir, const Hit& rec) {
    const auto& m = M(S, mi);
    if (m.type != MYPBR_MAT_DIELECTRIC || rec.front || (m.p[2] == 0 && m.p[3] == 0 && m.p[4] == 0))
        return V(1, 1, 1);
    double d = rec.t * r_dir.len();
    return {std::exp(-m.p[2] * d), std::exp(-m.p[3] * d), std::exp(-m.p[4] * d)};
}
bool lets_shadows_through(const Scene& S, int mi) {
    const auto& m = M(S, mi);
    return m.type == MYPBR_MAT_DIELECTRIC && m.p[1] == 0;
}
bool is_volume(const Scene& S, int mi) { return M(S, mi).type == MYPBR_MAT_PHASE; }

// ------------------------------------------------------------------ lights

// environment.h:334-348
void env_angles(const Scene& S, const V& dir, double& u, double& theta) {
    V d = unit(dir);
    theta = std::acos(std::clamp(d.y, -1.0, 1.0));
    u = 0.5 + std::atan2(d.x, -d.z) / (2 * PI) + S.f->environment.rotation;
    u -= std::floor(u);
}

// environment.h:202-215
V env_radiance(const Scene& S, const V& dir) {
    const auto& E = S.f->environment;
    double u, theta;
    env_angles(S, dir, u, theta);
    int w = E.width, h = E.height;
    double x = u * w - 0.5;
    double y = std::clamp(theta / PI * h - 0.5, 0.0, h - 1.0);
    double x0 = std::floor(x), y0 = std::floor(y), fx = x - x0, fy = y - y0;
    int i0 = (int(x0) + w) % w, i1 = (i0 + 1) % w;
    int j0 = int(y0), j1 = std::min(j0 + 1, h - 1);
    auto at = [&](int i, int j) {
        const float* p = E.pixels + (int64_t(j) * w + i) * 3;
        return V(p[0], p[1], p[2]);
    };
    V top = (1 - fx) * at(i0, j0) + fx * at(i1, j0);
    V bot = (1 - fx) * at(i0, j1) + fx * at(i1, j1);
    return E.intensity * ((1 - fy) * top + fy * bot);
}

// environment.h:283-312
void build_env(Scene& S) {
    const auto& E = S.f->environment;
    auto& D = S.env;
    D.w = E.width;
    D.h = E.height;
    if (D.w <= 0)
        return;
    int w = D.w, h = D.h;
    D.cond.assign(size_t(h) * (w + 1), 0.0);
    D.marg.assign(h + 1, 0.0);
    D.roww.assign(h, 0.0);
    for (int j = 0; j < h; j++) {
        double* c = &D.cond[size_t(j) * (w + 1)];
        double st = std::sin(PI * (j + 0.5) / h);
        for (int i = 0; i < w; i++) {
            const float* p = E.pixels + (int64_t(j) * w + i) * 3;
            c[i + 1] = c[i] + std::fmax(lum(V(p[0], p[1], p[2])) * st, 0.0);
        }
        D.roww[j] = c[w];
        for (int i = 1; i <= w; i++)
            c[i] = D.roww[j] > 0 ? c[i] / D.roww[j] : double(i) / w;
        D.marg[j + 1] = D.marg[j] + D.roww[j];
    }
    D.total = D.marg[h];
    if (D.total <= 0) {
        for (int j = 0; j < h; j++) {
            D.roww[j] = std::sin(PI * (j + 0.5) / h);
            D.marg[j + 1] = D.marg[j] + D.roww[j];
        }
        D.total = D.marg[h];
    }
    for (int j = 1; j <= h; j++)
        D.marg[j] /= D.total;
}

// environment.h:316-322
double sample_cdf(const double* cdf, int n, double xi) {
    int k = int(std::upper_bound(cdf, cdf + n + 1, xi) - cdf) - 1;
    k = std::clamp(k, 0, n - 1);
    double span = cdf[k + 1] - cdf[k];
    double fr = span > 0 ? (xi - cdf[k]) / span : 0.5;
    return k + std::clamp(fr, 0.0, 1.0 - 1e-9);
}

// environment.h:220-228, :326-331
double env_pdf(const Scene& S, const V& dir) {
    const auto& D = S.env;
    double u, theta;
    env_angles(S, dir, u, theta);
    double st = std::sin(theta);
    int i = std::clamp(int(u * D.w), 0, D.w - 1), j = std::clamp(int(theta / PI * D.h), 0, D.h - 1);
    if (st <= 0)
        return 0;
    double row = D.roww[j] / D.total;
    const double* c = &D.cond[size_t(j) * (D.w + 1)];
    return row * (c[i + 1] - c[i]) * D.w * D.h / (2 * PI * PI * st);
}

// environment.h:230-243
V env_random(const Scene& S, Rng& g) {
    const auto& D = S.env;
    double y = sample_cdf(D.marg.data(), D.h, g.next());
    int j = std::min(int(y), D.h - 1);
    double x = sample_cdf(&D.cond[size_t(j) * (D.w + 1)], D.w, g.next());
    double theta = PI * y / D.h, phi = 2 * PI * (x / D.w - 0.5 - S.f->environment.rotation);
    double st = std::sin(theta);
    return {st * std::sin(phi), std::cos(theta), -st * std::cos(phi)};
}

// sun.h:397-413
bool sun_in_cone(const Scene& S, const V& dir) { return dot(unit(dir), S.sun_frame.a[2]) >= S.sun_cos_max; }

// Density of one light member, as its own pdf_value (sphere.h:56-73,
// quad.h:65-74, mesh.h:115-124; instance.h:47-49 for a moved sphere).
double member_pdf(const Scene& S, const mypbr_light_member& mb, const V& o, const V& d) {
    Hit rec;
    switch (mb.prim_kind) {
        case MYPBR_PRIM_SPHERE: {
            const auto& s = S.f->spheres[mb.prim_index];
            V lo = o, ld = d;
            if (s.xform >= 0) {
                lo = S.xf[s.xform].ipoint(o);
                ld = S.xf[s.xform].ivec(d);
            }
            V c(s.center);
            if (!hit_sphere_local(c, s.radius, lo, ld, 0.001, INF, rec))
                return 0;
            double r = std::fabs(s.radius);
            double d2 = (c - lo).len2();
            if (d2 <= r * r) {
                double hd2 = rec.t * rec.t * ld.len2();
                double cosine = std::fabs(dot(unit(ld), (rec.p - c) / r));
                return hd2 / (cosine * 4 * PI * r * r);
            }
            double ctm = std::sqrt(1 - r * r / d2);
            return 1 / (2 * PI * (1 - ctm));
        }
        case MYPBR_PRIM_QUAD: {
            if (!hit_quad(S, mb.prim_index, o, d, 0.001, INF, rec))
                return 0;
            const auto& q = S.f->quads[mb.prim_index];
            double area = cross(V(q.u), V(q.v)).len();
            double d2 = rec.t * rec.t * d.len2();
            double cosine = std::fabs(dot(d, rec.normal) / d.len());
            return d2 / (cosine * area);
        }
        case MYPBR_PRIM_TRIANGLE: {
            if (!hit_triangle(S, mb.prim_index, o, d, 0.001, INF, rec, nullptr, false))
                return 0;
            const auto& tr = S.f->triangles[mb.prim_index];
            V p0 = pos(S, tr.v[0]);
            V c = cross(pos(S, tr.v[1]) - p0, pos(S, tr.v[2]) - p0);
            double area = 0.5 * c.len();
            V gn = unit(c);
            double d2 = rec.t * rec.t * d.len2();
            double cosine = std::fabs(dot(d, gn) / d.len());
            return d2 / (cosine * area);
        }
    }
    return 0;
}

// A direction towards a random point of one member (sphere.h:75-88,
// quad.h:76-79, mesh.h:127-136).
V member_random(const Scene& S, const mypbr_light_member& mb, const V& o, Rng& g) {
    switch (mb.prim_kind) {
        case MYPBR_PRIM_SPHERE: {
            const auto& s = S.f->spheres[mb.prim_index];
            const Xform* x = s.xform >= 0 ? &S.xf[s.xform] : nullptr;
            V lo = x ? x->ipoint(o) : o;
            V c(s.center);
            double r = std::fabs(s.radius);
            V dir = c - lo;
            double d2 = dir.len2();
            V out;
            if (d2 <= r * r) {
                out = c + r * random_unit_vector(g) - lo;
            } else {
                Onb uvw(dir);
                double r1 = g.next(), r2 = g.next();
                double z = 1 + r2 * (std::sqrt(1 - r * r / d2) - 1);
                double phi = 2 * PI * r1;
                out = uvw.to_world(V(std::cos(phi) * std::sqrt(1 - z * z), std::sin(phi) * std::sqrt(1 - z * z), z));
            }
            return x ? x->vec(out) : out;
        }
        case MYPBR_PRIM_QUAD: {
            const auto& q = S.f->quads[mb.prim_index];
            double a = g.next(), b = g.next();
            return V(q.q) + a * V(q.u) + b * V(q.v) - o;
        }
        case MYPBR_PRIM_TRIANGLE: {
            const auto& tr = S.f->triangles[mb.prim_index];
            double r1 = g.next(), r2 = g.next();
            if (r1 + r2 > 1) {
                r1 = 1 - r1;
                r2 = 1 - r2;
            }
            V p0 = pos(S, tr.v[0]);
            return p0 + r1 * (pos(S, tr.v[1]) - p0) + r2 * (pos(S, tr.v[2]) - p0) - o;
        }
    }
    return V(1, 0, 0);
}

double light_pdf_one(const Scene& S, int k, const V& o, const V& d) {
    const auto& L = S.f->lights[k];
    switch (L.kind) {
        case MYPBR_LIGHT_ENVIRONMENT: return S.env.w > 0 ? env_pdf(S, d) : 0;
        case MYPBR_LIGHT_SUN: return sun_in_cone(S, d) ? 1 / S.sun_solid_angle : 0;
        default: {
            double s = 0;
            for (int m = 0; m < L.member_count; m++) {
                const auto& mb = S.f->light_members[L.first_member + m];
                s += mb.weight * member_pdf(S, mb, o, d);
            }
            return s;
        }
    }
}

// light_list.h:106-113
double lights_pdf(const Scene& S, const V& o, const V& d) {
    double s = 0;
    for (int64_t k = 0; k < S.f->light_count; k++)
        s += S.f->lights[k].probability * light_pdf_one(S, int(k), o, d);
    return s;
}

// light_list.h:115-127
V lights_random(const Scene& S, const V& o, Rng& g) {
    int n = int(S.f->light_count);
    double xi = g.next();
    int k = int(std::upper_bound(S.light_cdf.begin(), S.light_cdf.end(), xi) - S.light_cdf.begin());
    k = std::clamp(k, 1, n) - 1;
    const auto& L = S.f->lights[k];
    switch (L.kind) {
        case MYPBR_LIGHT_ENVIRONMENT: return env_random(S, g);
        case MYPBR_LIGHT_SUN: {
            double ct = 1 - g.next() * (1 - S.sun_cos_max);
            double st = std::sqrt(std::fmax(0.0, 1 - ct * ct)), phi = 2 * PI * g.next();
            return S.sun_frame.to_world(V(std::cos(phi) * st, std::sin(phi) * st, ct));
        }
        default: {
            const auto& cdf = S.member_cdf[k];
            double x = g.next();
            int m = int(std::upper_bound(cdf.begin(), cdf.end(), x) - cdf.begin());
            m = std::clamp(m, 0, L.member_count - 1);
            return member_random(S, S.f->light_members[L.first_member + m], o, g);
        }
    }
}

// --------------------------------------------------------------- camera

struct Camera {
    int w, h, sqrt_spp;
    double recip_sqrt_spp;
    V center, p00, du, dv, u, v, wv, disk_u, disk_v;
    const mypbr_camera* c;
    // camera.h:142-179
    void init(const mypbr_camera& cam, int spp) {
        c = &cam;
        w = cam.image_width;
        h = cam.image_height;
        sqrt_spp = int(std::sqrt(double(spp)));
        recip_sqrt_spp = 1.0 / sqrt_spp;
        center = V(cam.lookfrom);
        double theta = cam.vfov * PI / 180.0;
        double hh = std::tan(theta / 2);
        double vh = cam.ortho_height > 0 ? cam.ortho_height : 2 * hh * cam.focus_dist;
        double vw = vh * (double(w) / h);
        wv = unit(V(cam.lookfrom) - V(cam.lookat));
        u = unit(cross(V(cam.vup), wv));
        v = cross(wv, u);
        V vu = vw * u, vv = vh * -v;
        du = vu / w;
        dv = vv / h;
        V ul = center - (cam.focus_dist * wv) - vu / 2 - vv / 2;
        p00 = ul + 0.5 * (du + dv);
        double dr = cam.focus_dist * std::tan(cam.defocus_angle / 2 * PI / 180.0);
        disk_u = u * dr;
        disk_v = v * dr;
    }
    // camera.h:291-339
    void get_ray(int i, int j, int pass, Rng& g, V& o, V& d) const {
        int strata = sqrt_spp * sqrt_spp;
        double ox, oy;
        if (pass >= strata) {
            ox = g.next() - 0.5;
            oy = g.next() - 0.5;
        } else {
            int cell = int((int64_t(pass) + int64_t(i) * 7919 + int64_t(j) * 104729) % strata);
            ox = ((cell % sqrt_spp + g.next()) * recip_sqrt_spp) - 0.5;
            oy = ((cell / sqrt_spp + g.next()) * recip_sqrt_spp) - 0.5;
        }
        V ps = p00 + ((i + ox) * du) + ((j + oy) * dv);
        V eye = c->ortho_height > 0 ? ps + c->focus_dist * wv : center;
        if (c->defocus_angle <= 0) {
            o = eye;
        } else {
            V p;
            if (c->blades >= 3) {
                int k = std::min(int(g.next() * c->blades), c->blades - 1);
                double a0 = c->blade_rotation * PI / 180.0 + 2 * PI * k / c->blades;
                double a1 = a0 + 2 * PI / c->blades;
                double s = g.next(), t = g.next();
                if (s + t > 1) {
                    s = 1 - s;
                    t = 1 - t;
                }
                p = s * V(std::cos(a0), std::sin(a0), 0) + t * V(std::cos(a1), std::sin(a1), 0);
            } else {
                p = random_in_unit_disk(g);
            }
            o = eye + (p.x * disk_u) + (p.y * disk_v);
        }
        d = ps - o;
    }
};

// ------------------------------------------------------------- integrator

struct Integrator {
    const Scene& S;
    const mypbr_render_opts& o;
    bool has_lights;

    // camera.h:515-529
    V escaped(const V& dir, bool camera_ray) const {
        V sky;
        const auto& F = *S.f;
        if (F.environment.width > 0) {
            sky = env_radiance(S, dir);
        } else if (!F.use_sky) {
            sky = V(F.background);
        } else {
            V ud = unit(dir);
            double a = 0.5 * (ud.y + 1.0);
            sky = (1.0 - a) * V(1, 1, 1) + a * V(0.5, 0.7, 1.0);
        }
        if (F.sun.enabled && (F.sun.disk_visible || !camera_ray) && sun_in_cone(S, dir))
            sky += S.sun_radiance;
        return sky;
    }

    static double power_heuristic(double a, double b) {
        double a2 = a * a, b2 = b * b;
        return (a2 + b2) > 0 ? a2 / (a2 + b2) : 0;
    }

    // camera.h:466-506
    V sample_light(const V& r_dir, const Hit& rec, const Pdf& bsdf, bool last, Rng& g, uint64_t& shadow_rays) const {
        V to_light = lights_random(S, rec.p, g);
        double lp = lights_pdf(S, rec.p, to_light);
        if (lp <= 0)
            return V();
        V f = eval(S, rec.mat, r_dir, rec, to_light);
        if (f.x <= 0 && f.y <= 0 && f.z <= 0)
            return V();
        V so = rec.p, sd = unit(to_light);
        V emission, through(1, 1, 1);
        Hit lr;
        for (int k = 0;; k++) {
            shadow_rays++;
            if (!world_hit(S, so, sd, 0.001, INF, lr, &g)) {
                emission = escaped(to_light, false);
                break;
            }
            if (o.transparent_shadows && k < 16 && lets_shadows_through(S, lr.mat)) {
                through = through * interior_transmittance(S, lr.mat, sd, lr);
                so = lr.p;
                continue;
            }
            emission = emitted(S, lr.mat, sd, lr);
            break;
        }
        emission = through * emission;
        double wgt = last ? 1.0 : power_heuristic(lp, bsdf.value(to_light));
        return f * emission * (wgt / lp);
    }

    // camera.h:356-461
    V ray_color(V ro, V rd, Rng& g, uint64_t& ext, uint64_t& shadow) const {
        V radiance, beta(1, 1, 1);
        bool specular = true, seen = false;
        double scatter_pdf = 0;
        V prev;
        int dc = 0, sc = 0, vc = 0;
        for (int depth = 0; depth < o.max_depth; depth++) {
            Hit rec;
            ext++;
            if (!world_hit(S, ro, rd, 0.001, INF, rec, &g)) {
                V sky = escaped(rd, depth == 0);
                if (seen)
                    break;
                if (specular || !has_lights)
                    radiance += beta * sky;
                else
                    radiance += beta * sky * power_heuristic(scatter_pdf, lights_pdf(S, prev, rd));
                break;
            }
            beta = beta * interior_transmittance(S, rec.mat, rd, rec);
            V em = emitted(S, rec.mat, rd, rec);
            if (!seen && (em.x > 0 || em.y > 0 || em.z > 0)) {
                if (specular || !has_lights)
                    radiance += beta * em;
                else
                    radiance += beta * em * power_heuristic(scatter_pdf, lights_pdf(S, prev, rd));
            }
            Scatter sr;
            if (!scatter(S, rec.mat, rd, rec, sr, g))
                break;
            if (sr.skip_pdf) {
                if (o.max_specular > 0 && ++sc > o.max_specular)
                    break;
                beta = beta * sr.attenuation;
                V nd = sr.skip_dir;
                if (o.transparent_shadows && lets_shadows_through(S, rec.mat) && has_lights && depth > 0 && !specular)
                    seen = true;
                ro = rec.p;
                rd = nd;
                specular = true;
            } else {
                bool vol = is_volume(S, rec.mat);
                int& cnt = vol ? vc : dc;
                int cap = vol ? o.max_scatter : o.max_diffuse;
                bool capped = cap > 0 && ++cnt >= cap;
                bool last = depth == o.max_depth - 1 || capped;
                seen = false;
                if (has_lights)
                    radiance += beta * sample_light(rd, rec, sr.pdf, last, g, shadow);
                if (capped)
                    break;
                V dir = sr.pdf.generate(g);
                scatter_pdf = sr.pdf.value(dir);
                if (scatter_pdf <= 0)
                    break;
                beta = beta * eval(S, rec.mat, rd, rec, dir) / scatter_pdf;
                prev = rec.p;
                ro = rec.p;
                rd = dir;
                specular = false;
            }
            if (depth >= 3) {
                double survive = std::fmin(std::fmax(beta.x, std::fmax(beta.y, beta.z)), 0.95);
                if (g.next() >= survive)
                    break;
                beta = beta / survive;
            }
        }
        return radiance;
    }

    // camera.h:253-277
    void first_surface(V ro, V rd, Rng& g, V& albedo, V& normal) const {
        V tint(1, 1, 1);
        for (int b = 0; b < 8; b++) {
            Hit rec;
            if (!world_hit(S, ro, rd, 0.001, INF, rec, &g))
                break;
            tint = tint * interior_transmittance(S, rec.mat, rd, rec);
            Scatter sr;
            if (!scatter(S, rec.mat, rd, rec, sr, g)) {
                albedo = tint;
                normal = rec.normal;
                return;
            }
            if (!sr.skip_pdf) {
                albedo = tint * sr.attenuation;
                normal = rec.normal;
                return;
            }
            tint = tint * sr.attenuation;
            ro = rec.p;
            rd = sr.skip_dir;
        }
        albedo = tint;
        normal = V();
    }
};

void setup(Scene& S, const mypbr_flat_scene* f);

}  // namespace

// ------------------------------------------------------------- C interface

extern "C" {

// The Kulla-Conty tables, restated (microfacet.h:299-337): out = E[32][32], E_avg[32].
void oracle_ggx_table(double* out) {
    const int size = 32, strata = 64;
    for (int j = 0; j < size; j++) {
        double r = double(j) / (size - 1);
        Ggx d{rough_to_alpha(r)};
        for (int i = 0; i < size; i++) {
            double mu = std::fmax(double(i) / (size - 1), 1e-3);
            V wo(std::sqrt(1 - mu * mu), 0, mu);
            double sum = 0;
            for (int a = 0; a < strata; a++)
                for (int b = 0; b < strata; b++) {
                    V h = d.sample_visible(wo, (a + 0.5) / strata, (b + 0.5) / strata);
                    V wi = -wo + 2 * dot(wo, h) * h;
                    if (wi.z > 0)
                        sum += d.G(wo, wi) / d.G1(wo);
                }
            out[j * size + i] = std::fmin(sum / (strata * strata), 1.0);
        }
        double integral = 0, h = 1.0 / (size - 1);
        for (int i = 0; i + 1 < size; i++) {
            double a = i * h, b = (i + 1) * h;
            integral += h * (out[j * size + i] * (2 * a + b) + out[j * size + i + 1] * (a + 2 * b)) / 6;
        }
        out[size * size + j] = std::fmin(2 * integral, 1.0);
    }
}

typedef struct oracle_scene oracle_scene;

oracle_scene* oracle_scene_create(const mypbr_flat_scene* f) {
    auto* S = new Scene();
    setup(*S, f);
    return reinterpret_cast<oracle_scene*>(S);
}

void oracle_scene_destroy(oracle_scene* s) { delete reinterpret_cast<Scene*>(s); }

// Closest hits of n rays (n x 8: o, d, tmin, tmax) without media. hits: n x 8
// (t, normal xyz, u, v, front_face, material); prim: n x 2 (kind, index; -1 on miss).
void oracle_trace(const oracle_scene* s, const double* rays, int64_t n, double* hits, int32_t* prim,
                  int brute_force) {
    const Scene& S = *reinterpret_cast<const Scene*>(s);
    for (int64_t k = 0; k < n; k++) {
        const double* r = rays + 8 * k;
        Hit rec;
        double* h = hits + 8 * k;
        if (world_hit(S, V(r), V(r + 3), r[6], r[7], rec, nullptr, brute_force != 0)) {
            h[0] = rec.t;
            h[1] = rec.normal.x;
            h[2] = rec.normal.y;
            h[3] = rec.normal.z;
            h[4] = rec.u;
            h[5] = rec.v;
            h[6] = rec.front ? 1 : 0;
            h[7] = rec.mat;
            prim[2 * k] = rec.kind;
            prim[2 * k + 1] = rec.index;
        } else {
            for (int c = 0; c < 8; c++)
                h[c] = 0;
            h[7] = -1;
            prim[2 * k] = -1;
            prim[2 * k + 1] = -1;
        }
    }
}

// BSDF eval and the scatter() pdf at given surface records. rec: n x 16 (p,
// normal, front_face, u, v, dpdu, dpdv, unused); r_in, wi: n x 3. out: n x 6
// (eval rgb, pdf, skip_pdf, scatters).
void oracle_bsdf(const oracle_scene* s, int material, const double* rec, const double* r_in, const double* wi,
                 int64_t n, double* out) {
    const Scene& S = *reinterpret_cast<const Scene*>(s);
    Rng g(1);
    for (int64_t k = 0; k < n; k++) {
        const double* r = rec + 16 * k;
        Hit h;
        h.p = V(r);
        h.normal = V(r + 3);
        h.front = r[6] != 0;
        h.u = r[7];
        h.v = r[8];
        h.dpdu = V(r + 9);
        h.dpdv = V(r + 12);
        h.mat = material;
        V rd(r_in + 3 * k), d(wi + 3 * k);
        V e = eval(S, material, rd, h, d);
        Scatter sr;
        bool sc = scatter(S, material, rd, h, sr, g);
        double* o = out + 6 * k;
        o[0] = e.x;
        o[1] = e.y;
        o[2] = e.z;
        o[3] = (sc && !sr.skip_pdf) ? sr.pdf.value(d) : 0;
        o[4] = sc && sr.skip_pdf;
        o[5] = sc;
    }
}

// The light list's density sum_k p_k pdf_k(origin, dir) (light_list.h:106-113).
void oracle_light_pdf(const oracle_scene* s, const double* origin, const double* dir, int64_t n, double* out) {
    const Scene& S = *reinterpret_cast<const Scene*>(s);
    for (int64_t k = 0; k < n; k++)
        out[k] = lights_pdf(S, V(origin + 3 * k), V(dir + 3 * k));
}

// n directions drawn by the light list from origin (light_list.h:115-117).
void oracle_light_sample(const oracle_scene* s, const double* origin, int64_t n, uint64_t seed, double* dirs) {
    const Scene& S = *reinterpret_cast<const Scene*>(s);
    Rng g(seed);
    V o(origin);
    for (int64_t k = 0; k < n; k++) {
        V d = lights_random(S, o, g);
        dirs[3 * k] = d.x;
        dirs[3 * k + 1] = d.y;
        dirs[3 * k + 2] = d.z;
    }
}

// Environment radiance and density along n directions (environment.h:202-228).
void oracle_environment(const oracle_scene* s, const double* dir, int64_t n, double* radiance, double* pdf) {
    const Scene& S = *reinterpret_cast<const Scene*>(s);
    for (int64_t k = 0; k < n; k++) {
        V d(dir + 3 * k);
        V L = S.env.w > 0 ? env_radiance(S, d) : V();
        radiance[3 * k] = L.x;
        radiance[3 * k + 1] = L.y;
        radiance[3 * k + 2] = L.z;
        pdf[k] = S.env.w > 0 ? env_pdf(S, d) : 0;
    }
}

// A full render (camera.h:79-105): radiance mean W*H*3 and, per channel, the
// variance of that mean (W*H*3, from the per-sample second moments). With
// features (may be NULL), also albedo, normal (W*H*3) and the luminance
// variance of camera.h:236-245 (W*H). counts (may be NULL): paths, extension
// rays, shadow rays. threads <= 0 uses every hardware thread. first_row /
// row_count restrict the render to a band of rows (the rest stays 0).
// Renders rows first_row, first_row + row_stride, ... (row_count of them;
// row_count <= 0: to the bottom of the image) of the camera's image.
int oracle_render_strided(const oracle_scene* s, const mypbr_camera* cam, const mypbr_render_opts* opts, int threads,
                          int first_row, int row_count, int row_stride, double* radiance, double* channel_var,
                          double* albedo, double* normal, double* lum_var, uint64_t* counts) {
    const Scene& S = *reinterpret_cast<const Scene*>(s);
    Camera C;
    C.init(*cam, opts->samples_per_pixel);
    Integrator I{S, *opts, S.f->light_count > 0};
    int W = C.w, H = C.h, spp = opts->samples_per_pixel;
    row_stride = std::max(row_stride, 1);
    first_row = std::clamp(first_row, 0, H - 1);
    int most = (H - 1 - first_row) / row_stride + 1;
    if (row_count <= 0 || row_count > most)
        row_count = most;
    int nt = threads > 0 ? threads : int(std::thread::hardware_concurrency());
    nt = std::max(nt, 1);
    std::atomic<int> next_row{0};
    std::atomic<uint64_t> tot_ext{0}, tot_sh{0};
    auto worker = [&]() {
        uint64_t ext = 0, sh = 0;
        while (true) {
            int k = next_row.fetch_add(1);
            if (k >= row_count)
                break;
            int j = first_row + k * row_stride;
            for (int i = 0; i < W; i++) {
                size_t p = size_t(j) * W + i;
                V sum, sum2, asum, nsum;
                double l2 = 0;
                for (int pass = 0; pass < spp; pass++) {
                    Rng g(opts->seed ^ (0x9e3779b97f4a7c15ull * (uint64_t(p) * 0x100000001ull + uint64_t(pass) + 1)));
                    V o, d;
                    C.get_ray(i, j, pass, g, o, d);
                    V c = I.ray_color(o, d, g, ext, sh);
                    if (!std::isfinite(c.x) || !std::isfinite(c.y) || !std::isfinite(c.z))
                        c = V();
                    sum += c;
                    sum2 += c * c;
                    if (opts->collect_features) {
                        V a, nn;
                        I.first_surface(o, d, g, a, nn);
                        asum += a;
                        nsum += nn;
                        double l = lum(c);
                        l2 += l * l;
                    }
                }
                double sc = 1.0 / spp;
                V mean = sc * sum;
                for (int k = 0; k < 3; k++) {
                    radiance[3 * p + k] = mean[k];
                    if (channel_var) {
                        double spread = std::fmax(sc * sum2[k] - mean[k] * mean[k], 0.0);
                        channel_var[3 * p + k] = spp > 1 ? spread / (spp - 1) : spread;
                    }
                }
                if (opts->collect_features) {
                    for (int k = 0; k < 3; k++) {
                        if (albedo)
                            albedo[3 * p + k] = sc * asum[k];
                        if (normal)
                            normal[3 * p + k] = sc * nsum[k];
                    }
                    if (lum_var) {
                        double m = lum(mean);
                        double spread = std::fmax(sc * l2 - m * m, 0.0);
                        lum_var[p] = spp > 1 ? spread / (spp - 1) : spread;
                    }
                }
            }
        }
        tot_ext += ext;
        tot_sh += sh;
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nt; t++)
        pool.emplace_back(worker);
    worker();
    for (auto& t : pool)
        t.join();
    if (counts) {
        counts[0] = uint64_t(W) * uint64_t(row_count) * uint64_t(spp);
        counts[1] = tot_ext.load();
        counts[2] = tot_sh.load();
    }
    return 0;
}

int oracle_render(const oracle_scene* s, const mypbr_camera* cam, const mypbr_render_opts* opts, int threads,
                  int first_row, int row_count, double* radiance, double* channel_var, double* albedo,
                  double* normal, double* lum_var, uint64_t* counts) {
    return oracle_render_strided(s, cam, opts, threads, first_row, row_count, 1, radiance, channel_var, albedo,
                                 normal, lum_var, counts);
}

}  // extern "C"

namespace {

void setup(Scene& S, const mypbr_flat_scene* f) {
    S.f = f;
    S.xf.resize(size_t(f->xform_count));
    for (int64_t k = 0; k < f->xform_count; k++) {
        const auto& x = f->xforms[k];
        auto& y = S.xf[size_t(k)];
        std::memcpy(y.m, x.m, sizeof(y.m));
        std::memcpy(y.t, x.t, sizeof(y.t));
        std::memcpy(y.im, x.inv_m, sizeof(y.im));
        std::memcpy(y.it, x.inv_t, sizeof(y.it));
    }
    // light CDF (light_list.h:92-95)
    int64_t n = f->light_count;
    S.light_cdf.assign(size_t(n) + 1, 0.0);
    for (int64_t k = 0; k < n; k++)
        S.light_cdf[size_t(k) + 1] = S.light_cdf[size_t(k)] + f->lights[k].probability;
    if (n > 0)
        S.light_cdf[size_t(n)] = 1;
    // members: a CDF over weights, for picking (mesh.h:211-216, hittable_list.h:120-124)
    S.member_cdf.resize(size_t(n));
    for (int64_t k = 0; k < n; k++) {
        const auto& L = f->lights[k];
        auto& c = S.member_cdf[size_t(k)];
        double acc = 0;
        for (int m = 0; m < L.member_count; m++) {
            acc += f->light_members[L.first_member + m].weight;
            c.push_back(acc);
        }
        if (!c.empty())
            c.back() = std::max(c.back(), 1.0);
    }
    build_env(S);
    double tab[32 * 32 + 32];
    oracle_ggx_table(tab);
    for (int j = 0; j < 32; j++) {
        for (int i = 0; i < 32; i++)
            S.E[j][i] = tab[j * 32 + i];
        S.Eavg[j] = tab[32 * 32 + j];
    }
    if (f->sun.enabled) {
        S.sun_frame = Onb(V(f->sun.direction));
        double half = std::fmax(f->sun.angular_diameter, 1e-3) * PI / 180.0 / 2;
        S.sun_cos_max = std::cos(half);
        S.sun_solid_angle = 2 * PI * (1 - S.sun_cos_max);
        S.sun_radiance = V(f->sun.irradiance) / S.sun_solid_angle;
    }
}

}  // namespace

// ------------------------------------------------------------- denoiser

namespace {

double lum3(const double* c) { return 0.2126 * c[0] + 0.7152 * c[1] + 0.0722 * c[2]; }

}  // namespace

extern "C" {

// denoiser::run (denoiser.h:45-193), FP64: firefly clamp, then `iterations`
// edge-avoiding a-trous passes (B3 5x5 taps spread 2^i apart) on lighting =
// radiance / (albedo + 1e-3), weighted by normal, albedo and the luminance
// within sigma_luminance standard deviations; out = lighting * (albedo + 1e-3).
// All arrays W*H(*3), rows from the top left.
void oracle_denoise(const double* radiance, const double* albedo, const double* normal, const double* variance,
                    int width, int height, int iterations, double sigma_luminance, double sigma_normal,
                    double sigma_albedo, double* out) {
    const double eps = 1e-3;
    size_t n = size_t(width) * height;
    std::vector<double> light(3 * n), var(n);
    for (size_t k = 0; k < n; k++) {
        double a[3] = {albedo[3 * k] + eps, albedo[3 * k + 1] + eps, albedo[3 * k + 2] + eps};
        for (int c = 0; c < 3; c++)
            light[3 * k + c] = radiance[3 * k + c] / a[c];
        double la = lum3(a);
        var[k] = variance[k] / (la * la);
    }
    // remove_fireflies (denoiser.h:90-111)
    std::vector<double> src = light;
    for (int j = 1; j < height - 1; j++)
        for (int i = 1; i < width - 1; i++) {
            size_t p = size_t(j) * width + i;
            double l = lum3(&src[3 * p]);
            if (l <= 0 || std::sqrt(var[p]) < 0.5 * l)
                continue;
            double brightest = 0;
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++)
                    if (dx || dy)
                        brightest = std::fmax(brightest, lum3(&src[3 * (p + dy * width + dx)]));
            if (l > brightest) {
                double s = brightest / l;
                for (int c = 0; c < 3; c++)
                    light[3 * p + c] = s * src[3 * p + c];
                var[p] *= s * s;
            }
        }
    static const double kern[5] = {1.0 / 16, 1.0 / 4, 3.0 / 8, 1.0 / 4, 1.0 / 16};
    std::vector<double> nl(3 * n), nv(n), bv(n);
    double inv_n = 1 / (sigma_normal * sigma_normal), inv_a = 1 / (sigma_albedo * sigma_albedo);
    for (int it = 0; it < iterations; it++) {
        // blur3x3 (denoiser.h:158-178)
        for (int j = 0; j < height; j++)
            for (int i = 0; i < width; i++) {
                static const double k3[3] = {0.25, 0.5, 0.25};
                double sum = 0, w = 0;
                for (int dy = -1; dy <= 1; dy++)
                    for (int dx = -1; dx <= 1; dx++) {
                        int x = i + dx, y = j + dy;
                        if (x < 0 || x >= width || y < 0 || y >= height)
                            continue;
                        double wt = k3[dx + 1] * k3[dy + 1];
                        sum += wt * var[size_t(y) * width + x];
                        w += wt;
                    }
                bv[size_t(j) * width + i] = sum / w;
            }
        int step = 1 << it;
        // filter_pixel (denoiser.h:113-156)
        for (int j = 0; j < height; j++)
            for (int i = 0; i < width; i++) {
                size_t p = size_t(j) * width + i;
                double lp = lum3(&light[3 * p]);
                double scale = sigma_luminance * std::sqrt(std::fmax(bv[p], 0.0)) + 1e-10;
                double s[3] = {0, 0, 0}, ws = 0, vs = 0;
                for (int dy = -2; dy <= 2; dy++) {
                    int y = j + dy * step;
                    if (y < 0 || y >= height)
                        continue;
                    for (int dx = -2; dx <= 2; dx++) {
                        int x = i + dx * step;
                        if (x < 0 || x >= width)
                            continue;
                        size_t q = size_t(y) * width + x;
                        double dn = 0, da = 0;
                        for (int c = 0; c < 3; c++) {
                            double a = normal[3 * p + c] - normal[3 * q + c], b = albedo[3 * p + c] - albedo[3 * q + c];
                            dn += a * a;
                            da += b * b;
                        }
                        double w = kern[dx + 2] * kern[dy + 2] * std::exp(-dn * inv_n) * std::exp(-da * inv_a) *
                                   std::exp(-std::fabs(lp - lum3(&light[3 * q])) / scale);
                        for (int c = 0; c < 3; c++)
                            s[c] += w * light[3 * q + c];
                        ws += w;
                        vs += w * w * var[q];
                    }
                }
                for (int c = 0; c < 3; c++)
                    nl[3 * p + c] = s[c] / ws;
                nv[p] = vs / (ws * ws);
            }
        std::swap(light, nl);
        std::swap(var, nv);
    }
    for (size_t k = 0; k < n; k++)
        for (int c = 0; c < 3; c++)
            out[3 * k + c] = light[3 * k + c] * (albedo[3 * k + c] + eps);
}

}  // extern "C"
