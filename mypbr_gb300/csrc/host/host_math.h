// Small FP64 vector, box and affine-transform helpers for the host scene layer.
//
// The host side keeps the reference's FP64 (include/vec3.h:11) so that the
// flat scene holds exactly the values the reference would compute from the
// same file; the device copy is converted to FP32 later.
#pragma once

#include <algorithm>
#include <cmath>
#include <limits>

namespace mypbr_host {

constexpr double kPi = 3.1415926535897932385;
constexpr double kInf = std::numeric_limits<double>::infinity();

inline double radians(double degrees) { return degrees * kPi / 180.0; }

struct V3 {
    double x = 0, y = 0, z = 0;
    V3() = default;
    V3(double a, double b, double c) : x(a), y(b), z(c) {}
    double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    double& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    V3 operator-() const { return {-x, -y, -z}; }
    double length_squared() const { return x * x + y * y + z * z; }
    double length() const { return std::sqrt(length_squared()); }
    bool near_zero() const { return std::fabs(x) < 1e-8 && std::fabs(y) < 1e-8 && std::fabs(z) < 1e-8; }
};
inline V3 operator+(const V3& a, const V3& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(const V3& a, const V3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(const V3& a, const V3& b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 operator*(double s, const V3& a) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 operator*(const V3& a, double s) { return {s * a.x, s * a.y, s * a.z}; }
inline V3 operator/(const V3& a, double s) { return (1 / s) * a; }
inline double dot(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(const V3& a, const V3& b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline V3 unit(const V3& a) { return a / a.length(); }
inline double luminance(const V3& c) { return 0.2126 * c.x + 0.7152 * c.y + 0.0722 * c.z; }

// An axis-aligned box with the reference's conventions (include/aabb.h):
// empty by default, and boxes made from points get every side at least
// 1e-4 wide so planar objects still have volume.
struct Box {
    V3 lo{kInf, kInf, kInf}, hi{-kInf, -kInf, -kInf};

    static Box from_points(const V3& a, const V3& b) {
        Box r;
        for (int k = 0; k < 3; k++) {
            r.lo[k] = std::fmin(a[k], b[k]);
            r.hi[k] = std::fmax(a[k], b[k]);
        }
        r.pad();
        return r;
    }
    void pad() {
        const double delta = 0.0001;
        for (int k = 0; k < 3; k++)
            if (hi[k] - lo[k] < delta) {
                lo[k] -= delta / 2;
                hi[k] += delta / 2;
            }
    }
    void grow(const Box& b) {
        for (int k = 0; k < 3; k++) {
            lo[k] = lo[k] <= b.lo[k] ? lo[k] : b.lo[k];
            hi[k] = hi[k] >= b.hi[k] ? hi[k] : b.hi[k];
        }
    }
    double size(int k) const { return hi[k] - lo[k]; }
    bool empty() const { return !(lo.x <= hi.x && lo.y <= hi.y && lo.z <= hi.z); }
    V3 centroid() const { return 0.5 * (lo + hi); }
    double surface_area() const {
        double dx = size(0), dy = size(1), dz = size(2);
        return 2 * (dx * dy + dy * dz + dz * dx);
    }
    int longest_axis() const {
        if (size(0) > size(1))
            return size(0) > size(2) ? 0 : 2;
        return size(1) > size(2) ? 1 : 2;
    }
};

// p -> M p + t with its inverse, composed like the reference's transform
// (include/transform.h:72-173).
struct Xf {
    double m[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    V3 t;
    double inv_m[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    V3 inv_t;

    static V3 mul(const double a[3][3], const V3& v) {
        return {a[0][0] * v.x + a[0][1] * v.y + a[0][2] * v.z, a[1][0] * v.x + a[1][1] * v.y + a[1][2] * v.z,
                a[2][0] * v.x + a[2][1] * v.y + a[2][2] * v.z};
    }
    static void mat_mul(const double a[3][3], const double b[3][3], double out[3][3]) {
        double r[3][3];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
                r[i][j] = a[i][0] * b[0][j] + a[i][1] * b[1][j] + a[i][2] * b[2][j];
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
                out[i][j] = r[i][j];
    }
    static Xf translate(const V3& d) {
        Xf x;
        x.t = d;
        x.inv_t = -d;
        return x;
    }
    static Xf scale(const V3& s) {
        Xf x;
        for (int k = 0; k < 3; k++) {
            x.m[k][k] = s[k];
            x.inv_m[k][k] = 1 / s[k];
        }
        return x;
    }
    // Counterclockwise about axis looking down it (Rodrigues).
    static Xf rotate(double degrees, const V3& axis) {
        V3 a = unit(axis);
        double th = radians(degrees);
        double c = std::cos(th), s = std::sin(th), C = 1 - c;
        double r[3][3] = {{a.x * a.x * C + c, a.x * a.y * C - a.z * s, a.x * a.z * C + a.y * s},
                          {a.y * a.x * C + a.z * s, a.y * a.y * C + c, a.y * a.z * C - a.x * s},
                          {a.z * a.x * C - a.y * s, a.z * a.y * C + a.x * s, a.z * a.z * C + c}};
        Xf x;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) {
                x.m[i][j] = r[i][j];
                x.inv_m[j][i] = r[i][j];
            }
        return x;
    }
    // This transform applied after `first`.
    Xf then_after(const Xf& first) const {
        Xf x;
        mat_mul(m, first.m, x.m);
        x.t = vec(first.t) + t;
        mat_mul(first.inv_m, inv_m, x.inv_m);
        x.inv_t = first.inv_vec(inv_t) + first.inv_t;
        return x;
    }
    V3 point(const V3& p) const { return vec(p) + t; }
    V3 vec(const V3& v) const { return mul(m, v); }
    V3 inv_point(const V3& p) const { return inv_vec(p) + inv_t; }
    V3 inv_vec(const V3& v) const { return mul(inv_m, v); }
    // Normals map by the inverse transpose.
    V3 normal(const V3& n) const {
        return {inv_m[0][0] * n.x + inv_m[1][0] * n.y + inv_m[2][0] * n.z,
                inv_m[0][1] * n.x + inv_m[1][1] * n.y + inv_m[2][1] * n.z,
                inv_m[0][2] * n.x + inv_m[1][2] * n.y + inv_m[2][2] * n.z};
    }
    double det() const {
        return m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
               m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
    }
    bool is_similarity() const {
        V3 c0(m[0][0], m[1][0], m[2][0]), c1(m[0][1], m[1][1], m[2][1]), c2(m[0][2], m[1][2], m[2][2]);
        double l = c0.length_squared();
        auto close = [l](double a, double b) { return std::fabs(a - b) <= 1e-9 * std::fmax(1.0, l); };
        return close(c1.length_squared(), l) && close(c2.length_squared(), l) && close(dot(c0, c1), 0) &&
               close(dot(c1, c2), 0) && close(dot(c0, c2), 0);
    }
    double area_scale() const { return std::pow(std::fabs(det()), 2.0 / 3.0); }
    // Bounding box of the eight transformed corners of b (include/instance.h:17-26).
    Box box(const Box& b) const {
        Box r;
        for (int i = 0; i < 2; i++)
            for (int j = 0; j < 2; j++)
                for (int k = 0; k < 2; k++) {
                    V3 c(i ? b.hi.x : b.lo.x, j ? b.hi.y : b.lo.y, k ? b.hi.z : b.lo.z);
                    V3 p = point(c);
                    r.grow(Box::from_points(p, p));
                }
        return r;
    }
};

}  // namespace mypbr_host
