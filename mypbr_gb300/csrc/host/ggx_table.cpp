// Kulla-Conty directional albedo table of single-scattering GGX, built on the
// host and uploaded to the device.
//
// The table is the reference's (include/microfacet.h:265-338): 32 x 32
// entries E(mu, alpha) of the F = 1 GGX lobe, rows evenly spaced in roughness
// (sqrt(alpha)), columns in mu, each the mean of G(wo, wi) / G1(wo) over a
// 64 x 64 stratified grid of visible-normal samples (Heitz 2018), then the
// exact integral E_avg = 2 * int E(mu) mu dmu over the piecewise-linear E.
// The device must use the same numbers for its energy compensation to match.
#include <cmath>

#include "bvh_build.h"

namespace mypbr_host {

namespace {

struct Ggx {
    double alpha;
    double lambda(const V3& w) const {
        double c2 = w.z * w.z;
        if (c2 <= 0)
            return kInf;
        double t2 = std::fmax(0.0, 1 - c2) / c2;
        return (-1 + std::sqrt(1 + alpha * alpha * t2)) / 2;
    }
    double g1(const V3& w) const { return 1 / (1 + lambda(w)); }
    double g(const V3& wo, const V3& wi) const { return 1 / (1 + lambda(wo) + lambda(wi)); }

    // Visible-normal sample for uniform numbers u1, u2 (Heitz 2018, section 4).
    V3 sample_visible(const V3& wo, double u1, double u2) const {
        V3 vh = unit(V3(alpha * wo.x, alpha * wo.y, wo.z));
        double len2 = vh.x * vh.x + vh.y * vh.y;
        V3 t1 = len2 > 0 ? V3(-vh.y, vh.x, 0) / std::sqrt(len2) : V3(1, 0, 0);
        V3 t2 = cross(vh, t1);
        double r = std::sqrt(u1), phi = 2 * kPi * u2;
        double p1 = r * std::cos(phi), p2 = r * std::sin(phi);
        double s = 0.5 * (1 + vh.z);
        p2 = (1 - s) * std::sqrt(std::fmax(0.0, 1 - p1 * p1)) + s * p2;
        V3 nh = p1 * t1 + p2 * t2 + std::sqrt(std::fmax(0.0, 1 - p1 * p1 - p2 * p2)) * vh;
        return unit(V3(alpha * nh.x, alpha * nh.y, std::fmax(1e-6, nh.z)));
    }
};

}  // namespace

void ggx_albedo_table(double* out) {
    const int size = 32, strata = 64;
    double* e = out;                 // [size][size]
    double* e_avg = out + size * size;
    for (int j = 0; j < size; j++) {
        double roughness = double(j) / (size - 1);
        Ggx d{std::max(roughness * roughness, 1e-3)};
        for (int i = 0; i < size; i++) {
            double mu = std::fmax(double(i) / (size - 1), 1e-3);
            V3 wo(std::sqrt(1 - mu * mu), 0, mu);
            double sum = 0;
            for (int a = 0; a < strata; a++)
                for (int b = 0; b < strata; b++) {
                    V3 h = d.sample_visible(wo, (a + 0.5) / strata, (b + 0.5) / strata);
                    V3 wi = -wo + 2 * dot(wo, h) * h;
                    if (wi.z > 0)
                        sum += d.g(wo, wi) / d.g1(wo);
                }
            e[j * size + i] = std::fmin(sum / (strata * strata), 1.0);
        }
        double integral = 0, h = 1.0 / (size - 1);
        for (int i = 0; i + 1 < size; i++) {
            double a = i * h, b = (i + 1) * h;
            integral += h * (e[j * size + i] * (2 * a + b) + e[j * size + i + 1] * (a + 2 * b)) / 6;
        }
        e_avg[j] = std::fmin(2 * integral, 1.0);
    }
}

}  // namespace mypbr_host
