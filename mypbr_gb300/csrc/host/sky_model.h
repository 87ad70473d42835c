// Single-scattering sky (the `sky atmosphere` of include/atmosphere.h), in
// FP64, compiled both for the host scene loader and for the device bake
// kernel (sky.cu). Sunlight scattered once by air molecules (Rayleigh,
// ~1/lambda^4), aerosols (Mie, Henyey-Greenstein phase) and absorbed by ozone,
// integrated by marching along the view ray (32 steps) with the sun's
// transmittance to each step marched again (16 steps). Earth's coefficients
// as tabulated by Hillaire, "A Scalable and Production Ready Sky and
// Atmosphere Rendering Technique" (EGSR 2020); planet and atmosphere radii
// 6360 km and 6460 km, viewer 200 m above the ground.
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define SKY_HD __host__ __device__
#else
#define SKY_HD
#endif

namespace mypbr_sky {

struct Settings {
    double rayleigh = 1, mie = 1, mie_g = 0.8, ozone = 1, intensity = 3;  // atmosphere.h:39-46
};

struct C3 {
    double r, g, b;
};

SKY_HD inline C3 c3(double r, double g, double b) { return C3{r, g, b}; }
SKY_HD inline C3 add(C3 a, C3 b) { return c3(a.r + b.r, a.g + b.g, a.b + b.b); }
SKY_HD inline C3 mul(double s, C3 a) { return c3(s * a.r, s * a.g, s * a.b); }
SKY_HD inline C3 mul(C3 a, C3 b) { return c3(a.r * b.r, a.g * b.g, a.b * b.b); }
SKY_HD inline C3 exp3(C3 a) { return c3(std::exp(a.r), std::exp(a.g), std::exp(a.b)); }

constexpr double kGround = 6360e3, kTop = 6460e3, kViewer = 6360e3 + 200;
constexpr double kPiD = 3.1415926535897932385;

// Extinction coefficients per metre at sea level (Hillaire 2020, table 1)
SKY_HD inline C3 beta_rayleigh(const Settings& s) { return mul(s.rayleigh, c3(5.802e-6, 13.558e-6, 33.1e-6)); }
SKY_HD inline C3 beta_mie(const Settings& s) { return mul(s.mie, c3(3.996e-6, 3.996e-6, 3.996e-6)); }
SKY_HD inline C3 beta_mie_ext(const Settings& s) { return mul(s.mie, c3(4.40e-6, 4.40e-6, 4.40e-6)); }
SKY_HD inline C3 beta_ozone(const Settings& s) { return mul(s.ozone, c3(0.650e-6, 1.881e-6, 0.085e-6)); }

// Relative densities at height h: exponential air (8 km) and aerosols
// (1.2 km), a tent of ozone centred at 25 km, 15 km each side.
SKY_HD inline void densities(double h, double& r, double& m, double& o) {
    r = std::exp(-h / 8000);
    m = std::exp(-h / 1200);
    o = std::fmax(0.0, 1 - std::fabs(h - 25000) / 15000);
}

SKY_HD inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// Along unit d from p inside the atmosphere: distance to its top, and to the
// ground (-1 when the ray misses the planet).
SKY_HD inline double to_top(const double* p, const double* d) {
    double b = dot3(p, d), c = dot3(p, p) - kTop * kTop;
    return -b + std::sqrt(std::fmax(0.0, b * b - c));
}
SKY_HD inline double to_ground(const double* p, const double* d) {
    double b = dot3(p, d), c = dot3(p, p) - kGround * kGround;
    double disc = b * b - c;
    if (disc < 0)
        return -1;
    double t = -b - std::sqrt(disc);
    return t > 0 ? t : -1;
}

SKY_HD inline C3 extinction(const Settings& s, double h) {
    double r, m, o;
    densities(h, r, m, o);
    return add(add(mul(r, beta_rayleigh(s)), mul(m, beta_mie_ext(s))), mul(o, beta_ozone(s)));
}

// Transmittance from p to space along unit d (0 if the ground is in the way).
SKY_HD inline C3 transmittance(const Settings& s, const double* p, const double* d) {
    if (to_ground(p, d) > 0)
        return c3(0, 0, 0);
    const int steps = 16;
    double dt = to_top(p, d) / steps;
    C3 depth = c3(0, 0, 0);
    for (int k = 0; k < steps; k++) {
        double q[3] = {p[0] + (k + 0.5) * dt * d[0], p[1] + (k + 0.5) * dt * d[1], p[2] + (k + 0.5) * dt * d[2]};
        double h = std::sqrt(dot3(q, q)) - kGround;
        depth = add(depth, mul(dt, extinction(s, h)));
    }
    return exp3(mul(-1.0, depth));
}

// unit_vector as vec3.h:95-97 forms it: (1 / |a|) a
SKY_HD inline void unit3(const double* a, double* out) {
    double inv = 1 / std::sqrt(dot3(a, a));
    out[0] = inv * a[0];
    out[1] = inv * a[1];
    out[2] = inv * a[2];
}

// Fraction of sunlight reaching the viewer along the sun's direction.
SKY_HD inline C3 sun_transmittance(const Settings& s, const double* sun_dir) {
    double d[3], o[3] = {0, kViewer, 0};
    unit3(sun_dir, d);
    return transmittance(s, o, d);
}

// Sky radiance in `dir` for a sun in `sun_dir` of irradiance `sun_irr` above the air.
SKY_HD inline C3 radiance(const Settings& st, const double* dir, const double* sun_dir, C3 sun_irr) {
    double d[3], sd[3], o[3] = {0, kViewer, 0};
    unit3(dir, d);
    unit3(sun_dir, sd);
    double t_max = to_top(o, d);
    double t_ground = to_ground(o, d);
    if (t_ground > 0)
        t_max = std::fmin(t_max, t_ground);
    double mu = dot3(d, sd);
    double phase_r = 3 / (16 * kPiD) * (1 + mu * mu);
    double g = st.mie_g;
    double den = 1 + g * g - 2 * g * mu;
    double phase_m = (1 - g * g) / (4 * kPiD * den * std::sqrt(den));
    const int steps = 32;
    double dt = t_max / steps;
    C3 depth = c3(0, 0, 0), sum = c3(0, 0, 0);
    for (int k = 0; k < steps; k++) {
        double p[3] = {o[0] + (k + 0.5) * dt * d[0], o[1] + (k + 0.5) * dt * d[1], o[2] + (k + 0.5) * dt * d[2]};
        double h = std::sqrt(dot3(p, p)) - kGround;
        double r, m, oz;
        densities(h, r, m, oz);
        C3 ext = add(add(mul(r, beta_rayleigh(st)), mul(m, beta_mie_ext(st))), mul(oz, beta_ozone(st)));
        depth = add(depth, mul(0.5 * dt, ext));  // midpoint: half a step to reach p
        C3 to_sun = transmittance(st, p, sd);
        C3 view = exp3(mul(-1.0, depth));
        C3 scat = add(mul(r * phase_r, beta_rayleigh(st)), mul(m * phase_m, beta_mie(st)));
        sum = add(sum, mul(dt, mul(mul(view, to_sun), scat)));
        depth = add(depth, mul(0.5 * dt, ext));
    }
    return mul(mul(st.intensity, sum), sun_irr);
}

// Pixel (i, j) of the equirectangular bake as environment_light reads it:
// theta = pi (j + 0.5) / h from +y, phi = 2 pi ((i + 0.5) / w - 0.5), -z at phi = 0.
SKY_HD inline C3 bake_pixel(const Settings& st, int i, int j, int w, int h, const double* sun_dir, C3 sun_irr) {
    double theta = kPiD * (j + 0.5) / h;
    double phi = 2 * kPiD * ((i + 0.5) / w - 0.5);
    double d[3] = {std::sin(theta) * std::sin(phi), std::cos(theta), -std::sin(theta) * std::cos(phi)};
    return radiance(st, d, sun_dir, sun_irr);
}

}  // namespace mypbr_sky
