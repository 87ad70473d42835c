// FP32 vector helpers, the counter-based random numbers and small utilities
// shared by the device kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#define MYPBR_DEV __device__ __forceinline__
#define MYPBR_HD __host__ __device__ __forceinline__

namespace mypbr_dev {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.31830988618379067154f;

MYPBR_HD float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
MYPBR_HD float3 f3(float s) { return make_float3(s, s, s); }
MYPBR_HD float3 f3(const float4& a) { return make_float3(a.x, a.y, a.z); }
MYPBR_HD float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
MYPBR_HD float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
MYPBR_HD float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
MYPBR_HD float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
MYPBR_HD float3 operator*(float s, float3 a) { return f3(s * a.x, s * a.y, s * a.z); }
MYPBR_HD float3 operator*(float3 a, float s) { return f3(s * a.x, s * a.y, s * a.z); }
MYPBR_HD float3 operator/(float3 a, float s) { return (1.0f / s) * a; }
MYPBR_HD float3& operator+=(float3& a, float3 b) {
    a = a + b;
    return a;
}
MYPBR_HD float3& operator*=(float3& a, float3 b) {
    a = a * b;
    return a;
}
MYPBR_HD float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
MYPBR_HD float3 cross(float3 a, float3 b) {
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
MYPBR_HD float len2(float3 a) { return dot(a, a); }
MYPBR_DEV float length(float3 a) { return sqrtf(dot(a, a)); }
MYPBR_DEV float3 normalize(float3 a) { return a * rsqrtf(dot(a, a)); }
MYPBR_HD float comp(float3 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : a.z); }
MYPBR_HD float comp4(float4 a, int i) { return i == 0 ? a.x : (i == 1 ? a.y : (i == 2 ? a.z : a.w)); }
MYPBR_HD void set_comp(float3& a, int i, float v) {
    if (i == 0)
        a.x = v;
    else if (i == 1)
        a.y = v;
    else
        a.z = v;
}
MYPBR_HD float maxc(float3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
MYPBR_HD float avg3(float3 a) { return (a.x + a.y + a.z) * (1.0f / 3.0f); }
MYPBR_HD float luminance(float3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }
MYPBR_HD float clampf(float x, float a, float b) { return fminf(fmaxf(x, a), b); }
MYPBR_HD bool nonzero(float3 c) { return c.x > 0.0f || c.y > 0.0f || c.z > 0.0f; }
MYPBR_DEV float3 reflect(float3 v, float3 n) { return v - 2.0f * dot(v, n) * n; }
// Refraction of unit uv through unit normal n with ratio eta_i / eta_t (vec3.h:324-329).
MYPBR_DEV float3 refract(float3 uv, float3 n, float ratio) {
    float c = fminf(dot(-uv, n), 1.0f);
    float3 perp = ratio * (uv + c * n);
    float3 par = -sqrtf(fabsf(1.0f - len2(perp))) * n;
    return perp + par;
}

// Orthonormal basis with w along n (onb.h:9-28).
struct Onb {
    float3 u, v, w;
    MYPBR_DEV explicit Onb(float3 n) {
        w = normalize(n);
        float3 a = fabsf(w.x) > 0.9f ? f3(0, 1, 0) : f3(1, 0, 0);
        v = normalize(cross(w, a));
        u = cross(w, v);
    }
    MYPBR_DEV float3 to_world(float3 a) const { return a.x * u + a.y * v + a.z * w; }
    MYPBR_DEV float3 to_local(float3 a) const { return f3(dot(a, u), dot(a, v), dot(a, w)); }
};

// ---------------------------------------------------------------- random

// PCG-XSH-RR 32 (O'Neill 2014) with a 64-bit state per path; one stream per
// (pixel, sample) from a hashed seed, so renders are reproducible.
MYPBR_HD uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

struct Rng {
    uint64_t state;
    MYPBR_DEV uint32_t next_u32() {
        uint64_t old = state;
        state = old * 6364136223846793005ull + 1442695040888963407ull;
        uint32_t xorshifted = uint32_t(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = uint32_t(old >> 59u);
        return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
    }
    // Uniform in [0, 1)
    MYPBR_DEV float next() { return float(next_u32() >> 8) * (1.0f / 16777216.0f); }
};

MYPBR_DEV Rng make_rng(uint64_t seed, uint64_t pixel, uint64_t sample) {
    Rng r;
    r.state = mix64(seed ^ mix64(pixel * 0x9e3779b97f4a7c15ull + sample + 1));
    r.next_u32();
    return r;
}

// A uniform number from a hash of (key, salt): free-flight sampling inside
// traversal, where a ray tests a medium once.
MYPBR_DEV float hash_uniform(uint64_t key, uint32_t salt) {
    uint64_t h = mix64(key ^ (uint64_t(salt) * 0xd6e8feb86659fd93ull));
    return float(uint32_t(h >> 40)) * (1.0f / 16777216.0f);
}

}  // namespace mypbr_dev
