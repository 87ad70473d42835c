// Textures, BSDFs, direction pdfs, lights and the sky, in FP32 on the device.
//
// Each function keeps the meaning of the reference function cited beside it
// (include/material.h, microfacet.h, pdf.h, light_list.h, environment.h,
// sun.h, camera.h), so that eval / pdf agree with the FP64 reference to FP32
// accuracy and renders agree statistically.
#pragma once

#include "dev_scene.cuh"

namespace mypbr_dev {

enum : int {
    kLambertian = 0, kMetal = 1, kDielectric = 2, kThinDielectric = 3, kPrincipled = 4, kDiffuseLight = 5, kPhase = 6
};
enum : int { kMatMeasured = 1, kMatCoat = 2, kMatCoatTint = 4 };

// -------------------------------------------------------------- textures

MYPBR_DEV float srgb_decode(int c) {
    float e = c * (1.0f / 255.0f);
    return e <= 0.04045f ? e * (1.0f / 12.92f) : powf((e + 0.055f) * (1.0f / 1.055f), 2.4f);
}

// texture.h:24-282: solid, checker and image textures, and the wrappers
// around them (scaled, channel, uv transform, normal scale). A chain holds at
// most two wrappers that change the value (checked at upload); they apply
// innermost first once the plain texture's value is known.
MYPBR_DEV float3 tex_value(const DeviceScene& S, int t, float u, float v, float3 p) {
    int outer0 = -1, outer1 = -1;
    float3 c = f3(0.0f);
    for (int guard = 0; guard < 8 && t >= 0; guard++) {
        const DevTexture& tx = S.textures[t];
        if (tx.type == 0) {
            c = f3(tx.p[0], tx.p[1], tx.p[2]);
            break;
        }
        if (tx.type == 1) {
            int x = int(floorf(tx.p[0] * p.x)), y = int(floorf(tx.p[0] * p.y)), z = int(floorf(tx.p[0] * p.z));
            t = ((x + y + z) % 2 == 0) ? tx.a : tx.b;
            continue;
        }
        if (tx.type == 2) {
            if (tx.flags & 4) {
                u -= floorf(u);
                v -= floorf(v);
            } else {
                u = clampf(u, 0.0f, 1.0f);
                v = clampf(v, 0.0f, 1.0f);
            }
            v = 1.0f - v;
            int i = min(max(int(u * tx.width), 0), tx.width - 1);
            int j = min(max(int(v * tx.height), 0), tx.height - 1);
            long long k = tx.offset + (long long)j * tx.width + i;
            if (tx.flags & 1) {
                const float* px = S.texels_hdr + 3 * k;
                c = f3(px[0], px[1], px[2]);
            } else {
                const uint8_t* px = S.texels_ldr + 4 * k;
                if (tx.flags & 2)
                    c = f3(px[0], px[1], px[2]) * (1.0f / 255.0f);
                else
                    c = f3(srgb_decode(px[0]), srgb_decode(px[1]), srgb_decode(px[2]));
            }
            break;
        }
        if (tx.type == 5) {
            // uv_transform_texture::value (texture.h:255-259), in glTF's
            // coordinates where v runs down the image; p[2], p[5] = cos, sin
            float su = tx.p[3] * u, sv = tx.p[4] * (1.0f - v);
            float tu = tx.p[2] * su + tx.p[5] * sv + tx.p[0];
            float tv = -tx.p[5] * su + tx.p[2] * sv + tx.p[1];
            u = tu;
            v = 1.0f - tv;
        } else if (outer0 < 0) {
            outer0 = t;
        } else {
            outer1 = t;
        }
        t = tx.a;
    }
    for (int k = 0; k < 2; k++) {
        int o = k == 0 ? outer1 : outer0;
        if (o < 0)
            continue;
        const DevTexture& tx = S.textures[o];
        if (tx.type == 3) {
            c = c * f3(tx.p[0], tx.p[1], tx.p[2]);
        } else if (tx.type == 4) {
            c = f3(tx.p[0] * comp(c, tx.b));
        } else {
            c = f3(0.5f + tx.p[0] * (c.x - 0.5f), 0.5f + tx.p[0] * (c.y - 0.5f), c.z);
        }
    }
    return c;
}

// ------------------------------------------------------- microfacet model

MYPBR_DEV float rough_to_alpha(float r) { return fmaxf(r * r, 1e-3f); }  // microfacet.h:17-19
MYPBR_DEV float pow5(float x) {
    float x2 = x * x;
    return x2 * x2 * x;
}
MYPBR_DEV float schlick(float c, float f0) { return f0 + (1.0f - f0) * pow5(1.0f - clampf(c, 0.0f, 1.0f)); }
MYPBR_DEV float3 schlick3(float c, float3 f0) {
    float k = pow5(1.0f - clampf(c, 0.0f, 1.0f));
    return f0 + (f3(1.0f) - f0) * k;
}

// microfacet.h:34-48
MYPBR_DEV float fresnel_dielectric(float ci, float eta) {
    ci = clampf(ci, -1.0f, 1.0f);
    if (ci < 0.0f) {
        eta = 1.0f / eta;
        ci = -ci;
    }
    float s2t = (1.0f - ci * ci) / (eta * eta);
    if (s2t >= 1.0f)
        return 1.0f;
    float ct = sqrtf(1.0f - s2t);
    float rp = (eta * ci - ct) / (eta * ci + ct), rs = (ci - eta * ct) / (ci + eta * ct);
    return 0.5f * (rp * rp + rs * rs);
}

// microfacet.h:57-65, complex arithmetic written out
MYPBR_DEV float fresnel_conductor(float ci, float eta, float k) {
    ci = clampf(ci, 0.0f, 1.0f);
    // n^2 = (eta^2 - k^2) + 2 i eta k; sin2_t = (1 - ci^2) / n^2
    float nr2 = eta * eta - k * k, ni2 = 2.0f * eta * k;
    float s2 = 1.0f - ci * ci;
    float inv = 1.0f / (nr2 * nr2 + ni2 * ni2);
    float sr = s2 * nr2 * inv, si = -s2 * ni2 * inv;  // sin2_t
    // cos_t = sqrt(1 - sin2_t), principal branch
    float zr = 1.0f - sr, zi = -si;
    float mag = sqrtf(zr * zr + zi * zi);
    float cr = sqrtf(fmaxf(0.5f * (mag + zr), 0.0f));
    float cim = copysignf(sqrtf(fmaxf(0.5f * (mag - zr), 0.0f)), zi);
    // r_parl = (n ci - cos_t) / (n ci + cos_t), r_perp = (ci - n cos_t) / (ci + n cos_t)
    float ar = eta * ci - cr, ai = k * ci - cim, br = eta * ci + cr, bi = k * ci + cim;
    float rp = (ar * ar + ai * ai) / (br * br + bi * bi);
    float ncr = eta * cr - k * cim, nci = eta * cim + k * cr;  // n * cos_t
    float pr = ci - ncr, pi_ = -nci, qr = ci + ncr, qi = nci;
    float rs = (pr * pr + pi_ * pi_) / (qr * qr + qi * qi);
    return 0.5f * (rp + rs);
}

// microfacet.h:145-212
struct Ggx {
    float a;
    // For unit h, h.z^2 (a^2 - 1) + 1 = a^2 h.z^2 + h.x^2 + h.y^2: the right-hand
    // form has no cancellation near the peak (h.z -> 1), where FP32 loses the
    // left-hand one for small alpha.
    MYPBR_DEV float D(float3 h) const {
        if (h.z <= 0.0f)
            return 0.0f;
        float a2 = a * a, d = a2 * h.z * h.z + (h.x * h.x + h.y * h.y);
        return a2 / (kPi * d * d);
    }
    // tan^2 of a unit w as (x^2 + y^2) / z^2, the same cancellation-free form
    MYPBR_DEV float lambda(float3 w) const {
        float c2 = w.z * w.z;
        if (c2 <= 0.0f)
            return 3.0e38f;
        float t2 = (w.x * w.x + w.y * w.y) / c2;
        return 0.5f * (-1.0f + sqrtf(1.0f + a * a * t2));
    }
    MYPBR_DEV float G1(float3 w) const { return 1.0f / (1.0f + lambda(w)); }
    MYPBR_DEV float G(float3 wo, float3 wi) const { return 1.0f / (1.0f + lambda(wo) + lambda(wi)); }
    MYPBR_DEV float visible_pdf(float3 wo, float3 h) const {
        if (wo.z <= 0.0f)
            return 0.0f;
        return G1(wo) / wo.z * D(h) * fabsf(dot(wo, h));
    }
    // Heitz 2018, "Sampling the GGX Distribution of Visible Normals"
    MYPBR_DEV float3 sample_visible(float3 wo, float u1, float u2) const {
        float3 vh = normalize(f3(a * wo.x, a * wo.y, wo.z));
        float l2 = vh.x * vh.x + vh.y * vh.y;
        float3 t1 = l2 > 0.0f ? f3(-vh.y, vh.x, 0.0f) * rsqrtf(l2) : f3(1, 0, 0);
        float3 t2 = cross(vh, t1);
        float r = sqrtf(u1), s_, c_;
        sincospif(2.0f * u2, &s_, &c_);
        float p1 = r * c_, p2 = r * s_;
        float s = 0.5f * (1.0f + vh.z);
        p2 = (1.0f - s) * sqrtf(fmaxf(0.0f, 1.0f - p1 * p1)) + s * p2;
        float3 nh = p1 * t1 + p2 * t2 + sqrtf(fmaxf(0.0f, 1.0f - p1 * p1 - p2 * p2)) * vh;
        return normalize(f3(a * nh.x, a * nh.y, fmaxf(1e-6f, nh.z)));
    }
};

// ggx_albedo_table (microfacet.h:276-293). The device holds the complements
// 1 - E and 1 - E_avg, computed in FP64 on the host: the compensation lobe
// divides products of (1 - E) by (1 - E_avg), all near zero for smooth
// surfaces, where forming 1 - E in FP32 would lose most digits. Bilinear
// interpolation of 1 - E equals 1 minus the interpolated E.
MYPBR_DEV float table_one_minus_E(const DeviceScene& S, float c, float alpha) {
    float x = clampf(c, 0.0f, 1.0f) * 31.0f, y = clampf(sqrtf(alpha), 0.0f, 1.0f) * 31.0f;
    int i = min(int(x), 30), j = min(int(y), 30);
    float tx = x - i, ty = y - j;
    const float* e = S.ggx_e;
    float lo = (1.0f - tx) * e[j * 32 + i] + tx * e[j * 32 + i + 1];
    float hi = (1.0f - tx) * e[(j + 1) * 32 + i] + tx * e[(j + 1) * 32 + i + 1];
    return (1.0f - ty) * lo + ty * hi;
}
MYPBR_DEV float table_E(const DeviceScene& S, float c, float alpha) { return 1.0f - table_one_minus_E(S, c, alpha); }
MYPBR_DEV float table_one_minus_Eavg(const DeviceScene& S, float alpha) {
    float y = clampf(sqrtf(alpha), 0.0f, 1.0f) * 31.0f;
    int j = min(int(y), 30);
    float ty = y - j;
    return (1.0f - ty) * S.ggx_eavg[j] + ty * S.ggx_eavg[j + 1];
}
MYPBR_DEV float table_Eavg(const DeviceScene& S, float alpha) { return 1.0f - table_one_minus_Eavg(S, alpha); }
// microfacet.h:341-373
MYPBR_DEV float ms_eval(const DeviceScene& S, float co, float ci, float alpha) {
    if (co <= 0.0f || ci <= 0.0f)
        return 0.0f;
    float miss = table_one_minus_Eavg(S, alpha);
    if (miss < 1e-6f)
        return 0.0f;
    return table_one_minus_E(S, co, alpha) * table_one_minus_E(S, ci, alpha) / (kPi * miss) * ci;
}
MYPBR_DEV float ms_albedo(const DeviceScene& S, float co, float alpha) {
    if (co <= 0.0f || table_one_minus_Eavg(S, alpha) < 1e-6f)
        return 0.0f;
    return table_one_minus_E(S, co, alpha);
}
MYPBR_DEV float3 ms_fresnel_avg(const DeviceScene& S, float3 fa, float alpha) {
    float m = table_one_minus_Eavg(S, alpha), e = 1.0f - m;
    return f3(fa.x * fa.x * e / (1.0f - fa.x * m), fa.y * fa.y * e / (1.0f - fa.y * m),
              fa.z * fa.z * e / (1.0f - fa.z * m));
}
MYPBR_DEV float3 ms_fresnel(const DeviceScene& S, float3 f0, float alpha) {
    return ms_fresnel_avg(S, f0 + (f3(1.0f) - f0) * (1.0f / 21.0f), alpha);
}

// rough_dielectric_bsdf (microfacet.h:384-470); frame +z is n on wo's side
struct RoughGlass {
    float3 n, wo;  // wo in the local frame of n
    float eta;
    Ggx d;
    MYPBR_DEV bool half_vector(float3 wiw, float3& wi, float3& wm, bool& refl) const {
        if (dot(wiw, wiw) == 0.0f || wo.z <= 0.0f)
            return false;
        Onb fr(n);
        wi = normalize(fr.to_local(wiw));
        if (wi.z == 0.0f)
            return false;
        refl = wi.z > 0.0f;
        wm = refl ? wo + wi : wi * eta + wo;
        if (dot(wm, wm) == 0.0f)
            return false;
        wm = normalize(wm);
        if (wm.z < 0.0f)
            wm = -wm;
        if (dot(wm, wi) * wi.z < 0.0f || dot(wm, wo) * wo.z < 0.0f)
            return false;
        return true;
    }
    MYPBR_DEV void eval_pdf(float3 wiw, float& f, float& pdf) const {
        f = pdf = 0.0f;
        float3 wi, wm;
        bool refl;
        if (!half_vector(wiw, wi, wm, refl))
            return;
        float F = fresnel_dielectric(dot(wo, wm), eta);
        if (refl) {
            f = F * d.D(wm) * d.G(wo, wi) / (4.0f * wo.z);
            pdf = F * d.visible_pdf(wo, wm) / (4.0f * fabsf(dot(wo, wm)));
            return;
        }
        float den = dot(wi, wm) + dot(wo, wm) / eta;
        den *= den;
        float ft = (1.0f - F) * d.D(wm) * d.G(wo, wi) * fabsf(dot(wi, wm) * dot(wo, wm) / (wi.z * wo.z * den));
        f = ft / (eta * eta) * fabsf(wi.z);
        pdf = (1.0f - F) * d.visible_pdf(wo, wm) * fabsf(dot(wi, wm)) / den;
    }
    MYPBR_DEV float3 sample(Rng& g) const {
        if (wo.z <= 0.0f)
            return f3(0.0f);
        float u1 = g.next(), u2 = g.next();
        float3 wm = d.sample_visible(wo, u1, u2);
        float F = fresnel_dielectric(dot(wo, wm), eta);
        float3 wi;
        if (g.next() < F) {
            wi = -wo + 2.0f * dot(wo, wm) * wm;
            if (wi.z <= 0.0f)
                return f3(0.0f);
        } else {
            wi = refract(-wo, wm, 1.0f / eta);
            if (wi.z >= 0.0f)
                return f3(0.0f);
        }
        return Onb(n).to_world(wi);
    }
};

// ---------------------------------------------------------- direction pdfs

enum : int { kLobeCosine = 0, kLobeGgx = 1, kLobeGlass = 2, kLobeHg = 3 };

// One strategy of a scatter() pdf: cosine (pdf.h:36-51), GGX visible-normal
// reflection (microfacet.h:215-245), rough glass (microfacet.h:472-482) or
// Henyey-Greenstein (pdf.h:57-89).
struct Lobe {
    int kind;
    float3 n;   // frame axis
    float3 wo;  // GGX / glass: wo in the local frame
    float alpha, eta;
    MYPBR_DEV float value(float3 dir) const {
        if (kind == kLobeCosine)
            return fmaxf(0.0f, dot(normalize(dir), normalize(n)) * kInvPi);
        if (kind == kLobeGgx) {
            if (dot(dir, dir) == 0.0f)
                return 0.0f;
            float3 wi = normalize(Onb(n).to_local(dir));
            if (wi.z <= 0.0f || wo.z <= 0.0f)
                return 0.0f;
            float3 h = normalize(wo + wi);
            Ggx d{alpha};
            return d.visible_pdf(wo, h) / (4.0f * fabsf(dot(wo, h)));
        }
        if (kind == kLobeGlass) {
            RoughGlass rg{n, wo, eta, Ggx{alpha}};
            float f, p;
            rg.eval_pdf(dir, f, p);
            return p;
        }
        float g = alpha;
        float c = dot(normalize(dir), normalize(n));
        float den = 1.0f + g * g - 2.0f * g * c;
        return (1.0f - g * g) / (4.0f * kPi * den * sqrtf(den));
    }
    MYPBR_DEV float3 generate(Rng& rng) const {
        if (kind == kLobeCosine) {
            float r1 = rng.next(), r2 = rng.next();
            float s, c;
            sincospif(2.0f * r1, &s, &c);
            float sr = sqrtf(r2);
            return Onb(n).to_world(f3(c * sr, s * sr, sqrtf(1.0f - r2)));
        }
        if (kind == kLobeGgx) {
            if (wo.z <= 0.0f)
                return f3(0.0f);
            float u1 = rng.next(), u2 = rng.next();
            Ggx d{alpha};
            float3 h = d.sample_visible(wo, u1, u2);
            float3 wi = -wo + 2.0f * dot(wo, h) * h;
            if (wi.z <= 0.0f)
                return f3(0.0f);
            return Onb(n).to_world(wi);
        }
        if (kind == kLobeGlass) {
            RoughGlass rg{n, wo, eta, Ggx{alpha}};
            return rg.sample(rng);
        }
        float g = alpha, xi = rng.next(), ct;
        if (fabsf(g) < 1e-3f) {
            ct = 1.0f - 2.0f * xi;
        } else {
            float s = (1.0f - g * g) / (1.0f - g + 2.0f * g * xi);
            ct = (1.0f + g * g - s * s) / (2.0f * g);
        }
        ct = clampf(ct, -1.0f, 1.0f);
        float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
        float s, c;
        sincospif(2.0f * rng.next(), &s, &c);
        return Onb(n).to_world(f3(c * st, s * st, ct));
    }
};

MYPBR_DEV Lobe cosine_lobe(float3 n) {
    Lobe l;
    l.kind = kLobeCosine;
    l.n = n;
    l.wo = f3(0.0f);
    l.alpha = l.eta = 0.0f;
    return l;
}
MYPBR_DEV Lobe ggx_lobe(float3 n, float3 wo_world, float alpha) {
    Lobe l;
    l.kind = kLobeGgx;
    l.n = n;
    l.wo = normalize(Onb(n).to_local(wo_world));
    l.alpha = alpha;
    l.eta = 0.0f;
    return l;
}

// A scatter() pdf: a mixture of up to three lobes (mixture_pdf nested, pdf.h:111-134).
struct Pdf {
    int n;
    Lobe lobe[3];
    float prob[3];
    // Loops with a constant trip count and static indices keep the lobes in
    // registers (a dynamically indexed array would live in local memory).
    MYPBR_DEV float value(float3 dir) const {
        float s = 0.0f;
#pragma unroll
        for (int k = 0; k < 3; k++)
            if (k < n && prob[k] > 0.0f)
                s += prob[k] * lobe[k].value(dir);
        return s;
    }
    MYPBR_DEV float3 generate(Rng& g) const {
        float xi = g.next();
        int pick = n - 1;
#pragma unroll
        for (int k = 2; k >= 0; k--) {  // the first lobe whose running sum passes xi
            float upto = 0.0f;
#pragma unroll
            for (int j = 0; j <= k; j++)
                upto += prob[j];
            if (k < n - 1 && xi < upto)
                pick = k;
        }
        Lobe l = lobe[0];
#pragma unroll
        for (int k = 1; k < 3; k++)
            if (pick == k)
                l = lobe[k];
        return l.generate(g);
    }
};

// --------------------------------------------------------------- materials

struct ScatterRec {
    float3 attenuation;
    bool skip_pdf;
    float3 skip_dir;
    Pdf pdf;
};

// normal_from_map (material.h:282-308)
MYPBR_DEV float3 normal_from_map(const DeviceScene& S, float3 r_dir, const Surface& rec, int map) {
    const float min_cos_o = 0.01f;
    float3 n = rec.front ? rec.normal : -rec.normal;
    float3 t = rec.dpdu - dot(rec.dpdu, n) * n;
    if (dot(t, t) <= 1e-12f * dot(rec.dpdu, rec.dpdu))
        return rec.normal;
    t = normalize(t);
    float3 b = cross(n, t);
    if (dot(b, rec.dpdv) < 0.0f)
        b = -b;
    float3 c = tex_value(S, map, rec.u, rec.v, rec.p);
    float nz = fmaxf(2.0f * c.z - 1.0f, 1e-3f);
    float3 m = normalize((2.0f * c.x - 1.0f) * t + (2.0f * c.y - 1.0f) * b + nz * n);
    if (!rec.front)
        m = -m;
    float3 wo = normalize(-r_dir);
    float co = dot(m, wo);
    if (co < min_cos_o)
        m = normalize(m + (min_cos_o - co) * wo);
    return m;
}

MYPBR_DEV float3 mat_vec(const DevMaterial& m, int k) { return f3(m.p[k], m.p[k + 1], m.p[k + 2]); }

// The metal's Fresnel curve: Schlick through f0 or the measured conductor (microfacet.h:125-131)
MYPBR_DEV float3 metal_fresnel_at(const DevMaterial& m, float c) {
    if (!(m.flags & kMatMeasured))
        return schlick3(c, mat_vec(m, 0));
    return f3(fresnel_conductor(c, m.p[4], m.p[7]), fresnel_conductor(c, m.p[5], m.p[8]),
              fresnel_conductor(c, m.p[6], m.p[9]));
}

// principled's texture-driven parameters (material.h:508-527)
struct PrincipledAt {
    float3 base;
    float metallic, alpha, coat, coat_alpha;
};
MYPBR_DEV PrincipledAt principled_at(const DeviceScene& S, const DevMaterial& m, const Surface& r) {
    PrincipledAt a;
    a.base = tex_value(S, m.tex[0], r.u, r.v, r.p);
    a.metallic = clampf(tex_value(S, m.tex[1], r.u, r.v, r.p).x, 0.0f, 1.0f);
    a.alpha = rough_to_alpha(clampf(tex_value(S, m.tex[2], r.u, r.v, r.p).x, 0.0f, 1.0f));
    a.coat = (m.flags & kMatCoat) ? clampf(tex_value(S, m.tex[4], r.u, r.v, r.p).x, 0.0f, 1.0f) : 0.0f;
    a.coat_alpha = (m.flags & kMatCoat) ? rough_to_alpha(clampf(tex_value(S, m.tex[5], r.u, r.v, r.p).x, 0.0f, 1.0f))
                                        : 1e-3f;
    return a;
}
MYPBR_DEV float3 spec_f0(const DevMaterial& m, float3 b, float mt) { return (1.0f - mt) * f3(m.p[0]) + mt * b; }
// material.h:536-549
MYPBR_DEV float3 spec_fresnel(const DevMaterial& m, float c, float3 b, float mt) {
    if (!(m.flags & kMatMeasured))
        return schlick3(c, spec_f0(m, b, mt));
    float fd = schlick(c, m.p[0]);
    return (1.0f - mt) * f3(fd) + mt * metal_fresnel_at(m, c);
}
MYPBR_DEV float3 principled_ms_fresnel(const DeviceScene& S, const DevMaterial& m, float3 b, float mt, float alpha) {
    if (!(m.flags & kMatMeasured))
        return ms_fresnel(S, spec_f0(m, b, mt), alpha);
    float fd = m.p[0] + (1.0f - m.p[0]) * (1.0f / 21.0f);
    return ms_fresnel_avg(S, (1.0f - mt) * f3(fd) + mt * mat_vec(m, 10), alpha);
}
// material.h:471-482
MYPBR_DEV float3 coat_transmittance(const DevMaterial& m, float w, float co, float ci) {
    if (!(m.flags & kMatCoatTint))
        return f3(1.0f);
    auto ct = [](float c) {
        c = clampf(c, 0.0f, 1.0f);
        return sqrtf(1.0f - (1.0f - c * c) * (1.0f / 2.25f));
    };
    float e = 0.5f * (1.0f / ct(co) + 1.0f / ct(ci));
    float3 t = f3(powf(m.p[13], e), powf(m.p[14], e), powf(m.p[15], e));
    return (1.0f - w) * f3(1.0f) + w * t;
}
// material.h:486-506
MYPBR_DEV float3 base_eval(const DeviceScene& S, const DevMaterial& m, const PrincipledAt& a, float3 n, float3 wow,
                           float3 wiw) {
    Onb fr(n);
    float3 wo = normalize(fr.to_local(wow)), wi = normalize(fr.to_local(wiw));
    if (wo.z <= 0.0f || wi.z <= 0.0f)
        return f3(0.0f);
    float3 h = normalize(wo + wi);
    Ggx d{a.alpha};
    float3 spec = spec_fresnel(m, dot(wi, h), a.base, a.metallic) * (d.D(h) * d.G(wo, wi) / (4.0f * wo.z)) +
                  principled_ms_fresnel(S, m, a.base, a.metallic, a.alpha) * ms_eval(S, wo.z, wi.z, a.alpha);
    float tr = (1.0f - schlick(wi.z, m.p[0])) * (1.0f - schlick(wo.z, m.p[0]));
    return spec + ((1.0f - a.metallic) * tr * wi.z * kInvPi) * a.base;
}

// scatter() of the material itself (no normal-map wrapper). ONLY >= 0 names
// the material type at compile time, which leaves only that case in the code.
template <int ONLY = -1>
MYPBR_DEV bool scatter_inner(const DeviceScene& S, const DevMaterial& m, float3 r_dir, const Surface& rec,
                             ScatterRec& sr, Rng& g) {
    sr.skip_pdf = false;
    sr.pdf.n = 0;
    switch (ONLY >= 0 ? ONLY : m.type) {
        case kLambertian:  // material.h:79-85
            sr.attenuation = tex_value(S, m.tex[0], rec.u, rec.v, rec.p);
            sr.pdf.n = 1;
            sr.pdf.lobe[0] = cosine_lobe(rec.normal);
            sr.pdf.prob[0] = 1.0f;
            return true;
        case kMetal: {  // material.h:123-150
            float roughness = m.p[3], alpha = rough_to_alpha(roughness);
            float3 wo = normalize(-r_dir);
            if (roughness == 0.0f) {
                sr.attenuation = (m.flags & kMatMeasured) ? metal_fresnel_at(m, dot(rec.normal, wo)) : mat_vec(m, 0);
                sr.skip_pdf = true;
                sr.skip_dir = reflect(normalize(r_dir), rec.normal);
                return true;
            }
            sr.attenuation = mat_vec(m, 0);
            float co = fmaxf(0.0f, dot(rec.normal, wo));
            float msw = ms_albedo(S, co, alpha) * avg3(ms_fresnel_avg(S, mat_vec(m, 10), alpha));
            float ssw = table_E(S, co, alpha) * avg3(metal_fresnel_at(m, co));
            sr.pdf.lobe[0] = ggx_lobe(rec.normal, wo, alpha);
            if (msw <= 0.0f) {
                sr.pdf.n = 1;
                sr.pdf.prob[0] = 1.0f;
                return true;
            }
            float ps = clampf(ssw / (ssw + msw), 0.1f, 1.0f);
            sr.pdf.n = 2;
            sr.pdf.lobe[1] = cosine_lobe(rec.normal);
            sr.pdf.prob[0] = ps;
            sr.pdf.prob[1] = 1.0f - ps;
            return true;
        }
        case kDielectric: {  // material.h:210-242
            float ior = m.p[0], roughness = m.p[1];
            sr.attenuation = f3(1.0f);
            if (roughness > 0.0f) {
                Lobe l;
                l.kind = kLobeGlass;
                l.n = rec.normal;
                l.wo = normalize(Onb(rec.normal).to_local(-r_dir));
                l.eta = rec.front ? ior : 1.0f / ior;
                l.alpha = rough_to_alpha(roughness);
                sr.pdf.n = 1;
                sr.pdf.lobe[0] = l;
                sr.pdf.prob[0] = 1.0f;
                return true;
            }
            sr.skip_pdf = true;
            float ri = rec.front ? 1.0f / ior : ior;
            float3 ud = normalize(r_dir);
            float ct = fminf(dot(-ud, rec.normal), 1.0f), st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
            bool cannot = ri * st > 1.0f;
            if (cannot || fresnel_dielectric(ct, 1.0f / ri) > g.next())
                sr.skip_dir = reflect(ud, rec.normal);
            else
                sr.skip_dir = refract(ud, rec.normal, ri);
            return true;
        }
        case kThinDielectric: {  // material.h:687-702
            float3 ud = normalize(r_dir);
            float ct = fminf(dot(-ud, rec.normal), 1.0f);
            float r = fresnel_dielectric(ct, m.p[0]);
            float refl = 2.0f * r / (1.0f + r);
            sr.skip_pdf = true;
            if (g.next() < refl) {
                sr.attenuation = f3(1.0f);
                sr.skip_dir = reflect(ud, rec.normal);
            } else {
                sr.attenuation = f3(m.p[2], m.p[3], m.p[4]);
                sr.skip_dir = ud;
            }
            return true;
        }
        case kPrincipled: {  // material.h:387-421
            PrincipledAt a = principled_at(S, m, rec);
            float3 wo = normalize(-r_dir);
            float3 nb = m.tex[3] >= 0 ? normal_from_map(S, r_dir, rec, m.tex[3]) : rec.normal;
            float co = fmaxf(0.0f, dot(nb, wo));
            float sw = avg3(spec_fresnel(m, co, a.base, a.metallic));
            float dw = (1.0f - a.metallic) * avg3(a.base) * (1.0f - schlick(co, m.p[0]));
            dw += ms_albedo(S, co, a.alpha) * avg3(principled_ms_fresnel(S, m, a.base, a.metallic, a.alpha));
            float ps = sw + dw > 0.0f ? sw / (sw + dw) : 1.0f;
            ps = clampf(ps, 0.1f, 1.0f);
            sr.attenuation = a.base;
            if (a.coat > 0.0f) {
                float3 nc = m.tex[6] >= 0 ? normal_from_map(S, r_dir, rec, m.tex[6]) : rec.normal;
                float cw = a.coat * schlick(dot(nc, wo), 0.04f);
                float below = (1.0f - cw) * (sw + dw) * avg3(coat_transmittance(m, a.coat, 1.0f, 1.0f));
                float pc = clampf(cw / (cw + below), 0.1f, 0.9f);
                sr.pdf.n = 3;
                sr.pdf.lobe[0] = ggx_lobe(nc, wo, a.coat_alpha);
                sr.pdf.lobe[1] = ggx_lobe(nb, wo, a.alpha);
                sr.pdf.lobe[2] = cosine_lobe(nb);
                sr.pdf.prob[0] = pc;
                sr.pdf.prob[1] = (1.0f - pc) * ps;
                sr.pdf.prob[2] = (1.0f - pc) * (1.0f - ps);
            } else {
                sr.pdf.n = 2;
                sr.pdf.lobe[0] = ggx_lobe(nb, wo, a.alpha);
                sr.pdf.lobe[1] = cosine_lobe(nb);
                sr.pdf.prob[0] = ps;
                sr.pdf.prob[1] = 1.0f - ps;
            }
            return true;
        }
        case kPhase: {  // medium.h:254-260
            sr.attenuation = mat_vec(m, 0);
            Lobe l;
            l.kind = kLobeHg;
            l.n = r_dir;
            l.wo = f3(0.0f);
            l.alpha = m.p[3];  // g
            l.eta = 0.0f;
            sr.pdf.n = 1;
            sr.pdf.lobe[0] = l;
            sr.pdf.prob[0] = 1.0f;
            return true;
        }
        default:
            return false;  // diffuse_light scatters nothing
    }
}

template <int ONLY = -1>
MYPBR_DEV float3 eval_inner(const DeviceScene& S, const DevMaterial& m, float3 r_dir, const Surface& rec, float3 dir) {
    switch (ONLY >= 0 ? ONLY : m.type) {
        case kLambertian: {  // material.h:88-97
            float c = dot(rec.normal, normalize(dir));
            return tex_value(S, m.tex[0], rec.u, rec.v, rec.p) * (c < 0.0f ? 0.0f : c * kInvPi);
        }
        case kMetal: {  // material.h:154-164
            float alpha = rough_to_alpha(m.p[3]);
            Onb fr(rec.normal);
            float3 wo = normalize(fr.to_local(-r_dir)), wi = normalize(fr.to_local(dir));
            if (wo.z <= 0.0f || wi.z <= 0.0f)
                return f3(0.0f);
            float3 h = normalize(wo + wi);
            Ggx d{alpha};
            return metal_fresnel_at(m, dot(wi, h)) * (d.D(h) * d.G(wo, wi) / (4.0f * wo.z)) +
                   ms_fresnel_avg(S, mat_vec(m, 10), alpha) * ms_eval(S, wo.z, wi.z, alpha);
        }
        case kDielectric: {  // material.h:244-249
            if (m.p[1] == 0.0f)
                return f3(0.0f);
            RoughGlass rg;
            rg.n = rec.normal;
            rg.wo = normalize(Onb(rec.normal).to_local(-r_dir));
            rg.eta = rec.front ? m.p[0] : 1.0f / m.p[0];
            rg.d = Ggx{rough_to_alpha(m.p[1])};
            float f, p;
            rg.eval_pdf(dir, f, p);
            return f3(f);
        }
        case kPrincipled: {  // material.h:423-453
            if (dot(dir, rec.normal) <= 0.0f)
                return f3(0.0f);
            PrincipledAt a = principled_at(S, m, rec);
            float3 wo = normalize(-r_dir), wi = normalize(dir);
            float3 nb = m.tex[3] >= 0 ? normal_from_map(S, r_dir, rec, m.tex[3]) : rec.normal;
            float3 below = base_eval(S, m, a, nb, wo, wi);
            if (a.coat <= 0.0f)
                return below;
            float3 nc = m.tex[6] >= 0 ? normal_from_map(S, r_dir, rec, m.tex[6]) : rec.normal;
            float co = dot(nc, wo), ci = dot(nc, wi);
            float through = (1.0f - a.coat * schlick(co, 0.04f)) * (1.0f - a.coat * schlick(ci, 0.04f));
            float3 result = through * coat_transmittance(m, a.coat, co, ci) * below;
            if (co > 0.0f && ci > 0.0f) {
                Onb fr(nc);
                float3 lo = normalize(fr.to_local(wo)), li = normalize(fr.to_local(wi));
                float3 h = normalize(lo + li);
                Ggx d{a.coat_alpha};
                float c = schlick(dot(li, h), 0.04f) * d.D(h) * d.G(lo, li) / (4.0f * lo.z);
                c += ms_fresnel(S, f3(0.04f), a.coat_alpha).x * ms_eval(S, lo.z, li.z, a.coat_alpha);
                result += f3(a.coat * c);
            }
            return result;
        }
        case kPhase: {  // medium.h:265-269
            float c = dot(normalize(r_dir), normalize(dir)), g = m.p[3];
            float den = 1.0f + g * g - 2.0f * g * c;
            return mat_vec(m, 0) * ((1.0f - g * g) / (4.0f * kPi * den * sqrtf(den)));
        }
        default:
            return f3(0.0f);
    }
}

// With the normal_mapped wrapper (material.h:631-674); principled bends its own normals.
MYPBR_DEV bool scatter(const DeviceScene& S, int mi, float3 r_dir, const Surface& rec, ScatterRec& sr, Rng& g) {
    const DevMaterial& m = S.materials[mi];
    if (m.normal_map < 0 || m.type == kPrincipled)
        return scatter_inner(S, m, r_dir, rec, sr, g);
    Surface sh = rec;
    sh.normal = normal_from_map(S, r_dir, rec, m.normal_map);
    if (!scatter_inner(S, m, r_dir, sh, sr, g))
        return false;
    if (sr.skip_pdf) {
        float3 d = sr.skip_dir;
        if (dot(d, sh.normal) > 0.0f && dot(d, rec.normal) < 0.0f)
            sr.skip_dir = d - 2.0f * dot(d, rec.normal) * rec.normal;
    }
    return true;
}

MYPBR_DEV float3 eval(const DeviceScene& S, int mi, float3 r_dir, const Surface& rec, float3 dir) {
    const DevMaterial& m = S.materials[mi];
    if (m.normal_map < 0 || m.type == kPrincipled)
        return eval_inner(S, m, r_dir, rec, dir);
    if (dot(dir, rec.normal) <= 0.0f)
        return f3(0.0f);
    Surface sh = rec;
    sh.normal = normal_from_map(S, r_dir, rec, m.normal_map);
    return eval_inner(S, m, r_dir, sh, dir);
}

// material.h:578-598 (diffuse_light) and :731-736 (emissive_surface)
MYPBR_DEV float3 emitted(const DeviceScene& S, int mi, float3 r_dir, const Surface& rec) {
    const DevMaterial& m = S.materials[mi];
    if (m.emission_tex >= 0)
        return rec.front ? tex_value(S, m.emission_tex, rec.u, rec.v, rec.p) : f3(0.0f);
    if (m.type != kDiffuseLight || !rec.front)
        return f3(0.0f);
    float3 e = mat_vec(m, 0);
    if (m.p[3] >= 180.0f)
        return e;
    float c = -dot(normalize(r_dir), rec.normal);
    if (c <= 0.0f)
        return f3(0.0f);
    float tt = sqrtf(fmaxf(0.0f, 1.0f - c * c)) / c;
    return e * fmaxf(0.0f, 1.0f - tt / m.p[4]);
}

MYPBR_DEV bool may_emit(const DeviceScene& S, int mi) {
    const DevMaterial& m = S.materials[mi];
    return m.emission_tex >= 0 || m.type == kDiffuseLight;
}

// material.h:201-206: Beer-Lambert over the segment that ended on a back face
MYPBR_DEV float3 interior_transmittance(const DeviceScene& S, int mi, float seg_len, bool front) {
    const DevMaterial& m = S.materials[mi];
    if (m.type != kDielectric || front || (m.p[2] == 0.0f && m.p[3] == 0.0f && m.p[4] == 0.0f))
        return f3(1.0f);
    return f3(expf(-m.p[2] * seg_len), expf(-m.p[3] * seg_len), expf(-m.p[4] * seg_len));
}
MYPBR_DEV bool lets_shadows_through(const DeviceScene& S, int mi) {
    const DevMaterial& m = S.materials[mi];
    return m.type == kDielectric && m.p[1] == 0.0f;
}
MYPBR_DEV bool is_volume(const DeviceScene& S, int mi) { return S.materials[mi].type == kPhase; }

// ------------------------------------------------------------------ lights

// environment.h:334-339
MYPBR_DEV void env_angles(const DeviceScene& S, float3 dir, float& u, float& theta) {
    float3 d = normalize(dir);
    theta = acosf(clampf(d.y, -1.0f, 1.0f));
    u = 0.5f + atan2f(d.x, -d.z) * (0.5f * kInvPi) + S.env_rotation;
    u -= floorf(u);
}

// environment.h:202-215 (bilinear)
MYPBR_DEV float3 env_radiance(const DeviceScene& S, float3 dir) {
    float u, theta;
    env_angles(S, dir, u, theta);
    int w = S.env_w, h = S.env_h;
    float x = u * w - 0.5f;
    float y = clampf(theta * kInvPi * h - 0.5f, 0.0f, h - 1.0f);
    float x0 = floorf(x), y0 = floorf(y), fx = x - x0, fy = y - y0;
    int i0 = (int(x0) + w) % w, i1 = (i0 + 1) % w;
    int j0 = int(y0), j1 = min(j0 + 1, h - 1);
    float3 a = f3(ldg4(S.env_pixels + j0 * w + i0)), b = f3(ldg4(S.env_pixels + j0 * w + i1));
    float3 c = f3(ldg4(S.env_pixels + j1 * w + i0)), e = f3(ldg4(S.env_pixels + j1 * w + i1));
    float3 top = (1.0f - fx) * a + fx * b, bot = (1.0f - fx) * c + fx * e;
    return S.env_intensity * ((1.0f - fy) * top + fy * bot);
}

// environment.h:220-228: the texel's probability times W H over 2 pi^2 sin(theta)
MYPBR_DEV float env_pdf(const DeviceScene& S, float3 dir) {
    float u, theta;
    env_angles(S, dir, u, theta);
    float st = sinf(theta);
    if (st <= 0.0f)
        return 0.0f;
    int i = min(max(int(u * S.env_w), 0), S.env_w - 1);
    int j = min(max(int(theta * kInvPi * S.env_h), 0), S.env_h - 1);
    return __ldg(S.env_texel_pdf + j * S.env_w + i) / (2.0f * kPi * kPi * st);
}

// Radiance and density together, from one evaluation of the angles
// (environment.h:202-228).
MYPBR_DEV void env_radiance_pdf(const DeviceScene& S, float3 dir, float3& L, float& pdf) {
    float u, theta;
    env_angles(S, dir, u, theta);
    int w = S.env_w, h = S.env_h;
    float x = u * w - 0.5f;
    float y = clampf(theta * kInvPi * h - 0.5f, 0.0f, h - 1.0f);
    float x0 = floorf(x), y0 = floorf(y), fx = x - x0, fy = y - y0;
    int i0 = (int(x0) + w) % w, i1 = (i0 + 1) % w;
    int j0 = int(y0), j1 = min(j0 + 1, h - 1);
    float3 a = f3(ldg4(S.env_pixels + j0 * w + i0)), b = f3(ldg4(S.env_pixels + j0 * w + i1));
    float3 c = f3(ldg4(S.env_pixels + j1 * w + i0)), e = f3(ldg4(S.env_pixels + j1 * w + i1));
    L = S.env_intensity * ((1.0f - fy) * ((1.0f - fx) * a + fx * b) + fy * ((1.0f - fx) * c + fx * e));
    float st = sinf(theta);
    int i = min(max(int(u * w), 0), w - 1), j = min(max(int(theta * kInvPi * h), 0), h - 1);
    pdf = st > 0.0f ? __ldg(S.env_texel_pdf + j * w + i) / (2.0f * kPi * kPi * st) : 0.0f;
}

// Draws a texel from the alias table (same per-texel probability as the
// reference's marginal / conditional CDFs, environment.h:230-243), then a
// uniform point inside it. With L and pdf, also returns the radiance there
// (bilinear, as env_radiance) and the density of this sampling, read from the
// texel instead of recomputing the angles of the direction.
MYPBR_DEV float3 env_sample(const DeviceScene& S, Rng& g, float3* L = nullptr, float* pdf = nullptr) {
    int n = S.env_w * S.env_h;
    float x = g.next() * n;
    int k = min(int(x), n - 1);
    float2 a = S.env_alias[k];
    float frac = x - k;
    if (frac >= a.x)
        k = __float_as_int(a.y);
    int i = k % S.env_w, j = k / S.env_w;
    float fx = g.next(), fy = g.next();
    float yy = j + fy, xx = i + fx;
    float theta = kPi * yy / S.env_h;
    float phi = 2.0f * kPi * (xx / S.env_w - 0.5f - S.env_rotation);
    float st = sinf(theta), ct = cosf(theta), sp, cp;
    sincosf(phi, &sp, &cp);
    if (L) {
        int w = S.env_w, h = S.env_h;
        float x = xx - 0.5f, y = clampf(yy - 0.5f, 0.0f, h - 1.0f);
        float x0 = floorf(x), y0 = floorf(y), ffx = x - x0, ffy = y - y0;
        int i0 = (int(x0) + w) % w, i1 = (i0 + 1) % w;
        int j0 = int(y0), j1 = min(j0 + 1, h - 1);
        float3 a = f3(ldg4(S.env_pixels + j0 * w + i0)), b = f3(ldg4(S.env_pixels + j0 * w + i1));
        float3 c = f3(ldg4(S.env_pixels + j1 * w + i0)), e = f3(ldg4(S.env_pixels + j1 * w + i1));
        *L = S.env_intensity * ((1.0f - ffy) * ((1.0f - ffx) * a + ffx * b) + ffy * ((1.0f - ffx) * c + ffx * e));
        *pdf = st > 0.0f ? __ldg(S.env_texel_pdf + k) / (2.0f * kPi * kPi * st) : 0.0f;
    }
    return f3(st * sp, ct, -st * cp);
}

// True when the light list is the environment alone and there is no sun:
// NEE then needs no pdf sum and no second angle evaluation.
MYPBR_DEV bool env_only(const DeviceScene& S) {
    return S.light_count == 1 && S.env_w > 0 && !S.sun_enabled && S.lights[0].kind == 1;
}

MYPBR_DEV bool sun_in_cone(const DeviceScene& S, float3 dir) {
    return dot(normalize(dir), S.sun_dir) >= S.sun_cos_max;
}

// One light member's solid-angle density (sphere.h:56-73, quad.h:65-74, mesh.h:115-124).
MYPBR_DEV float member_pdf(const DeviceScene& S, const DevMember& mb, float3 o, float3 d) {
    if (mb.kind == kSphere) {
        float4 sp = ldg4(S.spheres + mb.index);
        int xf = S.sphere_info[mb.index].y;
        float3 lo = o, ld = d;
        if (xf >= 0) {
            XformRef X;
            load_xform(S, xf, X);
            lo = xf_ipoint(X, o);
            ld = xf_ivec(X, d);
        }
        float3 c = f3(sp);
        float t;
        if (!sphere_root(c, sp.w, lo, ld, 0.001f, 3.0e38f, t))
            return 0.0f;
        float r = fabsf(sp.w);
        float d2 = len2(c - lo);
        if (d2 <= r * r) {
            float3 p = lo + t * ld;
            float hd2 = t * t * len2(ld);
            float cosine = fabsf(dot(normalize(ld), (p - c) / r));
            return hd2 / (cosine * 4.0f * kPi * r * r);
        }
        float ctm = sqrtf(fmaxf(0.0f, 1.0f - r * r / d2));
        return 1.0f / (2.0f * kPi * (1.0f - ctm));
    }
    if (mb.kind == kQuad) {
        float t, a, b;
        if (!hit_quad(S, mb.index, o, d, 0.001f, 3.0e38f, t, a, b))
            return 0.0f;
        const float4* q = S.quads + 5 * mb.index;
        float area = length(cross(f3(ldg4(q + 1)), f3(ldg4(q + 2))));
        float3 n = f3(ldg4(q + 3));
        float d2 = t * t * len2(d);
        float cosine = fabsf(dot(d, n)) * rsqrtf(len2(d));
        return d2 / (cosine * area);
    }
    // triangle
    TriRay tr = make_tri_ray(d);
    float t, b1, b2;
    if (!hit_triangle<false>(S, mb.index, o, tr, 0.001f, 3.0e38f, t, b1, b2))
        return 0.0f;
    const float4* tp = S.tris + 3 * mb.index;
    float3 v0 = f3(ldg4(tp));
    float3 c = cross(f3(ldg4(tp + 1)) - v0, f3(ldg4(tp + 2)) - v0);
    float area = 0.5f * length(c);
    float d2 = t * t * len2(d);
    float cosine = fabsf(dot(d, normalize(c))) * rsqrtf(len2(d));
    return d2 / (cosine * area);
}

// A direction towards a random point of the member (sphere.h:75-88, quad.h:76-79, mesh.h:127-136).
MYPBR_DEV float3 member_sample(const DeviceScene& S, const DevMember& mb, float3 o, Rng& g) {
    if (mb.kind == kSphere) {
        float4 sp = ldg4(S.spheres + mb.index);
        int xf = S.sphere_info[mb.index].y;
        XformRef X;
        float3 lo = o;
        if (xf >= 0) {
            load_xform(S, xf, X);
            lo = xf_ipoint(X, o);
        }
        float3 c = f3(sp);
        float r = fabsf(sp.w);
        float3 dir = c - lo;
        float d2 = len2(dir);
        float3 out;
        if (d2 <= r * r) {
            float z = 1.0f - 2.0f * g.next();
            float s, cc;
            sincospif(2.0f * g.next(), &s, &cc);
            float rr = sqrtf(fmaxf(0.0f, 1.0f - z * z));
            out = c + r * f3(rr * cc, rr * s, z) - lo;
        } else {
            float r1 = g.next(), r2 = g.next();
            float z = 1.0f + r2 * (sqrtf(fmaxf(0.0f, 1.0f - r * r / d2)) - 1.0f);
            float s, cc;
            sincospif(2.0f * r1, &s, &cc);
            float rr = sqrtf(fmaxf(0.0f, 1.0f - z * z));
            out = Onb(dir).to_world(f3(cc * rr, s * rr, z));
        }
        return xf >= 0 ? xf_vec(X, out) : out;
    }
    if (mb.kind == kQuad) {
        const float4* q = S.quads + 5 * mb.index;
        float a = g.next(), b = g.next();
        return (f3(ldg4(q)) - o) + a * f3(ldg4(q + 1)) + b * f3(ldg4(q + 2));
    }
    float r1 = g.next(), r2 = g.next();
    if (r1 + r2 > 1.0f) {
        r1 = 1.0f - r1;
        r2 = 1.0f - r2;
    }
    const float4* tp = S.tris + 3 * mb.index;
    float3 v0 = f3(ldg4(tp));
    return (v0 - o) + r1 * (f3(ldg4(tp + 1)) - v0) + r2 * (f3(ldg4(tp + 2)) - v0);
}

MYPBR_DEV float light_pdf_one(const DeviceScene& S, const DevLight& L, float3 o, float3 d) {
    if (L.kind == 1)
        return S.env_w > 0 ? env_pdf(S, d) : 0.0f;
    if (L.kind == 2)
        return sun_in_cone(S, d) ? 1.0f / S.sun_solid_angle : 0.0f;
    float s = 0.0f;
    for (int m = 0; m < L.member_count; m++) {
        DevMember mb = S.members[L.first_member + m];
        s += mb.weight * member_pdf(S, mb, o, d);
    }
    return s;
}

// light_list.h:106-113: sum_k p_k pdf_k
MYPBR_DEV float lights_pdf(const DeviceScene& S, float3 o, float3 d) {
    float s = 0.0f;
    for (int k = 0; k < S.light_count; k++) {
        DevLight L = S.lights[k];
        s += L.probability * light_pdf_one(S, L, o, d);
    }
    return s;
}

// light_list.h:115-127: pick a light by its CDF, then a direction towards it
MYPBR_DEV float3 lights_sample(const DeviceScene& S, float3 o, Rng& g) {
    float xi = g.next();
    int k = 0;
    while (k < S.light_count - 1 && S.lights[k].cdf_hi <= xi)
        k++;
    DevLight L = S.lights[k];
    if (L.kind == 1)
        return env_sample(S, g);
    if (L.kind == 2) {
        float ct = 1.0f - g.next() * (1.0f - S.sun_cos_max);
        float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
        float s, c;
        sincospif(2.0f * g.next(), &s, &c);
        return Onb(S.sun_dir).to_world(f3(c * st, s * st, ct));
    }
    float x = g.next();
    int lo = 0, hi = L.member_count - 1;
    while (lo < hi) {  // first member whose running sum exceeds x
        int mid = (lo + hi) >> 1;
        if (S.members[L.first_member + mid].cdf <= x)
            lo = mid + 1;
        else
            hi = mid;
    }
    return member_sample(S, S.members[L.first_member + lo], o, g);
}

// camera.h:515-529
MYPBR_DEV float3 escaped_radiance(const DeviceScene& S, float3 dir, bool camera_ray) {
    float3 sky;
    if (S.env_w > 0) {
        sky = env_radiance(S, dir);
    } else if (!S.use_sky) {
        sky = S.background;
    } else {
        float3 ud = normalize(dir);
        float a = 0.5f * (ud.y + 1.0f);
        sky = (1.0f - a) * f3(1.0f) + a * f3(0.5f, 0.7f, 1.0f);
    }
    if (S.sun_enabled && (S.sun_disk_visible || !camera_ray) && sun_in_cone(S, dir))
        sky += S.sun_radiance;
    return sky;
}

MYPBR_DEV float power_heuristic(float a, float b) {
    float a2 = a * a, b2 = b * b;
    return (a2 + b2) > 0.0f ? a2 / (a2 + b2) : 0.0f;
}

}  // namespace mypbr_dev
