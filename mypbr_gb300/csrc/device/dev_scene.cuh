// The scene as the kernels see it (FP32, in HBM) and the geometric queries on
// it: primitive intersection, the BVH walk and surface reconstruction.
//
// Layout (built by scene_gpu.cu from the flat FP64 scene):
//   bvh         4 float4 per interior node: child 0 box (lo.xyz | index),
//               (hi.xyz | count), child 1 likewise. count 0: index is an
//               interior node; count > 0: index is the first of `count` leaf
//               references. Boxes are rounded outwards to FP32. Loaded with
//               128-bit loads through the read-only path.
//   leaf_refs   (kind << 29 | index) per leaf slot.
//   spheres     float4 (centre, radius) + int2 (material, xform).
//   quads       5 float4: (Q | material), u, v, unit normal n, w = (u x v) / |u x v|^2.
//   triangles   3 float4 (v0 | material), (v1 | flags), (v2 | mesh); shading
//               indices in tri_shading (n0 n1 n2 t0) (t1 t2 - -).
//   media       3 float4: (a | density), (b | shape), (xform, material, -, -).
//   xforms      6 float4: forward rows (m | t), inverse rows (m^-1 | t^-1).
//   voxels      a model record each (DevVoxelModel); 2 int4 per block:
//               (model, lo xyz), (hi xyz, -); (material, kind) per palette
//               entry, 256 per model; one byte per cell, x fastest.
#pragma once

#include "dev_math.cuh"

namespace mypbr_dev {

// Primitive kinds in leaf references and hits: 0-4 as the flat scene's
// MYPBR_PRIM_*, then the unbounded objects tested beside the tree.
enum : int { kSphere = 0, kQuad = 1, kTriangle = 2, kMedium = 3, kVoxel = 4, kGround = 5, kHeightFog = 6 };

struct DevVoxelModel {
    int nx, ny, nz, xform;
    long long cells;  // offset into voxel_cells
    int palette, edge_material;
    float edge_width, pad0;
    long long kinds;  // offset into voxel_kinds (the cells' kinds under this model's palette)
};

constexpr int kBvhStack = 64;
constexpr int kVoxelBlockMax = 64;  // cells along each side of a voxel block, at most
constexpr uint32_t kKindShift = 29;
constexpr uint32_t kIndexMask = (1u << kKindShift) - 1;

struct DevUnbounded {
    int kind, material;
    float height, density, scale_height, pad0, pad1, pad2;
};

struct DevMaterial {
    int type, flags, normal_map, emission_tex;
    int tex[8];
    float p[16];
};

struct DevTexture {
    int type, a, b, width, height, flags;
    long long offset;
    float p[8];  // the ABI's six parameters (uv transforms: cos and sin of the rotation in p[2], p[5])
};

struct DevLight {
    int kind, first_member, member_count, pad;
    float probability, cdf_hi, pad1, pad2;  // cdf_hi: running sum up to and including this light
};

struct DevMember {
    int kind, index;
    float weight, cdf;  // cdf: running sum within the light up to and including this member
};

struct DeviceScene {
    // geometry
    const float4* bvh;
    const uint32_t* leaf_refs;
    const float4* bvh4;  // the same tree collapsed to 4 children per node (nullptr: not built)
    int bvh4_node_count;
    const uint4* bvh8;   // collapsed to 8 children with quantised boxes (nullptr: not built)
    int bvh8_node_count;
    int postponed_ok;    // leaves small enough to pack into walk_postponed's stack entries
    const float4* spheres;
    const int2* sphere_info;
    const float4* quads;
    const float4* tris;
    const int4* tri_shading;
    const float3* normals;
    const float2* uvs;
    const float4* media;
    const float4* xforms;
    const DevUnbounded* unbounded;
    const DevVoxelModel* voxel_models;
    const int4* voxel_blocks;      // 2 per block: (model, lo xyz), (hi xyz, -)
    const int2* voxel_palettes;    // (material, kind) per palette entry
    const uint8_t* voxel_cells;
    const uint8_t* voxel_kinds;    // per cell: 0 empty, 1 opaque, 2 transparent
    int unbounded_count;
    int has_bvh;
    int bvh_node_count;  // interior nodes; a walk visits each at most once
    int has_media;       // media or height fog present (free-flight sampling needs keys)
    int has_alpha;       // some triangle carries an alpha mask (its coverage test needs keys)
    int has_voxels;      // voxel blocks among the BVH's primitives
    int has_emitters;    // some hittable surface can emit (diffuse light or emissive texture)
    int has_clear_glass; // some hittable surface lets shadows through (smooth dielectric)
    const uint8_t* mat_class;  // shading class of each material
    int* error;          // sticky device error word (0 = none), read by the host after each call
    // appearance
    const DevMaterial* materials;
    const DevTexture* textures;
    const uint8_t* texels_ldr;
    const float* texels_hdr;
    const float* ggx_e;     // 1 - E(mu, alpha), 32 x 32
    const float* ggx_eavg;  // 1 - E_avg(alpha), 32
    // lights
    const DevLight* lights;
    const DevMember* members;
    int light_count;
    // environment
    int env_w, env_h;
    const float4* env_pixels;   // rgb, pad
    const float* env_texel_pdf; // p_ij * W * H
    const float2* env_alias;    // (probability, alias index as float bits)
    float env_intensity, env_rotation;
    // sun
    int sun_enabled, sun_disk_visible;
    float3 sun_dir;
    float sun_cos_max, sun_solid_angle;
    float3 sun_radiance;
    // sky without an environment
    int use_sky;
    float3 background;
};

MYPBR_DEV float4 ldg4(const float4* p) { return __ldg(p); }

// ------------------------------------------------------------- transforms

struct XformRef {
    float4 r[6];
};
MYPBR_DEV void load_xform(const DeviceScene& S, int x, XformRef& X) {
    const float4* p = S.xforms + 6 * x;
#pragma unroll
    for (int k = 0; k < 6; k++)
        X.r[k] = ldg4(p + k);
}
MYPBR_DEV float3 xf_point(const XformRef& X, float3 p) {
    return f3(X.r[0].x * p.x + X.r[0].y * p.y + X.r[0].z * p.z + X.r[0].w,
              X.r[1].x * p.x + X.r[1].y * p.y + X.r[1].z * p.z + X.r[1].w,
              X.r[2].x * p.x + X.r[2].y * p.y + X.r[2].z * p.z + X.r[2].w);
}
MYPBR_DEV float3 xf_vec(const XformRef& X, float3 v) {
    return f3(X.r[0].x * v.x + X.r[0].y * v.y + X.r[0].z * v.z, X.r[1].x * v.x + X.r[1].y * v.y + X.r[1].z * v.z,
              X.r[2].x * v.x + X.r[2].y * v.y + X.r[2].z * v.z);
}
MYPBR_DEV float3 xf_ipoint(const XformRef& X, float3 p) {
    return f3(X.r[3].x * p.x + X.r[3].y * p.y + X.r[3].z * p.z + X.r[3].w,
              X.r[4].x * p.x + X.r[4].y * p.y + X.r[4].z * p.z + X.r[4].w,
              X.r[5].x * p.x + X.r[5].y * p.y + X.r[5].z * p.z + X.r[5].w);
}
MYPBR_DEV float3 xf_ivec(const XformRef& X, float3 v) {
    return f3(X.r[3].x * v.x + X.r[3].y * v.y + X.r[3].z * v.z, X.r[4].x * v.x + X.r[4].y * v.y + X.r[4].z * v.z,
              X.r[5].x * v.x + X.r[5].y * v.y + X.r[5].z * v.z);
}
// Normals map by the inverse transpose.
MYPBR_DEV float3 xf_normal(const XformRef& X, float3 n) {
    return f3(X.r[3].x * n.x + X.r[4].x * n.y + X.r[5].x * n.z, X.r[3].y * n.x + X.r[4].y * n.y + X.r[5].y * n.z,
              X.r[3].z * n.x + X.r[4].z * n.y + X.r[5].z * n.z);
}

// ------------------------------------------------------------ primitives

// Ray/sphere roots in object space with the discriminant formed from the
// squared distance of the centre to the ray's line (Haines et al., "Precision
// Improvements for Ray/Sphere Intersection", Ray Tracing Gems 2019, ch. 7),
// which keeps FP32 accurate for large spheres such as a ground of radius 1000.
// Returns the nearest root in (tmin, tmax), the reference's rule (sphere.h:23-52).
MYPBR_DEV bool sphere_root(float3 c, float r, float3 o, float3 d, float tmin, float tmax, float& t) {
    float a = dot(d, d);
    float3 f = o - c;
    float b = -dot(f, d);  // = dot(d, c - o)
    float3 l = f + (b / a) * d;  // offset of the closest point of the line from the centre
    float disc = a * (r * r - dot(l, l));
    if (disc < 0.0f)
        return false;
    float sq = sqrtf(disc);
    float q = b + copysignf(sq, b);
    float cc = dot(f, f) - r * r;
    float r0 = cc / q, r1 = q / a;
    if (q == 0.0f) {
        r0 = r1 = b / a;
    }
    float lo = fminf(r0, r1), hi = fmaxf(r0, r1);
    if (lo > tmin && lo < tmax) {
        t = lo;
        return true;
    }
    if (hi > tmin && hi < tmax) {
        t = hi;
        return true;
    }
    return false;
}

MYPBR_DEV bool hit_sphere(const DeviceScene& S, int i, float3 o, float3 d, float tmin, float tmax, float& t) {
    float4 s = ldg4(S.spheres + i);
    int xf = __ldg(&S.sphere_info[i].y);
    if (xf < 0)
        return sphere_root(f3(s), s.w, o, d, tmin, tmax, t);
    XformRef X;
    load_xform(S, xf, X);
    return sphere_root(f3(s), s.w, xf_ipoint(X, o), xf_ivec(X, d), tmin, tmax, t);
}

// Plane t, then the parallelogram test 0 <= a, b <= 1 (quad.h:30-62).
MYPBR_DEV bool hit_quad(const DeviceScene& S, int i, float3 o, float3 d, float tmin, float tmax, float& t, float& a,
                        float& b) {
    const float4* q = S.quads + 5 * i;
    float4 Q = ldg4(q), n = ldg4(q + 3);
    float3 N = f3(n);
    float denom = dot(N, d);
    if (fabsf(denom) < 1e-8f)
        return false;
    float tt = dot(N, f3(Q) - o) / denom;
    if (!(tt >= tmin && tt <= tmax))
        return false;
    float3 hp = (o - f3(Q)) + tt * d;
    float3 u = f3(ldg4(q + 1)), v = f3(ldg4(q + 2)), w = f3(ldg4(q + 4));
    float al = dot(w, cross(hp, v)), be = dot(w, cross(u, hp));
    if (al < 0.0f || al > 1.0f || be < 0.0f || be > 1.0f)
        return false;
    t = tt;
    a = al;
    b = be;
    return true;
}

// Per-ray constants of the watertight ray/triangle test (Woop, Benthin and
// Wald, "Watertight Ray/Triangle Intersection", JCGT 2013).
struct TriRay {
    int kx, ky, kz;
    float sx, sy, sz;
};
MYPBR_DEV TriRay make_tri_ray(float3 d) {
    TriRay r;
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    r.kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    r.kx = r.kz == 2 ? 0 : r.kz + 1;
    r.ky = r.kx == 2 ? 0 : r.kx + 1;
    if (comp(d, r.kz) < 0.0f) {
        int tmp = r.kx;
        r.kx = r.ky;
        r.ky = tmp;
    }
    float dz = comp(d, r.kz);
    r.sx = comp(d, r.kx) / dz;
    r.sy = comp(d, r.ky) / dz;
    r.sz = 1.0f / dz;
    return r;
}

// Barycentrics b1, b2 are the weights of v1 and v2, the reference's (u, v)
// without texture coordinates (mesh.h:72-79).
// The coverage test of an alpha-masked triangle (mesh.h:23-26, 81-86): a ray
// meets the surface where the mask's coverage is a with probability a. The
// uniform number is a hash of the ray's key and the triangle, so the answer
// does not depend on the order the walk meets primitives in; with key 0 (a
// query without random numbers) the surface is there wherever a > 0.
// Coverage is the alpha byte / 255, or the grey level without an alpha
// channel (texture.h:132-136), at the nearest texel of the interpolated uv.
MYPBR_DEV bool alpha_covers(const DeviceScene& S, int i, float b1, float b2, uint64_t key) {
    int4 sb = S.tri_shading[2 * i + 1];
    if (sb.z < 0)
        return true;
    int4 sa = S.tri_shading[2 * i];
    float u = b1, v = b2;
    if (sa.w >= 0) {
        float2 t0 = S.uvs[sa.w], t1 = S.uvs[sb.x], t2 = S.uvs[sb.y];
        float b0 = 1.0f - b1 - b2;
        u = b0 * t0.x + b1 * t1.x + b2 * t2.x;
        v = b0 * t0.y + b1 * t1.y + b2 * t2.y;
    }
    const DevTexture& tx = S.textures[sb.z];
    if (tx.flags & 4) {
        u -= floorf(u);
        v -= floorf(v);
    } else {
        u = fminf(fmaxf(u, 0.0f), 1.0f);
        v = fminf(fmaxf(v, 0.0f), 1.0f);
    }
    v = 1.0f - v;
    int x = min(max(int(u * tx.width), 0), tx.width - 1);
    int y = min(max(int(v * tx.height), 0), tx.height - 1);
    long long k = tx.offset + (long long)y * tx.width + x;
    int a = S.texels_ldr[4 * k + ((tx.flags & 8) ? 0 : 3)];
    if (a >= 255)
        return true;
    if (key == 0)
        return a > 0;
    return hash_uniform(key, 0x80000000u | uint32_t(i)) * 255.0f < float(a);
}

// MASKED = false treats an alpha-masked triangle as solid (the light-sampling
// density of a mesh light, which ignores holes as its power estimate does,
// mesh.h:138).
// gamma_n = n u / (1 - n u), u = 2^-24: a bound on the relative error of n
// FP32 roundings (PBRT 3rd ed. section 3.9.1), taken at twice the IEEE
// figure for fast-math reciprocals and square roots.
MYPBR_DEV float err_gamma(int n) {
    const float u = 5.9604645e-8f;
    return 2.0f * float(n) * u / (1.0f - float(n) * u);
}

template <bool MASKED = true>
MYPBR_DEV bool hit_triangle(const DeviceScene& S, int i, float3 o, const TriRay& R, float tmin, float tmax, float& t,
                            float& b1, float& b2, uint64_t key = 0) {
    const float4* tp = S.tris + 3 * i;
    float3 A = f3(ldg4(tp)) - o, B = f3(ldg4(tp + 1)) - o, C = f3(ldg4(tp + 2)) - o;
    float Az = comp(A, R.kz), Bz = comp(B, R.kz), Cz = comp(C, R.kz);
    float Ax = comp(A, R.kx) - R.sx * Az, Ay = comp(A, R.ky) - R.sy * Az;
    float Bx = comp(B, R.kx) - R.sx * Bz, By = comp(B, R.ky) - R.sy * Bz;
    float Cx = comp(C, R.kx) - R.sx * Cz, Cy = comp(C, R.ky) - R.sy * Cz;
    float U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        // Exactly on an edge in FP32: decide in FP64, as the paper prescribes
        U = float(double(Cx) * double(By) - double(Cy) * double(Bx));
        V = float(double(Ax) * double(Cy) - double(Ay) * double(Cx));
        W = float(double(Bx) * double(Ay) - double(By) * double(Ax));
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f))
        return false;
    float det = U + V + W;
    if (det == 0.0f)
        return false;
    float T = R.sz * (U * Az + V * Bz + W * Cz);
    float inv = 1.0f / det;
    float tt = T * inv;
    if (!(tt > tmin && tt < tmax))
        return false;
    {
        // a hit only where t is surely positive: t above the bound on its
        // own rounding error (PBRT 3rd ed. section 3.9.6), from the largest
        // sheared vertex coordinates and edge functions. On long, thin
        // triangles that error can exceed a spawned ray's offset from the
        // surface it leaves, which is then met again just behind the origin.
        float zt = fabsf(R.sz) * fmaxf(fabsf(Az), fmaxf(fabsf(Bz), fabsf(Cz)));
        float xt = fmaxf(fabsf(Ax), fmaxf(fabsf(Bx), fabsf(Cx)));
        float yt = fmaxf(fabsf(Ay), fmaxf(fabsf(By), fabsf(Cy)));
        float dz = err_gamma(3) * zt;
        float dx = err_gamma(5) * (xt + zt), dy = err_gamma(5) * (yt + zt);
        float de = 2.0f * (err_gamma(2) * xt * yt + dy * xt + dx * yt);
        float me = fmaxf(fabsf(U), fmaxf(fabsf(V), fabsf(W)));
        float dt = 3.0f * (err_gamma(3) * me * zt + de * zt + dz * me) * fabsf(inv);
        if (tt <= dt)
            return false;
    }
    // checked before the caller's closest hit changes (mesh.h:81-86)
    if (MASKED && S.has_alpha && !alpha_covers(S, i, V * inv, W * inv, key))
        return false;
    t = tt;
    b1 = V * inv;
    b2 = W * inv;
    return true;
}

// Where a line enters and leaves a medium's convex boundary (medium.h:298-302).
MYPBR_DEV bool medium_span(const DeviceScene& S, int i, float3 o, float3 d, float& t_in, float& t_out, float& density,
                           int& material) {
    const float4* m = S.media + 3 * i;
    float4 A = ldg4(m), B = ldg4(m + 1), C = ldg4(m + 2);
    density = A.w;
    int shape = __float_as_int(B.w), xf = __float_as_int(C.x);
    material = __float_as_int(C.y);
    float3 lo = o, ld = d;
    if (xf >= 0) {
        XformRef X;
        load_xform(S, xf, X);
        lo = xf_ipoint(X, o);
        ld = xf_ivec(X, d);
    }
    if (shape == 0) {
        float3 c = f3(A);
        float r = B.x;
        float a = dot(ld, ld);
        float3 f = lo - c;
        float b = -dot(f, ld);
        float3 l = f + (b / a) * ld;
        float disc = a * (r * r - dot(l, l));
        if (disc < 0.0f)
            return false;
        float sq = sqrtf(disc);
        t_in = (b - sq) / a;
        t_out = (b + sq) / a;
        return t_out > t_in + 0.0001f;
    }
    float t0 = -3.0e38f, t1 = 3.0e38f;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        float mn = fminf(comp(f3(A), k), comp(f3(B), k)), mx = fmaxf(comp(f3(A), k), comp(f3(B), k));
        float dk = comp(ld, k), ok = comp(lo, k);
        if (dk == 0.0f) {
            if (ok < mn || ok > mx)
                return false;
            continue;
        }
        float ta = (mn - ok) / dk, tb = (mx - ok) / dk;
        t0 = fmaxf(t0, fminf(ta, tb));
        t1 = fminf(t1, fmaxf(ta, tb));
    }
    t_in = t0;
    t_out = t1;
    return t1 > t0 + 0.0001f;
}

// Free-flight sampling in a homogeneous medium (medium.h:295-323): xi is the
// ray's uniform number for this medium.
MYPBR_DEV bool hit_medium(const DeviceScene& S, int i, float3 o, float3 d, float tmin, float tmax, float xi, float& t) {
    float a, b, density;
    int mat;
    if (!medium_span(S, i, o, d, a, b, density, mat))
        return false;
    float t0 = fmaxf(a, tmin), t1 = fminf(b, tmax);
    if (t0 >= t1)
        return false;
    float len = length(d);
    float dist = -logf(1.0f - xi) / density;
    if (dist > (t1 - t0) * len)
        return false;
    t = t0 + dist / len;
    return true;
}

// ----------------------------------------------------------------- voxels

// The kind of a cell of the whole model (kinds hold one byte per cell:
// 0 empty, 1 opaque, 2 transparent, precomputed from the palette), 0 outside
// it (voxel.h:284-288).
MYPBR_DEV int voxel_kind_at(const DevVoxelModel& m, const uint8_t* kinds, int x, int y, int z) {
    if (unsigned(x) >= unsigned(m.nx) || unsigned(y) >= unsigned(m.ny) || unsigned(z) >= unsigned(m.nz))
        return 0;
    return __ldg(kinds + (size_t(z) * m.ny + y) * m.nx + x);
}

MYPBR_DEV bool voxel_face_visible(int k, int n) {  // voxel.h:100-106
    if (k == 0)
        return false;
    if (n == 0)
        return true;
    return k == 1 && n == 2;
}

// on_edge (voxel.h:313-331): within width of an outline of the shapes.
MYPBR_DEV bool voxel_on_edge(const DevVoxelModel& m, const uint8_t* kinds, float3 p, int axis, int sign,
                             const int cell[3]) {
    int k = voxel_kind_at(m, kinds, cell[0], cell[1], cell[2]);
    for (int side = 1; side <= 2; side++) {
        int tangent = (axis + side) % 3;
        float f = comp(p, tangent) - float(cell[tangent]);
        for (int dir = -1; dir <= 1; dir += 2) {
            if ((dir > 0 ? 1.0f - f : f) >= m.edge_width)
                continue;
            int beside[3] = {cell[0], cell[1], cell[2]};
            beside[tangent] += dir;
            int above[3] = {beside[0], beside[1], beside[2]};
            above[axis] += sign;
            if (voxel_face_visible(k, voxel_kind_at(m, kinds, beside[0], beside[1], beside[2])) ||
                voxel_kind_at(m, kinds, above[0], above[1], above[2]) != 0)
                return true;
        }
    }
    return false;
}

// The hit on the face of cell (x, y, z) whose outward normal is along axis
// with the given sign: material (the cell's palette entry, or the outline's).
MYPBR_DEV int voxel_face_material(const DeviceScene& S, const DevVoxelModel& m, const uint8_t* kinds, float3 p,
                                  int axis, int sign, int x, int y, int z) {
    int cell[3] = {x, y, z};
    if (m.edge_width > 0.0f && voxel_on_edge(m, kinds, p, axis, sign, cell))
        return m.edge_material;
    int idx = __ldg(S.voxel_cells + m.cells + (size_t(z) * m.ny + y) * m.nx + x);
    return __ldg(&S.voxel_palettes[m.palette + idx].x);
}

// A crossing from a cell of kind kf into one of kind kt along +-axis: which
// face is a surface, if any (crossing, voxel.h:294-305). 1: the entered
// cell's face; 2: the face of the cell being left, seen from inside; 0: none.
MYPBR_DEV int voxel_crossing(int kf, int kt) {
    if (kt != 0 && voxel_face_visible(kt, kf))
        return 1;
    return voxel_face_visible(kf, kt) ? 2 : 0;
}

// Block i of a placed voxel model, walked cell by cell with a 3D DDA
// (Amanatides and Woo 1987) in the model's space, as voxel_grid::hit
// (voxel.h:193-268). A surface is a crossing between cells of different kind.
// On a hit: t, the material and face = axis | (outward normal positive) << 2.
// The walk keeps its cell, step and next-plane distances in scalars (no
// dynamically indexed arrays, which would live in local memory).
MYPBR_DEV bool hit_voxel_block(const DeviceScene& S, int i, float3 ow, float3 dw, float tmin, float tmax, float& t_out,
                               int& mat_out, int& face_out) {
    int4 b0 = __ldg(S.voxel_blocks + 2 * i), b1 = __ldg(S.voxel_blocks + 2 * i + 1);
    const DevVoxelModel m = S.voxel_models[b0.x];
    XformRef X;
    load_xform(S, m.xform, X);
    float3 o = xf_ipoint(X, ow), d = xf_ivec(X, dw);
    const uint8_t* kinds = S.voxel_kinds + m.kinds;
    const float lox = float(b0.y), loy = float(b0.z), loz = float(b0.w);
    const float hix = float(b1.x), hiy = float(b1.y), hiz = float(b1.z);
    // where the ray's line enters and leaves the block
    float t_enter = -3.0e38f, t_exit = 3.0e38f;
    int enter_axis = 0;
#define MYPBR_SLAB(A, DA, OA, LO, HI)                  \
    if (DA == 0.0f) {                                  \
        if (OA < LO || OA > HI)                        \
            return false;                              \
    } else {                                           \
        float t0 = (LO - OA) / DA, t1 = (HI - OA) / DA; \
        if (t0 > t1) {                                 \
            float tmp = t0;                            \
            t0 = t1;                                   \
            t1 = tmp;                                  \
        }                                              \
        if (t0 > t_enter) {                            \
            t_enter = t0;                              \
            enter_axis = A;                            \
        }                                              \
        t_exit = fminf(t_exit, t1);                    \
    }
    MYPBR_SLAB(0, d.x, o.x, lox, hix)
    MYPBR_SLAB(1, d.y, o.y, loy, hiy)
    MYPBR_SLAB(2, d.z, o.z, loz, hiz)
#undef MYPBR_SLAB
    bool from_outside = t_enter >= tmin;
    float t_start = from_outside ? t_enter : tmin;
    if (t_start > fminf(t_exit, tmax))
        return false;
    float3 start = o + t_start * d;
    int cx = min(max(int(floorf(start.x)), b0.y), b1.x - 1);
    int cy = min(max(int(floorf(start.y)), b0.z), b1.y - 1);
    int cz = min(max(int(floorf(start.z)), b0.w), b1.z - 1);
    if (from_outside) {  // the layer just inside the entry face
        if (enter_axis == 0)
            cx = d.x > 0.0f ? b0.y : b1.x - 1;
        else if (enter_axis == 1)
            cy = d.y > 0.0f ? b0.z : b1.y - 1;
        else
            cz = d.z > 0.0f ? b0.w : b1.z - 1;
    }
    const int sx = d.x > 0.0f ? 1 : (d.x < 0.0f ? -1 : 0);
    const int sy = d.y > 0.0f ? 1 : (d.y < 0.0f ? -1 : 0);
    const int sz = d.z > 0.0f ? 1 : (d.z < 0.0f ? -1 : 0);
    float tnx = sx > 0 ? (cx + 1 - o.x) / d.x : (sx < 0 ? (cx - o.x) / d.x : 3.0e38f);
    float tny = sy > 0 ? (cy + 1 - o.y) / d.y : (sy < 0 ? (cy - o.y) / d.y : 3.0e38f);
    float tnz = sz > 0 ? (cz + 1 - o.z) / d.z : (sz < 0 ? (cz - o.z) / d.z : 3.0e38f);
    const float tdx = sx != 0 ? fabsf(1.0f / d.x) : 3.0e38f;
    const float tdy = sy != 0 ? fabsf(1.0f / d.y) : 3.0e38f;
    const float tdz = sz != 0 ? fabsf(1.0f / d.z) : 3.0e38f;
    int k_cur = voxel_kind_at(m, kinds, cx, cy, cz);
    if (from_outside) {
        // crossing into the block from the cell behind the entry face
        int bx = cx - (enter_axis == 0 ? sx : 0), by = cy - (enter_axis == 1 ? sy : 0),
            bz = cz - (enter_axis == 2 ? sz : 0);
        int stp = enter_axis == 0 ? sx : (enter_axis == 1 ? sy : sz);
        int which = voxel_crossing(voxel_kind_at(m, kinds, bx, by, bz), k_cur);
        if (which != 0) {
            int sign = which == 1 ? -stp : stp;
            t_out = t_enter;
            face_out = enter_axis | (sign > 0 ? 4 : 0);
            float3 p = o + t_enter * d;
            mat_out = which == 1 ? voxel_face_material(S, m, kinds, p, enter_axis, sign, cx, cy, cz)
                                 : voxel_face_material(S, m, kinds, p, enter_axis, sign, bx, by, bz);
            return true;
        }
    }
    // the walk stays inside the block: at most its three extents of steps
    for (int guard = 0; guard < 3 * kVoxelBlockMax + 4; guard++) {
        int a = tnx < tny ? (tnx < tnz ? 0 : 2) : (tny < tnz ? 1 : 2);
        float t;
        int px = cx, py = cy, pz = cz, stp;
        bool left;
        if (a == 0) {
            t = tnx;
            cx += sx;
            tnx += tdx;
            stp = sx;
            left = cx < b0.y || cx >= b1.x;
        } else if (a == 1) {
            t = tny;
            cy += sy;
            tny += tdy;
            stp = sy;
            left = cy < b0.z || cy >= b1.y;
        } else {
            t = tnz;
            cz += sz;
            tnz += tdz;
            stp = sz;
            left = cz < b0.w || cz >= b1.z;
        }
        if (t > tmax)
            return false;
        int k_next = voxel_kind_at(m, kinds, cx, cy, cz);
        int which = voxel_crossing(k_cur, k_next);
        if (which != 0) {
            int sign = which == 1 ? -stp : stp;
            t_out = t;
            face_out = a | (sign > 0 ? 4 : 0);
            float3 p = o + t * d;
            mat_out = which == 1 ? voxel_face_material(S, m, kinds, p, a, sign, cx, cy, cz)
                                 : voxel_face_material(S, m, kinds, p, a, sign, px, py, pz);
            return true;
        }
        if (left)
            return false;  // left the block
        k_cur = k_next;
    }
    return false;
}

// ------------------------------------------------------------- traversal

struct HitInfo {
    float t, b1, b2;
    uint32_t prim;  // kind << 29 | index; 0xffffffff: miss
};
constexpr uint32_t kMiss = 0xffffffffu;

MYPBR_DEV float safe_inv(float x) { return fabsf(x) > 1e-30f ? 1.0f / x : copysignf(1e30f, x); }

// The closest hit along o + t d, t in (tmin, tmax): the BVH, then the
// unbounded objects beside it (main.cpp:70-74 of the reference). media_key
// seeds free-flight sampling in media; media_key == 0 skips media (used by the
// deterministic ray-batch query).
// VOX: whether voxel blocks are tested (kernels for scenes without voxels
// leave that code out, and with it its registers).
// WALK: which walk. 0: the binary tree, leaves tested as soon as they are
// met; 1: the 4-wide tree (S.bvh4); 2: the binary tree with leaves postponed
// until every lane of the warp holds one (walk_postponed).
enum : int { kWalkBinary = 0, kWalkWide = 1, kWalkPostponed = 2, kWalkWide8 = 3 };
template <bool ANY, bool VOX = true, int WALK = kWalkBinary>
MYPBR_DEV HitInfo walk(const DeviceScene& S, float3 o, float3 d, float tmin, float tmax, uint64_t media_key);

template <bool VOX = true, int WALK = kWalkBinary>
MYPBR_DEV HitInfo closest_hit(const DeviceScene& S, float3 o, float3 d, float tmin, float tmax, uint64_t media_key) {
    return walk<false, VOX, WALK>(S, o, d, tmin, tmax, media_key);
}

// Whether anything at all lies along o + t d, t in (tmin, tmax): the walk stops
// at the first primitive it hits. For shadow rays in scenes where nothing
// hittable can emit, this is all the reference's closest-hit query decides.
template <bool VOX = true, int WALK = kWalkBinary>
MYPBR_DEV bool any_hit(const DeviceScene& S, float3 o, float3 d, float tmin, float tmax, uint64_t media_key) {
    return walk<true, VOX, WALK>(S, o, d, tmin, tmax, media_key).prim != 0xffffffffu;
}

// A ray's BVH walk, advanced one interior node at a time (walk_node), so that
// a persistent kernel can give a lane a new ray as soon as its last one is
// done instead of waiting for the slowest lane of its warp.
struct WalkState {
    float3 o, d, inv, oi;
    TriRay tr;
    float tmin;
    uint64_t media_key;
    HitInfo h;
    int node, sp, visits;
};
// The walk's stack lives beside its state (a kBvhStack-entry local array),
// so that the state's scalars can stay in registers.

MYPBR_DEV void walk_init(const DeviceScene& S, WalkState& W, float3 o, float3 d, float tmin, float tmax,
                         uint64_t media_key) {
    W.o = o;
    W.d = d;
    W.tmin = tmin;
    W.media_key = media_key;
    W.h.prim = kMiss;
    W.h.t = tmax;
    W.h.b1 = W.h.b2 = 0.0f;
    W.inv = f3(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
    W.oi = -1.0f * (o * W.inv);
    W.tr = make_tri_ray(d);
    W.node = 0;
    W.sp = S.has_bvh ? 0 : -1;  // -1: nothing (left) to walk
    W.visits = 0;
}

// One interior node: slab tests of both children, the primitives of child
// leaves, then the next node. Returns false once the walk is over (or, with
// ANY, a hit was found).
template <bool ANY, bool VOX>
MYPBR_DEV bool walk_node(const DeviceScene& S, WalkState& W, int* stack) {
    if (W.sp < 0)
        return false;
    // A tree walk enters each interior node at most once; the cap only guards
    // against a malformed tree, which it reports instead of spinning.
    if (++W.visits > S.bvh_node_count + 1) {
        atomicCAS(S.error, 0, 1);
        W.sp = -1;
        return false;
    }
    const float3 o = W.o, d = W.d, inv = W.inv, oi = W.oi;
    const float tmin = W.tmin;
    HitInfo& h = W.h;
    const float4* n = S.bvh + 4 * W.node;
    float4 a0 = ldg4(n), a1 = ldg4(n + 1), c0 = ldg4(n + 2), c1 = ldg4(n + 3);
    // slab tests of both children against (tmin, best)
    float lx0 = fmaf(a0.x, inv.x, oi.x), hx0 = fmaf(a1.x, inv.x, oi.x);
    float ly0 = fmaf(a0.y, inv.y, oi.y), hy0 = fmaf(a1.y, inv.y, oi.y);
    float lz0 = fmaf(a0.z, inv.z, oi.z), hz0 = fmaf(a1.z, inv.z, oi.z);
    float n0 = fmaxf(fmaxf(fminf(lx0, hx0), fminf(ly0, hy0)), fmaxf(fminf(lz0, hz0), tmin));
    float f0 = fminf(fminf(fmaxf(lx0, hx0), fmaxf(ly0, hy0)), fminf(fmaxf(lz0, hz0), h.t));
    float lx1 = fmaf(c0.x, inv.x, oi.x), hx1 = fmaf(c1.x, inv.x, oi.x);
    float ly1 = fmaf(c0.y, inv.y, oi.y), hy1 = fmaf(c1.y, inv.y, oi.y);
    float lz1 = fmaf(c0.z, inv.z, oi.z), hz1 = fmaf(c1.z, inv.z, oi.z);
    float n1 = fmaxf(fmaxf(fminf(lx1, hx1), fminf(ly1, hy1)), fmaxf(fminf(lz1, hz1), tmin));
    float f1 = fminf(fminf(fmaxf(lx1, hx1), fmaxf(ly1, hy1)), fminf(fmaxf(lz1, hz1), h.t));
    // A small relative widening keeps FP32 slab tests conservative
    bool h0 = n0 <= f0 * 1.00000024f + 1e-30f;
    bool h1 = n1 <= f1 * 1.00000024f + 1e-30f;
    int i0 = __float_as_int(a0.w), k0 = __float_as_int(a1.w);
    int i1 = __float_as_int(c0.w), k1 = __float_as_int(c1.w);
#pragma unroll
    for (int side = 0; side < 2; side++) {
        bool hit = side == 0 ? h0 : h1;
        int cnt = side == 0 ? k0 : k1;
        int first = side == 0 ? i0 : i1;
        if (!(hit && cnt > 0))
            continue;
        for (int k = 0; k < cnt; k++) {
            uint32_t ref = __ldg(S.leaf_refs + first + k);
            int kind = int(ref >> kKindShift), idx = int(ref & kIndexMask);
            float t, b1 = 0.0f, b2 = 0.0f;
            bool got = false;
            if (kind == kTriangle) {
                got = hit_triangle(S, idx, o, W.tr, tmin, h.t, t, b1, b2, W.media_key);
            } else if (kind == kSphere) {
                got = hit_sphere(S, idx, o, d, tmin, h.t, t);
            } else if (kind == kQuad) {
                got = hit_quad(S, idx, o, d, tmin, h.t, t, b1, b2);
            } else if (kind == kMedium && W.media_key != 0) {
                got = hit_medium(S, idx, o, d, tmin, h.t, hash_uniform(W.media_key, uint32_t(idx)), t);
            } else if (VOX && kind == kVoxel) {
                int mat, face;
                got = hit_voxel_block(S, idx, o, d, tmin, h.t, t, mat, face);
                b1 = __int_as_float(mat);
                b2 = __int_as_float(face);
            }
            if (got) {
                h.t = t;
                h.b1 = b1;
                h.b2 = b2;
                h.prim = ref;
                if (ANY) {
                    W.sp = -1;
                    return false;
                }
            }
        }
    }
    h0 = h0 && k0 == 0;
    h1 = h1 && k1 == 0;
    if (h0 && h1) {
        bool first0 = n0 <= n1;
        if (W.sp == kBvhStack) {  // deeper than the host-checked depth: report, stop
            atomicCAS(S.error, 0, 2);
            W.sp = -1;
            return false;
        }
        stack[W.sp++] = first0 ? i1 : i0;
        W.node = first0 ? i0 : i1;
    } else if (h0) {
        W.node = i0;
    } else if (h1) {
        W.node = i1;
    } else {
        if (W.sp == 0) {
            W.sp = -1;
            return false;
        }
        W.node = stack[--W.sp];
    }
    return true;
}

// The unbounded objects beside the BVH, after the walk.
template <bool ANY>
MYPBR_DEV void walk_unbounded(const DeviceScene& S, WalkState& W) {
    const float3 o = W.o, d = W.d;
    const float tmin = W.tmin;
    const uint64_t media_key = W.media_key;
    HitInfo& h = W.h;
    if (ANY && h.prim != kMiss)
        return;
    // The ground (plane.h:17-34) and height fog (medium.h:352-381) beside the BVH
    for (int k = 0; k < S.unbounded_count; k++) {
        DevUnbounded ub = S.unbounded[k];
        if (ub.kind == 0) {
            if (fabsf(d.y) < 1e-12f)
                continue;
            float t = (ub.height - o.y) / d.y;
            if (t > tmin && t < h.t) {
                h.t = t;
                h.prim = (uint32_t(kGround) << kKindShift) | uint32_t(k);
                if (ANY)
                    return;
            }
        } else if (media_key != 0) {
            float len = length(d);
            float kk = d.y / ub.scale_height;
            float start = ub.density * len * expf(-(o.y + tmin * d.y - ub.height) / ub.scale_height);
            if (!(start > 0.0f))
                continue;
            float tau = -logf(1.0f - hash_uniform(media_key, 0x40000000u + uint32_t(k)));
            float t;
            if (fabsf(kk) < 1e-12f) {
                t = tmin + tau / start;
            } else {
                float x = 1.0f - tau * kk / start;
                if (x <= 0.0f)
                    continue;
                t = tmin - logf(x) / kk;
            }
            if (t < h.t && isfinite(t)) {
                h.t = t;
                h.prim = (uint32_t(kHeightFog) << kKindShift) | uint32_t(k);
                if (ANY)
                    return;
            }
        }
    }
}

// The primitives of one leaf (count refs from first) against the ray; true
// when ANY and one was hit.
template <bool ANY, bool VOX>
MYPBR_DEV bool test_leaf(const DeviceScene& S, int first, int count, float3 o, float3 d, const TriRay& tr, float tmin,
                         uint64_t media_key, HitInfo& h) {
    for (int k = 0; k < count; k++) {
        uint32_t ref = __ldg(S.leaf_refs + first + k);
        int kind = int(ref >> kKindShift), idx = int(ref & kIndexMask);
        float t, b1 = 0.0f, b2 = 0.0f;
        bool got = false;
        if (kind == kTriangle) {
            got = hit_triangle(S, idx, o, tr, tmin, h.t, t, b1, b2, media_key);
        } else if (kind == kSphere) {
            got = hit_sphere(S, idx, o, d, tmin, h.t, t);
        } else if (kind == kQuad) {
            got = hit_quad(S, idx, o, d, tmin, h.t, t, b1, b2);
        } else if (kind == kMedium && media_key != 0) {
            got = hit_medium(S, idx, o, d, tmin, h.t, hash_uniform(media_key, uint32_t(idx)), t);
        } else if (VOX && kind == kVoxel) {
            int mat, face;
            got = hit_voxel_block(S, idx, o, d, tmin, h.t, t, mat, face);
            b1 = __int_as_float(mat);
            b2 = __int_as_float(face);
        }
        if (got) {
            h.t = t;
            h.b1 = b1;
            h.b2 = b2;
            h.prim = ref;
            if (ANY)
                return true;
        }
    }
    return false;
}

MYPBR_DEV int pick4(int4 v, int c) { return c == 0 ? v.x : (c == 1 ? v.y : (c == 2 ? v.z : v.w)); }

// The walk over the 4-wide tree. A node (8 float4, 128 B) holds its four
// children's boxes as rows (x lo, x hi, y lo, y hi, z lo, z hi; one lane per
// child), their indices and their kinds (count > 0: a leaf of that many
// references from the index; 0: an interior node; -1: an empty slot). Leaves
// among the children a ray meets are tested at once; the interior ones still
// nearer than the closest hit are visited nearest first (a five-comparison
// sorting network), the others pushed. The host bounds the stack (three
// entries per level) before it enables this walk.
constexpr int kBvh4Stack = 64;
template <bool ANY, bool VOX>
MYPBR_DEV bool walk_tree4(const DeviceScene& S, float3 o, float3 d, float tmin, uint64_t media_key, HitInfo& h) {
    float3 inv = f3(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
    float3 oi = -1.0f * (o * inv);
    TriRay tr = make_tri_ray(d);
    int stack[kBvh4Stack];
    int sp = 0;
    int node = 0;
    int visits = 0;
    while (true) {
        if (++visits > S.bvh4_node_count + 1) {  // a tree walk enters each node at most once
            atomicCAS(S.error, 0, 1);
            return false;
        }
        const float4* n = S.bvh4 + 8 * node;
        float4 xl = ldg4(n), xh = ldg4(n + 1), yl = ldg4(n + 2), yh = ldg4(n + 3), zl = ldg4(n + 4),
               zh = ldg4(n + 5);
        int4 child = __ldg(reinterpret_cast<const int4*>(n + 6));
        int4 count = __ldg(reinterpret_cast<const int4*>(n + 7));
        float near[4];
        unsigned leaves = 0, inner = 0;
#pragma unroll
        for (int c = 0; c < 4; c++) {
            float ax = comp4(xl, c), bx = comp4(xh, c), ay = comp4(yl, c), by = comp4(yh, c), az = comp4(zl, c),
                  bz = comp4(zh, c);
            float lx = fmaf(ax, inv.x, oi.x), hx = fmaf(bx, inv.x, oi.x);
            float ly = fmaf(ay, inv.y, oi.y), hy = fmaf(by, inv.y, oi.y);
            float lz = fmaf(az, inv.z, oi.z), hz = fmaf(bz, inv.z, oi.z);
            float tn = fmaxf(fmaxf(fminf(lx, hx), fminf(ly, hy)), fmaxf(fminf(lz, hz), tmin));
            float tf = fminf(fminf(fmaxf(lx, hx), fmaxf(ly, hy)), fminf(fmaxf(lz, hz), h.t));
            int cnt = pick4(count, c);
            // a small relative widening keeps FP32 slab tests conservative
            bool met = tn <= tf * 1.00000024f + 1e-30f && cnt >= 0;
            near[c] = tn;
            leaves |= (met && cnt > 0) ? 1u << c : 0u;
            inner |= (met && cnt == 0) ? 1u << c : 0u;
        }
        for (unsigned m = leaves; m; m &= m - 1) {
            int c = __ffs(m) - 1;
            if (test_leaf<ANY, VOX>(S, pick4(child, c), pick4(count, c), o, d, tr, tmin, media_key, h))
                return true;
        }
        // the interior children still nearer than the closest hit, nearest first
        float k0 = (inner & 1u) && near[0] <= h.t ? near[0] : INFINITY;
        float k1 = (inner & 2u) && near[1] <= h.t ? near[1] : INFINITY;
        float k2 = (inner & 4u) && near[2] <= h.t ? near[2] : INFINITY;
        float k3 = (inner & 8u) && near[3] <= h.t ? near[3] : INFINITY;
        int c0 = child.x, c1 = child.y, c2 = child.z, c3 = child.w;
        auto cswap = [](float& ka, int& ca, float& kb, int& cb) {
            if (kb < ka) {
                float tk = ka;
                ka = kb;
                kb = tk;
                int tc = ca;
                ca = cb;
                cb = tc;
            }
        };
        cswap(k0, c0, k1, c1);
        cswap(k2, c2, k3, c3);
        cswap(k0, c0, k2, c2);
        cswap(k1, c1, k3, c3);
        cswap(k1, c1, k2, c2);
        int pushes = (k1 < INFINITY) + (k2 < INFINITY) + (k3 < INFINITY);
        if (sp + pushes > kBvh4Stack) {  // deeper than the host-checked bound: report, stop
            atomicCAS(S.error, 0, 2);
            return false;
        }
        if (k3 < INFINITY)
            stack[sp++] = c3;
        if (k2 < INFINITY)
            stack[sp++] = c2;
        if (k1 < INFINITY)
            stack[sp++] = c1;
        if (k0 < INFINITY) {
            node = c0;
        } else {
            if (sp == 0)
                return false;
            node = stack[--sp];
        }
    }
}

// The binary walk with leaves postponed (Aila and Laine, "Understanding the
// Efficiency of Ray Traversal on GPUs", HPG 2009): a lane that meets a leaf
// keeps it aside and walks on through inner nodes until every active lane of
// its warp holds a leaf (or is done); then the warp tests its leaves
// together. The stack holds inner nodes (>= 0) and leaves (~(first << 4 |
// count), below 0); the host enables this walk only when every leaf has
// fewer than 16 references and the references number fewer than 2^26.
// Returns true when ANY and a hit was found.
constexpr int kWalkDone = int(0x80000000u);
template <bool ANY, bool VOX>
MYPBR_DEV bool walk_postponed(const DeviceScene& S, float3 o, float3 d, float tmin, uint64_t media_key, HitInfo& h) {
    float3 inv = f3(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
    float3 oi = -1.0f * (o * inv);
    TriRay tr = make_tri_ray(d);
    int stack[kBvhStack];
    int sp = 0;
    int node = 0;      // the entry being walked: an inner node, a leaf, or kWalkDone
    int leaf = 0;      // the postponed leaf (< 0), or 0 for none
    int visits = 0;
    while (node != kWalkDone || leaf < 0) {
        // inner nodes until this lane holds a leaf and the whole warp does
        while (node >= 0) {
            if (++visits > S.bvh_node_count + 1) {  // a tree walk enters each inner node at most once
                atomicCAS(S.error, 0, 1);
                return false;
            }
            const float4* n = S.bvh + 4 * node;
            float4 a0 = ldg4(n), a1 = ldg4(n + 1), c0 = ldg4(n + 2), c1 = ldg4(n + 3);
            float lx0 = fmaf(a0.x, inv.x, oi.x), hx0 = fmaf(a1.x, inv.x, oi.x);
            float ly0 = fmaf(a0.y, inv.y, oi.y), hy0 = fmaf(a1.y, inv.y, oi.y);
            float lz0 = fmaf(a0.z, inv.z, oi.z), hz0 = fmaf(a1.z, inv.z, oi.z);
            float n0 = fmaxf(fmaxf(fminf(lx0, hx0), fminf(ly0, hy0)), fmaxf(fminf(lz0, hz0), tmin));
            float f0 = fminf(fminf(fmaxf(lx0, hx0), fmaxf(ly0, hy0)), fminf(fmaxf(lz0, hz0), h.t));
            float lx1 = fmaf(c0.x, inv.x, oi.x), hx1 = fmaf(c1.x, inv.x, oi.x);
            float ly1 = fmaf(c0.y, inv.y, oi.y), hy1 = fmaf(c1.y, inv.y, oi.y);
            float lz1 = fmaf(c0.z, inv.z, oi.z), hz1 = fmaf(c1.z, inv.z, oi.z);
            float n1 = fmaxf(fmaxf(fminf(lx1, hx1), fminf(ly1, hy1)), fmaxf(fminf(lz1, hz1), tmin));
            float f1 = fminf(fminf(fmaxf(lx1, hx1), fmaxf(ly1, hy1)), fminf(fmaxf(lz1, hz1), h.t));
            bool h0 = n0 <= f0 * 1.00000024f + 1e-30f;
            bool h1 = n1 <= f1 * 1.00000024f + 1e-30f;
            int k0 = __float_as_int(a1.w), k1 = __float_as_int(c1.w);
            // a child as a walk entry: the inner node, or the leaf packed below 0
            int e0 = k0 > 0 ? ~((__float_as_int(a0.w) << 4) | k0) : __float_as_int(a0.w);
            int e1 = k1 > 0 ? ~((__float_as_int(c0.w) << 4) | k1) : __float_as_int(c0.w);
            if (h0 && h1) {
                bool first0 = n0 <= n1;
                if (sp == kBvhStack) {
                    atomicCAS(S.error, 0, 2);
                    return false;
                }
                stack[sp++] = first0 ? e1 : e0;
                node = first0 ? e0 : e1;
            } else if (h0) {
                node = e0;
            } else if (h1) {
                node = e1;
            } else {
                node = sp > 0 ? stack[--sp] : kWalkDone;
            }
            // a leaf met while none is held is put aside, and the walk goes on
            if (node < 0 && node != kWalkDone && leaf == 0) {
                leaf = node;
                node = sp > 0 ? stack[--sp] : kWalkDone;
            }
            if (__all_sync(__activemask(), leaf < 0 || node == kWalkDone))
                break;
        }
        // the leaves: the postponed one, then any the walk stands on
        while (leaf < 0) {
            int packed = ~leaf;
            if (test_leaf<ANY, VOX>(S, packed >> 4, packed & 15, o, d, tr, tmin, media_key, h))
                return true;
            leaf = 0;
            if (node < 0 && node != kWalkDone) {
                leaf = node;
                node = sp > 0 ? stack[--sp] : kWalkDone;
            }
        }
    }
    return false;
}

// The walk over the 8-wide tree with quantised boxes (96-byte nodes, the
// layout collapse_to_8q writes). Per node the eight child planes are decoded
// from bytes as t = q (s / d) + (p - o) / d per axis (one FMA each); leaves
// among the children the ray meets are tested at once, the interior ones
// still nearer than the closest hit are sorted near to far (a 19-comparator
// network) and all but the nearest pushed. The host bounds the stack (seven
// entries per level) before it enables this walk.
constexpr int kBvh8Stack = 64;
MYPBR_DEV float byte_at(uint32_t w, int c) { return float((w >> (8 * (c & 3))) & 0xffu); }
template <bool ANY, bool VOX>
MYPBR_DEV bool walk_tree8q(const DeviceScene& S, float3 o, float3 d, float tmin, uint64_t media_key, HitInfo& h) {
    const float3 inv = f3(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
    const TriRay tr = make_tri_ray(d);
    int stack[kBvh8Stack];
    int sp = 0;
    int node = 0;
    int visits = 0;
    while (true) {
        if (++visits > S.bvh8_node_count + 1) {  // a tree walk enters each node at most once
            atomicCAS(S.error, 0, 1);
            return false;
        }
        const uint4* n = S.bvh8 + 6 * node;
        const uint4 r0 = __ldg(n), rx = __ldg(n + 1), ry = __ldg(n + 2), rz = __ldg(n + 3), w03 = __ldg(n + 4),
                    w47 = __ldg(n + 5);
        const float sx = __uint_as_float((r0.w & 0xffu) << 23), sy = __uint_as_float(((r0.w >> 8) & 0xffu) << 23),
                    sz = __uint_as_float(((r0.w >> 16) & 0xffu) << 23);
        const float ax = sx * inv.x, ay = sy * inv.y, az = sz * inv.z;
        const float bx = (__uint_as_float(r0.x) - o.x) * inv.x, by = (__uint_as_float(r0.y) - o.y) * inv.y,
                    bz = (__uint_as_float(r0.z) - o.z) * inv.z;
        float key[8];
        int val[8];
        unsigned leaves = 0;
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const uint32_t w = c < 4 ? (c == 0 ? w03.x : c == 1 ? w03.y : c == 2 ? w03.z : w03.w)
                                     : (c == 4 ? w47.x : c == 5 ? w47.y : c == 6 ? w47.z : w47.w);
            const uint32_t lxw = c < 4 ? rx.x : rx.y, hxw = c < 4 ? rx.z : rx.w;
            const uint32_t lyw = c < 4 ? ry.x : ry.y, hyw = c < 4 ? ry.z : ry.w;
            const uint32_t lzw = c < 4 ? rz.x : rz.y, hzw = c < 4 ? rz.z : rz.w;
            const float lx = fmaf(byte_at(lxw, c), ax, bx), hx = fmaf(byte_at(hxw, c), ax, bx);
            const float ly = fmaf(byte_at(lyw, c), ay, by), hy = fmaf(byte_at(hyw, c), ay, by);
            const float lz = fmaf(byte_at(lzw, c), az, bz), hz = fmaf(byte_at(hzw, c), az, bz);
            const float tn = fmaxf(fmaxf(fminf(lx, hx), fminf(ly, hy)), fmaxf(fminf(lz, hz), tmin));
            const float tf = fminf(fminf(fmaxf(lx, hx), fmaxf(ly, hy)), fminf(fmaxf(lz, hz), h.t));
            // a small relative widening keeps FP32 slab tests conservative
            const bool met = w != 0xffffffffu && tn <= tf * 1.00000024f + 1e-30f;
            const bool leaf = (w >> 31) != 0u;
            leaves |= (met && leaf) ? 1u << c : 0u;
            key[c] = (met && !leaf) ? tn : INFINITY;
            val[c] = leaf ? int((w >> 4) & 0x7ffffffu) : int(w);
            if (met && leaf)
                key[c] = INFINITY;
        }
        for (unsigned m = leaves; m; m &= m - 1) {
            const int c = __ffs(m) - 1;
            const uint32_t w = c < 4 ? (c == 0 ? w03.x : c == 1 ? w03.y : c == 2 ? w03.z : w03.w)
                                     : (c == 4 ? w47.x : c == 5 ? w47.y : c == 6 ? w47.z : w47.w);
            if (test_leaf<ANY, VOX>(S, int((w >> 4) & 0x7ffffffu), int(w & 15u), o, d, tr, tmin, media_key, h))
                return true;
        }
        // the interior children still nearer than the closest hit, nearest first
#pragma unroll
        for (int c = 0; c < 8; c++)
            key[c] = key[c] <= h.t ? key[c] : INFINITY;
        auto cswap = [&](int i, int j) {
            if (key[j] < key[i]) {
                const float tk = key[i];
                key[i] = key[j];
                key[j] = tk;
                const int tv = val[i];
                val[i] = val[j];
                val[j] = tv;
            }
        };
        cswap(0, 2); cswap(1, 3); cswap(4, 6); cswap(5, 7);
        cswap(0, 4); cswap(1, 5); cswap(2, 6); cswap(3, 7);
        cswap(0, 1); cswap(2, 3); cswap(4, 5); cswap(6, 7);
        cswap(2, 4); cswap(3, 5);
        cswap(1, 4); cswap(3, 6);
        cswap(1, 2); cswap(3, 4); cswap(5, 6);
        int pushes = 0;
#pragma unroll
        for (int c = 1; c < 8; c++)
            pushes += key[c] < INFINITY;
        if (sp + pushes > kBvh8Stack) {  // deeper than the host-checked bound: report, stop
            atomicCAS(S.error, 0, 2);
            return false;
        }
#pragma unroll
        for (int c = 7; c >= 1; c--)
            if (key[c] < INFINITY)
                stack[sp++] = val[c];
        if (key[0] < INFINITY) {
            node = val[0];
        } else {
            if (sp == 0)
                return false;
            node = stack[--sp];
        }
    }
}

// The whole walk in one loop (the form the per-ray kernels use; walk_node
// above is the same step, resumable, for k_extend_pt).
template <bool ANY, bool VOX, int WALK>
MYPBR_DEV HitInfo walk(const DeviceScene& S, float3 o, float3 d, float tmin, float tmax, uint64_t media_key) {
    HitInfo h;
    h.prim = kMiss;
    h.t = tmax;
    h.b1 = h.b2 = 0.0f;
    if constexpr (WALK == kWalkWide) {
        if (S.has_bvh && walk_tree4<ANY, VOX>(S, o, d, tmin, media_key, h))
            return h;
    } else if constexpr (WALK == kWalkWide8) {
        if (S.has_bvh && walk_tree8q<ANY, VOX>(S, o, d, tmin, media_key, h))
            return h;
    } else if constexpr (WALK == kWalkPostponed) {
        if (S.has_bvh && walk_postponed<ANY, VOX>(S, o, d, tmin, media_key, h))
            return h;
    } else if (S.has_bvh) {
        float3 inv = f3(safe_inv(d.x), safe_inv(d.y), safe_inv(d.z));
        float3 oi = -1.0f * (o * inv);
        TriRay tr = make_tri_ray(d);
        int stack[kBvhStack];
        int sp = 0;
        int node = 0;
        // A tree walk enters each interior node at most once; the cap only
        // guards against a malformed tree, which it reports instead of spinning.
        int visits = 0;
        while (true) {
            if (++visits > S.bvh_node_count + 1) {
                atomicCAS(S.error, 0, 1);
                break;
            }
            const float4* n = S.bvh + 4 * node;
            float4 a0 = ldg4(n), a1 = ldg4(n + 1), c0 = ldg4(n + 2), c1 = ldg4(n + 3);
            // slab tests of both children against (tmin, best)
            float lx0 = fmaf(a0.x, inv.x, oi.x), hx0 = fmaf(a1.x, inv.x, oi.x);
            float ly0 = fmaf(a0.y, inv.y, oi.y), hy0 = fmaf(a1.y, inv.y, oi.y);
            float lz0 = fmaf(a0.z, inv.z, oi.z), hz0 = fmaf(a1.z, inv.z, oi.z);
            float n0 = fmaxf(fmaxf(fminf(lx0, hx0), fminf(ly0, hy0)), fmaxf(fminf(lz0, hz0), tmin));
            float f0 = fminf(fminf(fmaxf(lx0, hx0), fmaxf(ly0, hy0)), fminf(fmaxf(lz0, hz0), h.t));
            float lx1 = fmaf(c0.x, inv.x, oi.x), hx1 = fmaf(c1.x, inv.x, oi.x);
            float ly1 = fmaf(c0.y, inv.y, oi.y), hy1 = fmaf(c1.y, inv.y, oi.y);
            float lz1 = fmaf(c0.z, inv.z, oi.z), hz1 = fmaf(c1.z, inv.z, oi.z);
            float n1 = fmaxf(fmaxf(fminf(lx1, hx1), fminf(ly1, hy1)), fmaxf(fminf(lz1, hz1), tmin));
            float f1 = fminf(fminf(fmaxf(lx1, hx1), fmaxf(ly1, hy1)), fminf(fmaxf(lz1, hz1), h.t));
            // A small relative widening keeps FP32 slab tests conservative
            bool h0 = n0 <= f0 * 1.00000024f + 1e-30f;
            bool h1 = n1 <= f1 * 1.00000024f + 1e-30f;
            int i0 = __float_as_int(a0.w), k0 = __float_as_int(a1.w);
            int i1 = __float_as_int(c0.w), k1 = __float_as_int(c1.w);
#pragma unroll
            for (int side = 0; side < 2; side++) {
                bool hit = side == 0 ? h0 : h1;
                int cnt = side == 0 ? k0 : k1;
                int first = side == 0 ? i0 : i1;
                if (!(hit && cnt > 0))
                    continue;
                for (int k = 0; k < cnt; k++) {
                    uint32_t ref = __ldg(S.leaf_refs + first + k);
                    int kind = int(ref >> kKindShift), idx = int(ref & kIndexMask);
                    float t, b1 = 0.0f, b2 = 0.0f;
                    bool got = false;
                    if (kind == kTriangle) {
                        got = hit_triangle(S, idx, o, tr, tmin, h.t, t, b1, b2, media_key);
                    } else if (kind == kSphere) {
                        got = hit_sphere(S, idx, o, d, tmin, h.t, t);
                    } else if (kind == kQuad) {
                        got = hit_quad(S, idx, o, d, tmin, h.t, t, b1, b2);
                    } else if (kind == kMedium && media_key != 0) {
                        got = hit_medium(S, idx, o, d, tmin, h.t, hash_uniform(media_key, uint32_t(idx)), t);
                    } else if (VOX && kind == kVoxel) {
                        int mat, face;
                        got = hit_voxel_block(S, idx, o, d, tmin, h.t, t, mat, face);
                        b1 = __int_as_float(mat);
                        b2 = __int_as_float(face);
                    }
                    if (got) {
                        h.t = t;
                        h.b1 = b1;
                        h.b2 = b2;
                        h.prim = ref;
                        if (ANY)
                            return h;
                    }
                }
            }
            h0 = h0 && k0 == 0;
            h1 = h1 && k1 == 0;
            if (h0 && h1) {
                bool first0 = n0 <= n1;
                if (sp == kBvhStack) {  // deeper than the host-checked depth: report, stop
                    atomicCAS(S.error, 0, 2);
                    break;
                }
                stack[sp++] = first0 ? i1 : i0;
                node = first0 ? i0 : i1;
            } else if (h0) {
                node = i0;
            } else if (h1) {
                node = i1;
            } else {
                if (sp == 0)
                    break;
                node = stack[--sp];
            }
        }
    }
    // The ground (plane.h:17-34) and height fog (medium.h:352-381) beside the BVH
    for (int k = 0; k < S.unbounded_count; k++) {
        DevUnbounded ub = S.unbounded[k];
        if (ub.kind == 0) {
            if (fabsf(d.y) < 1e-12f)
                continue;
            float t = (ub.height - o.y) / d.y;
            if (t > tmin && t < h.t) {
                h.t = t;
                h.prim = (uint32_t(kGround) << kKindShift) | uint32_t(k);
                if (ANY)
                    return h;
            }
        } else if (media_key != 0) {
            float len = length(d);
            float kk = d.y / ub.scale_height;
            float start = ub.density * len * expf(-(o.y + tmin * d.y - ub.height) / ub.scale_height);
            if (!(start > 0.0f))
                continue;
            float tau = -logf(1.0f - hash_uniform(media_key, 0x40000000u + uint32_t(k)));
            float t;
            if (fabsf(kk) < 1e-12f) {
                t = tmin + tau / start;
            } else {
                float x = 1.0f - tau * kk / start;
                if (x <= 0.0f)
                    continue;
                t = tmin - logf(x) / kk;
            }
            if (t < h.t && isfinite(t)) {
                h.t = t;
                h.prim = (uint32_t(kHeightFog) << kKindShift) | uint32_t(k);
                if (ANY)
                    return h;
            }
        }
    }
    return h;
}

// ------------------------------------------------------- surface records

struct Surface {
    float3 p, normal, dpdu, dpdv;
    float u, v;
    int material;
    bool front;
    float3 ng;    // geometric normal (unit; either side), 0 where there is no surface (a medium)
    float3 perr;  // per component, a bound on |p - the exact point| from the FP32 arithmetic that made p
};

// ------------------------------------------------- error-bounded ray origins
//
// A hit point computed in FP32 lies off the exact surface by a rounding
// error whose bound follows from how it was computed (Pharr, Jakob and
// Humphreys, "Physically Based Rendering", 3rd ed., section 3.9: gamma_n =
// n u / (1 - n u) bounds n roundings, u = 2^-24). A new ray starts at the hit
// point moved along the geometric normal, to the side it leaves on, by that
// bound projected on the normal, then one float step further: the exact
// surface is then behind the origin. The bounds below are taken at twice the
// IEEE figure: fast-math reciprocals and square roots round less tightly.
MYPBR_DEV float3 abs3(float3 a) { return f3(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }

// The error of X p (+ translation) for a point p with error e: the rounding
// of the products and sums, and e carried through |M|.
MYPBR_DEV float3 xf_point_error(const XformRef& X, float3 p, float3 e) {
    float3 out;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float4 r = X.r[i];
        float mag = fabsf(r.x * p.x) + fabsf(r.y * p.y) + fabsf(r.z * p.z) + fabsf(r.w);
        float carried = fabsf(r.x) * e.x + fabsf(r.y) * e.y + fabsf(r.z) * e.z;
        set_comp(out, i, err_gamma(3) * mag + (1.0f + err_gamma(3)) * carried);
    }
    return out;
}

// The next float after x in the direction of `dir` (> 0: up, < 0: down).
MYPBR_DEV float float_step(float x, float dir) {
    if (dir == 0.0f)
        return x;
    if (x == 0.0f)
        return dir > 0.0f ? 1.4e-45f : -1.4e-45f;
    bool away = (dir > 0.0f) == (x > 0.0f);  // away from zero: the bit pattern grows
    return __int_as_float(__float_as_int(x) + (away ? 1 : -1));
}

// The smallest t a walk from o along d accepts: 8 FP32 steps of the
// origin's largest coordinate, in units of d. Below that the intersection
// arithmetic cannot tell on which side of the origin a surface lies; the
// spawn offset has already put the surface just left behind the origin.
MYPBR_DEV float spawn_tmin(float3 o, float3 d) {
    float m = fmaxf(fabsf(o.x), fmaxf(fabsf(o.y), fabsf(o.z)));
    return m * 9.5367431640625e-7f * rsqrtf(dot(d, d));
}

// Where a ray leaving surface s in direction w starts.
MYPBR_DEV float3 spawn_origin(const Surface& s, float3 w) {
    float dist = fabsf(s.ng.x) * s.perr.x + fabsf(s.ng.y) * s.perr.y + fabsf(s.ng.z) * s.perr.z;
    float3 off = dist * s.ng;
    if (dot(w, s.ng) < 0.0f)
        off = -1.0f * off;
    float3 o = s.p + off;
    return f3(float_step(o.x, off.x), float_step(o.y, off.y), float_step(o.z, off.z));
}

MYPBR_DEV void set_face(Surface& s, float3 d, float3 outward) {
    s.front = dot(d, outward) < 0.0f;
    s.normal = s.front ? outward : -outward;
}

// sphere.h:536-560: (u, v) and tangents of a point p on the unit sphere, radius r
MYPBR_DEV void sphere_uv_tangents(float3 p, float r, Surface& s) {
    float theta = acosf(clampf(-p.y, -1.0f, 1.0f));
    float phi = atan2f(-p.z, p.x) + kPi;
    s.u = phi * (0.5f * kInvPi);
    s.v = theta * kInvPi;
    float st = sqrtf(p.x * p.x + p.z * p.z);
    if (st < 1e-8f) {
        s.dpdu = s.dpdv = f3(0.0f);
        return;
    }
    s.dpdu = (2.0f * kPi * r) * f3(p.z, 0.0f, -p.x);
    s.dpdv = (kPi * r / st) * f3(-p.x * p.y, st * st, -p.y * p.z);
}

// Rebuilds the hit record (hittable.h:12-32) of a hit found by closest_hit.
MYPBR_DEV Surface make_surface(const DeviceScene& S, const HitInfo& h, float3 o, float3 d) {
    Surface s;
    int kind = int(h.prim >> kKindShift), idx = int(h.prim & kIndexMask);
    s.p = o + h.t * d;
    s.u = s.v = 0.0f;
    s.dpdu = s.dpdv = f3(0.0f);
    s.front = true;
    s.normal = f3(1, 0, 0);
    s.material = 0;
    s.ng = f3(0.0f);
    s.perr = f3(0.0f);
    if (kind == kSphere) {
        float4 sp = ldg4(S.spheres + idx);
        int2 info = S.sphere_info[idx];
        s.material = info.x;
        float3 c = f3(sp);
        float r = sp.w;
        if (info.y < 0) {
            float3 outward = (s.p - c) / r;
            outward = outward * rsqrtf(dot(outward, outward));
            s.p = c + fabsf(r) * (r < 0.0f ? -outward : outward);  // back onto the surface
            set_face(s, d, outward);
            sphere_uv_tangents(r < 0.0f ? -outward : outward, fabsf(r), s);
            s.ng = outward;
            s.perr = err_gamma(6) * (abs3(c) + fabsf(r) * abs3(outward));
        } else {
            XformRef X;
            load_xform(S, info.y, X);
            float3 lo = xf_ipoint(X, o), ld = xf_ivec(X, d);
            float3 lp = lo + h.t * ld;
            float3 outward = (lp - c) / r;
            Surface ls;
            set_face(ls, ld, outward);
            float3 un = r < 0.0f ? -outward : outward;
            un = un * rsqrtf(dot(un, un));
            sphere_uv_tangents(un, fabsf(r), ls);
            lp = c + fabsf(r) * un;  // back onto the surface, in the sphere's space
            s.u = ls.u;
            s.v = ls.v;
            s.front = ls.front;
            s.p = xf_point(X, lp);
            s.normal = normalize(xf_normal(X, ls.normal));
            s.dpdu = xf_vec(X, ls.dpdu);
            s.dpdv = xf_vec(X, ls.dpdv);
            s.ng = normalize(xf_normal(X, un));
            s.perr = xf_point_error(X, lp, err_gamma(6) * (abs3(c) + fabsf(r) * abs3(un)));
        }
    } else if (kind == kQuad) {
        const float4* q = S.quads + 5 * idx;
        float4 Q = ldg4(q);
        s.material = __float_as_int(Q.w);
        s.u = h.b1;
        s.v = h.b2;
        s.dpdu = f3(ldg4(q + 1));
        s.dpdv = f3(ldg4(q + 2));
        s.p = f3(Q) + h.b1 * s.dpdu + h.b2 * s.dpdv;
        set_face(s, d, f3(ldg4(q + 3)));
        s.ng = normalize(f3(ldg4(q + 3)));
        s.perr = err_gamma(5) * (abs3(f3(Q)) + fabsf(h.b1) * abs3(s.dpdu) + fabsf(h.b2) * abs3(s.dpdv));
    } else if (kind == kTriangle) {
        const float4* tp = S.tris + 3 * idx;
        float4 P0 = ldg4(tp), P1 = ldg4(tp + 1), P2 = ldg4(tp + 2);
        s.material = __float_as_int(P0.w);
        int flags = __float_as_int(P1.w);
        float b1 = h.b1, b2 = h.b2, b0 = 1.0f - b1 - b2;
        float3 v0 = f3(P0), e1 = f3(P1) - v0, e2 = f3(P2) - v0;
        s.p = v0 + b1 * e1 + b2 * e2;
        int4 sa = S.tri_shading[2 * idx], sb = S.tri_shading[2 * idx + 1];
        s.u = b1;
        s.v = b2;
        bool has_uv = sa.w >= 0;
        s.dpdu = e1;
        s.dpdv = e2;
        if (has_uv) {
            float2 t0 = S.uvs[sa.w], t1 = S.uvs[sb.x], t2 = S.uvs[sb.y];
            s.u = b0 * t0.x + b1 * t1.x + b2 * t2.x;
            s.v = b0 * t0.y + b1 * t1.y + b2 * t2.y;
            float du1 = t1.x - t0.x, dv1 = t1.y - t0.y, du2 = t2.x - t0.x, dv2 = t2.y - t0.y;
            float det = du1 * dv2 - du2 * dv1;
            if (fabsf(det) < 1e-12f) {
                s.dpdu = s.dpdv = f3(0.0f);
            } else {
                float iv = 1.0f / det;
                s.dpdu = (dv2 * e1 - dv1 * e2) * iv;
                s.dpdv = (du1 * e2 - du2 * e1) * iv;
            }
        }
        float3 g = normalize(cross(e1, e2));
        if (flags & 1)
            g = -g;
        set_face(s, d, g);
        s.ng = g;
        // the edges are differences of the stored corners: their rounding too
        s.perr = err_gamma(7) * (abs3(v0) + fabsf(b1) * (abs3(f3(P1)) + abs3(v0)) +
                                 fabsf(b2) * (abs3(f3(P2)) + abs3(v0)));
        if (sa.x >= 0) {
            float3 sh = b0 * S.normals[sa.x] + b1 * S.normals[sa.y] + b2 * S.normals[sa.z];
            if (dot(sh, sh) > 0.0f) {
                sh = normalize(sh);
                s.normal = dot(sh, s.normal) < 0.0f ? -sh : sh;
            }
        }
    } else if (kind == kMedium) {
        s.material = __float_as_int(ldg4(S.media + 3 * idx + 2).y);
    } else if (kind == kVoxel) {
        // voxel_grid::record (voxel.h:333-350) in the model's space, then the
        // placement as instance::hit does (instance.h:29-40)
        s.material = __float_as_int(h.b1);
        int face = __float_as_int(h.b2), axis = face & 3;
        float sign = (face & 4) ? 1.0f : -1.0f;
        const DevVoxelModel& m = S.voxel_models[__ldg(&S.voxel_blocks[2 * idx].x)];
        XformRef X;
        load_xform(S, m.xform, X);
        float3 lo = xf_ipoint(X, o), ld = xf_ivec(X, d);
        float3 lp = lo + h.t * ld;
        // the face lies on a whole-number plane of the model's cells: the
        // point is put on it exactly; along the face, the ray's rounding
        float3 lerr = err_gamma(4) * (abs3(lo) + abs3(h.t * ld));
        set_comp(lp, axis, rintf(comp(lp, axis)));
        set_comp(lerr, axis, 0.0f);
        float3 outward = f3(0.0f), tb = f3(0.0f), tc = f3(0.0f);
        set_comp(outward, axis, sign);
        set_comp(tb, (axis + 1) % 3, 1.0f);
        set_comp(tc, (axis + 2) % 3, 1.0f);
        float3 du = sign > 0.0f ? tb : tc, dv = sign > 0.0f ? tc : tb;
        float pu = dot(lp, du), pv = dot(lp, dv);
        s.u = pu - floorf(pu);
        s.v = pv - floorf(pv);
        Surface ls;
        set_face(ls, xf_ivec(X, d), outward);
        s.front = ls.front;
        s.p = xf_point(X, lp);
        s.normal = normalize(xf_normal(X, ls.normal));
        s.dpdu = xf_vec(X, du);
        s.dpdv = xf_vec(X, dv);
        s.ng = normalize(xf_normal(X, outward));
        s.perr = xf_point_error(X, lp, lerr);
    } else if (kind == kGround) {
        DevUnbounded ub = S.unbounded[idx];
        s.material = ub.material;
        s.p.y = ub.height;
        s.u = s.p.x;
        s.v = -s.p.z;
        s.dpdu = f3(1, 0, 0);
        s.dpdv = f3(0, 0, -1);
        set_face(s, d, f3(0, 1, 0));
        s.ng = f3(0, 1, 0);  // the point is on the plane exactly (y set to its height)
    } else if (kind == kHeightFog) {
        s.material = S.unbounded[idx].material;
    }
    return s;
}

}  // namespace mypbr_dev
