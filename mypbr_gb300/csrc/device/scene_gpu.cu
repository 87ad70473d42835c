// mypbr_gpu_scene_create / destroy: the flat FP64 scene becomes the compact
// FP32 layout of dev_scene.cuh in HBM.
//
// Every index of the flat scene is checked here, on the host, before anything
// reaches the device, so the kernels can index without bounds checks:
// materials, textures, texels, vertices, normals, uvs, transforms, BVH nodes
// and leaf references, light members. The BVH depth is checked against the
// traversal stack the kernels hold.
#include <algorithm>
#include <map>
#include <cmath>
#include <functional>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../host/bvh_build.h"
#include "gpu_scene.h"

namespace mypbr_host {
void set_error(const std::string& message);
}

namespace mypbr_dev {

void set_error_message(const std::string& m) { mypbr_host::set_error(m); }

int cuda_fail(cudaError_t e, const char* what) {
    set_error_message(std::string(what) + ": " + cudaGetErrorString(e));
    if (e == cudaErrorMemoryAllocation)
        return MYPBR_ERR_OUT_OF_MEMORY;
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
        return MYPBR_ERR_NO_DEVICE;
    return MYPBR_ERR_CUDA;
}

namespace {

float round_down(double x) {
    float f = float(x);
    if (double(f) > x)
        f = std::nextafter(f, -INFINITY);
    return f;
}
float round_up(double x) {
    float f = float(x);
    if (double(f) < x)
        f = std::nextafter(f, INFINITY);
    return f;
}

// The bits of an int in a float slot (host side of __float_as_int).
float ibits(int i) {
    float f;
    std::memcpy(&f, &i, sizeof f);
    return f;
}
int float_bits(float f) {
    int i;
    std::memcpy(&i, &f, sizeof i);
    return i;
}

int bad(const std::string& m) {
    set_error_message("mypbr_gpu_scene_create: " + m);
    return MYPBR_ERR_INVALID_ARGUMENT;
}

struct Uploader {
    mypbr_gpu_scene& G;
    template <typename T>
    int put(const std::vector<T>& v, const T*& out) {
        out = nullptr;
        if (v.empty())
            return MYPBR_OK;
        void* p = nullptr;
        MYPBR_CUDA(cudaMalloc(&p, v.size() * sizeof(T)));
        G.allocations.push_back(p);
        MYPBR_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
        out = static_cast<const T*>(p);
        return MYPBR_OK;
    }
};

const std::vector<double>& ggx_table_cached() {
    static std::vector<double> table;
    static std::once_flag once;
    std::call_once(once, [] {
        table.resize(32 * 32 + 32);
        mypbr_host::ggx_albedo_table(table.data());
    });
    return table;
}

int validate(const mypbr_flat_scene& F) {
    auto in = [](int64_t i, int64_t n) { return i >= 0 && i < n; };
    int64_t nm = F.material_count, nt = F.texture_count;
    if (nm <= 0)
        return bad("the scene has no materials");
    for (int64_t k = 0; k < nm; k++) {
        const auto& m = F.materials[k];
        if (m.type < 0 || m.type > MYPBR_MAT_PHASE)
            return bad("material " + std::to_string(k) + " has an unknown type");
        for (int t : m.tex)
            if (t != -1 && !in(t, nt))
                return bad("material " + std::to_string(k) + " names a missing texture");
        if ((m.normal_map != -1 && !in(m.normal_map, nt)) || (m.emission_tex != -1 && !in(m.emission_tex, nt)))
            return bad("material " + std::to_string(k) + " names a missing texture");
        if ((m.type == MYPBR_MAT_LAMBERTIAN && m.tex[0] < 0) ||
            (m.type == MYPBR_MAT_PRINCIPLED && (m.tex[0] < 0 || m.tex[1] < 0 || m.tex[2] < 0)) ||
            (m.type == MYPBR_MAT_PRINCIPLED && (m.flags & MYPBR_MATF_COAT) && (m.tex[4] < 0 || m.tex[5] < 0)))
            return bad("material " + std::to_string(k) + " lacks a texture it needs");
    }
    for (int64_t k = 0; k < nt; k++) {
        const auto& t = F.textures[k];
        auto plain = [&](int c) {
            return in(c, nt) && (F.textures[c].type == MYPBR_TEX_SOLID || F.textures[c].type == MYPBR_TEX_IMAGE);
        };
        if (t.type == MYPBR_TEX_CHECKER) {
            if (!plain(t.a) || !plain(t.b))
                return bad("checker texture " + std::to_string(k) + " must pick between two plain textures");
        } else if (t.type >= MYPBR_TEX_SCALED && t.type <= MYPBR_TEX_NORMAL_SCALE) {
            // wrappers name an earlier texture, so chains end; at most 6
            // deep, with at most two that change the value
            int depth = 0, value_ops = 0;
            for (int64_t c = k; c >= 0 && F.textures[c].type >= MYPBR_TEX_SCALED; c = F.textures[c].a) {
                if (!(F.textures[c].a >= 0 && F.textures[c].a < c) || ++depth > 6)
                    return bad("texture " + std::to_string(k) + " wraps a missing or later texture, or too deep");
                value_ops += F.textures[c].type != MYPBR_TEX_UV_TRANSFORM;
            }
            if (value_ops > 2)
                return bad("texture " + std::to_string(k) + " stacks more than two scaling wrappers");
            if (t.type == MYPBR_TEX_CHANNEL && (t.b < 0 || t.b > 2))
                return bad("channel texture " + std::to_string(k) + " names no color channel");
        } else if (t.type == MYPBR_TEX_IMAGE) {
            int64_t texels = int64_t(t.width) * t.height;
            if (t.width <= 0 || t.height <= 0 || t.offset < 0)
                return bad("image texture " + std::to_string(k) + " has no pixels");
            if (t.flags & MYPBR_TEXF_HDR) {
                if ((t.offset + texels) * 3 > F.texels_hdr_count)
                    return bad("image texture " + std::to_string(k) + " runs past texels_hdr");
            } else if ((t.offset + texels) * 4 > F.texels_ldr_bytes) {
                return bad("image texture " + std::to_string(k) + " runs past texels_ldr");
            }
        } else if (t.type != MYPBR_TEX_SOLID) {
            return bad("texture " + std::to_string(k) + " has an unknown type");
        }
    }
    for (int64_t k = 0; k < F.sphere_count; k++)
        if (!in(F.spheres[k].material, nm) || (F.spheres[k].xform != -1 && !in(F.spheres[k].xform, F.xform_count)) ||
            F.spheres[k].radius == 0)
            return bad("sphere " + std::to_string(k) + " is malformed");
    for (int64_t k = 0; k < F.quad_count; k++)
        if (!in(F.quads[k].material, nm))
            return bad("quad " + std::to_string(k) + " names a missing material");
    for (int64_t k = 0; k < F.triangle_count; k++) {
        const auto& t = F.triangles[k];
        if (!in(t.material, nm))
            return bad("triangle " + std::to_string(k) + " names a missing material");
        for (int c = 0; c < 3; c++) {
            if (!in(t.v[c], F.position_count) || (t.n[c] != -1 && !in(t.n[c], F.normal_count)) ||
                (t.t[c] != -1 && !in(t.t[c], F.uv_count)))
                return bad("triangle " + std::to_string(k) + " has an index out of range");
        }
        if ((t.n[0] < 0) != (t.n[1] < 0) || (t.n[0] < 0) != (t.n[2] < 0) || (t.t[0] < 0) != (t.t[1] < 0) ||
            (t.t[0] < 0) != (t.t[2] < 0))
            return bad("triangle " + std::to_string(k) + " mixes present and missing normals or uvs");
        if (t.flags & MYPBR_TRI_ALPHA_MASK) {
            if (!in(t.mesh, F.mesh_count))
                return bad("masked triangle " + std::to_string(k) + " names no mesh");
            int mask = F.meshes[t.mesh].alpha_mask;
            if (!in(mask, F.texture_count) || F.textures[mask].type != MYPBR_TEX_IMAGE)
                return bad("mesh " + std::to_string(t.mesh) + "'s alpha mask is not an image texture");
        }
    }
    for (int64_t k = 0; k < F.medium_count; k++) {
        const auto& m = F.media[k];
        if (!in(m.material, nm) || (m.xform != -1 && !in(m.xform, F.xform_count)) || m.shape < 0 || m.shape > 1 ||
            !(m.density > 0))
            return bad("medium " + std::to_string(k) + " is malformed");
    }
    for (int64_t k = 0; k < F.unbounded_count; k++) {
        const auto& u = F.unbounded[k];
        if (!in(u.material, nm) || u.kind < 0 || u.kind > 1 ||
            (u.kind == MYPBR_UNBOUNDED_HEIGHT_FOG && !(u.density > 0 && u.scale_height > 0)))
            return bad("unbounded object " + std::to_string(k) + " is malformed");
    }
    for (int64_t k = 0; k < F.voxel_palette_count; k++) {
        const auto& e = F.voxel_palettes[k];
        if (e.kind < MYPBR_VOXEL_EMPTY || e.kind > MYPBR_VOXEL_TRANSPARENT ||
            (e.kind != MYPBR_VOXEL_EMPTY && !in(e.material, nm)) || (k % 256 == 0 && e.kind != MYPBR_VOXEL_EMPTY))
            return bad("voxel palette entry " + std::to_string(k) + " is malformed");
    }
    for (int64_t k = 0; k < F.voxel_model_count; k++) {
        const auto& m = F.voxel_models[k];
        int64_t cells = int64_t(m.nx) * m.ny * m.nz;
        if (m.nx <= 0 || m.ny <= 0 || m.nz <= 0 || !in(m.xform, F.xform_count) || m.cells < 0 ||
            m.cells + cells > F.voxel_cell_bytes || m.palette < 0 || m.palette % 256 != 0 ||
            int64_t(m.palette) + 256 > F.voxel_palette_count || !(m.edge_width >= 0 && m.edge_width < 0.5) ||
            (m.edge_width > 0 && !in(m.edge_material, nm)))
            return bad("voxel model " + std::to_string(k) + " is malformed");
    }
    for (int64_t k = 0; k < F.voxel_block_count; k++) {
        const auto& b = F.voxel_blocks[k];
        if (!in(b.model, F.voxel_model_count))
            return bad("voxel block " + std::to_string(k) + " names a missing model");
        const auto& m = F.voxel_models[b.model];
        const int n[3] = {m.nx, m.ny, m.nz};
        for (int a = 0; a < 3; a++)
            if (b.lo[a] < 0 || b.hi[a] > n[a] || b.hi[a] <= b.lo[a] || b.hi[a] - b.lo[a] > kVoxelBlockMax)
                return bad("voxel block " + std::to_string(k) + " is out of its model or larger than " +
                           std::to_string(kVoxelBlockMax) + " cells a side");
    }
    auto prim_count = [&](int kind) -> int64_t {
        switch (kind) {
            case MYPBR_PRIM_SPHERE: return F.sphere_count;
            case MYPBR_PRIM_QUAD: return F.quad_count;
            case MYPBR_PRIM_TRIANGLE: return F.triangle_count;
            case MYPBR_PRIM_MEDIUM: return F.medium_count;
            case MYPBR_PRIM_VOXEL_BLOCK: return F.voxel_block_count;
            default: return -1;
        }
    };
    for (int64_t k = 0; k < F.bvh_prim_count; k++) {
        const auto& r = F.bvh_prims[k];
        int64_t n = prim_count(r.kind);
        if (n < 0 || !in(r.index, n) || r.index >= int64_t(kIndexMask))
            return bad("BVH primitive reference " + std::to_string(k) + " is out of range");
    }
    if (F.bvh_prim_count > 0) {
        if (F.bvh_node_count <= 0)
            return bad("primitives without BVH nodes");
        for (int64_t k = 0; k < F.bvh_node_count; k++) {
            const auto& n = F.bvh_nodes[k];
            if (n.count > 0) {
                if (n.offset < 0 || int64_t(n.offset) + n.count > F.bvh_prim_count)
                    return bad("BVH leaf " + std::to_string(k) + " runs past the primitive references");
            } else if (n.count == 0) {
                if (k + 1 >= F.bvh_node_count || n.offset <= k || n.offset >= F.bvh_node_count)
                    return bad("BVH node " + std::to_string(k) + " has a child out of range");
            } else {
                return bad("BVH node " + std::to_string(k) + " has a negative count");
            }
        }
    }
    for (int64_t k = 0; k < F.light_count; k++) {
        const auto& L = F.lights[k];
        if (L.kind == MYPBR_LIGHT_GROUP) {
            if (L.member_count <= 0 || L.first_member < 0 ||
                int64_t(L.first_member) + L.member_count > F.light_member_count)
                return bad("light " + std::to_string(k) + " has members out of range");
            for (int m = 0; m < L.member_count; m++) {
                const auto& mb = F.light_members[L.first_member + m];
                if (mb.prim_kind < 0 || mb.prim_kind > MYPBR_PRIM_TRIANGLE || !in(mb.prim_index, prim_count(mb.prim_kind)))
                    return bad("light member of light " + std::to_string(k) + " is out of range");
            }
        } else if (L.kind == MYPBR_LIGHT_ENVIRONMENT) {
            if (F.environment.width <= 0 || F.environment.height <= 0 || !F.environment.pixels)
                return bad("an environment light without an environment");
        } else if (L.kind == MYPBR_LIGHT_SUN) {
            if (!F.sun.enabled)
                return bad("a sun light without a sun");
        } else {
            return bad("light " + std::to_string(k) + " has an unknown kind");
        }
    }
    return MYPBR_OK;
}

// Depth of the DFS BVH below node k (iterative, no recursion on deep trees).
int bvh_depth(const mypbr_flat_scene& F) {
    int best = 0;
    std::vector<std::pair<int, int>> st{{0, 1}};
    while (!st.empty()) {
        auto [k, d] = st.back();
        st.pop_back();
        best = std::max(best, d);
        const auto& n = F.bvh_nodes[k];
        if (n.count == 0) {
            st.push_back({k + 1, d + 1});
            st.push_back({n.offset, d + 1});
        }
    }
    return best;
}

}  // namespace

int create_scene(const mypbr_flat_scene* Fp, mypbr_gpu_scene** out) {
    if (!Fp || !out)
        return bad("null argument");
    *out = nullptr;
    const mypbr_flat_scene& F = *Fp;
    if (F.abi_version != MYPBR_ABI_VERSION)
        return bad("ABI version mismatch");
    int status = validate(F);
    if (status != MYPBR_OK)
        return status;

    int device_count = 0;
    cudaError_t ce = cudaGetDeviceCount(&device_count);
    if (ce != cudaSuccess || device_count == 0) {
        set_error_message("mypbr_gpu_scene_create: no CUDA device is visible");
        return MYPBR_ERR_NO_DEVICE;
    }
    auto holder = std::make_unique<mypbr_gpu_scene>();
    mypbr_gpu_scene& G = *holder;
    MYPBR_CUDA(cudaGetDevice(&G.device));
    MYPBR_CUDA(cudaDeviceGetAttribute(&G.sm_count, cudaDevAttrMultiProcessorCount, G.device));
    MYPBR_CUDA(cudaStreamCreateWithFlags(&G.stream, cudaStreamNonBlocking));
    DeviceScene& D = G.dev;
    Uploader up{G};
    auto fail_cleanup = [&](int s) {
        for (void* p : G.allocations)
            cudaFree(p);
        G.allocations.clear();
        if (G.stream)
            cudaStreamDestroy(G.stream);
        G.stream = nullptr;
        return s;
    };
#define PUT(vec, dst)                          \
    do {                                       \
        int s_ = up.put((vec), (dst));         \
        if (s_ != MYPBR_OK)                    \
            return fail_cleanup(s_);           \
    } while (0)

    // ---- BVH: child boxes stored in the parent
    std::vector<float4> nodes;
    std::vector<uint32_t> refs;
    int interior = 0;
    D.has_bvh = F.bvh_prim_count > 0;
    if (D.has_bvh) {
        const auto& root = F.bvh_nodes[0];
        G.box_lo = make_float3(float(root.bmin[0]), float(root.bmin[1]), float(root.bmin[2]));
        G.box_hi = make_float3(float(root.bmax[0]), float(root.bmax[1]), float(root.bmax[2]));
        G.max_depth_bvh = bvh_depth(F);
        if (G.max_depth_bvh >= kBvhStack) {
            set_error_message("mypbr_gpu_scene_create: BVH depth " + std::to_string(G.max_depth_bvh) +
                              " exceeds the traversal stack (" + std::to_string(kBvhStack) + ")");
            return fail_cleanup(MYPBR_ERR_UNSUPPORTED);
        }
        std::vector<int> new_index(size_t(F.bvh_node_count), -1);
        for (int64_t k = 0; k < F.bvh_node_count; k++)
            if (F.bvh_nodes[k].count == 0)
                new_index[size_t(k)] = interior++;
        auto child_entry = [&](int64_t c, float4& lo, float4& hi) {
            const auto& n = F.bvh_nodes[c];
            lo = make_float4(round_down(n.bmin[0]), round_down(n.bmin[1]), round_down(n.bmin[2]), 0.0f);
            hi = make_float4(round_up(n.bmax[0]), round_up(n.bmax[1]), round_up(n.bmax[2]), 0.0f);
            int idx = n.count > 0 ? n.offset : new_index[size_t(c)];
            lo.w = ibits(idx);
            hi.w = ibits(n.count);
        };
        if (F.bvh_nodes[0].count > 0) {
            // A root leaf: one node holding it twice. The second copy's box sits
            // at +infinity on every axis, where the slab test fails for every
            // ray (both slab distances are +inf or both -inf); and were it ever
            // entered it would only test the same primitives again, never loop.
            float4 lo, hi;
            child_entry(0, lo, hi);
            float inf = INFINITY;
            nodes = {lo, hi, make_float4(inf, inf, inf, lo.w), make_float4(inf, inf, inf, hi.w)};
            interior = 1;
        } else {
            nodes.resize(size_t(interior) * 4);
            for (int64_t k = 0; k < F.bvh_node_count; k++) {
                const auto& n = F.bvh_nodes[k];
                if (n.count != 0)
                    continue;
                float4* dst = &nodes[size_t(new_index[size_t(k)]) * 4];
                child_entry(k + 1, dst[0], dst[1]);
                child_entry(n.offset, dst[2], dst[3]);
            }
        }
        refs.resize(size_t(F.bvh_prim_count));
        for (int64_t k = 0; k < F.bvh_prim_count; k++)
            refs[size_t(k)] = (uint32_t(F.bvh_prims[k].kind) << kKindShift) | uint32_t(F.bvh_prims[k].index);
    }
    PUT(nodes, D.bvh);
    PUT(refs, D.leaf_refs);
    D.bvh_node_count = interior;
    // walk_postponed packs a leaf as first << 4 | count in a stack entry
    D.postponed_ok = D.has_bvh && F.bvh_prim_count < (int64_t(1) << 26);
    {
        // leaves of triangles, quads, media or voxel blocks make the lanes of
        // a warp diverge in their tests (voxel blocks most: a DDA walk each);
        // spheres are one cheap test. Postponed leaves are the default unless
        // spheres fill most leaves.
        int64_t spheres = 0;
        for (int64_t k = 0; k < F.bvh_prim_count; k++)
            spheres += F.bvh_prims[k].kind == MYPBR_PRIM_SPHERE;
        G.prefer_postponed = 2 * spheres < F.bvh_prim_count;
    }
    for (size_t k = 0; D.postponed_ok && k < nodes.size(); k += 2)
        if (float_bits(nodes[k + 1].w) >= 16)
            D.postponed_ok = 0;
    {
        std::vector<float4> nodes4;
        int depth4 = 0;
        if (D.has_bvh)
            collapse_to_4(nodes, nodes4, depth4);
        // the 4-wide walk's stack takes at most three entries per level
        if (!nodes4.empty() && 3 * (depth4 + 1) <= kBvh4Stack) {
            PUT(nodes4, D.bvh4);
            D.bvh4_node_count = int(nodes4.size() / 8);
        } else {
            D.bvh4 = nullptr;
            D.bvh4_node_count = 0;
        }
    }
    {
        std::vector<uint4> nodes8;
        int depth8 = 0;
        // the 8-wide walk's stack takes at most seven entries per level
        if (D.has_bvh && collapse_to_8q(nodes, nodes8, depth8) && 7 * (depth8 + 1) <= kBvh8Stack) {
            PUT(nodes8, D.bvh8);
            D.bvh8_node_count = int(nodes8.size() / 6);
        } else {
            D.bvh8 = nullptr;
            D.bvh8_node_count = 0;
        }
    }
    {
        std::vector<int> zero(1, 0);
        const int* err = nullptr;
        PUT(zero, err);
        D.error = const_cast<int*>(err);
    }
    G.leaf_ref_count = refs.size();

    // ---- primitives
    std::vector<float4> spheres;
    std::vector<int2> sphere_info;
    for (int64_t k = 0; k < F.sphere_count; k++) {
        const auto& s = F.spheres[k];
        spheres.push_back(make_float4(float(s.center[0]), float(s.center[1]), float(s.center[2]), float(s.radius)));
        sphere_info.push_back(make_int2(s.material, s.xform));
    }
    PUT(spheres, D.spheres);
    PUT(sphere_info, D.sphere_info);

    std::vector<float4> quads;
    for (int64_t k = 0; k < F.quad_count; k++) {
        const auto& q = F.quads[k];
        mypbr_host::V3 u(q.u[0], q.u[1], q.u[2]), v(q.v[0], q.v[1], q.v[2]);
        mypbr_host::V3 c = mypbr_host::cross(u, v);
        mypbr_host::V3 w = c / mypbr_host::dot(c, c);
        quads.push_back(make_float4(float(q.q[0]), float(q.q[1]), float(q.q[2]), ibits(q.material)));
        quads.push_back(make_float4(float(u.x), float(u.y), float(u.z), 0.0f));
        quads.push_back(make_float4(float(v.x), float(v.y), float(v.z), 0.0f));
        quads.push_back(make_float4(float(q.normal[0]), float(q.normal[1]), float(q.normal[2]), 0.0f));
        quads.push_back(make_float4(float(w.x), float(w.y), float(w.z), 0.0f));
    }
    PUT(quads, D.quads);

    std::vector<float4> tris;
    std::vector<int4> tri_shading;
    tris.reserve(size_t(F.triangle_count) * 3);
    for (int64_t k = 0; k < F.triangle_count; k++) {
        const auto& t = F.triangles[k];
        for (int c = 0; c < 3; c++) {
            const double* p = F.positions + 3 * int64_t(t.v[c]);
            int w = c == 0 ? t.material : (c == 1 ? t.flags : t.mesh);
            tris.push_back(make_float4(float(p[0]), float(p[1]), float(p[2]), ibits(w)));
        }
        tri_shading.push_back(make_int4(t.n[0], t.n[1], t.n[2], t.t[0]));
        // an HDR image is opaque everywhere (texture.h:110-113): no test
        int mask = -1;
        if (t.flags & MYPBR_TRI_ALPHA_MASK) {
            int m = F.meshes[t.mesh].alpha_mask;
            if (!(F.textures[m].flags & MYPBR_TEXF_HDR)) {
                mask = m;
                D.has_alpha = 1;
            }
        }
        tri_shading.push_back(make_int4(t.t[1], t.t[2], mask, -1));
    }
    PUT(tris, D.tris);
    PUT(tri_shading, D.tri_shading);
    std::vector<float3> normals;
    for (int64_t k = 0; k < F.normal_count; k++)
        normals.push_back(make_float3(float(F.normals[3 * k]), float(F.normals[3 * k + 1]), float(F.normals[3 * k + 2])));
    PUT(normals, D.normals);
    std::vector<float2> uvs;
    for (int64_t k = 0; k < F.uv_count; k++)
        uvs.push_back(make_float2(float(F.uvs[2 * k]), float(F.uvs[2 * k + 1])));
    PUT(uvs, D.uvs);

    std::vector<float4> media;
    for (int64_t k = 0; k < F.medium_count; k++) {
        const auto& m = F.media[k];
        media.push_back(make_float4(float(m.a[0]), float(m.a[1]), float(m.a[2]), float(m.density)));
        media.push_back(make_float4(float(m.b[0]), float(m.b[1]), float(m.b[2]), ibits(m.shape)));
        media.push_back(make_float4(ibits(m.xform), ibits(m.material), 0.0f, 0.0f));
    }
    PUT(media, D.media);

    std::vector<float4> xforms;
    for (int64_t k = 0; k < F.xform_count; k++) {
        const auto& x = F.xforms[k];
        for (int r = 0; r < 3; r++)
            xforms.push_back(make_float4(float(x.m[r][0]), float(x.m[r][1]), float(x.m[r][2]), float(x.t[r])));
        for (int r = 0; r < 3; r++)
            xforms.push_back(
                make_float4(float(x.inv_m[r][0]), float(x.inv_m[r][1]), float(x.inv_m[r][2]), float(x.inv_t[r])));
    }
    PUT(xforms, D.xforms);

    std::vector<DevUnbounded> unb;
    for (int64_t k = 0; k < F.unbounded_count; k++) {
        const auto& u = F.unbounded[k];
        DevUnbounded d{};
        d.kind = u.kind;
        d.material = u.material;
        d.height = float(u.height);
        d.density = float(u.density);
        d.scale_height = float(u.scale_height);
        unb.push_back(d);
    }
    PUT(unb, D.unbounded);
    D.unbounded_count = int(unb.size());

    // Per (cells, palette) pair, the cells' kinds: the DDA then reads one byte
    // per step and looks the palette up only for the material of a hit.
    std::vector<DevVoxelModel> vmodels;
    std::vector<uint8_t> vkinds;
    std::map<std::pair<int64_t, int>, long long> kinds_at;
    for (int64_t k = 0; k < F.voxel_model_count; k++) {
        const auto& m = F.voxel_models[k];
        DevVoxelModel d{};
        d.nx = m.nx;
        d.ny = m.ny;
        d.nz = m.nz;
        d.xform = m.xform;
        d.cells = m.cells;
        d.palette = m.palette;
        d.edge_material = m.edge_material;
        d.edge_width = float(m.edge_width);
        auto key = std::make_pair(int64_t(m.cells), int(m.palette));
        auto it = kinds_at.find(key);
        if (it == kinds_at.end()) {
            size_t n = size_t(m.nx) * m.ny * m.nz;
            long long off = (long long)vkinds.size();
            vkinds.resize(vkinds.size() + n);
            for (size_t c = 0; c < n; c++)
                vkinds[size_t(off) + c] = uint8_t(F.voxel_palettes[m.palette + F.voxel_cells[m.cells + int64_t(c)]].kind);
            it = kinds_at.emplace(key, off).first;
        }
        d.kinds = it->second;
        vmodels.push_back(d);
    }
    PUT(vmodels, D.voxel_models);
    PUT(vkinds, D.voxel_kinds);
    D.has_voxels = F.voxel_block_count > 0;
    std::vector<int4> vblocks;
    for (int64_t k = 0; k < F.voxel_block_count; k++) {
        const auto& b = F.voxel_blocks[k];
        vblocks.push_back(make_int4(b.model, b.lo[0], b.lo[1], b.lo[2]));
        vblocks.push_back(make_int4(b.hi[0], b.hi[1], b.hi[2], 0));
    }
    PUT(vblocks, D.voxel_blocks);
    std::vector<int2> vpal;
    for (int64_t k = 0; k < F.voxel_palette_count; k++)
        vpal.push_back(make_int2(F.voxel_palettes[k].material, F.voxel_palettes[k].kind));
    PUT(vpal, D.voxel_palettes);
    std::vector<uint8_t> vcells(F.voxel_cells, F.voxel_cells + F.voxel_cell_bytes);
    PUT(vcells, D.voxel_cells);

    // ---- appearance
    std::vector<DevMaterial> mats;
    for (int64_t k = 0; k < F.material_count; k++) {
        const auto& m = F.materials[k];
        DevMaterial d{};
        d.type = m.type;
        d.flags = m.flags;
        d.normal_map = m.normal_map;
        d.emission_tex = m.emission_tex;
        for (int t = 0; t < 8; t++)
            d.tex[t] = m.tex[t];
        for (int p = 0; p < 16; p++)
            d.p[p] = float(m.p[p]);
        mats.push_back(d);
    }
    PUT(mats, D.materials);
    // Shading classes (render.cu): 1 lambertian, 2 metal, 3 dielectric,
    // 4 principled, 5 everything else (wrappers, lights, thin glass, media)
    std::vector<uint8_t> cls;
    for (int64_t k = 0; k < F.material_count; k++) {
        const auto& m = F.materials[k];
        bool plain = m.emission_tex < 0 && (m.normal_map < 0 || m.type == MYPBR_MAT_PRINCIPLED);
        uint8_t c = 5;
        if (plain && m.type == MYPBR_MAT_LAMBERTIAN)
            c = 1;
        else if (plain && m.type == MYPBR_MAT_METAL)
            c = 2;
        else if (plain && m.type == MYPBR_MAT_DIELECTRIC)
            c = 3;
        else if (plain && m.type == MYPBR_MAT_PRINCIPLED)
            c = 4;
        cls.push_back(c);
    }
    PUT(cls, D.mat_class);
    for (int64_t k = 0; k < F.material_count; k++) {
        const auto& m = F.materials[k];
        if (m.type == MYPBR_MAT_DIFFUSE_LIGHT || m.emission_tex >= 0)
            D.has_emitters = 1;
        if (m.type == MYPBR_MAT_DIELECTRIC && m.p[1] == 0)
            D.has_clear_glass = 1;
    }
    D.has_media = F.medium_count > 0;
    for (int64_t k = 0; k < F.unbounded_count; k++)
        if (F.unbounded[k].kind == MYPBR_UNBOUNDED_HEIGHT_FOG)
            D.has_media = 1;
    std::vector<DevTexture> texs;
    for (int64_t k = 0; k < F.texture_count; k++) {
        const auto& t = F.textures[k];
        DevTexture d{};
        d.type = t.type;
        d.a = t.a;
        d.b = t.b;
        d.width = t.width;
        d.height = t.height;
        d.flags = t.flags;
        d.offset = t.offset;
        for (int p = 0; p < 6; p++)
            d.p[p] = float(t.p[p]);
        if (t.type == MYPBR_TEX_UV_TRANSFORM) {
            d.p[2] = float(std::cos(t.p[2]));
            d.p[5] = float(std::sin(t.p[2]));
        }
        texs.push_back(d);
    }
    PUT(texs, D.textures);
    std::vector<uint8_t> ldr(F.texels_ldr, F.texels_ldr + F.texels_ldr_bytes);
    PUT(ldr, D.texels_ldr);
    std::vector<float> hdr(F.texels_hdr, F.texels_hdr + F.texels_hdr_count);
    PUT(hdr, D.texels_hdr);
    const auto& tab = ggx_table_cached();
    // complements 1 - E and 1 - E_avg, formed in FP64 (see table_one_minus_E)
    std::vector<float> ge(1024), ga(32);
    for (int k = 0; k < 1024; k++)
        ge[size_t(k)] = float(1.0 - tab[size_t(k)]);
    for (int k = 0; k < 32; k++)
        ga[size_t(k)] = float(1.0 - tab[size_t(1024 + k)]);
    PUT(ge, D.ggx_e);
    PUT(ga, D.ggx_eavg);

    // ---- lights
    std::vector<DevLight> lights;
    std::vector<DevMember> members(size_t(F.light_member_count));
    double acc = 0;
    for (int64_t k = 0; k < F.light_count; k++) {
        const auto& L = F.lights[k];
        DevLight d{};
        d.kind = L.kind;
        d.first_member = L.first_member;
        d.member_count = L.member_count;
        d.probability = float(L.probability);
        acc += L.probability;
        d.cdf_hi = k + 1 == F.light_count ? 2.0f : float(acc);  // the last light takes the rest
        lights.push_back(d);
        if (L.kind == MYPBR_LIGHT_GROUP) {
            double macc = 0;
            for (int m = 0; m < L.member_count; m++) {
                const auto& mb = F.light_members[L.first_member + m];
                macc += mb.weight;
                DevMember dm{};
                dm.kind = mb.prim_kind;
                dm.index = mb.prim_index;
                dm.weight = float(mb.weight);
                dm.cdf = m + 1 == L.member_count ? 2.0f : float(macc);
                members[size_t(L.first_member + m)] = dm;
            }
        }
    }
    PUT(lights, D.lights);
    PUT(members, D.members);
    D.light_count = int(lights.size());

    // ---- environment: pixels, per-texel pdf and alias table
    D.env_w = F.environment.width > 0 ? F.environment.width : 0;
    D.env_h = D.env_w > 0 ? F.environment.height : 0;
    D.env_intensity = float(F.environment.intensity);
    D.env_rotation = float(F.environment.rotation);
    if (D.env_w > 0) {
        int w = D.env_w, h = D.env_h;
        size_t n = size_t(w) * h;
        std::vector<float4> px(n);
        for (size_t k = 0; k < n; k++) {
            const float* p = F.environment.pixels + 3 * k;
            px[k] = make_float4(p[0], p[1], p[2], 0.0f);
        }
        PUT(px, D.env_pixels);
        // the sampling distribution, built on the device from the pixels
        float* rgb = nullptr;
        float* texel_pdf = nullptr;
        float2* alias = nullptr;
        if (cudaMalloc(&rgb, n * 3 * sizeof(float)) != cudaSuccess ||
            cudaMalloc(&texel_pdf, n * sizeof(float)) != cudaSuccess ||
            cudaMalloc(&alias, n * sizeof(float2)) != cudaSuccess) {
            cudaFree(rgb);
            cudaFree(texel_pdf);
            cudaFree(alias);
            set_error_message("mypbr_gpu_scene_create: out of device memory for the environment");
            return fail_cleanup(MYPBR_ERR_OUT_OF_MEMORY);
        }
        G.allocations.push_back(texel_pdf);
        G.allocations.push_back(alias);
        int st = MYPBR_OK;
        if (cudaMemcpy(rgb, F.environment.pixels, n * 3 * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
            st = cuda_fail(cudaGetLastError(), "environment upload");
        if (st == MYPBR_OK)
            st = build_env_distribution(rgb, w, h, texel_pdf, alias, G.stream);
        cudaFree(rgb);
        if (st != MYPBR_OK)
            return fail_cleanup(st);
        D.env_texel_pdf = texel_pdf;
        D.env_alias = alias;
    }

    // ---- sun (sun.h:23-43) and the plain sky
    D.sun_enabled = F.sun.enabled;
    D.sun_disk_visible = F.sun.disk_visible;
    if (F.sun.enabled) {
        mypbr_host::V3 d(F.sun.direction[0], F.sun.direction[1], F.sun.direction[2]);
        d = mypbr_host::unit(d);
        double half = std::fmax(F.sun.angular_diameter, 1e-3) * 3.1415926535897932385 / 180.0 / 2;
        double cmax = std::cos(half);
        double omega = 2 * 3.1415926535897932385 * (1 - cmax);
        D.sun_dir = make_float3(float(d.x), float(d.y), float(d.z));
        D.sun_cos_max = float(cmax);
        D.sun_solid_angle = float(omega);
        D.sun_radiance = make_float3(float(F.sun.irradiance[0] / omega), float(F.sun.irradiance[1] / omega),
                                     float(F.sun.irradiance[2] / omega));
    }
    G.material_count = F.material_count;
    D.use_sky = F.use_sky;
    D.background = make_float3(float(F.background[0]), float(F.background[1]), float(F.background[2]));
#undef PUT
    *out = holder.release();
    return MYPBR_OK;
}

}  // namespace mypbr_dev

namespace mypbr_dev {

// The environment's sampling tables on the host: per-texel weights
// luminance x sin(theta) (environment.h:147-176; rows by sin(theta) for a
// black sky, environment.h:302-309), the pdf table p n and Vose's alias table.
void env_distribution_host(const float* rgb, int w, int h, float* texel_pdf, float2* alias) {
    size_t n = size_t(w) * h;
    std::vector<double> wgt(n);
    const double kPiD = 3.1415926535897932385;
    double total = 0;
    for (int j = 0; j < h; j++) {
        double st = std::sin(kPiD * (j + 0.5) / h);
        for (int i = 0; i < w; i++) {
            const float* p = rgb + (size_t(j) * w + i) * 3;
            double l = 0.2126 * p[0] + 0.7152 * p[1] + 0.0722 * p[2];
            wgt[size_t(j) * w + i] = std::fmax(l * st, 0.0);
            total += wgt[size_t(j) * w + i];
        }
    }
    if (!(total > 0)) {
        total = 0;
        for (int j = 0; j < h; j++)
            for (int i = 0; i < w; i++) {
                wgt[size_t(j) * w + i] = std::sin(kPiD * (j + 0.5) / h);
                total += wgt[size_t(j) * w + i];
            }
    }
    std::vector<double> scaled(n);
    std::vector<uint32_t> small, large;
    for (size_t k = 0; k < n; k++) {
        double prob = wgt[k] / total;
        texel_pdf[k] = float(prob * double(n));
        scaled[k] = prob * double(n);
        (scaled[k] < 1.0 ? small : large).push_back(uint32_t(k));
    }
    while (!small.empty() && !large.empty()) {
        uint32_t s = small.back(), l = large.back();
        small.pop_back();
        alias[s] = make_float2(float(scaled[s]), ibits(int(l)));
        scaled[l] = (scaled[l] + scaled[s]) - 1.0;
        if (scaled[l] < 1.0) {
            large.pop_back();
            small.push_back(l);
        }
    }
    for (uint32_t l : large)
        alias[l] = make_float2(1.0f, ibits(int(l)));
    for (uint32_t s : small)
        alias[s] = make_float2(1.0f, ibits(int(s)));
}

// The binary tree (64-byte nodes holding both children's boxes) collapsed to
// four children per node: starting from a node's two children, the interior
// child of largest surface area is replaced by its own two children until
// there are four or none is interior. Node layout as walk_tree4 reads it.
// depth: the deepest level of the result (0 at the root).
void collapse_to_4(const std::vector<float4>& bin, std::vector<float4>& out, int& depth) {
    struct Child {
        float4 lo, hi;  // w: index, count (float bits) as in the binary node
        int index() const { return float_bits(lo.w); }
        int count() const { return float_bits(hi.w); }
    };
    auto children = [&](int i, Child* c) {
        c[0] = {bin[size_t(i) * 4], bin[size_t(i) * 4 + 1]};
        c[1] = {bin[size_t(i) * 4 + 2], bin[size_t(i) * 4 + 3]};
    };
    auto area = [](const Child& c) {
        double x = double(c.hi.x) - c.lo.x, y = double(c.hi.y) - c.lo.y, z = double(c.hi.z) - c.lo.z;
        if (!(x >= 0 && y >= 0 && z >= 0) || !std::isfinite(x + y + z))
            return -1.0;
        return x * y + y * z + z * x;
    };
    depth = 0;
    std::function<int(int, int)> build = [&](int i, int level) -> int {
        depth = std::max(depth, level);
        Child list[4];
        children(i, list);
        int n = 2;
        while (n < 4) {
            int best = -1;
            double best_area = -2;
            for (int k = 0; k < n; k++)
                if (list[k].count() == 0 && area(list[k]) > best_area) {
                    best = k;
                    best_area = area(list[k]);
                }
            if (best < 0)
                break;
            Child sub[2];
            children(list[best].index(), sub);
            list[best] = sub[0];
            list[n++] = sub[1];
        }
        int me = int(out.size() / 8);
        out.resize(out.size() + 8);
        int child[4], count[4];
        for (int k = 0; k < 4; k++) {
            if (k >= n) {
                child[k] = 0;
                count[k] = -1;
            } else if (list[k].count() > 0) {
                child[k] = list[k].index();
                count[k] = list[k].count();
            } else {
                child[k] = build(list[k].index(), level + 1);
                count[k] = 0;
            }
        }
        float4* row = &out[size_t(me) * 8];
        const float inf = INFINITY;
        float v[6][4];
        for (int k = 0; k < 4; k++) {
            bool used = k < n;
            v[0][k] = used ? list[k].lo.x : inf;
            v[1][k] = used ? list[k].hi.x : inf;
            v[2][k] = used ? list[k].lo.y : inf;
            v[3][k] = used ? list[k].hi.y : inf;
            v[4][k] = used ? list[k].lo.z : inf;
            v[5][k] = used ? list[k].hi.z : inf;
        }
        for (int r = 0; r < 6; r++)
            row[r] = make_float4(v[r][0], v[r][1], v[r][2], v[r][3]);
        row[6] = make_float4(ibits(child[0]), ibits(child[1]), ibits(child[2]), ibits(child[3]));
        row[7] = make_float4(ibits(count[0]), ibits(count[1]), ibits(count[2]), ibits(count[3]));
        return me;
    };
    build(0, 0);
}

// The binary tree collapsed to eight children per node (the interior child of
// largest surface area expanded first, as for four), each node 96 bytes:
//   row 0      the origin p (3 floats, at least one quantum below the
//              node's box) and, per axis, the biased exponent e of the
//              quantum 2^(e - 127) (bytes 0-2)
//   rows 1-3   per axis: the children's low planes as bytes (8), then their
//              high planes (8); a plane is p + q 2^(e - 127)
//   rows 4-5   per child a word: a node index, or 1 << 31 | first << 4 |
//              count for a leaf of `count` references from `first`, or
//              0xffffffff for an empty slot
// Quantised boxes contain the child's box with one to two quanta to spare on
// every side; the quantum is at least four float steps of the node's
// coordinates.
bool collapse_to_8q(const std::vector<float4>& bin, std::vector<uint4>& out, int& depth) {
    struct Child {
        float4 lo, hi;
        int index() const { return float_bits(lo.w); }
        int count() const { return float_bits(hi.w); }
    };
    auto children = [&](int i, Child* c) {
        c[0] = {bin[size_t(i) * 4], bin[size_t(i) * 4 + 1]};
        c[1] = {bin[size_t(i) * 4 + 2], bin[size_t(i) * 4 + 3]};
    };
    auto area = [](const Child& c) {
        double x = double(c.hi.x) - c.lo.x, y = double(c.hi.y) - c.lo.y, z = double(c.hi.z) - c.lo.z;
        if (!(x >= 0 && y >= 0 && z >= 0) || !std::isfinite(x + y + z))
            return -1.0;
        return x * y + y * z + z * x;
    };
    auto axis = [](const float4& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); };
    out.clear();
    depth = 0;
    bool ok = true;
    std::function<int(int, int)> build = [&](int i, int level) -> int {
        depth = std::max(depth, level);
        Child list[8];
        children(i, list);
        int n = 2;
        while (n < 8) {
            int best = -1;
            double best_area = -2;
            for (int k = 0; k < n; k++)
                if (list[k].count() == 0 && area(list[k]) > best_area) {
                    best = k;
                    best_area = area(list[k]);
                }
            if (best < 0)
                break;
            Child sub[2];
            children(list[best].index(), sub);
            list[best] = sub[0];
            list[n++] = sub[1];
        }
        // empty padding children (boxes at +infinity) take no slot
        int m = 0;
        for (int k = 0; k < n; k++)
            if (std::isfinite(list[k].lo.x) || list[k].count() == 0)
                list[m++] = list[k];
        n = m;
        const int me = int(out.size() / 6);
        out.resize(out.size() + 6);
        double lo[3], hi[3];
        for (int a = 0; a < 3; a++) {
            lo[a] = INFINITY;
            hi[a] = -INFINITY;
            for (int k = 0; k < n; k++) {
                lo[a] = std::min(lo[a], double(axis(list[k].lo, a)));
                hi[a] = std::max(hi[a], double(axis(list[k].hi, a)));
            }
            if (!(lo[a] <= hi[a]))
                lo[a] = hi[a] = 0.0;
        }
        // per axis: the quantum s = 2^e, at least four float steps of the
        // coordinates, and the origin p one quantum or more below the box;
        // every child plane then lies one to two quanta outside the child's
        // own (low planes rounded down, high planes up, one more quantum
        // each), so FP32 rounding of the slab distances cannot cut a child
        uint32_t ebias[3];
        double quantum[3], origin[3];
        for (int a = 0; a < 3; a++) {
            const double mag = std::max(std::fabs(lo[a]), std::fabs(hi[a])) + 1e-30;
            const double extent = hi[a] - lo[a];
            int e = std::max(std::ilogb(mag) - 21, -126);
            if (extent > 0)
                e = std::max(e, int(std::ceil(std::log2(extent / 250.0))));
            for (;; e++) {
                const double sq = std::ldexp(1.0, e);
                const float pf = std::nextafter(float(lo[a] - sq), -INFINITY);  // at or below lo - s
                if (e >= 127 || (std::ceil((hi[a] - double(pf)) / sq) + 1.0 <= 255.0 && double(pf) <= lo[a] - sq)) {
                    origin[a] = double(pf);
                    break;
                }
            }
            ebias[a] = uint32_t(std::min(e, 127) + 127);
            quantum[a] = std::ldexp(1.0, std::min(e, 127));
        }
        uint8_t qlo[3][8], qhi[3][8];
        uint32_t word[8];
        for (int k = 0; k < 8; k++) {
            for (int a = 0; a < 3; a++) {
                qlo[a][k] = 1;  // empty slots: an inverted box, and an empty word
                qhi[a][k] = 0;
            }
            word[k] = 0xffffffffu;
        }
        for (int k = 0; k < n; k++) {
            for (int a = 0; a < 3; a++) {
                const double p = origin[a], sq = quantum[a];
                const double cl = axis(list[k].lo, a), ch = axis(list[k].hi, a);
                const double ql = std::floor((cl - p) / sq) - 1.0, qh = std::ceil((ch - p) / sq) + 1.0;
                qlo[a][k] = uint8_t(std::min(std::max(ql, 0.0), 255.0));
                qhi[a][k] = uint8_t(std::min(std::max(qh, 0.0), 255.0));
            }
        }
        int child_node[8];
        for (int k = 0; k < n; k++)
            child_node[k] = list[k].count() == 0 ? build(list[k].index(), level + 1) : -1;
        for (int k = 0; k < n; k++) {
            if (list[k].count() == 0) {
                word[k] = uint32_t(child_node[k]);
            } else {
                const int first = list[k].index(), count = list[k].count();
                if (count >= 16 || first < 0 || first >= (1 << 27)) {
                    ok = false;
                    continue;
                }
                word[k] = 0x80000000u | (uint32_t(first) << 4) | uint32_t(count);
            }
        }
        uint4* row = &out[size_t(me) * 6];
        row[0] = make_uint4(uint32_t(float_bits(float(origin[0]))), uint32_t(float_bits(float(origin[1]))),
                            uint32_t(float_bits(float(origin[2]))), ebias[0] | (ebias[1] << 8) | (ebias[2] << 16));
        auto pack = [](const uint8_t* q, int from) {
            return uint32_t(q[from]) | (uint32_t(q[from + 1]) << 8) | (uint32_t(q[from + 2]) << 16) |
                   (uint32_t(q[from + 3]) << 24);
        };
        for (int a = 0; a < 3; a++)
            row[1 + a] = make_uint4(pack(qlo[a], 0), pack(qlo[a], 4), pack(qhi[a], 0), pack(qhi[a], 4));
        row[4] = make_uint4(word[0], word[1], word[2], word[3]);
        row[5] = make_uint4(word[4], word[5], word[6], word[7]);
        return me;
    };
    if (!bin.empty())
        build(0, 0);
    if (!ok)
        out.clear();
    return ok && !out.empty();
}

}  // namespace mypbr_dev

extern "C" int mypbr_gpu_scene_create(const mypbr_flat_scene* scene, mypbr_gpu_scene** out) {
    mypbr_dev::NvtxRange range("mypbr scene upload");
    try {
        return mypbr_dev::create_scene(scene, out);
    } catch (const std::bad_alloc&) {
        mypbr_dev::set_error_message("mypbr_gpu_scene_create: out of host memory");
        return MYPBR_ERR_OUT_OF_MEMORY;
    }
}

namespace mypbr_dev {
// Reads and clears the sticky device error word after a synchronised call.
int check_device_error(mypbr_gpu_scene* G) {
    int e = 0;
    MYPBR_CUDA(cudaMemcpy(&e, G->dev.error, sizeof e, cudaMemcpyDeviceToHost));
    if (e == 0)
        return MYPBR_OK;
    int zero = 0;
    MYPBR_CUDA(cudaMemcpy(G->dev.error, &zero, sizeof zero, cudaMemcpyHostToDevice));
    if (e == 3) {
        set_error_message("device wait: a tensor-core wait of the guiding network ran past its limit");
        return MYPBR_ERR_DEVICE_TIMEOUT;
    }
    set_error_message(e == 1 ? "device check: a BVH walk visited more nodes than the tree has"
                             : "device check: a BVH walk overflowed its stack");
    return MYPBR_ERR_DEVICE_CHECK;
}
}  // namespace mypbr_dev

extern "C" void mypbr_gpu_scene_destroy(mypbr_gpu_scene* scene) {
    if (!scene)
        return;
    mypbr_dev::release_batch_graph(scene);
    mypbr_dev::release_buffers(scene->rb);
    mypbr_dev::release_guide(scene->guide);
    for (void* p : scene->allocations)
        cudaFree(p);
    if (scene->stream)
        cudaStreamDestroy(scene->stream);
    delete scene;
}
