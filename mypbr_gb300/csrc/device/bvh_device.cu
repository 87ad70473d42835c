// A BVH built on the device: a linear BVH (LBVH) over the scene's primitives,
// for scenes whose load time the host SAH build (bvh_build.cpp, the
// reference's bvh.h:110-205) dominates. Morton codes of the primitive
// centroids (30 bits, 10 per axis, in the scene box) extended by the
// primitive's position to make every key unique; a radix sort (CUB); the
// hierarchy of Karras, "Maximizing Parallelism in the Construction of BVHs,
// Octrees, and k-d Trees" (HPG 2012), one thread per internal node; boxes
// fitted bottom-up, the second child to arrive at a node computing it.
// The result replaces the scene handle's device BVH in the same node layout
// (one primitive per leaf). Its SAH cost, and the host tree's, are reported so
// that the quality difference is visible: the host SAH build stays the
// reference's and the default.
#include <cub/cub.cuh>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "gpu_scene.h"

namespace mypbr_dev {
namespace {

struct Box3 {
    float3 lo, hi;
};

MYPBR_DEV void grow(Box3& b, float3 p) {
    b.lo = f3(fminf(b.lo.x, p.x), fminf(b.lo.y, p.y), fminf(b.lo.z, p.z));
    b.hi = f3(fmaxf(b.hi.x, p.x), fmaxf(b.hi.y, p.y), fmaxf(b.hi.z, p.z));
}

MYPBR_DEV Box3 empty_box() { return Box3{f3(3.0e38f), f3(-3.0e38f)}; }

// The 8 corners of an object-space box, placed by transform x.
MYPBR_DEV Box3 placed(const DeviceScene& S, int x, float3 lo, float3 hi) {
    if (x < 0)
        return Box3{lo, hi};
    XformRef X;
    load_xform(S, x, X);
    Box3 b = empty_box();
    for (int c = 0; c < 8; c++)
        grow(b, xf_point(X, f3((c & 1) ? hi.x : lo.x, (c & 2) ? hi.y : lo.y, (c & 4) ? hi.z : lo.z)));
    return b;
}

// World box of the primitive of leaf reference `ref`, widened by a few ulps
// of its extent so that FP32 rounding of the corners never shrinks it.
MYPBR_DEV Box3 prim_box(const DeviceScene& S, uint32_t ref) {
    int kind = int(ref >> kKindShift), idx = int(ref & kIndexMask);
    Box3 b = empty_box();
    if (kind == kSphere) {
        float4 s = S.spheres[idx];
        float r = fabsf(s.w);
        b = placed(S, S.sphere_info[idx].y, f3(s.x - r, s.y - r, s.z - r), f3(s.x + r, s.y + r, s.z + r));
    } else if (kind == kQuad) {
        const float4* q = S.quads + 5 * idx;
        float3 Q = f3(q[0]), u = f3(q[1]), v = f3(q[2]);
        grow(b, Q);
        grow(b, Q + u);
        grow(b, Q + v);
        grow(b, Q + u + v);
    } else if (kind == kTriangle) {
        const float4* t = S.tris + 3 * idx;
        grow(b, f3(t[0]));
        grow(b, f3(t[1]));
        grow(b, f3(t[2]));
    } else if (kind == kMedium) {
        float4 a = S.media[3 * idx], c = S.media[3 * idx + 1], e = S.media[3 * idx + 2];
        int shape = __float_as_int(c.w), xf = __float_as_int(e.x);
        float3 lo, hi;
        if (shape == 0) {
            float r = fabsf(c.x);
            lo = f3(a.x - r, a.y - r, a.z - r);
            hi = f3(a.x + r, a.y + r, a.z + r);
        } else {
            lo = f3(fminf(a.x, c.x), fminf(a.y, c.y), fminf(a.z, c.z));
            hi = f3(fmaxf(a.x, c.x), fmaxf(a.y, c.y), fmaxf(a.z, c.z));
        }
        b = placed(S, xf, lo, hi);
    } else if (kind == kVoxel) {
        int4 b0 = S.voxel_blocks[2 * idx], b1 = S.voxel_blocks[2 * idx + 1];
        b = placed(S, S.voxel_models[b0.x].xform, f3(float(b0.y), float(b0.z), float(b0.w)),
                   f3(float(b1.x), float(b1.y), float(b1.z)));
    }
    float3 ext = b.hi - b.lo;
    float pad = 4e-6f * (fmaxf(fmaxf(fabsf(b.lo.x), fabsf(b.hi.x)), fmaxf(fmaxf(fabsf(b.lo.y), fabsf(b.hi.y)),
                                                                     fmaxf(fabsf(b.lo.z), fabsf(b.hi.z)))) +
                          fmaxf(ext.x, fmaxf(ext.y, ext.z))) + 1e-30f;
    b.lo = b.lo - f3(pad);
    b.hi = b.hi + f3(pad);
    return b;
}

// Floats ordered as unsigned integers, for atomic min / max of the scene box.
MYPBR_DEV uint32_t ordered(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
MYPBR_HD float unordered(uint32_t u) {
    uint32_t v = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    float f;
    memcpy(&f, &v, 4);
    return f;
}

__global__ void k_prim_boxes(DeviceScene S, const uint32_t* refs, int n, Box3* boxes, uint32_t* scene_box) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        Box3 b = prim_box(S, refs[i]);
        boxes[i] = b;
        float3 c = 0.5f * (b.lo + b.hi);
        atomicMin(scene_box + 0, ordered(c.x));
        atomicMin(scene_box + 1, ordered(c.y));
        atomicMin(scene_box + 2, ordered(c.z));
        atomicMax(scene_box + 3, ordered(c.x));
        atomicMax(scene_box + 4, ordered(c.y));
        atomicMax(scene_box + 5, ordered(c.z));
    }
}

MYPBR_DEV uint32_t spread10(uint32_t v) {  // 10 bits -> every third bit
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__global__ void k_morton(const Box3* boxes, int n, const uint32_t* scene_box, unsigned long long* keys,
                         uint32_t* order) {
    float3 lo = f3(unordered(scene_box[0]), unordered(scene_box[1]), unordered(scene_box[2]));
    float3 hi = f3(unordered(scene_box[3]), unordered(scene_box[4]), unordered(scene_box[5]));
    float3 ext = hi - lo;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float3 c = 0.5f * (boxes[i].lo + boxes[i].hi);
        auto q = [](float v, float l, float e) {
            float t = e > 0.0f ? (v - l) / e : 0.5f;
            return uint32_t(fminf(fmaxf(t * 1024.0f, 0.0f), 1023.0f));
        };
        uint32_t m = (spread10(q(c.x, lo.x, ext.x)) << 2) | (spread10(q(c.y, lo.y, ext.y)) << 1) |
                     spread10(q(c.z, lo.z, ext.z));
        keys[i] = (unsigned long long)m << 32 | uint32_t(i);
        order[i] = uint32_t(i);
    }
}

// Common-prefix length of sorted keys i and j (-1 outside [0, n)).
MYPBR_DEV int delta(const unsigned long long* k, int n, int i, int j) {
    if (j < 0 || j >= n)
        return -1;
    return __clzll(k[i] ^ k[j]);
}

// Karras 2012, algorithm 2: the range and split of internal node i. Children
// are encoded as (index << 1) | leaf.
__global__ void k_hierarchy(const unsigned long long* k, int n, int2* children, int* parent) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n - 1; i += gridDim.x * blockDim.x) {
        int d = delta(k, n, i, i + 1) > delta(k, n, i, i - 1) ? 1 : -1;
        int dmin = delta(k, n, i, i - d);
        int lmax = 2;
        while (delta(k, n, i, i + lmax * d) > dmin)
            lmax <<= 1;
        int l = 0;
        for (int t = lmax >> 1; t >= 1; t >>= 1)
            if (delta(k, n, i, i + (l + t) * d) > dmin)
                l += t;
        int j = i + l * d;
        int dnode = delta(k, n, i, j);
        int s = 0;
        int len = l;
        for (int t = (len + 1) >> 1;; t = (t + 1) >> 1) {
            if (delta(k, n, i, i + (s + t) * d) > dnode)
                s += t;
            if (t == 1)
                break;
        }
        int gamma = i + s * d + min(d, 0);
        int lo = min(i, j), hi = max(i, j);
        int left = lo == gamma ? (gamma << 1) | 1 : (gamma << 1);
        int right = hi == gamma + 1 ? ((gamma + 1) << 1) | 1 : ((gamma + 1) << 1);
        children[i] = make_int2(left, right);
        // parents: internal nodes in parent[0, n-1), leaves in parent[n-1, 2n-1)
        parent[(left & 1) ? n - 1 + (left >> 1) : (left >> 1)] = i;
        parent[(right & 1) ? n - 1 + (right >> 1) : (right >> 1)] = i;
    }
}

// Bottom-up boxes: each leaf walks towards the root; at every node the first
// child to arrive stops, the second writes the node (both children's boxes
// and references) and goes on.
__global__ void k_fit(const Box3* sorted_boxes, const int2* children, const int* parent, int n, int* arrivals,
                      Box3* node_box, float4* nodes) {
    for (int leaf = blockIdx.x * blockDim.x + threadIdx.x; leaf < n; leaf += gridDim.x * blockDim.x) {
        int node = parent[n - 1 + leaf];
        int guard = 0;
        while (node >= 0 && guard++ < n) {
            __threadfence();
            if (atomicAdd(&arrivals[node], 1) == 0)
                break;  // the other child is not done yet
            __threadfence();
            int2 ch = children[node];
            Box3 b[2];
            int idx[2], cnt[2];
            for (int c = 0; c < 2; c++) {
                int e = c == 0 ? ch.x : ch.y;
                if (e & 1) {
                    b[c] = sorted_boxes[e >> 1];
                    idx[c] = e >> 1;
                    cnt[c] = 1;
                } else {
                    // written by another thread (maybe another SM): read past L1
                    const volatile float* v = reinterpret_cast<const volatile float*>(node_box + (e >> 1));
                    b[c] = Box3{f3(v[0], v[1], v[2]), f3(v[3], v[4], v[5])};
                    idx[c] = e >> 1;
                    cnt[c] = 0;
                }
            }
            float4* o = nodes + 4 * node;
            o[0] = make_float4(b[0].lo.x, b[0].lo.y, b[0].lo.z, __int_as_float(idx[0]));
            o[1] = make_float4(b[0].hi.x, b[0].hi.y, b[0].hi.z, __int_as_float(cnt[0]));
            o[2] = make_float4(b[1].lo.x, b[1].lo.y, b[1].lo.z, __int_as_float(idx[1]));
            o[3] = make_float4(b[1].hi.x, b[1].hi.y, b[1].hi.z, __int_as_float(cnt[1]));
            Box3 u{f3(fminf(b[0].lo.x, b[1].lo.x), fminf(b[0].lo.y, b[1].lo.y), fminf(b[0].lo.z, b[1].lo.z)),
                   f3(fmaxf(b[0].hi.x, b[1].hi.x), fmaxf(b[0].hi.y, b[1].hi.y), fmaxf(b[0].hi.z, b[1].hi.z))};
            node_box[node] = u;
            node = node == 0 ? -1 : parent[node];
        }
    }
}

// Depth of the deepest leaf (interior nodes on its path).
__global__ void k_depth(const int* parent, int n, int* max_depth) {
    for (int leaf = blockIdx.x * blockDim.x + threadIdx.x; leaf < n; leaf += gridDim.x * blockDim.x) {
        int depth = 0;
        for (int node = parent[n - 1 + leaf]; node >= 0 && depth <= n; node = node == 0 ? -1 : parent[node])
            depth++;
        atomicMax(max_depth, depth);
    }
}

__global__ void k_gather(const uint32_t* refs, const Box3* boxes, const uint32_t* order, int n, uint32_t* sorted_refs,
                         Box3* sorted_boxes) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        sorted_refs[i] = refs[order[i]];
        sorted_boxes[i] = boxes[order[i]];
    }
}

double area(float3 lo, float3 hi) {
    float3 e = f3(std::max(hi.x - lo.x, 0.0f), std::max(hi.y - lo.y, 0.0f), std::max(hi.z - lo.z, 0.0f));
    return 2.0 * (double(e.x) * e.y + double(e.y) * e.z + double(e.z) * e.x);
}

// SAH cost of a device tree (bvh.h's constants: 1 per primitive test, 0.125
// per node visited): sum over nodes of area / root area, from node 0.
double sah_cost(const std::vector<float4>& nodes) {
    if (nodes.empty())
        return 0;
    const float4* r = nodes.data();
    float3 lo = f3(std::min(r[0].x, r[2].x), std::min(r[0].y, r[2].y), std::min(r[0].z, r[2].z));
    float3 hi = f3(std::max(r[1].x, r[3].x), std::max(r[1].y, r[3].y), std::max(r[1].z, r[3].z));
    double root = std::max(area(lo, hi), 1e-30);
    double cost = 0.125;  // the root
    size_t count = nodes.size() / 4;
    for (size_t k = 0; k < count; k++)
        for (int c = 0; c < 2; c++) {
            const float4 a = nodes[4 * k + 2 * c], b = nodes[4 * k + 2 * c + 1];
            int cnt = 0;
            std::memcpy(&cnt, &b.w, 4);
            double p = area(f3(a.x, a.y, a.z), f3(b.x, b.y, b.z)) / root;
            cost += cnt > 0 ? p * cnt : p * 0.125;
        }
    return cost;
}

template <typename T>
struct DevArr {
    T* p = nullptr;
    ~DevArr() {
        if (p)
            cudaFree(p);
    }
    int alloc(size_t n) {
        MYPBR_CUDA(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
        return MYPBR_OK;
    }
};

}  // namespace
}  // namespace mypbr_dev

using namespace mypbr_dev;

extern "C" int mypbr_gpu_scene_rebuild_bvh(mypbr_gpu_scene* G, int32_t method, mypbr_bvh_report* report) {
    mypbr_dev::NvtxRange range("mypbr LBVH build");
    if (!G || method != MYPBR_BVH_LBVH) {
        set_error_message("mypbr_gpu_scene_rebuild_bvh: a scene and MYPBR_BVH_LBVH are required");
        return MYPBR_ERR_INVALID_ARGUMENT;
    }
    int n = int(G->leaf_ref_count);
    if (!G->dev.has_bvh || n < 2)
        return MYPBR_OK;  // nothing to build: the host tree stays
    MYPBR_CUDA(cudaSetDevice(G->device));
    DeviceScene& D = G->dev;
    std::vector<float4> before(size_t(D.bvh_node_count) * 4);
    MYPBR_CUDA(cudaMemcpy(before.data(), D.bvh, before.size() * sizeof(float4), cudaMemcpyDeviceToHost));

    DevArr<Box3> boxes, sorted_boxes, node_box;
    DevArr<uint32_t> scene_box, order, order_out, sorted_refs;
    DevArr<unsigned long long> keys, keys_out;
    DevArr<int2> children;
    DevArr<int> parent, arrivals, max_depth;
    DevArr<float4> nodes;
    DevArr<unsigned char> temp;
    int s;
    if ((s = boxes.alloc(n)) || (s = sorted_boxes.alloc(n)) || (s = node_box.alloc(n)) || (s = scene_box.alloc(6)) ||
        (s = order.alloc(n)) || (s = order_out.alloc(n)) || (s = keys.alloc(n)) || (s = keys_out.alloc(n)) ||
        (s = children.alloc(n)) || (s = parent.alloc(2 * size_t(n))) || (s = arrivals.alloc(n)) ||
        (s = max_depth.alloc(1)) || (s = nodes.alloc(4 * size_t(n))))
        return s;
    size_t temp_bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, temp_bytes, keys.p, keys_out.p, order.p, order_out.p, n);
    if ((s = temp.alloc(temp_bytes)))
        return s;
    if ((s = sorted_refs.alloc(n)))
        return s;

    cudaEvent_t e0, e1;
    MYPBR_CUDA(cudaEventCreate(&e0));
    MYPBR_CUDA(cudaEventCreate(&e1));
    const uint32_t init[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
    MYPBR_CUDA(cudaMemcpy(scene_box.p, init, sizeof init, cudaMemcpyHostToDevice));
    MYPBR_CUDA(cudaMemset(arrivals.p, 0, size_t(n) * sizeof(int)));
    MYPBR_CUDA(cudaMemset(max_depth.p, 0, sizeof(int)));
    MYPBR_CUDA(cudaMemset(parent.p, 0xff, 2 * size_t(n) * sizeof(int)));
    int grid = std::min((n + 255) / 256, G->sm_count * 16);
    cudaEventRecord(e0);
    k_prim_boxes<<<grid, 256>>>(D, D.leaf_refs, n, boxes.p, scene_box.p);
    k_morton<<<grid, 256>>>(boxes.p, n, scene_box.p, keys.p, order.p);
    cub::DeviceRadixSort::SortPairs(temp.p, temp_bytes, keys.p, keys_out.p, order.p, order_out.p, n);
    k_gather<<<grid, 256>>>(D.leaf_refs, boxes.p, order_out.p, n, sorted_refs.p, sorted_boxes.p);
    k_hierarchy<<<grid, 256>>>(keys_out.p, n, children.p, parent.p);
    k_fit<<<grid, 256>>>(sorted_boxes.p, children.p, parent.p, n, arrivals.p, node_box.p, nodes.p);
    k_depth<<<grid, 256>>>(parent.p, n, max_depth.p);
    cudaEventRecord(e1);
    MYPBR_CUDA(cudaGetLastError());
    MYPBR_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    int depth = 0;
    MYPBR_CUDA(cudaMemcpy(&depth, max_depth.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (depth + 1 >= kBvhStack) {
        set_error_message("mypbr_gpu_scene_rebuild_bvh: the LBVH is " + std::to_string(depth) +
                          " levels deep, more than the traversal stack holds; the host tree stays");
        return MYPBR_ERR_UNSUPPORTED;
    }
    std::vector<float4> after(size_t(n - 1) * 4);
    MYPBR_CUDA(cudaMemcpy(after.data(), nodes.p, after.size() * sizeof(float4), cudaMemcpyDeviceToHost));
    // the new tree replaces the old one (whose arrays stay until the handle goes)
    G->allocations.push_back(nodes.p);
    G->allocations.push_back(sorted_refs.p);
    // and its 4-wide form, when the 4-wide walk's stack can hold it
    std::vector<float4> wide;
    int depth4 = 0;
    collapse_to_4(after, wide, depth4);
    float4* wide_p = nullptr;
    if (3 * (depth4 + 1) <= kBvh4Stack) {
        MYPBR_CUDA(cudaMalloc(&wide_p, wide.size() * sizeof(float4)));
        MYPBR_CUDA(cudaMemcpy(wide_p, wide.data(), wide.size() * sizeof(float4), cudaMemcpyHostToDevice));
        G->allocations.push_back(wide_p);
    }
    // and its 8-wide quantised form, likewise
    std::vector<uint4> wide8;
    int depth8 = 0;
    uint4* wide8_p = nullptr;
    if (collapse_to_8q(after, wide8, depth8) && 7 * (depth8 + 1) <= kBvh8Stack) {
        MYPBR_CUDA(cudaMalloc(&wide8_p, wide8.size() * sizeof(uint4)));
        MYPBR_CUDA(cudaMemcpy(wide8_p, wide8.data(), wide8.size() * sizeof(uint4), cudaMemcpyHostToDevice));
        G->allocations.push_back(wide8_p);
    }
    D.bvh = nodes.p;
    D.leaf_refs = sorted_refs.p;
    D.bvh_node_count = n - 1;
    D.bvh4 = wide_p;
    D.bvh8 = wide8_p;
    D.bvh8_node_count = wide8_p ? int(wide8.size() / 6) : 0;
    D.postponed_ok = n < (1 << 26);  // one reference per leaf
    D.bvh4_node_count = wide_p ? int(wide.size() / 8) : 0;
    nodes.p = nullptr;
    sorted_refs.p = nullptr;
    G->max_depth_bvh = depth;
    if (report) {
        report->primitives = n;
        report->nodes = n - 1;
        report->depth = depth;
        report->build_ms = ms;
        report->sah_cost = sah_cost(after);
        report->sah_cost_before = sah_cost(before);
    }
    return MYPBR_OK;
}
