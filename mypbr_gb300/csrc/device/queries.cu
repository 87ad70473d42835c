// Pointwise queries for parity checks: ray batches through the BVH walk, and
// BSDF eval / pdf at given surface records. Both run the same device
// functions the renderer runs.
#include <algorithm>
#include <string>

#include "dev_shading.cuh"
#include "gpu_scene.h"

namespace mypbr_dev {

template <int WALK>
__global__ void k_trace(DeviceScene S, const float* rays, long long n, float* hits, int* prim) {
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
        const float* r = rays + 8 * k;
        float3 o = f3(r[0], r[1], r[2]), d = f3(r[3], r[4], r[5]);
        HitInfo h = closest_hit<true, WALK>(S, o, d, r[6], r[7], 0);
        float* out = hits + 8 * k;
        if (h.prim == kMiss) {
            for (int c = 0; c < 8; c++)
                out[c] = 0.0f;
            prim[2 * k] = -1;
            prim[2 * k + 1] = -1;
            continue;
        }
        Surface s = make_surface(S, h, o, d);
        out[0] = h.t;
        out[1] = s.normal.x;
        out[2] = s.normal.y;
        out[3] = s.normal.z;
        out[4] = s.u;
        out[5] = s.v;
        out[6] = s.front ? 1.0f : 0.0f;
        out[7] = float(s.material);
        prim[2 * k] = int(h.prim >> kKindShift);
        prim[2 * k + 1] = int(h.prim & kIndexMask);
    }
}

__global__ void k_bsdf(DeviceScene S, int material, const float* rec, const float* r_in, const float* wi, long long n,
                       float* out) {
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
        const float* r = rec + 16 * k;
        Surface s;
        s.p = f3(r[0], r[1], r[2]);
        s.normal = f3(r[3], r[4], r[5]);
        s.front = r[6] != 0.0f;
        s.u = r[7];
        s.v = r[8];
        s.dpdu = f3(r[9], r[10], r[11]);
        s.dpdv = f3(r[12], r[13], r[14]);
        s.material = material;
        float3 d = f3(r_in[3 * k], r_in[3 * k + 1], r_in[3 * k + 2]);
        float3 w = f3(wi[3 * k], wi[3 * k + 1], wi[3 * k + 2]);
        float3 e = eval(S, material, d, s, w);
        Rng g = make_rng(1, uint64_t(k), 0);
        ScatterRec sr;
        bool sc = scatter(S, material, d, s, sr, g);
        out[4 * k] = e.x;
        out[4 * k + 1] = e.y;
        out[4 * k + 2] = e.z;
        out[4 * k + 3] = (sc && !sr.skip_pdf) ? sr.pdf.value(w) : 0.0f;
    }
}

// Self-intersection probe of the spawned rays: each ray's closest hit, then
// from there a reflected ray (about the geometric normal) and a ray going on
// through the surface, both from spawn_origin with spawn_tmin as the
// renderer starts them. out (n x 8, 32-bit words): kind of the first hit
// (-1: miss); per spawned ray whether it met the surface it left (a planar
// primitive, quad, triangle or ground, met again at all; a voxel block's face
// on the same plane with the same orientation; a sphere within 1e-4 of the
// hit point's scale); the kind of the reflected ray's hit; then, as float
// bits, for the first spawned ray that met its surface (else the reflected
// one): its t, the origin's offset from the hit point, the cosine of its
// direction to the normal and the t_min of its walk.
__global__ void k_spawn_probe(DeviceScene S, const float* rays, long long n, int* out) {
    long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
        const float* r = rays + 8 * k;
        float3 o = f3(r[0], r[1], r[2]), d = f3(r[3], r[4], r[5]);
        HitInfo h = closest_hit<true>(S, o, d, r[6], r[7], 0);
        int* res = out + 8 * k;
        res[0] = h.prim == kMiss ? -1 : int(h.prim >> kKindShift);
        res[1] = res[2] = 0;
        res[3] = -1;
        for (int c = 4; c < 8; c++)
            res[c] = 0;
        if (h.prim == kMiss)
            continue;
        Surface s = make_surface(S, h, o, d);
        if (s.ng.x == 0.0f && s.ng.y == 0.0f && s.ng.z == 0.0f)
            continue;  // a medium: no surface
        const int kind = int(h.prim >> kKindShift);
        const bool planar = kind == kQuad || kind == kTriangle || kind == kGround;
        const float scale = fmaxf(1.0f, fmaxf(fabsf(s.p.x), fmaxf(fabsf(s.p.y), fabsf(s.p.z))));
        float3 dn = normalize(d);
        float3 dirs[2] = {dn - 2.0f * dot(dn, s.ng) * s.ng, dn};
        bool noted = false;
        for (int m = 0; m < 2; m++) {
            float3 w = dirs[m];
            float3 o2 = spawn_origin(s, w);
            float tmin = spawn_tmin(o2, w);
            HitInfo h2 = closest_hit<true>(S, o2, w, tmin, 3.0e38f, 0);
            if (m == 0)
                res[3] = h2.prim == kMiss ? -1 : int(h2.prim >> kKindShift);
            bool self = false;
            if (h2.prim == h.prim) {
                if (kind == kVoxel) {
                    Surface s2 = make_surface(S, h2, o2, w);
                    // the face codes are integers held as float bits: compare the bits
                    self = __float_as_int(h2.b2) == __float_as_int(h.b2) && fabsf(dot(s2.p - s.p, s.ng)) < 1e-3f;
                } else {
                    self = planar || h2.t * length(w) < 1e-4f * scale;
                }
            }
            res[1 + m] = self ? 1 : 0;
            if ((self && !noted) || m == 0) {
                res[4] = __float_as_int(h2.prim == kMiss ? -1.0f : h2.t);
                res[5] = __float_as_int(length(o2 - s.p));
                res[6] = __float_as_int(dot(w, s.ng));
                res[7] = __float_as_int(tmin);
                noted = noted || self;
            }
        }
    }
}

namespace {
struct Buf {
    void* p = nullptr;
    ~Buf() {
        if (p)
            cudaFree(p);
    }
};
int bad_arg(const std::string& m) {
    set_error_message(m);
    return MYPBR_ERR_INVALID_ARGUMENT;
}
}  // namespace

}  // namespace mypbr_dev

using namespace mypbr_dev;

// The walk the handle's traversal setting names (mypbr_gpu_set_launch): 2 the
// 4-wide tree, 3 postponed leaves, 5 the quantised 8-wide tree, where the
// scene's tree allows it; the plain binary walk otherwise.
static void (*trace_kernel(const mypbr_gpu_scene* G))(DeviceScene, const float*, long long, float*, int*) {
    if (G->tuned_traversal == 2 && G->dev.bvh4)
        return k_trace<kWalkWide>;
    if (G->tuned_traversal == 3 && G->dev.postponed_ok)
        return k_trace<kWalkPostponed>;
    if (G->tuned_traversal == 5 && G->dev.bvh8)
        return k_trace<kWalkWide8>;
    return k_trace<kWalkBinary>;
}

extern "C" int mypbr_gpu_trace(mypbr_gpu_scene* G, const float* rays, int64_t n, float* hits, int32_t* prim,
                               int on_device) {
    if (!G || (n > 0 && (!rays || !hits || !prim)) || n < 0)
        return bad_arg("mypbr_gpu_trace: bad argument");
    if (n == 0)
        return MYPBR_OK;
    MYPBR_CUDA(cudaSetDevice(G->device));
    int blocks = int(std::min<int64_t>((n + 127) / 128, int64_t(G->sm_count) * 16));
    auto k_trace_walk = trace_kernel(G);
    if (on_device) {
        k_trace_walk<<<blocks, 128>>>(G->dev, rays, (long long)n, hits, prim);
        MYPBR_CUDA(cudaGetLastError());
        MYPBR_CUDA(cudaDeviceSynchronize());
        return check_device_error(G);
    }
    Buf dr, dh, dp;
    MYPBR_CUDA(cudaMalloc(&dr.p, size_t(n) * 8 * sizeof(float)));
    MYPBR_CUDA(cudaMalloc(&dh.p, size_t(n) * 8 * sizeof(float)));
    MYPBR_CUDA(cudaMalloc(&dp.p, size_t(n) * 2 * sizeof(int)));
    MYPBR_CUDA(cudaMemcpy(dr.p, rays, size_t(n) * 8 * sizeof(float), cudaMemcpyHostToDevice));
    k_trace_walk<<<blocks, 128>>>(G->dev, static_cast<float*>(dr.p), (long long)n, static_cast<float*>(dh.p),
                                  static_cast<int*>(dp.p));
    MYPBR_CUDA(cudaGetLastError());
    MYPBR_CUDA(cudaMemcpy(hits, dh.p, size_t(n) * 8 * sizeof(float), cudaMemcpyDeviceToHost));
    MYPBR_CUDA(cudaMemcpy(prim, dp.p, size_t(n) * 2 * sizeof(int), cudaMemcpyDeviceToHost));
    return check_device_error(G);
}

extern "C" int mypbr_gpu_bsdf_eval(mypbr_gpu_scene* G, int32_t material, const float* rec, const float* r_in,
                                   const float* wi, int64_t n, float* out) {
    if (!G || n < 0 || (n > 0 && (!rec || !r_in || !wi || !out)))
        return bad_arg("mypbr_gpu_bsdf_eval: bad argument");
    if (material < 0 || material >= G->material_count)
        return bad_arg("mypbr_gpu_bsdf_eval: material index out of range");
    if (n == 0)
        return MYPBR_OK;
    MYPBR_CUDA(cudaSetDevice(G->device));
    Buf a, b, c, d;
    MYPBR_CUDA(cudaMalloc(&a.p, size_t(n) * 16 * sizeof(float)));
    MYPBR_CUDA(cudaMalloc(&b.p, size_t(n) * 3 * sizeof(float)));
    MYPBR_CUDA(cudaMalloc(&c.p, size_t(n) * 3 * sizeof(float)));
    MYPBR_CUDA(cudaMalloc(&d.p, size_t(n) * 4 * sizeof(float)));
    MYPBR_CUDA(cudaMemcpy(a.p, rec, size_t(n) * 16 * sizeof(float), cudaMemcpyHostToDevice));
    MYPBR_CUDA(cudaMemcpy(b.p, r_in, size_t(n) * 3 * sizeof(float), cudaMemcpyHostToDevice));
    MYPBR_CUDA(cudaMemcpy(c.p, wi, size_t(n) * 3 * sizeof(float), cudaMemcpyHostToDevice));
    int blocks = int(std::min<int64_t>((n + 127) / 128, 4096));
    k_bsdf<<<blocks, 128>>>(G->dev, material, static_cast<float*>(a.p), static_cast<float*>(b.p),
                            static_cast<float*>(c.p), (long long)n, static_cast<float*>(d.p));
    MYPBR_CUDA(cudaGetLastError());
    MYPBR_CUDA(cudaMemcpy(out, d.p, size_t(n) * 4 * sizeof(float), cudaMemcpyDeviceToHost));
    return check_device_error(G);
}

extern "C" int mypbr_gpu_test_spawn(mypbr_gpu_scene* G, const float* rays, int64_t n, int32_t* out) {
    if (!G || n < 0 || (n > 0 && (!rays || !out)))
        return bad_arg("mypbr_gpu_test_spawn: bad argument");
    if (n == 0)
        return MYPBR_OK;
    MYPBR_CUDA(cudaSetDevice(G->device));
    Buf dr, dout;
    MYPBR_CUDA(cudaMalloc(&dr.p, size_t(n) * 8 * sizeof(float)));
    MYPBR_CUDA(cudaMalloc(&dout.p, size_t(n) * 8 * sizeof(int)));
    MYPBR_CUDA(cudaMemcpy(dr.p, rays, size_t(n) * 8 * sizeof(float), cudaMemcpyHostToDevice));
    int blocks = int(std::min<int64_t>((n + 127) / 128, int64_t(G->sm_count) * 16));
    k_spawn_probe<<<blocks, 128>>>(G->dev, static_cast<float*>(dr.p), (long long)n, static_cast<int*>(dout.p));
    MYPBR_CUDA(cudaGetLastError());
    MYPBR_CUDA(cudaMemcpy(out, dout.p, size_t(n) * 8 * sizeof(int), cudaMemcpyDeviceToHost));
    return check_device_error(G);
}
