// The wavefront path tracer: camera::render / ray_color of the reference
// (include/camera.h:79-461) as kernels over queues in HBM.
//
// A wave holds every pixel times `npass` passes, one path per slot. Each
// bounce runs three kernels:
//   extend  closest hit of every ray in the extension queue (BVH walk);
//   shade   per path: sky or emission with MIS, Beer-Lambert, scatter();
//           for non-specular vertices next-event estimation writes a shadow
//           ray into the shadow queue; the BSDF sample, Russian roulette, and
//           the surviving path goes to the next extension queue;
//   shadow  closest hit of every shadow ray; adds f L w / pdf to its path and,
//           for a path that ended at this bounce, writes it to the film.
// Queues hold slot indices and are appended with warp-aggregated atomics; the
// per-bounce counters live in device memory, so the host never waits on them.
// Kernels are persistent-style (grid = SMs x resident blocks, grid-stride over
// the queue length they read on the device).
#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <atomic>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../host/host_math.h"
#include "dev_shading.cuh"
#include "gpu_scene.h"

namespace mypbr_dev {

// Path flags, kept in the w lane of the origin: bit 0 specular, bit 1 seen by a
// shadow ray, then the diffuse / specular / scatter bounce counts (8 bits each).
constexpr uint32_t kFlagSpecular = 1u;
constexpr uint32_t kFlagSeen = 2u;

// Shading classes: each has its own queue and kernel, so a warp shades one
// kind of material and each kernel carries only that material's code.
constexpr int kShadeClasses = 6;

enum : int { kClassMiss = 0, kClassLambert = 1, kClassMetal = 2, kClassDielectric = 3, kClassPrincipled = 4,
             kClassGeneric = 5 };

struct CameraParams {
    float3 center, p00, du, dv, wv, disk_u, disk_v;
    int width, height, sqrt_spp, blades;
    float recip_sqrt_spp, focus_dist, ortho_height, defocus_angle, blade_rotation;
};

struct WaveParams {
    DeviceScene S;
    CameraParams cam;
    RenderBuffers B;
    int max_depth, max_diffuse, max_specular, max_scatter;
    int transparent_shadows, collect_features, has_lights;
    int keyed;  // rays carry random keys: media, height fog or alpha masks
    unsigned long long seed;
    int pass0, npass;
    int first_row, band_rows;  // the rows rendered: [first_row, first_row + band_rows)
    unsigned long long* totals;  // extension rays, shadow rays, bounces run by a replayed wave graph
    // path guiding
    int guided;                // mixtures were computed for this wave's guidable vertices
    float guide_alpha;         // probability of sampling the mixture there (one-sample MIS), first bounce
    float guide_alpha_deep;    // the same at later bounces
    int guide_depths;          // bounces below this sample the mixture
    int record;                // write training records
    GuideRecords rec;          // slots below rec_slots record their first rec.depth vertices
    uint32_t rec_slots;
    GuidePacked* guide_mix;    // per slot
    float3 guide_lo, guide_inv;
};

// Counters: extension queue length entering bounce d; shadow queue length of
// bounce d; length of shading class c's queue at bounce d.
MYPBR_DEV uint32_t* ext_counter(const WaveParams& P, int d) { return P.B.counters + d; }
MYPBR_DEV uint32_t* sh_counter(const WaveParams& P, int d) { return P.B.counters + P.B.depth_slots + d; }
MYPBR_DEV uint32_t* class_counter(const WaveParams& P, int d, int c) {
    return P.B.counters + 2 * P.B.depth_slots + d * kShadeClasses + c;
}
MYPBR_DEV uint32_t* class_queue(const WaveParams& P, int c) { return P.B.class_queue + size_t(c) * P.B.capacity; }
// Rays of bounce d's extension queue handed out so far (the persistent extend kernel).
MYPBR_DEV uint32_t* fetch_counter(const WaveParams& P, int d) {
    return P.B.counters + (2 + kShadeClasses) * P.B.depth_slots + d;
}

// One atomic per warp: the active lanes that push get consecutive slots.
MYPBR_DEV uint32_t warp_push(uint32_t* counter) {
    unsigned mask = __activemask();
    int lane = threadIdx.x & 31;
    int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader)
        base = atomicAdd(counter, uint32_t(__popc(mask)));
    base = __shfl_sync(mask, base, leader);
    return base + uint32_t(__popc(mask & ((1u << lane) - 1u)));
}

// The same for lanes pushing to different counters: one atomic per distinct counter.
MYPBR_DEV uint32_t warp_push_keyed(uint32_t* counter) {
    unsigned mask = __activemask();
    unsigned peers = __match_any_sync(mask, reinterpret_cast<unsigned long long>(counter));
    int lane = threadIdx.x & 31;
    int leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (lane == leader)
        base = atomicAdd(counter, uint32_t(__popc(peers)));
    base = __shfl_sync(peers, base, leader);
    return base + uint32_t(__popc(peers & ((1u << lane) - 1u)));
}

MYPBR_DEV void film_add(const WaveParams& P, uint32_t pixel, float3 c) {
    // NaN or infinite estimates count as black (camera.h:281-287)
    if (!isfinite(c.x) || !isfinite(c.y) || !isfinite(c.z))
        c = f3(0.0f);
    double* f = P.B.film + 3 * size_t(pixel);
    double* f2 = P.B.film2 + 3 * size_t(pixel);
    atomicAdd(f, double(c.x));
    atomicAdd(f + 1, double(c.y));
    atomicAdd(f + 2, double(c.z));
    atomicAdd(f2, double(c.x) * c.x);
    atomicAdd(f2 + 1, double(c.y) * c.y);
    atomicAdd(f2 + 2, double(c.z) * c.z);
    if (P.collect_features) {
        double l = luminance(c);
        atomicAdd(P.B.feat + 7 * size_t(pixel) + 6, l * l);
    }
}

// Keys of the random numbers: everything random in a path depends only on
// (seed, pixel, pass, bounce, stage), never on where the path sits in a wave.
MYPBR_DEV uint64_t media_key(const WaveParams& P, uint32_t pixel, uint32_t pass, uint32_t depth, uint32_t kind) {
    return mix64(P.seed ^ mix64((uint64_t(pixel) << 24) ^ (uint64_t(pass) << 8) ^ (uint64_t(depth) << 2) ^ kind)) | 1ull;
}
MYPBR_DEV Rng bounce_rng(const WaveParams& P, uint32_t pixel, uint32_t pass, int depth, uint32_t stage) {
    return make_rng(P.seed ^ (0x9e3779b97f4a7c15ull * (uint64_t(depth) * 8 + stage + 1)), pixel, pass);
}

// camera.h:291-339: a ray through pixel (i, j) for pass `pass`, stratified over
// the first sqrt_spp^2 passes with the per-pixel cell offset of camera.h:205.
MYPBR_DEV void camera_ray(const CameraParams& C, int i, int j, int pass, Rng& g, float3& o, float3& d) {
    int strata = C.sqrt_spp * C.sqrt_spp;
    float ox, oy;
    if (pass >= strata) {
        ox = g.next() - 0.5f;
        oy = g.next() - 0.5f;
    } else {
        long long cell = (long long)pass + (long long)i * 7919 + (long long)j * 104729;
        int c = int(cell % strata);
        float rx = g.next(), ry = g.next();
        ox = ((c % C.sqrt_spp) + rx) * C.recip_sqrt_spp - 0.5f;
        oy = ((c / C.sqrt_spp) + ry) * C.recip_sqrt_spp - 0.5f;
    }
    float3 ps = C.p00 + (float(i) + ox) * C.du + (float(j) + oy) * C.dv;
    float3 eye = C.ortho_height > 0.0f ? ps + C.focus_dist * C.wv : C.center;
    if (C.defocus_angle <= 0.0f) {
        o = eye;
    } else {
        float px, py;
        if (C.blades >= 3) {  // camera.h:329-339
            int k = min(int(g.next() * C.blades), C.blades - 1);
            float a0 = C.blade_rotation + 2.0f * kPi * k / C.blades;
            float a1 = a0 + 2.0f * kPi / C.blades;
            float s = g.next(), t = g.next();
            if (s + t > 1.0f) {
                s = 1.0f - s;
                t = 1.0f - t;
            }
            px = s * cosf(a0) + t * cosf(a1);
            py = s * sinf(a0) + t * sinf(a1);
        } else {  // vec3.h:309-315
            do {
                px = 2.0f * g.next() - 1.0f;
                py = 2.0f * g.next() - 1.0f;
            } while (px * px + py * py >= 1.0f);
        }
        o = eye + px * C.disk_u + py * C.disk_v;
    }
    d = ps - o;
}

MYPBR_DEV float bits_f(uint32_t u) { return __uint_as_float(u); }
MYPBR_DEV uint32_t f_bits(float f) { return __float_as_uint(f); }

// (first pass, number of passes) of the current wave: from device memory when
// a captured graph replays the wave, else from the kernel arguments.
MYPBR_DEV int2 wave_of(const WaveParams& P) {
    return P.B.wave_state ? make_int2(P.B.wave_state[0], P.B.wave_state[1]) : make_int2(P.pass0, P.npass);
}

// The bounce a kernel works on: its argument, or, given -1 (the kernels of a
// replayed wave graph, which loops over bounces on the device), the bounce
// counter in device memory.
MYPBR_DEV int bounce_of(const WaveParams& P, int depth) { return depth >= 0 ? depth : P.B.wave_state[2]; }

__global__ void k_set_wave(int* state, int pass0, int npass) {
    state[0] = pass0;
    state[1] = npass;
    state[2] = 0;  // bounce
}

// Ends one bounce of a replayed wave graph's loop: the next bounce runs while
// it is below max_depth and its extension queue holds paths (once a bounce
// has none, no later one has any). Counts the bounces run.
__global__ void k_next_bounce(WaveParams P, cudaGraphConditionalHandle loop) {
    int next = P.B.wave_state[2] + 1;
    P.B.wave_state[2] = next;
    atomicAdd(&P.totals[2], 1ull);
    cudaGraphSetConditional(loop, next < P.max_depth && *ext_counter(P, next) > 0 ? 1u : 0u);
}

// A job of a batch graph, before its loop: the first wave's state (passes
// [0, min(per_wave, spp)), bounce 0, starting) and cleared queue counters.
__global__ void k_job_begin(WaveParams P, int per_wave, int spp, int counter_words) {
    if (threadIdx.x == 0) {
        P.B.wave_state[0] = 0;
        P.B.wave_state[1] = min(per_wave, spp);
        P.B.wave_state[2] = 0;
        P.B.wave_state[3] = 1;
    }
    for (int k = threadIdx.x; k < counter_words; k += blockDim.x)
        P.B.counters[k] = 0;
}

// Ends one iteration of a job's loop in a batch graph (one bounce of one
// wave): the next bounce of this wave while it is below max_depth and has
// paths, else the next wave (counters cleared, camera rays generated by the
// next iteration) while passes remain, else the job is done. Each iteration
// advances the bounce or the pass range, so the loop ends after
// waves x max_depth iterations at most.
__global__ void k_job_step(WaveParams P, cudaGraphConditionalHandle loop, int per_wave, int spp, int counter_words) {
    __shared__ int new_wave;
    if (threadIdx.x == 0) {
        int* ws = P.B.wave_state;
        ws[3] = 0;
        atomicAdd(&P.totals[2], 1ull);
        int next = ws[2] + 1;
        unsigned go = 1;
        new_wave = 0;
        if (next < P.max_depth && *ext_counter(P, next) > 0) {
            ws[2] = next;
        } else if (ws[0] + ws[1] < spp) {
            int pass0 = ws[0] + ws[1];
            ws[0] = pass0;
            ws[1] = min(per_wave, spp - pass0);
            ws[2] = 0;
            ws[3] = 1;
            new_wave = 1;
        } else {
            go = 0;
        }
        cudaGraphSetConditional(loop, go);
    }
    __syncthreads();
    if (new_wave)
        for (int k = threadIdx.x; k < counter_words; k += blockDim.x)
            P.B.counters[k] = 0;
}

// gated: only when the wave state says a wave starts (a job's device-side
// loop in a batch graph runs this kernel every iteration).
MYPBR_DEV bool wave_starting(const WaveParams& P, int gated) { return !gated || P.B.wave_state[3] != 0; }

__global__ void k_generate(WaveParams P, int gated) {
    if (!wave_starting(P, gated))
        return;
    const int2 wv = wave_of(P);
    size_t npix = size_t(P.cam.width) * P.band_rows;
    size_t n = npix * size_t(wv.y);
    size_t stride = size_t(gridDim.x) * blockDim.x;
    size_t first_pixel = size_t(P.first_row) * P.cam.width;
    for (size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x; t < n; t += stride) {
        uint32_t pixel = uint32_t(first_pixel + t % npix);
        uint32_t pass = uint32_t(wv.x + int(t / npix));
        int i = int(pixel % uint32_t(P.cam.width)), j = int(pixel / uint32_t(P.cam.width));
        Rng g = make_rng(P.seed, pixel, pass);
        float3 o, d;
        camera_ray(P.cam, i, j, int(pass), g, o, d);
        P.B.ray_o[t] = make_float4(o.x, o.y, o.z, bits_f(kFlagSpecular));
        P.B.ray_d[t] = make_float4(d.x, d.y, d.z, 0.0f);
        P.B.beta[t] = make_float4(1.0f, 1.0f, 1.0f, bits_f(pass));
        P.B.radiance[t] = make_float4(0.0f, 0.0f, 0.0f, bits_f(pixel));
        P.B.queue[0][t] = uint32_t(t);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
        *ext_counter(P, 0) = uint32_t(n);
}

// camera.h:253-277: albedo and normal of the first non-specular surface
__global__ void k_features(WaveParams P, int gated) {
    if (!wave_starting(P, gated))
        return;
    size_t n = size_t(P.cam.width) * P.band_rows * size_t(wave_of(P).y);
    size_t stride = size_t(gridDim.x) * blockDim.x;
    for (size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x; t < n; t += stride) {
        float4 ro = P.B.ray_o[t], rd = P.B.ray_d[t];
        uint32_t pixel = f_bits(P.B.radiance[t].w), pass = f_bits(P.B.beta[t].w);
        float3 o = f3(ro), d = f3(rd);
        Rng g = make_rng(P.seed ^ 0x5bd1e995ull, pixel, pass);
        float3 tint = f3(1.0f), albedo = f3(1.0f), normal = f3(0.0f);
        bool done = false;
        for (int b = 0; b < 8 && !done; b++) {
            HitInfo h = closest_hit<true>(P.S, o, d, spawn_tmin(o, d), 3.0e38f, media_key(P, pixel, pass, 100 + b, 3));
            if (h.prim == kMiss)
                break;
            Surface s = make_surface(P.S, h, o, d);
            tint *= interior_transmittance(P.S, s.material, h.t * length(d), s.front);
            ScatterRec sr;
            if (!scatter(P.S, s.material, d, s, sr, g)) {
                albedo = tint;
                normal = s.normal;
                done = true;
            } else if (!sr.skip_pdf) {
                albedo = tint * sr.attenuation;
                normal = s.normal;
                done = true;
            } else {
                tint *= sr.attenuation;
                d = sr.skip_dir;
                o = spawn_origin(s, d);
            }
        }
        if (!done) {
            albedo = tint;
            normal = f3(0.0f);
        }
        double* f = P.B.feat + 7 * size_t(pixel);
        atomicAdd(f, double(albedo.x));
        atomicAdd(f + 1, double(albedo.y));
        atomicAdd(f + 2, double(albedo.z));
        atomicAdd(f + 3, double(normal.x));
        atomicAdd(f + 4, double(normal.y));
        atomicAdd(f + 5, double(normal.z));
    }
}

// The material index of a hit (a voxel face carries its own in b1).
MYPBR_DEV int hit_material(const DeviceScene& S, const HitInfo& h) {
    int kind = int(h.prim >> kKindShift), idx = int(h.prim & kIndexMask);
    switch (kind) {
        case kSphere: return __ldg(&S.sphere_info[idx].x);
        case kQuad: return __float_as_int(ldg4(S.quads + 5 * idx).w);
        case kTriangle: return __float_as_int(ldg4(S.tris + 3 * idx).w);
        case kMedium: return __float_as_int(ldg4(S.media + 3 * idx + 2).y);
        case kVoxel: return __float_as_int(h.b1);
        default: return S.unbounded[idx].material;
    }
}

// Closest hits of the extension queue; each ray then joins its shading class's queue.
template <bool VOX, int WALK>
__global__ void __launch_bounds__(256, 3) k_extend(WaveParams P, int depth) {
    depth = bounce_of(P, depth);
    uint32_t n = *ext_counter(P, depth);
    if (blockIdx.x == 0 && threadIdx.x == 0 && n > 0)
        atomicAdd(&P.totals[0], (unsigned long long)n);
    const uint32_t* q = P.B.queue[depth & 1];
    uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
        uint32_t slot = q[k];
        float4 ro = P.B.ray_o[slot], rd = P.B.ray_d[slot];
        uint64_t key = 0;
        if (P.keyed) {
            uint32_t pixel = f_bits(P.B.radiance[slot].w), pass = f_bits(P.B.beta[slot].w);
            key = media_key(P, pixel, pass, uint32_t(depth), 0);
        }
        HitInfo h = closest_hit<VOX, WALK>(P.S, f3(ro), f3(rd), spawn_tmin(f3(ro), f3(rd)), 3.0e38f, key);
        P.B.hit[slot] = make_float4(h.t, h.b1, h.b2, __uint_as_float(h.prim));
        int c = h.prim == kMiss ? kClassMiss : int(P.S.mat_class[hit_material(P.S, h)]);
        uint32_t* counter = class_counter(P, depth, c);
        class_queue(P, c)[warp_push_keyed(counter)] = slot;
    }
}

// k_extend with lanes that take a new ray as soon as theirs is done: a warp
// advances all its rays one BVH node per step, and when at least a quarter of
// its lanes are idle (or all), it takes that many rays from the queue with
// one atomic. Lanes then do not wait for the slowest ray of their warp (the
// replacement of terminated rays of Aila and Laine, "Understanding the
// Efficiency of Ray Traversal on GPUs", HPG 2009). Same hits as k_extend.
template <bool VOX>
__global__ void __launch_bounds__(256, 3) k_extend_pt(WaveParams P, int depth) {
    depth = bounce_of(P, depth);
    const uint32_t n = *ext_counter(P, depth);
    if (blockIdx.x == 0 && threadIdx.x == 0 && n > 0)
        atomicAdd(&P.totals[0], (unsigned long long)n);
    const uint32_t* q = P.B.queue[depth & 1];
    uint32_t* fetch = fetch_counter(P, depth);
    const int lane = threadIdx.x & 31;
    const unsigned lanes_below = (1u << lane) - 1u;
    WalkState W;
    int stack[kBvhStack];
    uint32_t slot = 0;
    bool active = false, exhausted = false;
    // every lane's walk is bounded (node visits); this bounds the warp's steps
    // by the rays one warp could ever be given, were it given all of them
    const long long max_steps = (long long)(n + 32) * (long long)(P.S.bvh_node_count + 2) + 64;
    for (long long step = 0; step < max_steps; step++) {
        unsigned idle = __ballot_sync(0xffffffffu, !active && !exhausted);
        unsigned busy = __ballot_sync(0xffffffffu, active);
        if (idle != 0 && (__popc(idle) >= 8 || busy == 0)) {
            int leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if (lane == leader)
                base = atomicAdd(fetch, uint32_t(__popc(idle)));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (!active && !exhausted) {
                uint32_t k = base + uint32_t(__popc(idle & lanes_below));
                if (k < n) {
                    slot = q[k];
                    float4 ro = P.B.ray_o[slot], rd = P.B.ray_d[slot];
                    uint64_t key = 0;
                    if (P.keyed) {
                        uint32_t pixel = f_bits(P.B.radiance[slot].w), pass = f_bits(P.B.beta[slot].w);
                        key = media_key(P, pixel, pass, uint32_t(depth), 0);
                    }
                    walk_init(P.S, W, f3(ro), f3(rd), spawn_tmin(f3(ro), f3(rd)), 3.0e38f, key);
                    active = true;
                } else {
                    exhausted = true;
                }
            }
        }
        if (__all_sync(0xffffffffu, exhausted))
            break;
        if (active && !walk_node<false, VOX>(P.S, W, stack)) {
            walk_unbounded<false>(P.S, W);
            const HitInfo& h = W.h;
            P.B.hit[slot] = make_float4(h.t, h.b1, h.b2, __uint_as_float(h.prim));
            int c = h.prim == kMiss ? kClassMiss : int(P.S.mat_class[hit_material(P.S, h)]);
            class_queue(P, c)[warp_push_keyed(class_counter(P, depth, c))] = slot;
            active = false;
        }
    }
}

// scatter() restricted to one class: the compiler keeps only that material's code.
template <int C>
constexpr int class_type() {
    return C == kClassLambert ? kLambertian
         : C == kClassMetal ? kMetal
         : C == kClassDielectric ? kDielectric
         : C == kClassPrincipled ? kPrincipled : -1;
}
template <int C>
MYPBR_DEV bool class_scatter(const DeviceScene& S, int mi, float3 d, const Surface& s, ScatterRec& sr, Rng& g) {
    if constexpr (C == kClassGeneric)
        return scatter(S, mi, d, s, sr, g);
    else
        return scatter_inner<class_type<C>()>(S, S.materials[mi], d, s, sr, g);
}
template <int C>
MYPBR_DEV float3 class_eval(const DeviceScene& S, int mi, float3 d, const Surface& s, float3 dir) {
    if constexpr (C == kClassGeneric)
        return eval(S, mi, d, s, dir);
    else
        return eval_inner<class_type<C>()>(S, S.materials[mi], d, s, dir);
}

// Classes whose non-specular vertices the guiding network serves.
template <int C>
constexpr bool kGuidable() {
    return C == kClassLambert || C == kClassMetal || C == kClassPrincipled || C == kClassGeneric;
}

// One bounce of ray_color (camera.h:370-457) for the paths of shading class C.
// GUIDED: the variant of guided renders, which reads the learned mixtures and
// writes training records (plain renders keep the leaner code).
template <int C, bool GUIDED>
__device__ __forceinline__ void shade_body(const WaveParams& P, int depth) {
    uint32_t n = *class_counter(P, depth, C);
    const uint32_t* q = class_queue(P, C);
    uint32_t* q_next = P.B.queue[(depth + 1) & 1];
    const DeviceScene& S = P.S;
    uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
        uint32_t slot = q[k];
        float4 ro = P.B.ray_o[slot], rd = P.B.ray_d[slot];
        float4 bt = P.B.beta[slot], rad4 = P.B.radiance[slot];
        uint32_t pixel = f_bits(rad4.w), pass = f_bits(bt.w), flags = f_bits(ro.w);
        float3 o = f3(ro), d = f3(rd), beta = f3(bt), rad = f3(rad4);
        float scatter_pdf = rd.w;
        bool specular = flags & kFlagSpecular, seen = flags & kFlagSeen;
        uint32_t diffuse_count = (flags >> 8) & 0xff, specular_count = (flags >> 16) & 0xff;
        uint32_t scatter_count = flags >> 24;
        bool terminate = false, pushed_shadow = false;
        float3 new_o = o, new_d = d;
        int rec_at = -1;  // record written at this vertex (index), listed if the path goes on
        if (GUIDED && P.record && slot < P.rec_slots && depth >= 1 && depth - 1 < P.rec.depth) {
            // what the previous vertex's record needs: radiance and throughput on arrival here
            uint32_t r = slot * uint32_t(P.rec.depth) + uint32_t(depth - 1);
            P.rec.mark[r] = make_float4(rad.x, rad.y, rad.z, 0.0f);
            P.rec.bnext[r] = make_float4(beta.x, beta.y, beta.z, 0.0f);
        }
        if constexpr (C == kClassMiss) {
            // camera.h:373-387: the sky is a light, weighted like emission
            if (!seen) {
                if (env_only(S)) {
                    float3 sky;
                    float lp;
                    env_radiance_pdf(S, d, sky, lp);
                    rad += beta * sky * (specular ? 1.0f : power_heuristic(scatter_pdf, lp));
                } else {
                    float3 sky = escaped_radiance(S, d, depth == 0);
                    if (specular || !P.has_lights)
                        rad += beta * sky;
                    else
                        rad += beta * sky * power_heuristic(scatter_pdf, lights_pdf(S, o, d));
                }
            }
            terminate = true;
        } else {
            Rng g = bounce_rng(P, pixel, pass, depth, 0);
            float4 hb = P.B.hit[slot];
            HitInfo h;
            h.t = hb.x;
            h.b1 = hb.y;
            h.b2 = hb.z;
            h.prim = __float_as_uint(hb.w);
            Surface s = make_surface(S, h, o, d);
            int mat = s.material;
            if constexpr (C == kClassDielectric || C == kClassGeneric)  // camera.h:396
                beta *= interior_transmittance(S, mat, h.t * length(d), s.front);
            if constexpr (C == kClassGeneric) {  // camera.h:399-407
                if (!seen && may_emit(S, mat)) {
                    float3 em = emitted(S, mat, d, s);
                    if (nonzero(em)) {
                        if (specular || !P.has_lights)
                            rad += beta * em;
                        else
                            rad += beta * em * power_heuristic(scatter_pdf, lights_pdf(S, o, d));
                    }
                }
            }
            ScatterRec sr;
            if (!class_scatter<C>(S, mat, d, s, sr, g)) {
                terminate = true;
            } else if (sr.skip_pdf) {  // camera.h:413-423
                if (P.max_specular > 0 && ++specular_count > uint32_t(P.max_specular)) {
                    terminate = true;
                } else {
                    beta *= sr.attenuation;
                    new_d = sr.skip_dir;
                    new_o = spawn_origin(s, new_d);
                    if (P.transparent_shadows && lets_shadows_through(S, mat) && P.has_lights && depth > 0 && !specular)
                        seen = true;
                    specular = true;
                }
            } else {  // camera.h:424-448
                bool vol = (C == kClassGeneric) && is_volume(S, mat);
                uint32_t& cnt = vol ? scatter_count : diffuse_count;
                int cap = vol ? P.max_scatter : P.max_diffuse;
                bool capped = cap > 0 && ++cnt >= uint32_t(cap);
                bool last = depth == P.max_depth - 1 || capped;
                seen = false;
                // The learned mixture as one more proposal: directions come from
                // it with probability alpha, else from the BSDF, and every MIS
                // weight and throughput uses the combined density.
                GuideMix gm;
                bool use_guide = false;
                const float ga = depth == 0 ? P.guide_alpha : P.guide_alpha_deep;
                if constexpr (GUIDED && kGuidable<C>()) {
                    if (P.guided && ga > 0.0f && !vol && depth < P.guide_depths) {
                        guide_unpack(P.guide_mix[slot], gm);
                        use_guide = true;
                    }
                }
                auto mis_pdf = [&](float3 dir) {
                    float pb = sr.pdf.value(dir);
                    return use_guide ? ga * guide_pdf(gm, normalize(dir)) + (1.0f - ga) * pb : pb;
                };
                if (P.has_lights) {  // camera.h:466-506; the shadow ray is traced by k_shadow
                    // With the sky as the only light, the sample carries its own
                    // radiance and density; the shadow ray then only tests visibility
                    bool sky_only = env_only(S) && !S.has_emitters && !(P.transparent_shadows && S.has_clear_glass);
                    float3 to_light, sky = f3(1.0f);
                    float lp;
                    if (sky_only) {
                        to_light = env_sample(S, g, &sky, &lp);
                    } else {
                        to_light = lights_sample(S, s.p, g);
                        lp = lights_pdf(S, s.p, to_light);
                    }
                    if (lp > 0.0f) {
                        float3 f = class_eval<C>(S, mat, d, s, to_light);
                        if (f.x > 0.0f || f.y > 0.0f || f.z > 0.0f) {
                            float w = last ? 1.0f : power_heuristic(lp, mis_pdf(to_light));
                            float3 c = beta * f * sky * (w / lp);
                            float3 sd = normalize(to_light);
                            float3 so = spawn_origin(s, sd);
                            P.B.sh_o[slot] = make_float4(so.x, so.y, so.z, 0.0f);
                            P.B.sh_d[slot] = make_float4(sd.x, sd.y, sd.z, 0.0f);
                            P.B.sh_c[slot] = make_float4(c.x, c.y, c.z, sky_only ? 1.0f : 0.0f);
                            P.B.shadow_queue[warp_push(sh_counter(P, depth))] = slot;
                            pushed_shadow = true;
                        }
                    }
                }
                if (capped) {
                    terminate = true;
                } else {
                    float3 dir;
                    if (use_guide && g.next() < ga) {
                        float u0 = g.next(), u1 = g.next();
                        dir = guide_sample(gm, u0, u1, g.next());
                    } else {
                        dir = sr.pdf.generate(g);
                    }
                    float spdf = mis_pdf(dir);
                    if (!(spdf > 0.0f)) {
                        terminate = true;
                    } else {
                        float3 factor = class_eval<C>(S, mat, d, s, dir) / spdf;
                        beta *= factor;
                        scatter_pdf = spdf;
                        new_d = dir;
                        new_o = spawn_origin(s, new_d);
                        specular = false;
                        if constexpr (GUIDED && kGuidable<C>()) {
                            if (P.record && !vol && slot < P.rec_slots && depth < P.rec.depth) {
                                float sc[7];
                                guide_scalars(s.p, s.normal, normalize(-1.0f * d), P.guide_lo, P.guide_inv, sc);
                                float3 wd = normalize(dir);
                                uint32_t r = slot * uint32_t(P.rec.depth) + uint32_t(depth);
                                P.rec.in0[r] = make_float4(sc[0], sc[1], sc[2], sc[3]);
                                P.rec.in1[r] = make_float4(sc[4], sc[5], sc[6], 0.0f);
                                P.rec.dir[r] = make_float4(wd.x, wd.y, wd.z, 0.0f);
                                P.rec.fac[r] = make_float4(factor.x, factor.y, factor.z, 0.0f);
                                rec_at = int(r);
                            }
                        }
                    }
                }
            }
            // Russian roulette (camera.h:452-457)
            if (!terminate && depth >= 3) {
                float survive = fminf(maxc(beta), 0.95f);
                if (g.next() >= survive)
                    terminate = true;
                else
                    beta = beta / survive;
            }
            if (!terminate && depth + 1 >= P.max_depth)
                terminate = true;
        }
        if (terminate) {
            if (pushed_shadow) {
                P.B.radiance[slot] = make_float4(rad.x, rad.y, rad.z, rad4.w);
                P.B.sh_d[slot].w = 1.0f;  // the shadow kernel finishes this path
            } else {
                film_add(P, pixel, rad);
                if (GUIDED && P.record && slot < P.rec_slots)
                    P.rec.fin[slot] = make_float4(rad.x, rad.y, rad.z, 0.0f);
            }
            continue;
        }
        if (GUIDED && rec_at >= 0)  // the path goes on: the next vertex completes the record
            P.rec.list[warp_push(P.rec.count)] = uint32_t(rec_at);
        uint32_t nflags = (specular ? kFlagSpecular : 0u) | (seen ? kFlagSeen : 0u) | (diffuse_count << 8) |
                          (specular_count << 16) | (scatter_count << 24);
        P.B.ray_o[slot] = make_float4(new_o.x, new_o.y, new_o.z, bits_f(nflags));
        P.B.ray_d[slot] = make_float4(new_d.x, new_d.y, new_d.z, scatter_pdf);
        P.B.beta[slot] = make_float4(beta.x, beta.y, beta.z, bt.w);
        P.B.radiance[slot] = make_float4(rad.x, rad.y, rad.z, rad4.w);
        q_next[warp_push(ext_counter(P, depth + 1))] = slot;
    }
}

// The shading kernels. The plain ones leave registers to the compiler
// (requiring one or three resident blocks instead, with more registers or a
// few spills, measured 2.5 % slower on the sphere field); the guided ones
// would take up to 211 registers, one block of 256 per multiprocessor, and
// are held to two (a guided render 19 % faster).
template <int C>
__global__ void __launch_bounds__(256) k_shade(WaveParams P, int depth) {
    shade_body<C, false>(P, bounce_of(P, depth));
}
template <int C>
__global__ void __launch_bounds__(256, 2) k_shade_guided(WaveParams P, int depth) {
    shade_body<C, true>(P, bounce_of(P, depth));
}

template <bool VOX, int WALK>
__global__ void __launch_bounds__(256, 3) k_shadow(WaveParams P, int depth) {
    depth = bounce_of(P, depth);
    uint32_t n = *sh_counter(P, depth);
    if (blockIdx.x == 0 && threadIdx.x == 0 && n > 0)
        atomicAdd(&P.totals[1], (unsigned long long)n);
    const DeviceScene& S = P.S;
    uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
        uint32_t slot = P.B.shadow_queue[k];
        float4 so = P.B.sh_o[slot], sd = P.B.sh_d[slot], sc = P.B.sh_c[slot];
        float3 o = f3(so), d = f3(sd);
        uint64_t key = 0;
        uint32_t pixel = 0, pass = 0;
        if (P.keyed) {
            pixel = f_bits(P.B.radiance[slot].w);
            pass = f_bits(P.B.beta[slot].w);
        }
        float3 through = f3(1.0f), emission = f3(0.0f);
        if (!S.has_emitters && !(P.transparent_shadows && S.has_clear_glass)) {
            // Nothing the ray can reach emits, and nothing lets it through:
            // only whether it escapes matters (camera.h:488-503). A sky-only
            // sample already holds the sky's radiance (sc.w = 1).
            if (P.keyed)
                key = media_key(P, pixel, pass, uint32_t(depth), 1);
            if (!any_hit<VOX, WALK>(S, o, d, spawn_tmin(o, d), 3.0e38f, key))
                emission = sc.w != 0.0f ? f3(1.0f) : escaped_radiance(S, d, false);
        } else
        for (int hop = 0; hop <= 16; hop++) {
            if (P.keyed)
                key = media_key(P, pixel, pass, uint32_t(depth), 1 + 4 * hop);
            HitInfo h = closest_hit<VOX, WALK>(S, o, d, spawn_tmin(o, d), 3.0e38f, key);
            if (h.prim == kMiss) {
                emission = escaped_radiance(S, d, false);
                break;
            }
            int kind = int(h.prim >> kKindShift);
            int mat = (kind == kSphere || kind == kQuad || kind == kTriangle || kind == kVoxel) ? hit_material(S, h) : -1;
            // media, the ground and fog neither emit nor let shadows through
            bool through_glass = P.transparent_shadows && hop < 16 && mat >= 0 && lets_shadows_through(S, mat);
            if (!through_glass && (mat < 0 || !may_emit(S, mat)))
                break;  // blocked by something dark
            Surface s = make_surface(S, h, o, d);
            if (through_glass) {
                through *= interior_transmittance(S, mat, h.t * length(d), s.front);
                o = spawn_origin(s, d);
                continue;
            }
            emission = emitted(S, mat, d, s);
            break;
        }
        float4 r4 = P.B.radiance[slot];
        float3 rad = f3(r4) + f3(sc) * through * emission;
        if (sd.w != 0.0f) {
            film_add(P, f_bits(r4.w), rad);
            if (P.record && slot < P.rec_slots)
                P.rec.fin[slot] = make_float4(rad.x, rad.y, rad.z, 0.0f);
        } else
            P.B.radiance[slot] = make_float4(rad.x, rad.y, rad.z, r4.w);
    }
}

// Averages (camera.h:223-246): radiance, albedo, normal over `samples`, and
// the variance of the mean luminance.
__global__ void k_resolve(WaveParams P, int samples, double* radiance, double* albedo, double* normal,
                          double* variance) {
    size_t first = size_t(P.first_row) * P.cam.width;
    size_t end = first + size_t(P.cam.width) * P.band_rows;
    double scale = 1.0 / samples;
    size_t stride = size_t(gridDim.x) * blockDim.x;
    for (size_t p = first + size_t(blockIdx.x) * blockDim.x + threadIdx.x; p < end; p += stride) {
        double r0 = scale * P.B.film[3 * p], r1 = scale * P.B.film[3 * p + 1], r2 = scale * P.B.film[3 * p + 2];
        radiance[3 * p] = r0;
        radiance[3 * p + 1] = r1;
        radiance[3 * p + 2] = r2;
        if (!P.collect_features)
            continue;
        const double* f = P.B.feat + 7 * p;
        if (albedo) {
            albedo[3 * p] = scale * f[0];
            albedo[3 * p + 1] = scale * f[1];
            albedo[3 * p + 2] = scale * f[2];
        }
        if (normal) {
            normal[3 * p] = scale * f[3];
            normal[3 * p + 1] = scale * f[4];
            normal[3 * p + 2] = scale * f[5];
        }
        if (variance) {
            double mean = 0.2126 * r0 + 0.7152 * r1 + 0.0722 * r2;
            double spread = fmax(scale * f[6] - mean * mean, 0.0);
            variance[p] = samples > 1 ? spread / (samples - 1) : spread;
        }
    }
}

// Per-channel variance of the mean radiance, from the second moments
// (for the statistical parity checks).
__global__ void k_channel_variance(WaveParams P, int samples, double* out) {
    size_t first = size_t(P.first_row) * P.cam.width * 3;
    size_t end = first + size_t(P.cam.width) * P.band_rows * 3;
    double scale = 1.0 / samples;
    size_t stride = size_t(gridDim.x) * blockDim.x;
    for (size_t k = first + size_t(blockIdx.x) * blockDim.x + threadIdx.x; k < end; k += stride) {
        double m = scale * P.B.film[k];
        double spread = fmax(scale * P.B.film2[k] - m * m, 0.0);
        out[k] = samples > 1 ? spread / (samples - 1) : spread;
    }
}

// ------------------------------------------------------------ host side

int release_buffers(RenderBuffers& rb) {
    void* ptrs[] = {rb.ray_o, rb.ray_d, rb.beta, rb.radiance, rb.hit, rb.sh_o, rb.sh_d, rb.sh_c, rb.queue[0],
                    rb.queue[1], rb.class_queue, rb.shadow_queue, rb.counters, rb.wave_state, rb.film, rb.film2,
                    rb.feat};
    for (void* p : ptrs)
        if (p)
            cudaFree(p);
    rb = RenderBuffers();
    return MYPBR_OK;
}

// The guiding network's rows at a bounce: the vertices of the guidable
// shading classes' queues, one after another.
MYPBR_HD constexpr int guided_class(int c) {
    return c == 0 ? kClassLambert : c == 1 ? kClassMetal : c == 2 ? kClassPrincipled : kClassGeneric;
}

MYPBR_DEV uint32_t guided_slot(const WaveParams& P, int depth, long long i) {
#pragma unroll
    for (int c = 0; c < 4; c++) {
        long long n = *class_counter(P, depth, guided_class(c));
        if (i < n)
            return class_queue(P, guided_class(c))[i];
        i -= n;
    }
    return 0;  // not reached: i < count()
}

// The guidable vertices of a bounce (depth -1: the bounce in device memory),
// none past the guided depths. A row is the vertex's path slot and, once
// finished, its 7 network scalars; load starts the reads of the ray and hit
// records, finish turns them into the surface point and its scalars.
struct GuideQueueSource {
    WaveParams P;
    int depth;
    struct Row {
        float4 ro, rd, hb;
        float s[kGuideScalars];
        uint32_t slot;
        bool valid;
    };
    MYPBR_DEV long long count(long long) const {
        const int d = bounce_of(P, depth);
        if (d >= P.guide_depths)
            return 0;
        long long n = 0;
#pragma unroll
        for (int c = 0; c < 4; c++)
            n += *class_counter(P, d, guided_class(c));
        return n;
    }
    MYPBR_DEV void load(long long i, Row& r) const {
        r.valid = i >= 0;
        if (!r.valid)
            return;
        r.slot = guided_slot(P, bounce_of(P, depth), i);
        r.ro = P.B.ray_o[r.slot];
        r.rd = P.B.ray_d[r.slot];
        r.hb = P.B.hit[r.slot];
    }
    MYPBR_DEV void finish(Row& r) const {
        if (!r.valid) {  // a padding row: its outputs are never used
#pragma unroll
            for (int k = 0; k < kGuideScalars; k++)
                r.s[k] = 0.0f;
            return;
        }
        HitInfo h;
        h.t = r.hb.x;
        h.b1 = r.hb.y;
        h.b2 = r.hb.z;
        h.prim = __float_as_uint(r.hb.w);
        Surface sf = make_surface(P.S, h, f3(r.ro), f3(r.rd));
        guide_scalars(sf.p, sf.normal, normalize(-1.0f * f3(r.rd)), P.guide_lo, P.guide_inv, r.s);
    }
    MYPBR_DEV void encode(const Row& r, __nv_bfloat16* A, int row) const { guide_encode_row(r.s, A, row); }
};

struct GuidePackSink {
    WaveParams P;
    MYPBR_DEV void put(long long, const GuideQueueSource::Row& r, const float* v) const {
        GuidePacked pk;
        guide_pack(v, pk);
        P.guide_mix[r.slot] = pk;
    }
};

size_t counter_words(int depth_slots) { return size_t(depth_slots) * (3 + kShadeClasses) + 8; }

namespace {

template <typename T>
int alloc(T*& p, size_t count) {
    MYPBR_CUDA(cudaMalloc(reinterpret_cast<void**>(&p), std::max<size_t>(count, 1) * sizeof(T)));
    return MYPBR_OK;
}

int ensure_buffers(RenderBuffers& rb, size_t capacity, size_t pixels, int depth_slots) {
    if (rb.capacity >= capacity && rb.pixels >= pixels && rb.depth_slots >= depth_slots)
        return MYPBR_OK;
    capacity = std::max(capacity, rb.capacity);
    pixels = std::max(pixels, rb.pixels);
    depth_slots = std::max(depth_slots, rb.depth_slots);
    release_buffers(rb);
    int s = MYPBR_OK;
#define A(ptr, n) \
    if (s == MYPBR_OK) s = alloc(ptr, n)
    A(rb.ray_o, capacity);
    A(rb.ray_d, capacity);
    A(rb.beta, capacity);
    A(rb.radiance, capacity);
    A(rb.hit, capacity);
    A(rb.sh_o, capacity);
    A(rb.sh_d, capacity);
    A(rb.sh_c, capacity);
    A(rb.queue[0], capacity);
    A(rb.queue[1], capacity);
    A(rb.class_queue, capacity * kShadeClasses);
    A(rb.shadow_queue, capacity);
    A(rb.counters, counter_words(depth_slots));
    A(rb.wave_state, 4);
    A(rb.film, 3 * pixels);
    A(rb.film2, 3 * pixels);
    A(rb.feat, 7 * pixels);
#undef A
    if (s != MYPBR_OK) {
        release_buffers(rb);
        return s;
    }
    rb.capacity = capacity;
    rb.pixels = pixels;
    rb.depth_slots = depth_slots;
    return MYPBR_OK;
}

// camera.h:142-179 in FP64, handed to the device in FP32
CameraParams make_camera(const mypbr_camera& c, int spp) {
    using mypbr_host::V3;
    CameraParams C{};
    int w = c.image_width;
    int h = c.image_height > 0 ? c.image_height : std::max(1, int(c.image_width / c.aspect_ratio));
    C.width = w;
    C.height = h;
    C.sqrt_spp = std::max(1, int(std::sqrt(double(spp))));
    C.recip_sqrt_spp = float(1.0 / C.sqrt_spp);
    const double pi = 3.1415926535897932385;
    V3 from(c.lookfrom[0], c.lookfrom[1], c.lookfrom[2]), at(c.lookat[0], c.lookat[1], c.lookat[2]),
        vup(c.vup[0], c.vup[1], c.vup[2]);
    double theta = c.vfov * pi / 180.0;
    double hh = std::tan(theta / 2);
    double vh = c.ortho_height > 0 ? c.ortho_height : 2 * hh * c.focus_dist;
    double vw = vh * (double(w) / h);
    V3 wv = mypbr_host::unit(from - at);
    V3 u = mypbr_host::unit(mypbr_host::cross(vup, wv));
    V3 v = mypbr_host::cross(wv, u);
    V3 vu = vw * u, vv = vh * -v;
    V3 du = vu / w, dv = vv / h;
    V3 ul = from - (c.focus_dist * wv) - vu / 2 - vv / 2;
    V3 p00 = ul + 0.5 * (du + dv);
    double dr = c.focus_dist * std::tan(c.defocus_angle / 2 * pi / 180.0);
    auto F = [](const V3& a) { return make_float3(float(a.x), float(a.y), float(a.z)); };
    C.center = F(from);
    C.p00 = F(p00);
    C.du = F(du);
    C.dv = F(dv);
    C.wv = F(wv);
    C.disk_u = F(u * dr);
    C.disk_v = F(v * dr);
    C.focus_dist = float(c.focus_dist);
    C.ortho_height = float(c.ortho_height);
    C.defocus_angle = float(c.defocus_angle);
    C.blades = c.blades;
    C.blade_rotation = float(c.blade_rotation * pi / 180.0);
    return C;
}

int bad_arg(const std::string& m) {
    set_error_message(m);
    return MYPBR_ERR_INVALID_ARGUMENT;
}

struct Launch {
    int grid_extend, grid_shade, grid_shadow, grid_stream;
    int block = 256;              // threads per block of extend, shade and shadow
    bool persistent = false;      // extend with lanes that take new rays (k_extend_pt)
    int walk = kWalkBinary;       // which walk extend and shadow use
    bool guided_kernels = false;  // the shading variants of guided renders
    int grid_guide = 0;
    size_t guide_smem = 0;
    GuideNetView net{};
};

// A bounce kernel (WaveParams, depth) launched through its address, so that
// graph capture records it like a <<<>>> launch.
void launch_bounce_kernel(const void* fn, int grid, int block, cudaStream_t st, WaveParams& P, int depth) {
    void* args[2] = {&P, &depth};
    cudaLaunchKernel(fn, dim3(grid), dim3(block), args, 0, st);
}

// The extend and shadow kernels of a walk, with or without the voxel code.
const void* extend_kernel(bool vox, int walk) {
    if (walk == kWalkWide8)
        return vox ? (const void*)k_extend<true, kWalkWide8> : (const void*)k_extend<false, kWalkWide8>;
    if (walk == kWalkWide)
        return vox ? (const void*)k_extend<true, kWalkWide> : (const void*)k_extend<false, kWalkWide>;
    if (walk == kWalkPostponed)
        return vox ? (const void*)k_extend<true, kWalkPostponed> : (const void*)k_extend<false, kWalkPostponed>;
    return vox ? (const void*)k_extend<true, kWalkBinary> : (const void*)k_extend<false, kWalkBinary>;
}
const void* shadow_kernel(bool vox, int walk) {
    if (walk == kWalkWide8)
        return vox ? (const void*)k_shadow<true, kWalkWide8> : (const void*)k_shadow<false, kWalkWide8>;
    if (walk == kWalkWide)
        return vox ? (const void*)k_shadow<true, kWalkWide> : (const void*)k_shadow<false, kWalkWide>;
    if (walk == kWalkPostponed)
        return vox ? (const void*)k_shadow<true, kWalkPostponed> : (const void*)k_shadow<false, kWalkPostponed>;
    return vox ? (const void*)k_shadow<true, kWalkBinary> : (const void*)k_shadow<false, kWalkBinary>;
}

// The path kernels keep their data in L1 (tree nodes, voxel cells, material
// records): they ask for the largest L1 share of each SM's on-chip memory.
// Without the request an SM keeps the split of the kernel before, and after
// the guiding network's kernels (213 KB of shared memory each) that leaves
// the walks a small L1. Set once per device.
void prefer_l1(int device) {
    static std::atomic<uint64_t> done{0};
    const uint64_t bit = uint64_t(1) << (device & 63);
    if (done.load() & bit)
        return;
    const void* kernels[] = {
        (const void*)k_generate, (const void*)k_features,
        (const void*)k_extend<true, kWalkBinary>, (const void*)k_extend<false, kWalkBinary>,
        (const void*)k_extend<true, kWalkWide>, (const void*)k_extend<false, kWalkWide>,
        (const void*)k_extend<true, kWalkPostponed>, (const void*)k_extend<false, kWalkPostponed>,
        (const void*)k_extend<true, kWalkWide8>, (const void*)k_extend<false, kWalkWide8>,
        (const void*)k_shadow<true, kWalkWide8>, (const void*)k_shadow<false, kWalkWide8>,
        (const void*)k_extend_pt<true>, (const void*)k_extend_pt<false>,
        (const void*)k_shadow<true, kWalkBinary>, (const void*)k_shadow<false, kWalkBinary>,
        (const void*)k_shadow<true, kWalkWide>, (const void*)k_shadow<false, kWalkWide>,
        (const void*)k_shadow<true, kWalkPostponed>, (const void*)k_shadow<false, kWalkPostponed>,
        (const void*)k_shade<kClassMiss>, (const void*)k_shade<kClassLambert>, (const void*)k_shade<kClassMetal>,
        (const void*)k_shade<kClassDielectric>, (const void*)k_shade<kClassPrincipled>,
        (const void*)k_shade<kClassGeneric>, (const void*)k_shade_guided<kClassMiss>,
        (const void*)k_shade_guided<kClassLambert>, (const void*)k_shade_guided<kClassMetal>,
        (const void*)k_shade_guided<kClassDielectric>, (const void*)k_shade_guided<kClassPrincipled>,
        (const void*)k_shade_guided<kClassGeneric>};
    for (const void* k : kernels)
        cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, int(cudaSharedmemCarveoutMaxL1));
    cudaGetLastError();  // a hint: a driver that ignores it changes nothing
    done.fetch_or(bit);
}

// Grids of `block` threads: SMs x resident blocks (persistent-style loops).
Launch launch_config(const mypbr_gpu_scene& G, int block = 0) {
    prefer_l1(G.device);
    Launch L{};
    // 128-thread blocks suit the postponed-leaf walk (6 % faster on the
    // 2 M-triangle room, 6 % on the guided voxel hall), 256 the rest
    int default_block = G.prefer_postponed && G.tuned_traversal == 0 ? 128 : 256;
    L.block = block == 128 || block == 256 ? block : (G.tuned_block ? G.tuned_block : default_block);
    // traversal 0 is the scene's default: leaves postponed unless spheres fill
    // most of the leaves (other leaves' tests diverge), the plain binary walk else
    int trav = G.tuned_traversal;
    if (trav == 0)
        trav = G.prefer_postponed && G.dev.postponed_ok ? 3 : 4;
    L.persistent = trav == 1;
    if (trav == 2 && G.dev.bvh4 != nullptr)
        L.walk = kWalkWide;
    else if (trav == 3 && G.dev.postponed_ok)
        L.walk = kWalkPostponed;
    else if (trav == 5 && G.dev.bvh8 != nullptr)
        L.walk = kWalkWide8;
    int per_sm = 0;
    bool vox = G.dev.has_voxels;
    const void* extend = extend_kernel(vox, L.walk);
    const void* shadow = shadow_kernel(vox, L.walk);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, extend, L.block, 0);
    L.grid_extend = G.sm_count * std::max(per_sm, 1);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, shadow, L.block, 0);
    L.grid_shadow = G.sm_count * std::max(per_sm, 1);
    L.grid_stream = G.sm_count * 8;
    int worst = 1;
    for (auto f : {(const void*)k_shade<kClassMiss>, (const void*)k_shade<kClassLambert>,
                   (const void*)k_shade<kClassMetal>, (const void*)k_shade<kClassDielectric>,
                   (const void*)k_shade<kClassPrincipled>, (const void*)k_shade<kClassGeneric>}) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, L.block, 0);
        worst = std::max(worst, per_sm);
    }
    L.grid_shade = G.sm_count * worst;
    return L;
}

// CUDA events around each launch, summed per kernel kind after the render.
struct KernelTimer {
    bool on = false;
    cudaStream_t st = nullptr;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pool;
    std::vector<int> kinds;  // 0 generate, 1 extend, 2 shade, 3 shadow, 4 other
    size_t used = 0;
    ~KernelTimer() {
        for (auto& e : pool) {
            cudaEventDestroy(e.first);
            cudaEventDestroy(e.second);
        }
    }
    int begin(int kind) {
        if (!on)
            return MYPBR_OK;
        if (used == pool.size()) {
            cudaEvent_t a, b;
            MYPBR_CUDA(cudaEventCreate(&a));
            MYPBR_CUDA(cudaEventCreate(&b));
            pool.push_back({a, b});
            kinds.push_back(kind);
        }
        kinds[used] = kind;
        MYPBR_CUDA(cudaEventRecord(pool[used].first, st));
        return MYPBR_OK;
    }
    int end() {
        if (!on)
            return MYPBR_OK;
        MYPBR_CUDA(cudaEventRecord(pool[used].second, st));
        used++;
        return MYPBR_OK;
    }
    int collect(mypbr_render_stats* s) {
        if (!on || !s)
            return MYPBR_OK;
        double ms[5] = {0, 0, 0, 0, 0};
        uint64_t cnt[5] = {0, 0, 0, 0, 0};
        for (size_t k = 0; k < used; k++) {
            MYPBR_CUDA(cudaEventSynchronize(pool[k].second));
            float t = 0;
            MYPBR_CUDA(cudaEventElapsedTime(&t, pool[k].first, pool[k].second));
            ms[kinds[k]] += t;
            cnt[kinds[k]]++;
        }
        s->ms_generate = ms[0];
        s->ms_extend = ms[1];
        s->ms_shade = ms[2];
        s->ms_shadow = ms[3];
        s->ms_other = ms[4];
        s->launches_extend = cnt[1];
        s->launches_shade = cnt[2];
        s->launches_shadow = cnt[3];
        return MYPBR_OK;
    }
};

#define TIMED(kind, launch)                      \
    do {                                         \
        int s_ = T.begin(kind);                  \
        if (s_ != MYPBR_OK)                      \
            return s_;                           \
        launch;                                  \
        s_ = T.end();                            \
        if (s_ != MYPBR_OK)                      \
            return s_;                           \
    } while (0)

// A wave's start: cleared queue counters, camera rays, feature guides.
int run_prefix(WaveParams& P, const Launch& L, cudaStream_t st, uint64_t& launches, KernelTimer& T) {
    MYPBR_CUDA(cudaMemsetAsync(P.B.counters, 0, sizeof(uint32_t) * counter_words(P.B.depth_slots), st));
    TIMED(0, (k_generate<<<L.grid_stream, 256, 0, st>>>(P, 0)));
    launches++;
    if (P.collect_features) {
        TIMED(4, (k_features<<<L.grid_shade, 256, 0, st>>>(P, 0)));
        launches++;
    }
    return MYPBR_OK;
}

// One bounce: extend, the guiding network's mixtures (guided renders), the
// shading classes, shadow rays. depth -1: the bounce counter in device memory.
int run_bounce(WaveParams& P, const Launch& L, cudaStream_t st, uint64_t& launches, KernelTimer& T, int depth) {
    if (L.persistent && P.S.has_voxels)
        TIMED(1, (k_extend_pt<true><<<L.grid_extend, L.block, 0, st>>>(P, depth)));
    else if (L.persistent)
        TIMED(1, (k_extend_pt<false><<<L.grid_extend, L.block, 0, st>>>(P, depth)));
    else
        TIMED(1, (launch_bounce_kernel(extend_kernel(P.S.has_voxels, L.walk), L.grid_extend, L.block, st, P, depth)));
    if (P.guided && (depth < 0 || depth < P.guide_depths)) {  // the mixtures of this bounce's guidable vertices
        TIMED(4, (k_guide_forward<GuideQueueSource, GuidePackSink><<<L.grid_guide, 128 * kGuideGroups, L.guide_smem, st>>>(
                     L.net, GuideQueueSource{P, depth}, GuidePackSink{P}, 0)));
        launches++;
    }
    if (L.guided_kernels) {
        TIMED(2, (k_shade_guided<kClassMiss><<<L.grid_shade, L.block, 0, st>>>(P, depth)));
        TIMED(2, (k_shade_guided<kClassLambert><<<L.grid_shade, L.block, 0, st>>>(P, depth)));
        TIMED(2, (k_shade_guided<kClassMetal><<<L.grid_shade, L.block, 0, st>>>(P, depth)));
        TIMED(2, (k_shade_guided<kClassDielectric><<<L.grid_shade, L.block, 0, st>>>(P, depth)));
        TIMED(2, (k_shade_guided<kClassPrincipled><<<L.grid_shade, L.block, 0, st>>>(P, depth)));
        TIMED(2, (k_shade_guided<kClassGeneric><<<L.grid_shade, L.block, 0, st>>>(P, depth)));
    } else {
        TIMED(2, (k_shade<kClassMiss><<<L.grid_shade, L.block, 0, st>>>(P, depth)));
        TIMED(2, (k_shade<kClassLambert><<<L.grid_shade, L.block, 0, st>>>(P, depth)));
        TIMED(2, (k_shade<kClassMetal><<<L.grid_shade, L.block, 0, st>>>(P, depth)));
        TIMED(2, (k_shade<kClassDielectric><<<L.grid_shade, L.block, 0, st>>>(P, depth)));
        TIMED(2, (k_shade<kClassPrincipled><<<L.grid_shade, L.block, 0, st>>>(P, depth)));
        TIMED(2, (k_shade<kClassGeneric><<<L.grid_shade, L.block, 0, st>>>(P, depth)));
    }
    TIMED(3, (launch_bounce_kernel(shadow_kernel(P.S.has_voxels, L.walk), L.grid_shadow, L.block, st, P, depth)));
    launches += 2 + kShadeClasses;
    return MYPBR_OK;
}

// Renders passes [pass0, pass0 + npass) of every pixel of the band into the
// film, every bounce up to max_depth launched from the host.
int run_wave(WaveParams& P, const Launch& L, cudaStream_t st, uint64_t& launches, KernelTimer& T) {
    int s = run_prefix(P, L, st, launches, T);
    for (int depth = 0; depth < P.max_depth && s == MYPBR_OK; depth++)
        s = run_bounce(P, L, st, launches, T, depth);
    if (s != MYPBR_OK)
        return s;
    MYPBR_CUDA(cudaGetLastError());
    return MYPBR_OK;
}

// A wave's bounces as a CUDA graph replayed for every wave with the same
// settings: one conditional WHILE node whose body is one bounce's kernels
// (they read the bounce from device memory) followed by k_next_bounce, which
// lets the loop go on while the next bounce has paths and is below
// max_depth. Bounces with no paths are not launched at all, and the loop ends
// after max_depth bodies at most. The wave's start (counters, camera rays,
// features) is launched before the graph, with the pass range in device
// memory (wave_state) set by a one-thread kernel.
struct WaveGraph {
    cudaGraphExec_t exec = nullptr;
    int key = -1;
    uint64_t per_bounce = 0;  // kernels in one body, k_next_bounce included
    ~WaveGraph() {
        if (exec)
            cudaGraphExecDestroy(exec);
    }
};

int build_wave_graph(WaveParams& P, const Launch& L, cudaStream_t st, WaveGraph* graph) {
    cudaGraph_t g = nullptr;
    MYPBR_CUDA(cudaGraphCreate(&g, 0));
    struct Owned {
        cudaGraph_t g;
        ~Owned() { cudaGraphDestroy(g); }
    } owned{g};
    cudaGraphConditionalHandle loop;
    MYPBR_CUDA(cudaGraphConditionalHandleCreate(&loop, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = loop;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    MYPBR_CUDA(cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    MYPBR_CUDA(cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    uint64_t n = 0;
    KernelTimer off;  // no events inside a graph
    off.st = st;
    int s = run_bounce(P, L, st, n, off, -1);
    if (s == MYPBR_OK)
        k_next_bounce<<<1, 1, 0, st>>>(P, loop);
    cudaGraph_t captured = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &captured);
    if (s != MYPBR_OK)
        return s;
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaStreamEndCapture (wave graph body)");
    MYPBR_CUDA(cudaGetLastError());
    e = cudaGraphInstantiate(&graph->exec, g, 0);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGraphInstantiate");
    graph->per_bounce = n + 1;
    return MYPBR_OK;
}

int launch_wave(WaveParams& P, const Launch& L, cudaStream_t st, uint64_t& launches, KernelTimer& T,
                WaveGraph* graph) {
    if (!graph)
        return run_wave(P, L, st, launches, T);
    // the wave's launches depend on these; the kernels' parameters (captured
    // by value) on the mixing probability too
    int key = (P.guided ? 1 : 0) | (P.record ? 2 : 0) | (P.guide_alpha > 0.0f ? 4 : 0) |
              (P.guided ? (std::min(P.guide_depths, 255) << 3) | (int(P.guide_alpha * 1000.0f + 0.5f) << 11) |
                              (int(P.guide_alpha_deep * 1000.0f + 0.5f) << 21)
                        : 0);
    if (!graph->exec || graph->key != key) {
        if (graph->exec) {
            cudaGraphExecDestroy(graph->exec);
            graph->exec = nullptr;
        }
        int s = build_wave_graph(P, L, st, graph);
        if (s != MYPBR_OK)
            return s;
        graph->key = key;
    }
    k_set_wave<<<1, 1, 0, st>>>(P.B.wave_state, P.pass0, P.npass);
    launches++;
    int s = run_prefix(P, L, st, launches, T);
    if (s != MYPBR_OK)
        return s;
    MYPBR_CUDA(cudaGraphLaunch(graph->exec, st));
    return MYPBR_OK;
}

// Whether waves on stream st may be captured: not the legacy default stream,
// and not a stream the caller is capturing already (our launches then go
// into the caller's graph as they are).
bool graphs_allowed(cudaStream_t st) {
    if (st == nullptr || st == cudaStreamLegacy)
        return false;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess)
        return false;
    return cs == cudaStreamCaptureStatusNone;
}

}  // namespace

struct RenderSetup {
    WaveParams P;
    Launch L;
    int spp, per_wave;
    size_t npix;  // pixels of the band
    bool timing;
    bool guided = false, fixed_waves = false;
    int per_wave_train = 0;  // passes per training wave of a guided render
};

// Guided renders: the first waves are small and recorded, each followed by
// Adam steps on their vertices; later waves keep training online, lightly.
constexpr int kGuideTrainWaves = 8;
constexpr int kGuideBatchTilesPerSm = 2;  // 128-sample tiles per SM in one step (39K samples on 152 SMs)
constexpr float kGuideLr = 4e-3f;

// plain_wave: the default paths per wave of a plain render (batches keep
// 32M per job, since every job holds its own buffers at once)
int prepare(mypbr_gpu_scene* G, const mypbr_camera* cam, const mypbr_render_opts* o, int save_every, RenderSetup& R,
            size_t plain_wave = size_t(128) << 20) {
    if (!G || !cam || !o)
        return bad_arg("mypbr_gpu_render: null argument");
    if (cam->image_width < 1 || o->samples_per_pixel < 1 || o->max_depth < 1 || o->max_depth > 4096)
        return bad_arg("mypbr_gpu_render: image_width, samples_per_pixel and max_depth must be positive");
    if (o->guided < 0)
        return bad_arg("mypbr_gpu_render: guided must be 0 (off), 1 (default network) or 2, 4, 8 hidden layers");
    if (o->max_diffuse > 255 || o->max_specular > 255 || o->max_diffuse < 0 || o->max_specular < 0 ||
        o->max_scatter < 0)
        return bad_arg("mypbr_gpu_render: bounce caps must be in [0, 255]");
    MYPBR_CUDA(cudaSetDevice(G->device));
    WaveParams& P = R.P;
    P = WaveParams{};
    P.S = G->dev;
    P.cam = make_camera(*cam, o->samples_per_pixel);
    P.max_depth = o->max_depth;
    P.max_diffuse = o->max_diffuse;
    P.max_specular = o->max_specular;
    P.max_scatter = o->max_scatter;
    P.transparent_shadows = o->transparent_shadows;
    P.collect_features = o->collect_features;
    P.has_lights = G->dev.light_count > 0;
    P.keyed = G->dev.has_media || G->dev.has_alpha;
    P.seed = o->seed;
    if (size_t(P.cam.width) * P.cam.height > (size_t(1) << 31))
        return bad_arg("mypbr_gpu_render: image too large");
    P.first_row = o->first_row;
    P.band_rows = o->row_count > 0 ? o->row_count : P.cam.height - o->first_row;
    if (o->first_row < 0 || o->row_count < 0 || P.band_rows <= 0 || P.first_row + P.band_rows > P.cam.height)
        return bad_arg("mypbr_gpu_render: first_row / row_count outside the image");
    R.npix = size_t(P.cam.width) * P.band_rows;
    R.timing = o->timing != 0;
    R.spp = o->samples_per_pixel;
    // Paths in flight per wave: the autotuned size, or what the caller asks, or
    // about 128M for a plain render (fewer waves, fewer sparse last bounces:
    // the 1000-sphere field renders 4 % faster than with 32M) and 32M for a
    // guided one (whose network trains after every wave)
    size_t wave_paths = G->tuned_wave_paths ? G->tuned_wave_paths
                                            : (o->guided != 0 ? std::min(plain_wave, size_t(32) << 20) : plain_wave);
    int per_wave = o->samples_per_wave > 0 ? o->samples_per_wave
                                           : int(std::max<size_t>(1, wave_paths / std::max<size_t>(R.npix, 1)));
    per_wave = std::min(per_wave, R.spp);
    if (save_every > 0)
        per_wave = std::min(per_wave, save_every);
    while (per_wave > 1 && R.npix * size_t(per_wave) > (size_t(1) << 30))
        per_wave /= 2;
    R.per_wave = per_wave;
    int s = ensure_buffers(G->rb, R.npix * size_t(per_wave), size_t(P.cam.width) * P.cam.height, P.max_depth + 1);
    if (s != MYPBR_OK)
        return s;
    P.B = G->rb;
    R.L = launch_config(*G);
    R.guided = o->guided != 0;
    R.fixed_waves = o->samples_per_wave > 0;
    if (R.guided) {
        int hidden = (o->guided == 2 || o->guided == 4 || o->guided == 8) ? o->guided : 8;
        s = guide_ensure(G, hidden, o->seed ^ 0x9d2c5680ull);
        if (s != MYPBR_OK)
            return s;
        size_t slots = R.npix * size_t(per_wave);
        // training waves: about 2M paths each, every one recorded
        R.per_wave_train = std::max(1, std::min(per_wave, int((size_t(2) << 20) / std::max<size_t>(R.npix, 1))));
        if (R.fixed_waves)
            R.per_wave_train = per_wave;
        size_t rec_slots = std::min(slots, std::max(R.npix * size_t(R.per_wave_train), size_t(1)));
        s = guide_ensure_records(G, slots, rec_slots, kGuideRecordDepth);
        if (s != MYPBR_OK)
            return s;
        GuideState& g = G->guide;
        P.rec = g.rec;
        P.rec_slots = uint32_t(g.rec_slots);
        P.guide_mix = reinterpret_cast<GuidePacked*>(g.packed);
        P.guide_lo = g.box_lo;
        P.guide_inv = g.box_inv;
        R.L.net = GuideNetView{g.hidden, g.w, g.wt, g.grad, G->dev.error};
        R.L.guide_smem = guide_forward_smem(g.hidden);
        auto k = k_guide_forward<GuideQueueSource, GuidePackSink>;
        MYPBR_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(R.L.guide_smem)));
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 128 * kGuideGroups, R.L.guide_smem);
        R.L.grid_guide = G->sm_count * std::max(per_sm, 1);
        R.L.guided_kernels = true;
    }
    return MYPBR_OK;
}

// Wave number `wave` of a render, starting at pass0: its size, the guiding
// state, the kernels (replayed from `graph` when given), then for guided
// renders the training steps on what the wave recorded.
int render_wave(mypbr_gpu_scene* G, RenderSetup& R, int wave, int pass0, int save_every, cudaStream_t st,
                uint64_t& launches, KernelTimer& T, WaveGraph* graph) {
    NvtxRange range("mypbr wave");
    WaveParams& P = R.P;
    bool train_wave = R.guided && wave < kGuideTrainWaves;
    P.pass0 = pass0;
    P.npass = std::min(train_wave ? R.per_wave_train : R.per_wave, R.spp - pass0);
    if (save_every > 0)  // waves end on every multiple of save_every
        P.npass = std::min(P.npass, save_every - pass0 % save_every);
    if (R.guided) {
        const GuideState& g = G->guide;
        P.guided = g.steps >= g.use_after;
        P.guide_alpha = P.guided ? g.alpha : 0.0f;
        P.guide_alpha_deep = P.guided ? (g.alpha_deep >= 0.0f ? g.alpha_deep : g.alpha) : 0.0f;
        P.guide_depths = std::min(g.depths, P.max_depth);
        P.record = g.steps < g.max_steps;
        if (P.record)
            MYPBR_CUDA(cudaMemsetAsync(P.rec.count, 0, sizeof(uint32_t), st));
    }
    int s = launch_wave(P, R.L, st, launches, T, graph);
    if (s != MYPBR_OK)
        return s;
    if (R.guided && P.record && !G->guide.box_fitted && G->guide.steps == 0) {
        // a fresh network: its position encoding is narrowed to where this
        // wave's vertices lie before it learns anything
        int version = G->guide.box_version;
        if ((s = guide_fit_box(G, st)) != MYPBR_OK)
            return s;
        if (G->guide.box_version != version) {
            P.guide_lo = G->guide.box_lo;
            P.guide_inv = G->guide.box_inv;
            if (graph)
                graph->key = -1;  // the captured kernels hold the old box
        }
    }
    if (R.guided && P.record) {
        if ((s = T.begin(4)) != MYPBR_OK)
            return s;
        const long long left = std::max(0LL, (long long)G->guide.max_steps - G->guide.steps);
        const int steps = (int)std::min<long long>(train_wave ? G->guide.steps_early : G->guide.steps_late, left);
        s = guide_train(G, steps, kGuideBatchTilesPerSm * G->sm_count,
                        kGuideLr, st);
        if (s != MYPBR_OK || (s = T.end()) != MYPBR_OK)
            return s;
        launches += 4 * steps;  // two weight passes, the step, Adam
    }
    return MYPBR_OK;
}

struct Totals {
    unsigned long long* d = nullptr;
    ~Totals() {
        if (d)
            cudaFree(d);
    }
};

int render_all(mypbr_gpu_scene* G, RenderSetup& R, cudaStream_t st, double* d_rad, double* d_alb, double* d_nrm,
               double* d_var, double* d_chvar, int save_every, mypbr_pass_callback cb, void* user,
               double* h_rad, double* h_alb, double* h_nrm, double* h_var, mypbr_render_stats* stats) {
    NvtxRange range("mypbr render");
    WaveParams& P = R.P;
    Totals tot;
    MYPBR_CUDA(cudaMalloc(&tot.d, 3 * sizeof(unsigned long long)));
    MYPBR_CUDA(cudaMemsetAsync(tot.d, 0, 3 * sizeof(unsigned long long), st));
    P.totals = tot.d;
    size_t full = size_t(P.cam.width) * P.cam.height;
    MYPBR_CUDA(cudaMemsetAsync(P.B.film, 0, 3 * full * sizeof(double), st));
    MYPBR_CUDA(cudaMemsetAsync(P.B.film2, 0, 3 * full * sizeof(double), st));
    if (P.collect_features)
        MYPBR_CUDA(cudaMemsetAsync(P.B.feat, 0, 7 * full * sizeof(double), st));
    uint64_t launches = 0;
    KernelTimer T;
    T.on = R.timing;
    T.st = st;
    // per-kernel timing needs events around each launch: no graph then
    WaveGraph graph;
    bool use_graph = !T.on && graphs_allowed(st);
    P.B.wave_state = use_graph ? G->rb.wave_state : nullptr;
    int wave = 0;
    for (int pass0 = 0; pass0 < R.spp; pass0 += P.npass, wave++) {
        int s = render_wave(G, R, wave, pass0, save_every, st, launches, T, use_graph ? &graph : nullptr);
        if (s != MYPBR_OK)
            return s;
        int done = pass0 + P.npass;
        if (cb && save_every > 0 && done % save_every == 0 && done < R.spp) {
            k_resolve<<<R.L.grid_stream, 256, 0, st>>>(P, done, d_rad, d_alb, d_nrm, d_var);
            launches++;
            MYPBR_CUDA(cudaGetLastError());
            if (h_rad) {
                size_t off = size_t(P.first_row) * P.cam.width;
                MYPBR_CUDA(cudaMemcpyAsync(h_rad + 3 * off, d_rad + 3 * off, 3 * R.npix * sizeof(double),
                                           cudaMemcpyDeviceToHost, st));
                if (P.collect_features) {
                    if (h_alb)
                        MYPBR_CUDA(cudaMemcpyAsync(h_alb + 3 * off, d_alb + 3 * off, 3 * R.npix * sizeof(double),
                                                   cudaMemcpyDeviceToHost, st));
                    if (h_nrm)
                        MYPBR_CUDA(cudaMemcpyAsync(h_nrm + 3 * off, d_nrm + 3 * off, 3 * R.npix * sizeof(double),
                                                   cudaMemcpyDeviceToHost, st));
                    if (h_var)
                        MYPBR_CUDA(cudaMemcpyAsync(h_var + off, d_var + off, R.npix * sizeof(double),
                                                   cudaMemcpyDeviceToHost, st));
                }
            }
            MYPBR_CUDA(cudaStreamSynchronize(st));
            cb(done, user);
        }
    }
    k_resolve<<<R.L.grid_stream, 256, 0, st>>>(P, R.spp, d_rad, d_alb, d_nrm, d_var);
    launches++;
    if (d_chvar) {
        k_channel_variance<<<R.L.grid_stream, 256, 0, st>>>(P, R.spp, d_chvar);
        launches++;
    }
    MYPBR_CUDA(cudaGetLastError());
    if (stats) {
        *stats = mypbr_render_stats{};
        unsigned long long t[3];
        MYPBR_CUDA(cudaMemcpyAsync(t, tot.d, sizeof t, cudaMemcpyDeviceToHost, st));
        MYPBR_CUDA(cudaStreamSynchronize(st));
        stats->paths = uint64_t(R.npix) * uint64_t(R.spp);
        stats->extension_rays = t[0];
        stats->shadow_rays = t[1];
        // host launches, plus the kernels of every bounce the wave graphs ran
        stats->kernel_launches = launches + t[2] * graph.per_bounce;
        int s = T.collect(stats);
        if (s != MYPBR_OK)
            return s;
        return check_device_error(G);
    }
    return MYPBR_OK;
}

}  // namespace mypbr_dev

using namespace mypbr_dev;

extern "C" int mypbr_gpu_render_device(mypbr_gpu_scene* G, const mypbr_camera* cam, const mypbr_render_opts* opts,
                                       double* d_radiance, double* d_albedo, double* d_normal, double* d_variance,
                                       void* cuda_stream, mypbr_render_stats* stats) {
    if (!d_radiance)
        return bad_arg("mypbr_gpu_render_device: radiance is required");
    RenderSetup R;
    int s = prepare(G, cam, opts, 0, R);
    if (s != MYPBR_OK)
        return s;
    return render_all(G, R, static_cast<cudaStream_t>(cuda_stream), d_radiance, d_albedo, d_normal, d_variance,
                      nullptr, 0, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, stats);
}

namespace {
struct DevBuf {
    double* p = nullptr;
    ~DevBuf() {
        if (p)
            cudaFree(p);
    }
};
}  // namespace

// The render with host outputs, plus (channel_variance != NULL) the per-channel
// variance of the mean radiance (W*H*3) used by the statistical parity tests.
extern "C" int mypbr_gpu_render_ex(mypbr_gpu_scene* G, const mypbr_camera* cam, const mypbr_render_opts* opts,
                                   double* radiance, double* albedo, double* normal, double* variance,
                                   double* channel_variance, int save_every, mypbr_pass_callback on_pass, void* user,
                                   mypbr_render_stats* stats) {
    if (!radiance)
        return bad_arg("mypbr_gpu_render: radiance is required");
    RenderSetup R;
    int s = prepare(G, cam, opts, save_every, R);
    if (s != MYPBR_OK)
        return s;
    bool feats = opts->collect_features != 0;
    // Device outputs cover the whole image (kernels index by image pixel);
    // only the band's rows come back.
    size_t full = size_t(R.P.cam.width) * R.P.cam.height;
    size_t off = size_t(R.P.first_row) * R.P.cam.width, n = R.npix;
    DevBuf rad, alb, nrm, var, chv;
    MYPBR_CUDA(cudaMalloc(&rad.p, 3 * full * sizeof(double)));
    if (feats) {
        MYPBR_CUDA(cudaMalloc(&alb.p, 3 * full * sizeof(double)));
        MYPBR_CUDA(cudaMalloc(&nrm.p, 3 * full * sizeof(double)));
        MYPBR_CUDA(cudaMalloc(&var.p, full * sizeof(double)));
    }
    if (channel_variance)
        MYPBR_CUDA(cudaMalloc(&chv.p, 3 * full * sizeof(double)));
    cudaStream_t st = G->stream;
    s = render_all(G, R, st, rad.p, alb.p, nrm.p, var.p, chv.p, save_every, on_pass, user, radiance,
                   feats ? albedo : nullptr, feats ? normal : nullptr, feats ? variance : nullptr, stats);
    if (s != MYPBR_OK)
        return s;
    auto back = [&](double* host, const double* dev, size_t per_pixel) {
        return cudaMemcpyAsync(host + per_pixel * off, dev + per_pixel * off, per_pixel * n * sizeof(double),
                               cudaMemcpyDeviceToHost, st);
    };
    MYPBR_CUDA(back(radiance, rad.p, 3));
    if (feats) {
        if (albedo)
            MYPBR_CUDA(back(albedo, alb.p, 3));
        if (normal)
            MYPBR_CUDA(back(normal, nrm.p, 3));
        if (variance)
            MYPBR_CUDA(back(variance, var.p, 1));
    }
    if (channel_variance)
        MYPBR_CUDA(back(channel_variance, chv.p, 3));
    MYPBR_CUDA(cudaStreamSynchronize(st));
    return check_device_error(G);
}

extern "C" int mypbr_gpu_render(mypbr_gpu_scene* G, const mypbr_camera* cam, const mypbr_render_opts* opts,
                                double* radiance, double* albedo, double* normal, double* variance, int save_every,
                                mypbr_pass_callback on_pass, void* user) {
    return mypbr_gpu_render_ex(G, cam, opts, radiance, albedo, normal, variance, nullptr, save_every, on_pass, user,
                               nullptr);
}

// ------------------------------------------------------------ batches
//
// Many renders at once: every job's waves are launched in turn, one wave per
// job per round, each job on its scene handle's own stream, so renders of
// different scenes overlap on the GPU while their waves replay as captured
// graphs. Jobs that share a scene handle run one after another (they share
// its path buffers and network).

namespace mypbr_dev {
namespace {

struct BatchJob {
    RenderSetup R;
    WaveGraph graph;
    KernelTimer T;
    Totals tot;
    uint64_t launches = 0;
    int pass0 = 0, wave = 0;
    bool started = false;
};

int job_start(mypbr_batch_job& jb, BatchJob& j) {
    mypbr_gpu_scene* G = jb.scene;
    if (!jb.radiance)
        return bad_arg("mypbr_gpu_render_batch: every job needs a radiance buffer");
    int s = prepare(G, jb.camera, jb.opts, 0, j.R, size_t(32) << 20);
    if (s != MYPBR_OK)
        return s;
    WaveParams& P = j.R.P;
    cudaStream_t st = G->stream;
    MYPBR_CUDA(cudaMalloc(&j.tot.d, 3 * sizeof(unsigned long long)));
    MYPBR_CUDA(cudaMemsetAsync(j.tot.d, 0, 3 * sizeof(unsigned long long), st));
    P.totals = j.tot.d;
    size_t full = size_t(P.cam.width) * P.cam.height;
    MYPBR_CUDA(cudaMemsetAsync(P.B.film, 0, 3 * full * sizeof(double), st));
    MYPBR_CUDA(cudaMemsetAsync(P.B.film2, 0, 3 * full * sizeof(double), st));
    if (P.collect_features)
        MYPBR_CUDA(cudaMemsetAsync(P.B.feat, 0, 7 * full * sizeof(double), st));
    P.B.wave_state = G->rb.wave_state;
    j.T.st = st;
    j.started = true;
    return MYPBR_OK;
}

// ----------------------------------------------- a batch as one graph
//
// Every job of a batch of plain renders becomes one device-side loop: a
// conditional WHILE node whose body is one bounce (camera rays and feature
// guides are generated only in the iteration that starts a wave) ending in
// k_job_step, which moves to the next bounce, the next wave or the end. The
// jobs of one scene handle follow one another (they share its buffers);
// jobs of different handles are independent branches of the same graph, so
// the whole batch is one graph launch and the GPU schedules the branches.

// Captures job `jb` at the end of the capture running on `st` (whose graph
// is g); the loop body is captured on `side`.
int capture_job(const mypbr_batch_job& jb, RenderSetup& R, cudaStream_t st, cudaStream_t side, cudaGraph_t g) {
    WaveParams& P = R.P;
    size_t full = size_t(P.cam.width) * P.cam.height;
    MYPBR_CUDA(cudaMemsetAsync(P.totals, 0, 3 * sizeof(unsigned long long), st));
    MYPBR_CUDA(cudaMemsetAsync(P.B.film, 0, 3 * full * sizeof(double), st));
    MYPBR_CUDA(cudaMemsetAsync(P.B.film2, 0, 3 * full * sizeof(double), st));
    if (P.collect_features)
        MYPBR_CUDA(cudaMemsetAsync(P.B.feat, 0, 7 * full * sizeof(double), st));
    const int words = int(counter_words(P.B.depth_slots));
    k_job_begin<<<1, 256, 0, st>>>(P, R.per_wave, R.spp, words);
    cudaGraphConditionalHandle loop;
    MYPBR_CUDA(cudaGraphConditionalHandleCreate(&loop, g, 1, cudaGraphCondAssignDefault));
    cudaStreamCaptureStatus status;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    MYPBR_CUDA(cudaStreamGetCaptureInfo(st, &status, nullptr, nullptr, &deps, nullptr, &ndeps));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = loop;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    MYPBR_CUDA(cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &cp));
    MYPBR_CUDA(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    MYPBR_CUDA(cudaStreamBeginCaptureToGraph(side, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                             cudaStreamCaptureModeThreadLocal));
    uint64_t n = 0;
    KernelTimer off;  // no events inside a graph
    off.st = side;
    k_generate<<<R.L.grid_stream, 256, 0, side>>>(P, 1);
    if (P.collect_features)
        k_features<<<R.L.grid_shade, 256, 0, side>>>(P, 1);
    int s = run_bounce(P, R.L, side, n, off, -1);
    if (s == MYPBR_OK)
        k_job_step<<<1, 256, 0, side>>>(P, loop, R.per_wave, R.spp, words);
    cudaGraph_t body = nullptr;
    cudaError_t e = cudaStreamEndCapture(side, &body);
    if (s != MYPBR_OK)
        return s;
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaStreamEndCapture (batch job body)");
    k_resolve<<<R.L.grid_stream, 256, 0, st>>>(P, R.spp, jb.radiance, jb.albedo, jb.normal, jb.variance);
    MYPBR_CUDA(cudaGetLastError());
    return MYPBR_OK;
}

void append_bytes(std::vector<unsigned char>& k, const void* p, size_t n) {
    const unsigned char* c = static_cast<const unsigned char*>(p);
    k.insert(k.end(), c, c + n);
}

}  // namespace

// The instantiated graph of a batch and the key it was captured for: every
// job's wave parameters (all device pointers, camera, options, buffers; the
// totals pointer left out, it belongs to the cache), launch shapes, output
// pointers, in capture order. A batch whose key equals it would capture the
// same nodes with the same arguments, so the graph is launched again as it is.
struct BatchGraphCache {
    std::vector<unsigned char> key;
    cudaGraphExec_t exec = nullptr;
    unsigned long long* totals = nullptr;  // 3 per job
    ~BatchGraphCache() {
        if (exec)
            cudaGraphExecDestroy(exec);
        if (totals)
            cudaFree(totals);
    }
};

void release_batch_graph(mypbr_gpu_scene* G) {
    delete G->batch_graph;
    G->batch_graph = nullptr;
}

namespace {

// The batch as one graph; MYPBR_OK when it ran (every job's status set).
// The graph is kept on the first job's scene handle and replayed by the next
// batch that would capture the same launches.
int batch_one_graph(mypbr_batch_job* jobs, int n, const std::vector<mypbr_gpu_scene*>& scenes,
                    const std::vector<std::vector<int>>& order) {
    const size_t count = size_t(n);
    std::vector<RenderSetup> R(count);
    for (int i = 0; i < n; i++) {
        if (!jobs[i].radiance)
            return bad_arg("mypbr_gpu_render_batch: every job needs a radiance buffer");
        int s = prepare(jobs[i].scene, jobs[i].camera, jobs[i].opts, 0, R[size_t(i)], size_t(32) << 20);
        if (s != MYPBR_OK)
            return s;
    }
    std::vector<unsigned char> key;
    for (size_t k = 0; k < scenes.size(); k++) {
        uint32_t jobs_here = uint32_t(order[k].size());
        append_bytes(key, &jobs_here, sizeof(jobs_here));
        for (int i : order[k]) {
            RenderSetup& r = R[size_t(i)];
            r.P.B = jobs[i].scene->rb;  // the buffers as they are once every job has grown them
            r.P.totals = nullptr;
            append_bytes(key, &r.P, sizeof(r.P));
            append_bytes(key, &r.L, sizeof(r.L));
            append_bytes(key, &r.spp, sizeof(r.spp));
            append_bytes(key, &r.per_wave, sizeof(r.per_wave));
            void* outs[4] = {jobs[i].radiance, jobs[i].albedo, jobs[i].normal, jobs[i].variance};
            append_bytes(key, outs, sizeof(outs));
        }
    }
    mypbr_gpu_scene* owner = scenes[0];
    cudaStream_t st = owner->stream;
    if (!owner->batch_graph || owner->batch_graph->key != key) {
        release_batch_graph(owner);
        std::unique_ptr<BatchGraphCache> c(new BatchGraphCache());
        c->key = std::move(key);
        MYPBR_CUDA(cudaMalloc(&c->totals, 3 * count * sizeof(unsigned long long)));
        for (int i = 0; i < n; i++)
            R[size_t(i)].P.totals = c->totals + 3 * size_t(i);
        struct Owned {
            cudaGraph_t g = nullptr;
            cudaStream_t side = nullptr;
            ~Owned() {
                if (g)
                    cudaGraphDestroy(g);
                if (side)
                    cudaStreamDestroy(side);
            }
        } o;
        MYPBR_CUDA(cudaStreamCreateWithFlags(&o.side, cudaStreamNonBlocking));
        MYPBR_CUDA(cudaGraphCreate(&o.g, 0));
        for (size_t k = 0; k < scenes.size(); k++) {
            cudaStream_t sk = scenes[k]->stream;
            MYPBR_CUDA(cudaStreamBeginCaptureToGraph(sk, o.g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
            int s = MYPBR_OK;
            for (int i : order[k]) {
                s = capture_job(jobs[i], R[size_t(i)], sk, o.side, o.g);
                if (s != MYPBR_OK)
                    break;
            }
            cudaGraph_t captured = nullptr;
            cudaError_t e = cudaStreamEndCapture(sk, &captured);
            if (s != MYPBR_OK)
                return s;
            if (e != cudaSuccess)
                return cuda_fail(e, "cudaStreamEndCapture (batch)");
        }
        MYPBR_CUDA(cudaGraphInstantiate(&c->exec, o.g, 0));
        owner->batch_graph = c.release();
    }
    {
        NvtxRange range("mypbr batch graph");
        MYPBR_CUDA(cudaGraphLaunch(owner->batch_graph->exec, st));
        MYPBR_CUDA(cudaStreamSynchronize(st));
    }
    int first_error = MYPBR_OK;
    for (mypbr_gpu_scene* G : scenes) {
        int s = check_device_error(G);
        for (int i = 0; i < n; i++)
            if (jobs[i].scene == G)
                jobs[i].status = s;
        if (s != MYPBR_OK && first_error == MYPBR_OK)
            first_error = s;
    }
    return first_error;
}

}  // namespace
}  // namespace mypbr_dev

extern "C" int mypbr_gpu_render_batch(mypbr_batch_job* jobs, int32_t n) {
    if (n < 0 || (n > 0 && !jobs))
        return bad_arg("mypbr_gpu_render_batch: bad job list");
    std::vector<std::unique_ptr<BatchJob>> J;
    std::vector<mypbr_gpu_scene*> scenes;            // in first-use order
    std::vector<std::vector<int>> order;             // job indices per scene
    for (int i = 0; i < n; i++) {
        jobs[i].status = MYPBR_ERR_INVALID_ARGUMENT;
        J.emplace_back(new BatchJob());
        if (!jobs[i].scene || !jobs[i].camera || !jobs[i].opts)
            continue;
        auto it = std::find(scenes.begin(), scenes.end(), jobs[i].scene);
        if (it == scenes.end()) {
            scenes.push_back(jobs[i].scene);
            order.emplace_back();
            it = scenes.end() - 1;
        }
        order[size_t(it - scenes.begin())].push_back(i);
    }
    // plain jobs on capturable streams: the whole batch as one graph launch
    // (MYPBR_BATCH_ONE_GRAPH=0 keeps the per-wave host loop, for comparison)
    const char* env = std::getenv("MYPBR_BATCH_ONE_GRAPH");
    bool one_graph = n > 0 && !scenes.empty() && !(env && env[0] == '0');
    for (int i = 0; i < n && one_graph; i++)
        one_graph = jobs[i].scene && jobs[i].camera && jobs[i].opts && jobs[i].opts->guided == 0 &&
                    jobs[i].opts->timing == 0;
    for (mypbr_gpu_scene* G : scenes)
        one_graph = one_graph && graphs_allowed(G->stream);
    if (one_graph) {
        int s = batch_one_graph(jobs, n, scenes, order);
        for (int i = 0; i < n; i++)
            if (s != MYPBR_OK && jobs[i].status == MYPBR_OK)
                jobs[i].status = s;
        if (s != MYPBR_OK)
            for (int i = 0; i < n; i++)
                if (jobs[i].status == MYPBR_ERR_INVALID_ARGUMENT && s != MYPBR_ERR_INVALID_ARGUMENT)
                    jobs[i].status = s;
        return s;
    }
    std::vector<size_t> next(scenes.size(), 0);
    int first_error = MYPBR_OK;
    bool any = true;
    while (any) {
        any = false;
        for (size_t k = 0; k < scenes.size(); k++) {
            if (next[k] >= order[k].size())
                continue;
            any = true;
            int i = order[k][next[k]];
            mypbr_batch_job& jb = jobs[i];
            BatchJob& j = *J[size_t(i)];
            mypbr_gpu_scene* G = scenes[k];
            int s = MYPBR_OK;
            if (!j.started)
                s = job_start(jb, j);
            if (s == MYPBR_OK && j.pass0 < j.R.spp) {
                s = render_wave(G, j.R, j.wave, j.pass0, 0, G->stream, j.launches, j.T, &j.graph);
                j.pass0 += j.R.P.npass;
                j.wave++;
                if (s == MYPBR_OK)
                    continue;  // this job's next wave in the next round
            }
            if (s == MYPBR_OK) {  // all waves launched: the averages into the caller's buffers
                WaveParams& P = j.R.P;
                k_resolve<<<j.R.L.grid_stream, 256, 0, G->stream>>>(P, j.R.spp, jb.radiance, jb.albedo, jb.normal,
                                                                   jb.variance);
                cudaError_t e = cudaGetLastError();
                s = e == cudaSuccess ? MYPBR_OK : cuda_fail(e, "k_resolve");
                // the next job of this scene reuses the buffers: the stream orders it
            }
            jb.status = s;
            if (s != MYPBR_OK && first_error == MYPBR_OK)
                first_error = s;
            next[k]++;
        }
    }
    for (mypbr_gpu_scene* G : scenes) {
        cudaError_t e = cudaStreamSynchronize(G->stream);
        int s = e == cudaSuccess ? check_device_error(G) : cuda_fail(e, "mypbr_gpu_render_batch");
        if (s != MYPBR_OK) {
            for (int i = 0; i < n; i++)
                if (jobs[i].scene == G && jobs[i].status == MYPBR_OK)
                    jobs[i].status = s;
            if (first_error == MYPBR_OK)
                first_error = s;
        }
    }
    for (int i = 0; i < n; i++)
        if (jobs[i].status != MYPBR_OK && first_error == MYPBR_OK)
            first_error = jobs[i].status;
    return first_error;
}

// ------------------------------------------------------------ autotuner
//
// Tries the threads per block of the bounce kernels (128, 256) and the paths
// per wave (16M, 32M, 64M, 128M: the queue capacity) on short renders of the
// given view (about 256M paths each, two waves of the largest size), and
// keeps the fastest on the scene handle for later renders.

extern "C" int mypbr_gpu_autotune(mypbr_gpu_scene* G, const mypbr_camera* cam, const mypbr_render_opts* opts,
                                  mypbr_tune_result* out) {
    if (!G || !cam || !opts)
        return bad_arg("mypbr_gpu_autotune: null argument");
    mypbr_render_opts o = *opts;
    o.samples_per_wave = 0;
    o.timing = 0;
    o.guided = 0;
    int w = cam->image_width;
    int h = cam->image_height > 0 ? cam->image_height : std::max(1, int(cam->image_width / cam->aspect_ratio));
    size_t npix = size_t(w) * h;
    // about 256M paths per trial, at most the caller's spp
    o.samples_per_pixel = int(std::max<size_t>(1, std::min<size_t>(size_t(opts->samples_per_pixel),
                                                                       (size_t(256) << 20) / std::max<size_t>(npix, 1))));
    DevBuf rad;
    MYPBR_CUDA(cudaMalloc(&rad.p, 3 * npix * sizeof(double)));
    const int blocks[2] = {128, 256};
    const size_t waves[4] = {size_t(16) << 20, size_t(32) << 20, size_t(64) << 20, size_t(128) << 20};
    mypbr_tune_result res{};
    double best = -1;
    size_t keep_paths = G->tuned_wave_paths;
    int keep_block = G->tuned_block, keep_trav = G->tuned_traversal;
    cudaEvent_t e0, e1;
    MYPBR_CUDA(cudaEventCreate(&e0));
    MYPBR_CUDA(cudaEventCreate(&e1));
    int status = MYPBR_OK;
    int trial = 0;
    for (int trav = 1; trav <= 5; trav++)
    for (int b : blocks) {
        if ((trav == 2 && G->dev.bvh4 == nullptr) || (trav == 3 && !G->dev.postponed_ok) ||
            (trav == 5 && G->dev.bvh8 == nullptr)) {
            trial += 4;  // a walk this scene's tree does not allow: trials skipped
            continue;
        }
        for (size_t wp : waves) {
            G->tuned_traversal = trav;
            G->tuned_block = b;
            G->tuned_wave_paths = wp;
            float ms = 0;
            for (int rep = 0; rep < 2 && status == MYPBR_OK; rep++) {  // the first run warms up
                cudaEventRecord(e0, G->stream);
                status = mypbr_gpu_render_device(G, cam, &o, rad.p, nullptr, nullptr, nullptr, G->stream, nullptr);
                cudaEventRecord(e1, G->stream);
                cudaEventSynchronize(e1);
                cudaEventElapsedTime(&ms, e0, e1);
            }
            if (status != MYPBR_OK)
                break;
            double mp = double(npix) * o.samples_per_pixel / (ms * 1e-3) / 1e6;
            res.trial_mpaths[trial++] = mp;
            if (mp > best) {
                best = mp;
                res.block = b;
                res.traversal = trav;
                res.wave_paths = int64_t(wp);
                res.mpaths_per_s = mp;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (status != MYPBR_OK) {
        G->tuned_wave_paths = keep_paths;
        G->tuned_block = keep_block;
        G->tuned_traversal = keep_trav;
        return status;
    }
    G->tuned_block = res.block;
    G->tuned_traversal = res.traversal;
    G->tuned_wave_paths = size_t(res.wave_paths);
    if (out)
        *out = res;
    return MYPBR_OK;
}

extern "C" int mypbr_gpu_set_launch(mypbr_gpu_scene* G, int32_t block, int64_t wave_paths, int32_t traversal) {
    if (!G || (block != 0 && block != 128 && block != 256) || wave_paths < 0 || traversal < 0 || traversal > 5)
        return bad_arg("mypbr_gpu_set_launch: block 0, 128 or 256; wave_paths >= 0; traversal 0 to 5");
    G->tuned_block = block;
    G->tuned_wave_paths = size_t(wave_paths);
    G->tuned_traversal = traversal;
    return MYPBR_OK;
}

// ------------------------------------------------- render without allocation
//
// mypbr_gpu_render_noalloc: the same render, with every scratch buffer (path
// state, queues, queue counters, FP64 film, ray totals) carved from one
// file-scope device array instead of cudaMalloc. It serves callers that may
// not allocate device memory while they render: a host application that hands
// this library a fixed device-memory budget up front and forbids allocation
// afterwards, or a per-frame callback of an interactive viewer in which the
// device-wide synchronisation an allocation can cause would stall the frame.
// The scene must already be on the device (mypbr_gpu_scene_create) and the
// caller passes device output buffers.
//
// Limits: at most kNoAllocMaxPixels (65,536) pixels in the rendered rows
// (width x row_count; a band of a larger image is fine), max_depth at most
// kNoAllocMaxDepth. The array (kNoAllocBytes, 18 MiB) exists on every GPU that
// loads this library, for as long as the library is loaded. Every call reuses
// it and it keeps the previous call's contents, so the film and counters are
// cleared at the start of each call; two calls whose work overlaps on the GPU
// (different streams, or different host threads) race on it and must not be
// issued. The first call on a device looks the array's device address up
// (cudaGetSymbolAddress) with that device current and keeps it; make that
// first call before any stream capture begins, and do not reset the device
// (cudaDeviceReset) while the library is loaded, since the kept address would
// then be stale.

namespace mypbr_dev {
namespace {

constexpr size_t kNoAllocMaxPixels = 65536;  // path slots and film pixels
constexpr int kNoAllocMaxDepth = 1024;
constexpr size_t kNoAllocAlign = 256;

constexpr size_t align_up(size_t x) { return (x + kNoAllocAlign - 1) / kNoAllocAlign * kNoAllocAlign; }
constexpr size_t kSlotBytes = 8 * sizeof(float4) + (3 + kShadeClasses) * sizeof(uint32_t);
constexpr size_t kPixelBytes = (3 + 3 + 7) * sizeof(double);
constexpr size_t kCounterBytes = ((3 + kShadeClasses) * (kNoAllocMaxDepth + 1) + 8) * sizeof(uint32_t);
constexpr size_t kNoAllocNeed = 16 * kNoAllocAlign + kNoAllocMaxPixels * (kSlotBytes + kPixelBytes) + kCounterBytes +
                                2 * sizeof(unsigned long long);
constexpr size_t kNoAllocBytes = size_t(18) << 20;
static_assert(kNoAllocNeed <= kNoAllocBytes, "scratch layout exceeds the static array");

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[kMaxDevices] = {};

// The array's device address on the current device, looked up once per device.
int noalloc_scratch(int device, unsigned char** out) {
    if (device < 0 || device >= kMaxDevices)
        return bad_arg("mypbr_gpu_render_noalloc: device index out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_noalloc_ptr[device] = p;
    }
    *out = static_cast<unsigned char*>(g_noalloc_ptr[device]);
    return MYPBR_OK;
}

// Carves the render buffers out of the array (each start 256-byte aligned).
RenderBuffers carve(unsigned char* base, unsigned long long** totals) {
    RenderBuffers rb;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        unsigned char* p = base + off;
        off = align_up(off + bytes);
        return p;
    };
    const size_t n = kNoAllocMaxPixels;
    rb.ray_o = reinterpret_cast<float4*>(take(n * sizeof(float4)));
    rb.ray_d = reinterpret_cast<float4*>(take(n * sizeof(float4)));
    rb.beta = reinterpret_cast<float4*>(take(n * sizeof(float4)));
    rb.radiance = reinterpret_cast<float4*>(take(n * sizeof(float4)));
    rb.hit = reinterpret_cast<float4*>(take(n * sizeof(float4)));
    rb.sh_o = reinterpret_cast<float4*>(take(n * sizeof(float4)));
    rb.sh_d = reinterpret_cast<float4*>(take(n * sizeof(float4)));
    rb.sh_c = reinterpret_cast<float4*>(take(n * sizeof(float4)));
    rb.queue[0] = reinterpret_cast<uint32_t*>(take(n * sizeof(uint32_t)));
    rb.queue[1] = reinterpret_cast<uint32_t*>(take(n * sizeof(uint32_t)));
    rb.class_queue = reinterpret_cast<uint32_t*>(take(kShadeClasses * n * sizeof(uint32_t)));
    rb.shadow_queue = reinterpret_cast<uint32_t*>(take(n * sizeof(uint32_t)));
    rb.counters = reinterpret_cast<uint32_t*>(take(kCounterBytes));
    rb.film = reinterpret_cast<double*>(take(3 * n * sizeof(double)));
    rb.film2 = reinterpret_cast<double*>(take(3 * n * sizeof(double)));
    rb.feat = reinterpret_cast<double*>(take(7 * n * sizeof(double)));
    *totals = reinterpret_cast<unsigned long long*>(take(2 * sizeof(unsigned long long)));
    rb.capacity = n;
    rb.pixels = n;
    rb.depth_slots = kNoAllocMaxDepth + 1;
    return rb;
}

}  // namespace
}  // namespace mypbr_dev

extern "C" int mypbr_gpu_render_noalloc(mypbr_gpu_scene* G, const mypbr_camera* cam, const mypbr_render_opts* o,
                                        double* d_radiance, double* d_albedo, double* d_normal, double* d_variance,
                                        void* cuda_stream) {
    if (!G || !cam || !o || !d_radiance)
        return bad_arg("mypbr_gpu_render_noalloc: null argument");
    if (cam->image_width < 1 || o->samples_per_pixel < 1 || o->max_depth < 1)
        return bad_arg("mypbr_gpu_render_noalloc: image_width, samples_per_pixel and max_depth must be positive");
    if (o->max_depth > kNoAllocMaxDepth)
        return bad_arg("mypbr_gpu_render_noalloc: max_depth is limited to " + std::to_string(kNoAllocMaxDepth));
    if (o->guided != 0) {
        set_error_message("mypbr_gpu_render_noalloc: guided rendering is not supported by the render without "
                          "allocation (it has no scratch for the network's training records)");
        return MYPBR_ERR_UNSUPPORTED;
    }
    if (o->max_diffuse > 255 || o->max_specular > 255 || o->max_scatter > 255 || o->max_diffuse < 0 ||
        o->max_specular < 0 || o->max_scatter < 0)
        return bad_arg("mypbr_gpu_render_noalloc: bounce caps must be in [0, 255]");
    MYPBR_CUDA(cudaSetDevice(G->device));
    WaveParams P{};
    P.S = G->dev;
    P.cam = make_camera(*cam, o->samples_per_pixel);
    P.first_row = o->first_row;
    P.band_rows = o->row_count > 0 ? o->row_count : P.cam.height - o->first_row;
    if (o->first_row < 0 || o->row_count < 0 || P.band_rows <= 0 || P.first_row + P.band_rows > P.cam.height)
        return bad_arg("mypbr_gpu_render_noalloc: first_row / row_count outside the image");
    size_t npix = size_t(P.cam.width) * P.band_rows;
    if (npix > kNoAllocMaxPixels)
        return bad_arg("mypbr_gpu_render_noalloc: " + std::to_string(P.cam.width) + " x " +
                       std::to_string(P.band_rows) + " rendered pixels exceed the " +
                       std::to_string(kNoAllocMaxPixels) + "-pixel limit of the render without allocation");
    P.max_depth = o->max_depth;
    P.max_diffuse = o->max_diffuse;
    P.max_specular = o->max_specular;
    P.max_scatter = o->max_scatter;
    P.transparent_shadows = o->transparent_shadows;
    P.collect_features = o->collect_features;
    P.has_lights = G->dev.light_count > 0;
    P.keyed = G->dev.has_media || G->dev.has_alpha;
    P.seed = o->seed;
    unsigned char* base = nullptr;
    int s = noalloc_scratch(G->device, &base);
    if (s != MYPBR_OK)
        return s;
    P.B = carve(base, &P.totals);
    int spp = o->samples_per_pixel;
    int per_wave = int(std::max<size_t>(1, kNoAllocMaxPixels / npix));
    per_wave = std::min(per_wave, spp);
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    // The array keeps the last call's contents: clear what accumulates (the
    // band's film only, which starts at the array's film buffers)
    MYPBR_CUDA(cudaMemsetAsync(P.B.film, 0, 3 * npix * sizeof(double), st));
    MYPBR_CUDA(cudaMemsetAsync(P.B.film2, 0, 3 * npix * sizeof(double), st));
    if (P.collect_features)
        MYPBR_CUDA(cudaMemsetAsync(P.B.feat, 0, 7 * npix * sizeof(double), st));
    MYPBR_CUDA(cudaMemsetAsync(P.totals, 0, 2 * sizeof(unsigned long long), st));
    // The kernels index the film by the pixel's place in the whole image; the
    // array holds only the band's pixels, so the film pointers are moved back
    // by the band's first pixel (only indices from that pixel on are used)
    size_t first_pixel = size_t(P.first_row) * P.cam.width;
    P.B.film -= 3 * first_pixel;
    P.B.film2 -= 3 * first_pixel;
    P.B.feat -= 7 * first_pixel;
    Launch L = launch_config(*G);
    uint64_t launches = 0;
    KernelTimer T;  // off: no events are created
    T.st = st;
    for (int pass0 = 0; pass0 < spp; pass0 += per_wave) {
        P.pass0 = pass0;
        P.npass = std::min(per_wave, spp - pass0);
        s = run_wave(P, L, st, launches, T);
        if (s != MYPBR_OK)
            return s;
    }
    k_resolve<<<L.grid_stream, 256, 0, st>>>(P, spp, d_radiance, d_albedo, d_normal, d_variance);
    MYPBR_CUDA(cudaGetLastError());
    MYPBR_CUDA(cudaStreamSynchronize(st));
    return check_device_error(G);
}
