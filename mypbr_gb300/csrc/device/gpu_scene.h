// The device scene handle behind mypbr_gpu_scene and the helpers the
// translation units share.
#pragma once

#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../../include/mypbr_gpu.h"
#include "guide.cuh"

namespace mypbr_dev {

struct BatchGraphCache;  // render.cu

// Scratch memory of one render: path state in slots, queues of slot indices,
// the FP64 film. Kept on the scene handle and grown on demand.
struct RenderBuffers {
    size_t capacity = 0;   // path slots
    size_t pixels = 0;     // film pixels
    int depth_slots = 0;   // per-bounce queue counters
    // path state (slot-indexed, 64 B)
    float4* ray_o = nullptr;     // origin, path flags (bits)
    float4* ray_d = nullptr;     // direction, scatter pdf of the direction
    float4* beta = nullptr;      // throughput, pass (bits)
    float4* radiance = nullptr;  // path radiance so far, pixel (bits)
    float4* hit = nullptr;       // t, b1, b2, prim (bits)
    float4* sh_o = nullptr;      // shadow ray: origin, -
    float4* sh_d = nullptr;      // direction, final flag
    float4* sh_c = nullptr;      // contribution rgb, -
    uint32_t* queue[2] = {nullptr, nullptr};  // extension queues (ping-pong)
    uint32_t* class_queue = nullptr;          // one queue per shading class, capacity each
    uint32_t* shadow_queue = nullptr;
    uint32_t* counters = nullptr;
    int* wave_state = nullptr;   // (first pass, passes) of the wave a captured graph replays; null: kernel arguments
    // film (pixel-indexed, FP64 sums)
    double* film = nullptr;   // radiance sum rgb
    double* film2 = nullptr;  // radiance squared sum rgb
    double* feat = nullptr;   // albedo rgb, normal rgb, luminance^2 (7 per pixel)
};

// The guiding network of a scene and what training it needs on the device.
struct GuideState {
    int hidden = 0;                  // 0: no network yet
    int params = 0;
    __nv_bfloat16* w = nullptr;      // canonical BF16 copies the kernels read
    __nv_bfloat16* wt = nullptr;
    float* master = nullptr;         // FP32 weights, Adam moments, gradients ([out][in] per matrix)
    float* m = nullptr;
    float* v = nullptr;
    float* grad = nullptr;
    float* stats = nullptr;          // [0] loss sum, [1] weight sum of the current batch
    __nv_bfloat16* scratch = nullptr;  // per training group: the layer inputs of its tile
    float* partial = nullptr;          // per training group: its FP32 weight gradients
    int train_ctas = 0;
    long long steps = 0;             // Adam steps taken
    float3 box_lo{}, box_inv{};      // box of the position encoding: the scene's, then where paths go
    bool box_fitted = false;         // narrowed to the recorded vertices (once per fresh network)
    int box_version = 0;             // bumped when the box changes (waves captured before must be re-captured)
    // sampling: the mixture is drawn with probability alpha (else the BSDF) at
    // the first `depths` bounces of a path (mypbr_guide_configure); by default
    // at the kGuideRecordDepth vertices the network is trained on
    float alpha = 0.5f;
    float alpha_deep = -1.0f;  // alpha at bounces after the first (below 0: alpha)
    int depths = 4;
    // training schedule (mypbr_guide_schedule): Adam steps after each of the
    // first recorded waves and after each later one, and the total after
    // which recording and training stop
    int steps_early = 16, steps_late = 4, max_steps = 1500;
    int use_after = 128;  // steps before the mixture is sampled at all
    float weight_cap = 256.0f;  // a record's training weight at most this x the batch's mean (0: no cap)
    // recording buffers (slot-indexed, grown with the render buffers)
    GuideRecords rec{};
    size_t rec_slots = 0;
    __half* packed = nullptr;        // per slot: the vertex's decoded mixture (GuidePacked)
    size_t packed_slots = 0;
};

}  // namespace mypbr_dev

struct mypbr_gpu_scene {
    mypbr_dev::DeviceScene dev{};
    std::vector<void*> allocations;
    int device = 0;
    int sm_count = 0;
    int max_depth_bvh = 0;
    size_t leaf_ref_count = 0;
    int64_t material_count = 0;
    mypbr_dev::RenderBuffers rb;
    mypbr_dev::GuideState guide;
    float3 box_lo{-1.0f, -1.0f, -1.0f}, box_hi{1.0f, 1.0f, 1.0f};  // bounds of the BVH's primitives
    cudaStream_t stream = nullptr;  // the handle's own stream, for renders with host buffers (graph capture needs one)
    // autotuned launch settings (0: built-in defaults)
    size_t tuned_wave_paths = 0;
    int tuned_block = 0;
    int tuned_traversal = 0;  // 0: the scene's default (3 or 4); 1: lanes take new rays (k_extend_pt);
                              // 2: the 4-wide tree; 3: postponed leaves; 4: the plain binary walk
    bool prefer_postponed = false;  // spheres fill fewer than half the leaves: traversal 0 means 3
    // the instantiated graph of the last batch whose first job used this
    // handle, replayed while a batch captures to the same launches
    mypbr_dev::BatchGraphCache* batch_graph = nullptr;
};

namespace mypbr_dev {

// An NVTX range around a stage (render, wave, training, uploads, builds), for
// profilers that show them; nothing is recorded unless a tool is attached.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

void set_error_message(const std::string& m);
int cuda_fail(cudaError_t e, const char* what);
int release_buffers(RenderBuffers& rb);
int check_device_error(mypbr_gpu_scene* G);
int release_guide(GuideState& g);
void release_batch_graph(mypbr_gpu_scene* G);
// Creates the network (seeded initial weights) if the scene has none of this size.
int guide_ensure(mypbr_gpu_scene* G, int hidden, unsigned long long seed);
// Mixture buffers for `mix_slots` path slots, training records for the first `rec_slots`.
int guide_ensure_records(mypbr_gpu_scene* G, size_t mix_slots, size_t rec_slots, int depth);
// `steps` Adam steps on batches drawn from the recorded vertices.
int guide_train(mypbr_gpu_scene* G, int steps, int batch_tiles, float lr, cudaStream_t st);
// Narrows a fresh network's position box to where the recorded vertices lie
// (1st to 99th percentile per axis, plus a margin) and re-expresses the
// records in it. Synchronises the stream once.
int guide_fit_box(mypbr_gpu_scene* G, cudaStream_t st);
// The binary tree's device nodes collapsed to four children per node (walk_tree4's layout); depth: deepest level.
void collapse_to_4(const std::vector<float4>& bin, std::vector<float4>& out, int& depth);
// The binary tree collapsed to 8 children per node with quantised child boxes
// (the layout walk_tree8q reads); false (out empty) when a leaf holds 16 or
// more references or starts past 2^27.
bool collapse_to_8q(const std::vector<float4>& bin, std::vector<uint4>& out, int& depth);
// The environment's pdf table (p n per texel) and alias table (probability, alias index bits) from its
// pixels (w x h x 3 floats): on the device (device pointers, env_dist.cu) or on the host (Vose's method).
int build_env_distribution(const float* rgb, int w, int h, float* texel_pdf, float2* alias, cudaStream_t st);
void env_distribution_host(const float* rgb, int w, int h, float* texel_pdf, float2* alias);

}  // namespace mypbr_dev

#define MYPBR_CUDA(call)                                       \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess)                                 \
            return ::mypbr_dev::cuda_fail(e_, #call);          \
    } while (0)
