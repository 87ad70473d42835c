// The denoiser of the reference (include/denoiser.h:45-193) on the device:
// firefly clamp, then edge-avoiding a-trous iterations with the SVGF
// variance-guided luminance weight, on lighting = radiance / (albedo + 1e-3).
//
// Iteration i spreads its 5 x 5 B3-spline taps 2^i pixels apart, so the taps
// of pixel (x, y) all lie on the lattice {(x + a s, y + b s)} of spacing s.
// A block takes one phase (x mod s, y mod s) of the image and a 16 x 16 tile
// of that phase's lattice: it stages the 20 x 20 lattice points the tile's
// taps reach (lighting + variance, albedo, normal: 48 B each) in shared
// memory once, and every staged point then serves up to 25 outputs. The
// variance blur (3 x 3 at step 1, denoiser.h:158-178) is a separate pass.
// Arithmetic is FP32; the frame comes in and goes out in FP64.
#include <algorithm>
#include <string>

#include "dev_math.cuh"
#include "gpu_scene.h"

namespace mypbr_dev {
namespace {

constexpr int kTile = 16;
constexpr int kHalo = 2;
constexpr int kSpan = kTile + 2 * kHalo;

MYPBR_DEV float lum(float4 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

// lighting = radiance / (albedo + eps), its variance over luminance(albedo + eps)^2
__global__ void k_dn_prepare(const double* rad, const double* alb, const double* nrm, const double* var, int n,
                             float4* L, float4* A, float4* N) {
    const float eps = 1e-3f;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        float a0 = float(alb[3 * k]), a1 = float(alb[3 * k + 1]), a2 = float(alb[3 * k + 2]);
        float e0 = a0 + eps, e1 = a1 + eps, e2 = a2 + eps;
        float la = 0.2126f * e0 + 0.7152f * e1 + 0.0722f * e2;
        L[k] = make_float4(float(rad[3 * k]) / e0, float(rad[3 * k + 1]) / e1, float(rad[3 * k + 2]) / e2,
                           float(var[k]) / (la * la));
        A[k] = make_float4(a0, a1, a2, 0.0f);
        N[k] = make_float4(float(nrm[3 * k]), float(nrm[3 * k + 1]), float(nrm[3 * k + 2]), 0.0f);
    }
}

// remove_fireflies (denoiser.h:90-111): a pixel brighter than its eight
// neighbours whose deviation exceeds half its luminance is scaled down to the
// brightest neighbour. Reads src, writes dst (every pixel).
__global__ void k_dn_fireflies(const float4* src, float4* dst, int w, int h) {
    int n = w * h;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        float4 c = src[k];
        int i = k % w, j = k / w;
        if (i >= 1 && i < w - 1 && j >= 1 && j < h - 1) {
            float l = lum(c);
            if (l > 0.0f && !(sqrtf(c.w) < 0.5f * l)) {
                float brightest = 0.0f;
                for (int dy = -1; dy <= 1; dy++)
                    for (int dx = -1; dx <= 1; dx++)
                        if (dx || dy)
                            brightest = fmaxf(brightest, lum(src[k + dy * w + dx]));
                if (l > brightest) {
                    float s = brightest / l;
                    c = make_float4(s * c.x, s * c.y, s * c.z, c.w * s * s);
                }
            }
        }
        dst[k] = c;
    }
}

// blur3x3 of the variance (denoiser.h:158-178), normalised by the weights inside the image
__global__ void k_dn_blur(const float4* L, float* bv, int w, int h) {
    int n = w * h;
    const float k3[3] = {0.25f, 0.5f, 0.25f};
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        int i = k % w, j = k / w;
        float sum = 0.0f, wt = 0.0f;
        for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++) {
                int x = i + dx, y = j + dy;
                if (x < 0 || x >= w || y < 0 || y >= h)
                    continue;
                float c = k3[dx + 1] * k3[dy + 1];
                sum += c * L[y * w + x].w;
                wt += c;
            }
        bv[k] = sum / wt;
    }
}

// One a-trous iteration (filter_pixel, denoiser.h:113-156) at spacing `step`.
// grid: (tiles_x * step, tiles_y * step); block (16, 16).
__global__ void __launch_bounds__(256) k_dn_atrous(const float4* L, const float* bv, const float4* A,
                                                     const float4* N, float4* out, int w, int h, int step,
                                                     float sigma_l, float inv_n, float inv_a) {
    __shared__ float4 sL[kSpan][kSpan];
    __shared__ float4 sA[kSpan][kSpan];
    __shared__ float4 sN[kSpan][kSpan];
    // which phase of the lattice, and which tile of that phase
    int tiles_x = (gridDim.x + step - 1) / step;  // tiles per phase column (gridDim.x = tiles_x * step)
    int phase_x = blockIdx.x / tiles_x, tile_x = blockIdx.x % tiles_x;
    int tiles_y = (gridDim.y + step - 1) / step;
    int phase_y = blockIdx.y / tiles_y, tile_y = blockIdx.y % tiles_y;
    int lx0 = tile_x * kTile - kHalo, ly0 = tile_y * kTile - kHalo;  // lattice origin of the staged span
    int tid = threadIdx.y * kTile + threadIdx.x;
    for (int e = tid; e < kSpan * kSpan; e += kTile * kTile) {
        int sx = e % kSpan, sy = e / kSpan;
        int x = phase_x + (lx0 + sx) * step, y = phase_y + (ly0 + sy) * step;
        if (x >= 0 && x < w && y >= 0 && y < h) {
            int q = y * w + x;
            sL[sy][sx] = L[q];
            sA[sy][sx] = A[q];
            sN[sy][sx] = N[q];
        } else {
            sA[sy][sx] = make_float4(0.0f, 0.0f, 0.0f, -1.0f);  // outside the image: no tap
        }
    }
    __syncthreads();
    int cx = threadIdx.x + kHalo, cy = threadIdx.y + kHalo;
    int x = phase_x + (lx0 + cx) * step, y = phase_y + (ly0 + cy) * step;
    if (x >= w || y >= h || phase_x >= step || phase_y >= step)
        return;
    const float kern[5] = {1.0f / 16, 1.0f / 4, 3.0f / 8, 1.0f / 4, 1.0f / 16};
    float4 cp = sL[cy][cx], ap = sA[cy][cx], np = sN[cy][cx];
    float lp = lum(cp);
    float scale = sigma_l * sqrtf(fmaxf(bv[y * w + x], 0.0f)) + 1e-10f;
    float inv_scale = 1.0f / scale;
    float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, ws = 0.0f, vs = 0.0f;
#pragma unroll
    for (int dy = 0; dy < 5; dy++) {
#pragma unroll
        for (int dx = 0; dx < 5; dx++) {
            float4 aq = sA[cy + dy - 2][cx + dx - 2];
            if (aq.w < 0.0f)
                continue;
            float4 cq = sL[cy + dy - 2][cx + dx - 2], nq = sN[cy + dy - 2][cx + dx - 2];
            float n0 = np.x - nq.x, n1 = np.y - nq.y, n2 = np.z - nq.z;
            float a0 = ap.x - aq.x, a1 = ap.y - aq.y, a2 = ap.z - aq.z;
            float e = (n0 * n0 + n1 * n1 + n2 * n2) * inv_n + (a0 * a0 + a1 * a1 + a2 * a2) * inv_a +
                      fabsf(lp - lum(cq)) * inv_scale;
            float wgt = kern[dx] * kern[dy] * __expf(-e);
            s0 += wgt * cq.x;
            s1 += wgt * cq.y;
            s2 += wgt * cq.z;
            ws += wgt;
            vs += wgt * wgt * cq.w;
        }
    }
    float iw = 1.0f / ws;
    out[y * w + x] = make_float4(s0 * iw, s1 * iw, s2 * iw, vs * iw * iw);
}

__global__ void k_dn_finish(const float4* L, const double* alb, double* out, int n) {
    const double eps = 1e-3;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        float4 c = L[k];
        out[3 * k] = double(c.x) * (alb[3 * k] + eps);
        out[3 * k + 1] = double(c.y) * (alb[3 * k + 1] + eps);
        out[3 * k + 2] = double(c.z) * (alb[3 * k + 2] + eps);
    }
}

struct Buf {
    void* p = nullptr;
    ~Buf() {
        if (p)
            cudaFree(p);
    }
};

int bad(const std::string& m) {
    set_error_message(m);
    return MYPBR_ERR_INVALID_ARGUMENT;
}

}  // namespace
}  // namespace mypbr_dev

using namespace mypbr_dev;

extern "C" void mypbr_denoise_opts_init(mypbr_denoise_opts* o) {
    if (!o)
        return;
    *o = mypbr_denoise_opts{};
    o->iterations = 5;          // denoiser.h:39-42
    o->sigma_luminance = 4;
    o->sigma_normal = 0.1;
    o->sigma_albedo = 0.1;
}

extern "C" int mypbr_gpu_denoise(const double* radiance, const double* albedo, const double* normal,
                                 const double* variance, int32_t width, int32_t height, const mypbr_denoise_opts* opts,
                                 double* out, int on_device) {
    mypbr_dev::NvtxRange range("mypbr denoise");
    if (!radiance || !albedo || !normal || !variance || !out || width < 1 || height < 1)
        return bad("mypbr_gpu_denoise: bad argument");
    mypbr_denoise_opts o;
    mypbr_denoise_opts_init(&o);
    if (opts)
        o = *opts;
    if (o.iterations < 0 || o.iterations > 16 || !(o.sigma_normal > 0) || !(o.sigma_albedo > 0))
        return bad("mypbr_gpu_denoise: iterations must be in [0, 16] and the sigmas positive");
    size_t n = size_t(width) * height;
    if (n > (size_t(1) << 30))
        return bad("mypbr_gpu_denoise: image too large");
    int dev = 0;
    MYPBR_CUDA(cudaGetDevice(&dev));
    int sms = 1;
    MYPBR_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    Buf bL0, bL1, bA, bN, bBV, din[4], dout;
    MYPBR_CUDA(cudaMalloc(&bL0.p, n * sizeof(float4)));
    MYPBR_CUDA(cudaMalloc(&bL1.p, n * sizeof(float4)));
    MYPBR_CUDA(cudaMalloc(&bA.p, n * sizeof(float4)));
    MYPBR_CUDA(cudaMalloc(&bN.p, n * sizeof(float4)));
    MYPBR_CUDA(cudaMalloc(&bBV.p, n * sizeof(float)));
    const double* in[4] = {radiance, albedo, normal, variance};
    double* dst = out;
    if (!on_device) {
        size_t sizes[4] = {3 * n, 3 * n, 3 * n, n};
        for (int k = 0; k < 4; k++) {
            MYPBR_CUDA(cudaMalloc(&din[k].p, sizes[k] * sizeof(double)));
            MYPBR_CUDA(cudaMemcpy(din[k].p, in[k], sizes[k] * sizeof(double), cudaMemcpyHostToDevice));
            in[k] = static_cast<const double*>(din[k].p);
        }
        MYPBR_CUDA(cudaMalloc(&dout.p, 3 * n * sizeof(double)));
        dst = static_cast<double*>(dout.p);
    }
    float4* L0 = static_cast<float4*>(bL0.p);
    float4* L1 = static_cast<float4*>(bL1.p);
    float4* A = static_cast<float4*>(bA.p);
    float4* N = static_cast<float4*>(bN.p);
    float* BV = static_cast<float*>(bBV.p);
    int blocks = int(std::min<size_t>((n + 255) / 256, size_t(sms) * 16));
    k_dn_prepare<<<blocks, 256>>>(in[0], in[1], in[2], in[3], int(n), L0, A, N);
    k_dn_fireflies<<<blocks, 256>>>(L0, L1, width, height);
    float4* cur = L1;
    float4* nxt = L0;
    float inv_n = float(1.0 / (o.sigma_normal * o.sigma_normal)), inv_a = float(1.0 / (o.sigma_albedo * o.sigma_albedo));
    for (int it = 0; it < o.iterations; it++) {
        int step = 1 << it;
        k_dn_blur<<<blocks, 256>>>(cur, BV, width, height);
        // lattice of each phase: ceil(width / step) points wide (at most)
        int lw = (width + step - 1) / step, lh = (height + step - 1) / step;
        int tx = (lw + kTile - 1) / kTile, ty = (lh + kTile - 1) / kTile;
        dim3 grid(unsigned(tx * step), unsigned(ty * step));
        k_dn_atrous<<<grid, dim3(kTile, kTile)>>>(cur, BV, A, N, nxt, width, height, step, float(o.sigma_luminance),
                                                  inv_n, inv_a);
        std::swap(cur, nxt);
    }
    k_dn_finish<<<blocks, 256>>>(cur, in[1], dst, int(n));
    MYPBR_CUDA(cudaGetLastError());
    if (!on_device)
        MYPBR_CUDA(cudaMemcpy(out, dst, 3 * n * sizeof(double), cudaMemcpyDeviceToHost));
    else
        MYPBR_CUDA(cudaDeviceSynchronize());
    return MYPBR_OK;
}
