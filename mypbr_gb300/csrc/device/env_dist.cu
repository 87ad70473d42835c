// The environment's sampling distribution built on the device
// (environment.h:147-176 builds its CDFs on the host): per-texel weights
// luminance x sin(theta) (rows by sin(theta) alone for a black sky,
// environment.h:302-309), the per-texel pdf table, and an alias table.
//
// The alias table comes from the sweep of the alias method restated with
// prefix sums so that every entry is computed independently: with q = n p
// (mean 1), "light" entries (q < 1) in index order have deficits 1 - q and
// "heavy" ones excesses q - 1, laid end to end on two lines (exclusive
// prefix sums D and E). A sequential sweep hands light i to the heavy entry
// active when i is reached: the j with E_j <= D_i < E_j+1. Heavy j runs out
// (falls below 1) at the first light whose cumulative deficit C_i = D_i + d_i
// passes E_j+1; it keeps 1 - (C_i - E_j+1) and hands the rest to j + 1, and
// is never used up if no C_i passes E_j+1. Each entry's probability and alias
// are therefore binary searches in C or E, and the table holds exactly the
// distribution p (its implied per-entry mass is checked against p by the
// tests). Prefix sums in FP64 (CUB scans); partitions by a flag scan.
#include <cub/cub.cuh>

#include <cmath>
#include <string>
#include <vector>

#include "gpu_scene.h"

namespace mypbr_dev {
namespace {

template <class T>
struct Scratch {
    T* p = nullptr;
    ~Scratch() {
        if (p)
            cudaFree(p);
    }
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)); }
};

constexpr double kPiD = 3.1415926535897932385;

// weights and their row-free total (FP64), one thread per texel
__global__ void k_env_weights(const float* rgb, int w, int h, int black, double* weight) {
    size_t n = size_t(w) * h;
    for (size_t k = blockIdx.x * size_t(blockDim.x) + threadIdx.x; k < n; k += size_t(gridDim.x) * blockDim.x) {
        int j = int(k / size_t(w));
        double st = sin(kPiD * (j + 0.5) / h);
        if (black) {
            weight[k] = st;
        } else {
            const float* p = rgb + 3 * k;
            double l = __dadd_rn(__dadd_rn(__dmul_rn(0.2126, double(p[0])), __dmul_rn(0.7152, double(p[1]))),
                                 __dmul_rn(0.0722, double(p[2])));
            weight[k] = fmax(__dmul_rn(l, st), 0.0);
        }
    }
}

// q = n p, the pdf table (p w h = p n) and the light / heavy flags
__global__ void k_env_scale(const double* weight, const double* total, size_t n, double* q, float* texel_pdf,
                            int* light) {
    double inv = 1.0 / *total;
    for (size_t k = blockIdx.x * size_t(blockDim.x) + threadIdx.x; k < n; k += size_t(gridDim.x) * blockDim.x) {
        double p = weight[k] * inv;
        q[k] = p * double(n);
        texel_pdf[k] = float(p * double(n));
        light[k] = q[k] < 1.0 ? 1 : 0;
    }
}

// stable split of the indices: lights first (in index order), heavies after;
// deficit / excess of each in its list's order
__global__ void k_env_split(const double* q, const int* light, const int* light_pos, size_t n, int n_light,
                            uint32_t* order, double* amount) {
    for (size_t k = blockIdx.x * size_t(blockDim.x) + threadIdx.x; k < n; k += size_t(gridDim.x) * blockDim.x) {
        size_t slot = light[k] ? size_t(light_pos[k]) : size_t(n_light) + (k - size_t(light_pos[k]));
        order[slot] = uint32_t(k);
        amount[slot] = light[k] ? 1.0 - q[k] : q[k] - 1.0;
    }
}

// first index in [lo, hi) of a sorted array whose value is > x (upper bound)
__device__ size_t upper(const double* a, size_t lo, size_t hi, double x) {
    while (lo < hi) {
        size_t mid = lo + (hi - lo) / 2;
        if (a[mid] <= x)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// prefix: exclusive sums of amount (lights' deficits D in [0, L), heavies'
// excesses E - D_total in [L, n)); entries written as (probability, alias)
__global__ void k_env_alias(const double* q, const uint32_t* order, const double* amount, const double* prefix,
                            size_t n, size_t n_light, float2* alias) {
    size_t n_heavy = n - n_light;
    double d_total = n_light ? prefix[n_light - 1] + amount[n_light - 1] : 0.0;
    for (size_t s = blockIdx.x * size_t(blockDim.x) + threadIdx.x; s < n; s += size_t(gridDim.x) * blockDim.x) {
        uint32_t k = order[s];
        if (n_heavy == 0) {  // rounding left no entry at or above the mean
            alias[k] = make_float2(1.0f, __int_as_float(int(k)));
            continue;
        }
        if (s < n_light) {
            // the heavy entry whose excess range holds D_i: E_j <= D_i < E_j+1
            double D = prefix[s];
            size_t j = upper(prefix, n_light, n, D + d_total);  // E stored offset by d_total
            j = j > n_light ? j - 1 : n_light;
            alias[k] = make_float2(float(q[k]), __int_as_float(int(order[j])));
        } else {
            size_t j = s;
            if (j + 1 == n) {  // the last heavy entry is never used up (up to rounding)
                alias[k] = make_float2(1.0f, __int_as_float(int(k)));
                continue;
            }
            double e_next = prefix[j + 1] - d_total;  // E_j+1
            // the first light whose cumulative deficit C_i = D_i + d_i passes E_j+1
            size_t lo = 0, hi = n_light;
            while (lo < hi) {
                size_t mid = lo + (hi - lo) / 2;
                if (prefix[mid] + amount[mid] <= e_next)
                    lo = mid + 1;
                else
                    hi = mid;
            }
            if (lo == n_light) {
                alias[k] = make_float2(1.0f, __int_as_float(int(k)));
            } else {
                double keep = 1.0 - ((prefix[lo] + amount[lo]) - e_next);
                keep = fmin(fmax(keep, 0.0), 1.0);
                alias[k] = make_float2(float(keep), __int_as_float(int(order[j + 1])));
            }
        }
    }
}

}  // namespace

// rgb: device, w * h * 3 floats. Writes device texel_pdf (n floats) and
// alias (n float2: probability, alias index bits).
int build_env_distribution(const float* rgb, int w, int h, float* texel_pdf, float2* alias, cudaStream_t st) {
    NvtxRange range("mypbr environment tables");
    size_t n = size_t(w) * h;
    if (n == 0)
        return MYPBR_OK;
    Scratch<double> weight, q, amount, prefix, total;
    Scratch<int> light, light_pos;
    Scratch<uint32_t> order;
    Scratch<unsigned char> temp;
    MYPBR_CUDA(weight.alloc(n));
    MYPBR_CUDA(q.alloc(n));
    MYPBR_CUDA(amount.alloc(n));
    MYPBR_CUDA(prefix.alloc(n));
    MYPBR_CUDA(total.alloc(1));
    MYPBR_CUDA(light.alloc(n + 1));
    MYPBR_CUDA(light_pos.alloc(n + 1));
    MYPBR_CUDA(order.alloc(n));
    size_t tb = 0, need = 0;
    cub::DeviceReduce::Sum(nullptr, need, weight.p, total.p, n, st);
    tb = std::max(tb, need);
    cub::DeviceScan::ExclusiveSum(nullptr, need, light.p, light_pos.p, n + 1, st);
    tb = std::max(tb, need);
    cub::DeviceScan::ExclusiveSum(nullptr, need, amount.p, prefix.p, n, st);
    tb = std::max(tb, need);
    MYPBR_CUDA(temp.alloc(tb));
    int grid = 4 * 152, block = 256;
    k_env_weights<<<grid, block, 0, st>>>(rgb, w, h, 0, weight.p);
    MYPBR_CUDA(cub::DeviceReduce::Sum(temp.p, tb, weight.p, total.p, n, st));
    double sum = 0;
    MYPBR_CUDA(cudaMemcpyAsync(&sum, total.p, sizeof sum, cudaMemcpyDeviceToHost, st));
    MYPBR_CUDA(cudaStreamSynchronize(st));
    if (!(sum > 0)) {  // a black sky: rows by sin(theta)
        k_env_weights<<<grid, block, 0, st>>>(rgb, w, h, 1, weight.p);
        MYPBR_CUDA(cub::DeviceReduce::Sum(temp.p, tb, weight.p, total.p, n, st));
    }
    k_env_scale<<<grid, block, 0, st>>>(weight.p, total.p, n, q.p, texel_pdf, light.p);
    MYPBR_CUDA(cudaMemsetAsync(light.p + n, 0, sizeof(int), st));
    MYPBR_CUDA(cub::DeviceScan::ExclusiveSum(temp.p, tb, light.p, light_pos.p, n + 1, st));
    int n_light = 0;
    MYPBR_CUDA(cudaMemcpyAsync(&n_light, light_pos.p + n, sizeof n_light, cudaMemcpyDeviceToHost, st));
    MYPBR_CUDA(cudaStreamSynchronize(st));
    k_env_split<<<grid, block, 0, st>>>(q.p, light.p, light_pos.p, n, n_light, order.p, amount.p);
    // one scan over both lists: the heavies' prefix is offset by the lights' total
    MYPBR_CUDA(cub::DeviceScan::ExclusiveSum(temp.p, tb, amount.p, prefix.p, n, st));
    k_env_alias<<<grid, block, 0, st>>>(q.p, order.p, amount.p, prefix.p, n, size_t(n_light), alias);
    MYPBR_CUDA(cudaGetLastError());
    MYPBR_CUDA(cudaStreamSynchronize(st));
    return MYPBR_OK;
}

}  // namespace mypbr_dev

// The tables for a caller's pixels (host arrays), built on the device
// (on_gpu) or on the host, for the parity tests and for tools.
extern "C" int mypbr_env_distribution(const float* rgb, int32_t width, int32_t height, float* texel_pdf,
                                      float* alias, int on_gpu) {
    using namespace mypbr_dev;
    if (!rgb || !texel_pdf || !alias || width <= 0 || height <= 0) {
        set_error_message("mypbr_env_distribution: pixels, outputs and a positive size are required");
        return MYPBR_ERR_INVALID_ARGUMENT;
    }
    size_t n = size_t(width) * height;
    if (!on_gpu) {
        env_distribution_host(rgb, width, height, texel_pdf, reinterpret_cast<float2*>(alias));
        return MYPBR_OK;
    }
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        set_error_message("mypbr_env_distribution: no CUDA device");
        return MYPBR_ERR_NO_DEVICE;
    }
    Scratch<float> d_rgb, d_pdf;
    Scratch<float2> d_alias;
    MYPBR_CUDA(d_rgb.alloc(n * 3));
    MYPBR_CUDA(d_pdf.alloc(n));
    MYPBR_CUDA(d_alias.alloc(n));
    MYPBR_CUDA(cudaMemcpy(d_rgb.p, rgb, n * 3 * sizeof(float), cudaMemcpyHostToDevice));
    int s = build_env_distribution(d_rgb.p, width, height, d_pdf.p, d_alias.p, nullptr);
    if (s != MYPBR_OK)
        return s;
    MYPBR_CUDA(cudaMemcpy(texel_pdf, d_pdf.p, n * sizeof(float), cudaMemcpyDeviceToHost));
    MYPBR_CUDA(cudaMemcpy(alias, d_alias.p, n * sizeof(float2), cudaMemcpyDeviceToHost));
    return MYPBR_OK;
}
