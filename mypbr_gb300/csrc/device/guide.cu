// Training of the guiding network on the tensor cores, its Adam optimiser,
// and pointwise entry points that the tests compare with the CPU oracle.
//
// One training step: k_guide_prep, twice, sums the sample weights of a batch
// drawn from the recorded vertices (their mean, then the sum with each weight
// capped at a multiple of it); k_guide_train runs forward and backward for
// tiles of 128 samples (groups of 128 threads, a thread per sample, sharing
// the CTA's resident weights) and adds the weight gradients into per-CTA
// FP32 partial sums; k_guide_adam sums the partials, updates the FP32 master
// weights and rewrites the BF16 copies the kernels read.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "dev_shading.cuh"
#include "gpu_scene.h"

namespace mypbr_dev {

namespace {

MYPBR_DEV uint32_t hash_u32(uint32_t a, uint32_t b) {
    uint64_t z = mix64((uint64_t(a) << 32) ^ b ^ 0x5bd1e995ull);
    return uint32_t(z ^ (z >> 32));
}

// Loss weight of a recorded vertex: luminance of (f cos / pdf) * L_i, with
// L_i = (final radiance - radiance at the next vertex) / throughput there.
MYPBR_DEV float record_weight(const GuideRecords& R, uint32_t r, uint32_t slot) {
    float4 f = R.fac[r], mk = R.mark[r], bn = R.bnext[r], fin = R.fin[slot];
    float li_r = bn.x > 0.0f ? (fin.x - mk.x) / bn.x : 0.0f;
    float li_g = bn.y > 0.0f ? (fin.y - mk.y) / bn.y : 0.0f;
    float li_b = bn.z > 0.0f ? (fin.z - mk.z) / bn.z : 0.0f;
    float c = 0.2126f * f.x * li_r + 0.7152f * f.y * li_g + 0.0722f * f.z * li_b;
    return isfinite(c) ? fminf(fmaxf(c, 0.0f), 1e6f) : 0.0f;
}

// Training rows drawn from the recorded vertices (uniformly, by a hash of
// the step and the row). A record's weight can be capped at a multiple of
// the batch's mean weight (mypbr_guide_schedule's weight_cap): a rare path
// that carries a very large contribution (a caustic, a glint of the sun)
// would otherwise take most of a batch's loss and pull a lobe toward its one
// direction. The cap shapes only what the network is fitted to; the
// renderer's estimator stays unbiased whatever it learns.
struct RecordSource {
    GuideRecords R;
    uint32_t step;
    const float* stats;  // [1]: sum of the batch's capped weights; [2]: the rows drawn; [3]: the uncapped sum
    float cap;           // the cap as a multiple of the batch's mean weight; 0: none
    // The cap on one record's weight: `cap` x the batch's mean uncapped weight.
    MYPBR_DEV float weight_cap() const { return cap > 0.0f ? cap * stats[3] / fmaxf(stats[2], 1.0f) : 3.0e38f; }
    MYPBR_DEV bool pick(long long i, uint32_t& r) const {
        uint32_t n = *R.count;
        if (i < 0 || n == 0)
            return false;
        r = R.list[hash_u32(step, uint32_t(i)) % n];
        return true;
    }
    MYPBR_DEV void fill(long long i, __nv_bfloat16* A, int row) const {
        uint32_t r;
        if (!pick(i, r)) {
            guide_encode_row(nullptr, A, row);
            return;
        }
        float4 a = R.in0[r], b = R.in1[r];
        float s[7] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z};
        guide_encode_row(s, A, row);
    }
    MYPBR_DEV float dout(long long i, const float* v, float* g) const {
#pragma unroll
        for (int k = 0; k < kGuideOut; k++)
            g[k] = 0.0f;
        uint32_t r;
        float total = stats[1];
        if (!pick(i, r) || !(total > 0.0f))
            return 0.0f;
        float c = fminf(record_weight(R, r, r / uint32_t(R.depth)), weight_cap()) / total;
        if (c <= 0.0f)
            return 0.0f;
        float4 d = R.dir[r];
        return guide_loss_grad(v, f3(d.x, d.y, d.z), c, g);
    }
};

// Rows given by the caller: encoded inputs and output gradients (tests).
struct GivenSource {
    const float* inputs;  // n x 128
    const float* grads;   // n x 64
    struct Row {
        long long i;
    };
    MYPBR_DEV long long count(long long rows) const { return rows; }
    MYPBR_DEV void load(long long i, Row& r) const { r.i = i; }
    MYPBR_DEV void finish(Row&) const {}
    MYPBR_DEV void encode(const Row& r, __nv_bfloat16* A, int row) const { fill(r.i, A, row); }
    MYPBR_DEV void fill(long long i, __nv_bfloat16* A, int row) const {
#pragma unroll 1
        for (int b = 0; b < kGuideIn / 8; b++) {
            float v[8];
#pragma unroll
            for (int e = 0; e < 8; e++)
                v[e] = i >= 0 ? inputs[i * kGuideIn + 8 * b + e] : 0.0f;
            uint4 u;
            u.x = pack_bf16(v[0], v[1]);
            u.y = pack_bf16(v[2], v[3]);
            u.z = pack_bf16(v[4], v[5]);
            u.w = pack_bf16(v[6], v[7]);
            *reinterpret_cast<uint4*>(A + canon(row, 8 * b, kGuideIn)) = u;
        }
    }
    MYPBR_DEV float dout(long long i, const float*, float* g) const {
#pragma unroll
        for (int k = 0; k < kGuideOut; k++)
            g[k] = i >= 0 ? grads[i * kGuideOut + k] : 0.0f;
        return 0.0f;
    }
};

struct RowSink {
    float* out;  // n x 64
    template <class Row>
    MYPBR_DEV void put(long long i, const Row&, const float* v) const {
        float4* o = reinterpret_cast<float4*>(out + i * kGuideOut);
#pragma unroll
        for (int k = 0; k < kGuideOut / 4; k++)
            o[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
    }
};

// Training CTA: kTrainGroups groups of 128 threads (a thread per sample row),
// each group on its own tile of 128 samples, all sharing one resident copy
// of the weights. Shared memory: the weights (canonical [64 out][in] per
// matrix), then per group a 128 x 128 activation tile and a 128 x 64
// output-gradient tile, then the groups' mbarriers and the TMEM address.
constexpr int kTrainGroups = 2;
// (16 KB of slack after the barriers: every operand an MMA addresses lies in
// its tile, the slack keeps any layout misreading inside the allocation)
MYPBR_HD size_t train_smem(int hidden) {
    return size_t(guide_params(hidden)) * 2 + size_t(kTrainGroups) * (128 * 128 + 128 * 64) * 2 + 64 + 16384;
}
// Per group of a training CTA: the layer inputs of its current tile kept for
// the backward pass (canonical K-major, the input encoding then each hidden
// layer's activations), in global memory (L2 resident).
MYPBR_HD size_t train_scratch_per_group(int hidden) { return size_t(128) * 128 + size_t(hidden) * 128 * 64; }
MYPBR_HD size_t train_scratch_offset(int l) { return l == 0 ? 0 : size_t(128) * 128 + size_t(l - 1) * 128 * 64; }

// Copies row `row` of a canonical K-major BF16 tile with K columns from src
// to dst (K / 8 16-byte chunks, the row's own).
MYPBR_DEV void copy_row_u4(__nv_bfloat16* dst, const __nv_bfloat16* src, int row, int K) {
    for (int b = 0; b < K / 8; b++) {
        const int e = canon(row, 8 * b, K);
        *reinterpret_cast<uint4*>(dst + e) = *reinterpret_cast<const uint4*>(src + e);
    }
}

// One training step's forward and backward passes. Per layer l with input H
// (batch x in) and output gradient dZ (batch x 64), both BF16 in shared
// memory:
//   forward  Z = H W^T           (M = 128 batch, N = 64, K = in; A = H K-major,
//                                 B = W K-major)
//   dW^T = H^T dZ                (M = 128 in (rows past `in` unused), N = 64,
//                                 K = 128 batch; A = the H tile read MN-major,
//                                 B = the dZ tile read MN-major)
//   dX   = dZ W                  (M = 128 batch, N = in, K = 64; A = dZ
//                                 K-major, B = W read MN-major)
// so no transposed copy of anything is made. Each group writes its tiles'
// dW into its own FP32 partial ([out][in] per matrix; plain stores for its
// first tile, additions by the same thread for later ones, zeros if it had
// none); the Adam kernel sums the groups' partials.
template <int HIDDEN, class Src>
__global__ void __launch_bounds__(128 * kTrainGroups) k_guide_train(GuideNetView net, Src src, long long rows,
                                                                    __nv_bfloat16* scratch, float* partial,
                                                                    float* loss_sum) {
    extern __shared__ __align__(1024) uint8_t smem[];
    constexpr int P = kGuideWidth * kGuideIn + HIDDEN * kGuideWidth * kGuideWidth;
    const int group = threadIdx.x >> 7, row = threadIdx.x & 127, warp = threadIdx.x >> 5;
    __nv_bfloat16* W = reinterpret_cast<__nv_bfloat16*>(smem);
    __nv_bfloat16* A = W + P + size_t(group) * (128 * 128 + 128 * 64);  // 128 x 128
    __nv_bfloat16* DZ = A + 128 * 128;                                   // 128 x 64
    uint64_t* bars = reinterpret_cast<uint64_t*>(W + P + size_t(kTrainGroups) * (128 * 128 + 128 * 64));
    uint64_t* bar = bars + group;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + kTrainGroups);
    float* part = partial + (size_t(blockIdx.x) * kTrainGroups + group) * P;
    __nv_bfloat16* scr = scratch + (size_t(blockIdx.x) * kTrainGroups + group) * train_scratch_per_group(HIDDEN);
    {
        const uint4* g = reinterpret_cast<const uint4*>(net.w);
        uint4* w = reinterpret_cast<uint4*>(W);
        for (int k = threadIdx.x; k < P / 8; k += blockDim.x)
            w[k] = g[k];
    }
    if (warp == 0)
        tc::tmem_alloc(tmem_slot, 128 * kTrainGroups);
    if (row == 0)
        tc::bar_init(bar, 1);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t t_acc = *tmem_slot + uint32_t(128 * group), t_dw = t_acc + 64;
    const int bar_id = 1 + group;  // named barrier 0 is __syncthreads
    uint32_t phase = 0;
    bool failed = false, first = true;
    float loss_acc = 0.0f;
    const long long tiles = (rows + 127) / 128;
    // Every thread of the group waits for the MMAs of the group's issuing
    // thread; false (error recorded) on a timeout.
    auto wait_mma = [&]() {
        bool ok = tc::bar_wait(bar, phase);
        phase ^= 1;
        if (tc::group_sync_or(bar_id, 128, !ok)) {
            if (row == 0)
                atomicCAS(net.error, 0, 3);
            tc::bar_wait(bar, phase ^ 1);  // once more, bounded, for the MMAs in flight
            return false;
        }
        tc::fence_after();
        return true;
    };
    for (long long tile = (long long)blockIdx.x * kTrainGroups + group; tile < tiles && !failed;
         tile += (long long)gridDim.x * kTrainGroups) {
        const long long i = tile * 128 + row;
        const long long src_i = i < rows ? i : -1;
        src.fill(src_i, A, row);
        copy_row_u4(scr, A, row, kGuideIn);  // the encoding, for layer 0's weight gradient
        uint32_t mask[2 * HIDDEN + 2];
        float dz[64];
        // ---- forward
#pragma unroll 1
        for (int l = 0; l <= HIDDEN; l++) {
            const int K = guide_in(l);
            tc::fence_smem();
            tc::group_sync(bar_id, 128);
            if (row == 0) {
                tc::fence_after();
                const uint32_t a0 = tc::smem_u32(A), b0 = tc::smem_u32(W + guide_offset(l));
                const uint32_t idesc = tc::idesc_bf16(128, 64);
                for (int s = 0; s < K / 16; s++)
                    tc::mma(t_acc, tc::desc(a0 + 256 * s, 128, K * 16), tc::desc(b0 + 256 * s, 128, K * 16), idesc,
                            s > 0);
                tc::commit(bar);
            }
            if (!wait_mma()) {
                failed = true;
                break;
            }
            float v[64];
            tc::tmem_row64(t_acc, 0, v);
            tc::fence_before();
            if (l < HIDDEN) {
                uint32_t m0 = 0, m1 = 0;
#pragma unroll
                for (int k = 0; k < 32; k++) {
                    m0 |= v[k] > 0.0f ? (1u << k) : 0u;
                    m1 |= v[k + 32] > 0.0f ? (1u << k) : 0u;
                }
                mask[2 * l] = m0;
                mask[2 * l + 1] = m1;
                store_row_bf16_relu(A, row, v);  // the next layer's input, K = 64
                if (l + 1 < HIDDEN)              // the last one stays in A for the backward pass
                    copy_row_u4(scr + train_scratch_offset(l + 1), A, row, kGuideWidth);
            } else {
                loss_acc += src.dout(src_i, v, dz);
            }
        }
        if (failed)
            break;
        // ---- backward
        uint4 pre[8];  // the next layer's input row (its first 64 values), read while this layer's MMAs run
#pragma unroll 1
        for (int l = HIDDEN; l >= 0; l--) {
            const int in = guide_in(l);
            store_row_bf16(DZ, row, kGuideWidth, 0, dz);
            if (l < HIDDEN) {  // this layer's input, back from the scratch
#pragma unroll
                for (int b = 0; b < 8; b++)
                    *reinterpret_cast<uint4*>(A + canon(row, 8 * b, in)) = pre[b];
                for (int b = 8; b < in / 8; b++) {
                    const int e = canon(row, 8 * b, in);
                    *reinterpret_cast<uint4*>(A + e) =
                        *reinterpret_cast<const uint4*>(scr + train_scratch_offset(l) + e);
                }
            }
            tc::fence_smem();
            tc::group_sync(bar_id, 128);
            if (row == 0) {
                tc::fence_after();
                const uint32_t h0 = tc::smem_u32(A), z0 = tc::smem_u32(DZ), w0 = tc::smem_u32(W + guide_offset(l));
                // dW^T: K = batch in steps of 16 rows (two row groups of each tile)
                const uint32_t id_w = tc::idesc_bf16_mn(128, 64, true, true);
                for (int s = 0; s < 8; s++)
                    tc::mma(t_dw, tc::desc(h0 + uint32_t(s) * 32u * uint32_t(in), uint32_t(in) * 16u, 128),
                            tc::desc(z0 + uint32_t(s) * 2048u, 1024, 128), id_w, s > 0);
                if (l > 0) {  // dX: K = the 64 outputs in steps of 16 (two row groups of W)
                    const uint32_t id_x = tc::idesc_bf16_mn(128, 64, false, true);
                    for (int s = 0; s < 4; s++)
                        tc::mma(t_acc, tc::desc(z0 + 256u * uint32_t(s), 128, 1024),
                                tc::desc(w0 + uint32_t(s) * 32u * uint32_t(in), uint32_t(in) * 16u, 128), id_x,
                                s > 0);
                }
                tc::commit(bar);
            }
            if (l > 0) {
                const int nin = guide_in(l - 1);
                const __nv_bfloat16* src_row = scr + train_scratch_offset(l - 1);
#pragma unroll
                for (int b = 0; b < 8; b++)
                    pre[b] = *reinterpret_cast<const uint4*>(src_row + canon(row, 8 * b, nin));
            }
            if (!wait_mma()) {
                failed = true;
                break;
            }
            float gw[64];
            tc::tmem_row64(t_dw, 0, gw);  // lane = input feature `row`
            if (row < in) {  // element (j, row) of the [out][in] matrix: a warp writes 32 neighbours
                float* gp = part + guide_offset(l) + row;
                if (first) {
#pragma unroll 8
                    for (int j = 0; j < 64; j++)
                        gp[j * in] = gw[j];
                } else {
#pragma unroll 8
                    for (int j = 0; j < 64; j++)
                        gp[j * in] += gw[j];
                }
            }
            if (l > 0) {
                float dx[64];
                tc::tmem_row64(t_acc, 0, dx);
                const uint32_t m0 = mask[2 * (l - 1)], m1 = mask[2 * (l - 1) + 1];
#pragma unroll
                for (int k = 0; k < 32; k++) {
                    dz[k] = (m0 >> k) & 1u ? dx[k] : 0.0f;
                    dz[k + 32] = (m1 >> k) & 1u ? dx[k + 32] : 0.0f;
                }
            }
            tc::fence_before();
        }
        first = false;
    }
    if (first)  // no tile for this group: its partial is zero
        for (int k = row; k < P / 4; k += 128)
            reinterpret_cast<float4*>(part)[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int o = 16; o > 0; o >>= 1)
        loss_acc += __shfl_xor_sync(0xffffffffu, loss_acc, o);
    if ((threadIdx.x & 31) == 0 && loss_sum && loss_acc != 0.0f)
        atomicAdd(loss_sum, loss_acc);
    tc::fence_before();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after();
        tc::tmem_free(*tmem_slot, 128 * kTrainGroups);
    }
}

// Sums the training groups' partial gradients into grad (test entry points).
__global__ void k_guide_sum_partials(const float* partial, int ctas, int params, float* grad) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < params; p += gridDim.x * blockDim.x) {
        float acc = 0.0f;
        for (int c = 0; c < ctas; c++)
            acc += partial[size_t(c) * params + p];
        grad[p] = acc;
    }
}

// The batch's weights: pass 0 sums them uncapped (stats[3]) and counts the
// rows drawn (stats[2]); pass 1 sums them capped (stats[1], which normalises
// the loss so the weights used sum to 1).
__global__ void k_guide_prep(RecordSource src, long long rows, float* stats, int pass) {
    const float cap = pass == 1 ? src.weight_cap() : 0.0f;
    float acc = 0.0f, drawn = 0.0f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < rows;
         i += (long long)gridDim.x * blockDim.x) {
        uint32_t r;
        if (src.pick(i, r)) {
            const float w = record_weight(src.R, r, r / uint32_t(src.R.depth));
            acc += pass == 1 ? fminf(w, cap) : w;
            drawn += 1.0f;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        acc += __shfl_xor_sync(0xffffffffu, acc, o);
        drawn += __shfl_xor_sync(0xffffffffu, drawn, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (acc != 0.0f)
            atomicAdd(stats + (pass == 1 ? 1 : 3), acc);
        if (pass == 0 && drawn != 0.0f)
            atomicAdd(stats + 2, drawn);
    }
}

MYPBR_DEV void param_coords(int p, int& l, int& j, int& t, int& in) {
    if (p < kGuideWidth * kGuideIn) {
        l = 0;
        in = kGuideIn;
    } else {
        l = 1 + (p - kGuideWidth * kGuideIn) / (kGuideWidth * kGuideWidth);
        in = kGuideWidth;
    }
    int local = p - guide_offset(l);
    j = local / in;
    t = local % in;
}

// Adam (Kingma and Ba 2015) on the FP32 masters, then the BF16 copies.
// lr == 0 only republishes the copies.
// The gradient is the sum of the training groups' partials.
__global__ void k_guide_adam(float* master, float* m, float* v, const float* partial, int ctas, __nv_bfloat16* w,
                             __nv_bfloat16* wt, int params, float lr, float b1t, float b2t) {
    const float b1 = 0.9f, b2 = 0.99f, eps = 1e-8f;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < params; p += gridDim.x * blockDim.x) {
        float x = master[p];
        if (lr > 0.0f) {
            float g = 0.0f;
#pragma unroll 8
            for (int c = 0; c < ctas; c++)
                g += partial[size_t(c) * params + p];
            g = isfinite(g) ? g : 0.0f;
            float mm = b1 * m[p] + (1.0f - b1) * g;
            float vv = b2 * v[p] + (1.0f - b2) * g * g;
            m[p] = mm;
            v[p] = vv;
            x -= lr * (mm / (1.0f - b1t)) / (sqrtf(vv / (1.0f - b2t)) + eps);
            master[p] = x;
        }
        int l, j, t, in;
        param_coords(p, l, j, t, in);
        __nv_bfloat16 h = __float2bfloat16_rn(x);
        w[guide_offset(l) + canon(j, t, in)] = h;
        wt[guide_offset(l) + canon(t, j, kGuideWidth)] = h;
    }
}

__global__ void k_loss_test(const float* raw, const float* dirs, const float* c, long long n, float* grad,
                            float* loss) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float g[kGuideOut];
        float3 w = f3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]);
        loss[i] = guide_loss_grad(raw + i * kGuideOut, w, c[i], g);
        for (int k = 0; k < kGuideOut; k++)
            grad[i * kGuideOut + k] = k < kGuideUsed ? g[k] : 0.0f;
    }
}

__global__ void k_mixture_test(const float* raw, const float* u, const float* dirs, long long n, float* samples,
                               float* pdf_sample, float* pdf_dir) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        GuidePacked pk;
        guide_pack(raw + i * kGuideOut, pk);
        GuideMix m;
        guide_unpack(pk, m);
        float3 s = guide_sample(m, u[3 * i], u[3 * i + 1], u[3 * i + 2]);
        samples[3 * i] = s.x;
        samples[3 * i + 1] = s.y;
        samples[3 * i + 2] = s.z;
        pdf_sample[i] = guide_pdf(m, s);
        pdf_dir[i] = guide_pdf(m, normalize(f3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2])));
    }
}

template <class Kernel>
int set_smem(Kernel k, size_t bytes) {
    MYPBR_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes)));
    return MYPBR_OK;
}

template <int H, class Src>
int launch_train(GuideNetView net, Src src, long long rows, int ctas, __nv_bfloat16* scratch, float* partial,
                 float* loss, cudaStream_t st) {
    auto k = k_guide_train<H, Src>;
    const size_t smem = train_smem(H);
    int rc = set_smem(k, smem);
    if (rc != MYPBR_OK)
        return rc;
    k<<<ctas, 128 * kTrainGroups, smem, st>>>(net, src, rows, scratch, partial, loss);
    MYPBR_CUDA(cudaGetLastError());
    return MYPBR_OK;
}

// `ctas` training CTAs (each kTrainGroups tiles at a time); scratch holds
// ctas * kTrainGroups * train_scratch_per_group(hidden) BF16 values and
// partial ctas * kTrainGroups * params floats.
template <class Src>
int train_dispatch(int hidden, GuideNetView net, Src src, long long rows, int ctas, __nv_bfloat16* scratch,
                   float* partial, float* loss, cudaStream_t st) {
    switch (hidden) {
        case 2: return launch_train<2>(net, src, rows, ctas, scratch, partial, loss, st);
        case 4: return launch_train<4>(net, src, rows, ctas, scratch, partial, loss, st);
        case 8: return launch_train<8>(net, src, rows, ctas, scratch, partial, loss, st);
        default:
            set_error_message("guiding networks have 2, 4 or 8 hidden layers");
            return MYPBR_ERR_UNSUPPORTED;
    }
}

// Seeded He-uniform initial weights (the output layer scaled by 1/2).
std::vector<float> initial_weights(int hidden, unsigned long long seed) {
    std::vector<float> w(size_t(guide_params(hidden)));
    uint64_t state = seed * 0x9e3779b97f4a7c15ull + 0x632be59bd9b4e019ull;
    auto uniform = [&]() {
        state = state * 6364136223846793005ull + 1442695040888963407ull;
        return double(state >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int l = 0; l <= hidden; l++) {
        int in = guide_in(l);
        double b = std::sqrt(6.0 / in) * (l == hidden ? 0.5 : 1.0);
        for (int k = 0; k < kGuideWidth * in; k++)
            w[size_t(guide_offset(l) + k)] = float((2 * uniform() - 1) * b);
    }
    return w;
}

template <typename T>
int dalloc(T*& p, size_t n) {
    MYPBR_CUDA(cudaMalloc(&p, n * sizeof(T)));
    return MYPBR_OK;
}

// A network for the test entry points: weights given by the caller.
struct TempNet {
    GuideState g;
    int* err = nullptr;
    ~TempNet() {
        release_guide(g);
        cudaFree(err);
    }
};

int temp_net(TempNet& T, int hidden, const float* weights) {
    if (hidden != 2 && hidden != 4 && hidden != 8) {
        set_error_message("guiding networks have 2, 4 or 8 hidden layers");
        return MYPBR_ERR_INVALID_ARGUMENT;
    }
    GuideState& g = T.g;
    g.hidden = hidden;
    g.params = guide_params(hidden);
    size_t P = size_t(g.params);
    int rc;
    if ((rc = dalloc(g.w, P)) || (rc = dalloc(g.wt, P)) || (rc = dalloc(g.master, P)) || (rc = dalloc(g.m, P)) ||
        (rc = dalloc(g.v, P)) || (rc = dalloc(g.grad, P)) || (rc = dalloc(T.err, 1)))
        return rc;
    MYPBR_CUDA(cudaMemcpy(g.master, weights, P * 4, cudaMemcpyHostToDevice));
    MYPBR_CUDA(cudaMemset(g.grad, 0, P * 4));
    MYPBR_CUDA(cudaMemset(T.err, 0, 4));
    k_guide_adam<<<64, 256>>>(g.master, g.m, g.v, nullptr, 0, g.w, g.wt, g.params, 0.0f, 0.0f, 0.0f);
    MYPBR_CUDA(cudaGetLastError());
    return MYPBR_OK;
}

GuideNetView view_of(GuideState& g, int* err) { return GuideNetView{g.hidden, g.w, g.wt, g.grad, err}; }

int read_error(int* err) {
    int e = 0;
    MYPBR_CUDA(cudaMemcpy(&e, err, 4, cudaMemcpyDeviceToHost));
    if (e != 0) {
        set_error_message("a tensor-core wait of the guiding network timed out");
        return MYPBR_ERR_DEVICE_TIMEOUT;
    }
    return MYPBR_OK;
}

// One CTA waits, through the same bounded wait the tensor-core kernels use,
// on an mbarrier phase nothing completes: after the wait's limit (about a
// second of clocks) it records the timeout in the error word and returns.
__global__ void k_wait_probe(int* err) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0)
        tc::bar_init(&bar, 1);
    __syncthreads();
    if (threadIdx.x == 0 && !tc::bar_wait(&bar, 0))
        atomicCAS(err, 0, 3);
}

}  // namespace

int release_guide(GuideState& g) {
    void* ptrs[] = {g.w, g.wt, g.master, g.m, g.v, g.grad, g.stats, g.scratch, g.partial, g.rec.in0, g.rec.in1, g.rec.dir,
                    g.rec.fac, g.rec.mark, g.rec.bnext, g.rec.fin, g.rec.list, g.rec.count, g.packed};
    for (void* p : ptrs)
        if (p)
            cudaFree(p);
    g = GuideState{};
    return MYPBR_OK;
}

// The position encoding's box: the scene's bounding box, until a fresh
// network's first recorded wave narrows it (guide_fit_box).
void set_scene_box(mypbr_gpu_scene* G) {
    GuideState& g = G->guide;
    float3 lo = G->box_lo, hi = G->box_hi;
    g.box_lo = lo;
    g.box_inv = f3(1.0f / fmaxf(hi.x - lo.x, 1e-6f), 1.0f / fmaxf(hi.y - lo.y, 1e-6f), 1.0f / fmaxf(hi.z - lo.z, 1e-6f));
    g.box_fitted = false;
    g.box_version++;
}

constexpr int kBoxBins = 1024;

// histograms of the recorded vertices' positions (in the current box), per axis
__global__ void k_guide_box_histogram(GuideRecords rec, uint32_t* hist) {
    uint32_t n = min(*rec.count, rec.capacity);
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        float4 s = rec.in0[rec.list[k]];
        atomicAdd(&hist[0 * kBoxBins + min(int(s.x * kBoxBins), kBoxBins - 1)], 1u);
        atomicAdd(&hist[1 * kBoxBins + min(int(s.y * kBoxBins), kBoxBins - 1)], 1u);
        atomicAdd(&hist[2 * kBoxBins + min(int(s.z * kBoxBins), kBoxBins - 1)], 1u);
    }
}

// the records' positions re-expressed in the sub-box [a, b] of the current one
__global__ void k_guide_box_rescale(GuideRecords rec, float3 a, float3 inv_width) {
    uint32_t n = min(*rec.count, rec.capacity);
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        uint32_t r = rec.list[k];
        float4 s = rec.in0[r];
        s.x = clampf((s.x - a.x) * inv_width.x, 0.0f, 1.0f);
        s.y = clampf((s.y - a.y) * inv_width.y, 0.0f, 1.0f);
        s.z = clampf((s.z - a.z) * inv_width.z, 0.0f, 1.0f);
        rec.in0[r] = s;
    }
}

int guide_fit_box(mypbr_gpu_scene* G, cudaStream_t st) {
    GuideState& g = G->guide;
    if (g.box_fitted)
        return MYPBR_OK;
    g.box_fitted = true;
    uint32_t* hist = nullptr;
    MYPBR_CUDA(cudaMalloc(&hist, 3 * kBoxBins * sizeof(uint32_t)));
    std::vector<uint32_t> h(3 * kBoxBins);
    int rc = MYPBR_OK;
    if (cudaMemsetAsync(hist, 0, 3 * kBoxBins * sizeof(uint32_t), st) != cudaSuccess)
        rc = cuda_fail(cudaGetLastError(), "guide_fit_box");
    if (rc == MYPBR_OK) {
        k_guide_box_histogram<<<4 * G->sm_count, 256, 0, st>>>(g.rec, hist);
        if (cudaMemcpyAsync(h.data(), hist, h.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            rc = cuda_fail(cudaGetLastError(), "guide_fit_box");
    }
    cudaFree(hist);
    if (rc != MYPBR_OK)
        return rc;
    // per axis: the 1st and 99th percentiles, widened by a tenth of their span
    float a[3], b[3];
    bool narrower = false;
    for (int axis = 0; axis < 3; axis++) {
        const uint32_t* H = &h[size_t(axis) * kBoxBins];
        uint64_t total = 0;
        for (int k = 0; k < kBoxBins; k++)
            total += H[k];
        if (total < 1024)
            return MYPBR_OK;  // too few vertices to go by: the scene box stays
        uint64_t run = 0;
        int lo = 0, hi = kBoxBins - 1;
        for (int k = 0; k < kBoxBins; k++) {
            run += H[k];
            if (run * 100 >= total) {
                lo = k;
                break;
            }
        }
        run = 0;
        for (int k = kBoxBins - 1; k >= 0; k--) {
            run += H[k];
            if (run * 100 >= total) {
                hi = k;
                break;
            }
        }
        float x0 = float(lo) / kBoxBins, x1 = float(hi + 1) / kBoxBins;
        float margin = 0.1f * (x1 - x0) + 1.0f / kBoxBins;
        a[axis] = fmaxf(0.0f, x0 - margin);
        b[axis] = fminf(1.0f, x1 + margin);
        narrower = narrower || (b[axis] - a[axis]) < 0.8f;
    }
    if (!narrower)
        return MYPBR_OK;
    float3 A = make_float3(a[0], a[1], a[2]);
    float3 inv = make_float3(1.0f / (b[0] - a[0]), 1.0f / (b[1] - a[1]), 1.0f / (b[2] - a[2]));
    k_guide_box_rescale<<<4 * G->sm_count, 256, 0, st>>>(g.rec, A, inv);
    MYPBR_CUDA(cudaGetLastError());
    // the new box in world units: lo + a / inv_old, width (b - a) / inv_old
    float3 lo0 = g.box_lo, inv0 = g.box_inv;
    g.box_lo = make_float3(lo0.x + a[0] / inv0.x, lo0.y + a[1] / inv0.y, lo0.z + a[2] / inv0.z);
    g.box_inv = make_float3(inv0.x / (b[0] - a[0]), inv0.y / (b[1] - a[1]), inv0.z / (b[2] - a[2]));
    g.box_version++;
    return MYPBR_OK;
}

int guide_ensure(mypbr_gpu_scene* G, int hidden, unsigned long long seed) {
    GuideState& g = G->guide;
    if (g.hidden == hidden)
        return MYPBR_OK;
    if (hidden != 2 && hidden != 4 && hidden != 8) {
        set_error_message("guiding networks have 2, 4 or 8 hidden layers");
        return MYPBR_ERR_INVALID_ARGUMENT;
    }
    GuideRecords keep = g.rec;
    size_t keep_slots = g.rec_slots;
    __half* keep_packed = g.packed;
    size_t keep_packed_slots = g.packed_slots;
    g.rec = GuideRecords{};
    g.packed = nullptr;
    release_guide(g);
    g.rec = keep;
    g.rec_slots = keep_slots;
    g.packed = keep_packed;
    g.packed_slots = keep_packed_slots;
    g.hidden = hidden;
    g.params = guide_params(hidden);
    size_t P = size_t(g.params);
    g.train_ctas = G->sm_count;
    int rc;
    if ((rc = dalloc(g.w, P)) || (rc = dalloc(g.wt, P)) || (rc = dalloc(g.master, P)) || (rc = dalloc(g.m, P)) ||
        (rc = dalloc(g.v, P)) || (rc = dalloc(g.grad, P)) || (rc = dalloc(g.stats, 4)) ||
        (rc = dalloc(g.scratch, size_t(g.train_ctas) * kTrainGroups * train_scratch_per_group(hidden))) ||
        (rc = dalloc(g.partial, size_t(g.train_ctas) * kTrainGroups * P)))
        return rc;
    std::vector<float> w0 = initial_weights(hidden, seed);
    MYPBR_CUDA(cudaMemcpy(g.master, w0.data(), P * 4, cudaMemcpyHostToDevice));
    MYPBR_CUDA(cudaMemset(g.m, 0, P * 4));
    MYPBR_CUDA(cudaMemset(g.v, 0, P * 4));
    MYPBR_CUDA(cudaMemset(g.grad, 0, P * 4));
    k_guide_adam<<<64, 256>>>(g.master, g.m, g.v, nullptr, 0, g.w, g.wt, g.params, 0.0f, 0.0f, 0.0f);
    MYPBR_CUDA(cudaGetLastError());
    g.steps = 0;
    set_scene_box(G);
    return MYPBR_OK;
}

int guide_ensure_records(mypbr_gpu_scene* G, size_t mix_slots, size_t slots, int depth) {
    GuideState& g = G->guide;
    if (g.packed_slots < mix_slots) {
        if (g.packed)
            cudaFree(g.packed);
        g.packed = nullptr;
        g.packed_slots = 0;
        int rc = dalloc(g.packed, mix_slots * sizeof(GuidePacked) / sizeof(__half));
        if (rc != MYPBR_OK)
            return rc;
        g.packed_slots = mix_slots;
    }
    if (g.rec_slots >= slots && g.rec.depth == depth)
        return MYPBR_OK;
    void* old[] = {g.rec.in0, g.rec.in1, g.rec.dir, g.rec.fac, g.rec.mark, g.rec.bnext, g.rec.fin, g.rec.list,
                   g.rec.count};
    for (void* p : old)
        if (p)
            cudaFree(p);
    g.rec = GuideRecords{};
    g.rec_slots = 0;
    size_t n = slots * size_t(depth);
    int rc;
    if ((rc = dalloc(g.rec.in0, n)) || (rc = dalloc(g.rec.in1, n)) || (rc = dalloc(g.rec.dir, n)) ||
        (rc = dalloc(g.rec.fac, n)) || (rc = dalloc(g.rec.mark, n)) || (rc = dalloc(g.rec.bnext, n)) ||
        (rc = dalloc(g.rec.fin, slots)) || (rc = dalloc(g.rec.list, n)) || (rc = dalloc(g.rec.count, 1)))
        return rc;
    g.rec.depth = depth;
    g.rec.capacity = uint32_t(n);
    g.rec_slots = slots;
    MYPBR_CUDA(cudaMemset(g.rec.count, 0, 4));
    return MYPBR_OK;
}

int guide_train(mypbr_gpu_scene* G, int steps, int batch_tiles, float lr, cudaStream_t st) {
    NvtxRange range("mypbr guide training");
    GuideState& g = G->guide;
    if (g.hidden == 0 || g.rec.count == nullptr)
        return MYPBR_OK;
    long long rows = (long long)batch_tiles * 128;
    GuideNetView net = view_of(g, G->dev.error);
    for (int s = 0; s < steps; s++) {
        RecordSource src{g.rec, uint32_t(g.steps * 7919 + 17), g.stats, g.weight_cap};
        MYPBR_CUDA(cudaMemsetAsync(g.stats, 0, 4 * sizeof(float), st));
        k_guide_prep<<<G->sm_count * 2, 256, 0, st>>>(src, rows, g.stats, 0);
        k_guide_prep<<<G->sm_count * 2, 256, 0, st>>>(src, rows, g.stats, 1);
        MYPBR_CUDA(cudaGetLastError());
        int rc = train_dispatch(g.hidden, net, src, rows, g.train_ctas, g.scratch, g.partial, g.stats, st);
        if (rc != MYPBR_OK)
            return rc;
        g.steps++;
        float b1t = std::pow(0.9f, float(g.steps)), b2t = std::pow(0.99f, float(g.steps));
        k_guide_adam<<<(g.params + 255) / 256, 256, 0, st>>>(g.master, g.m, g.v, g.partial,
                                                            g.train_ctas * kTrainGroups, g.w, g.wt, g.params, lr,
                                                            b1t, b2t);
        MYPBR_CUDA(cudaGetLastError());
    }
    return MYPBR_OK;
}

}  // namespace mypbr_dev

using namespace mypbr_dev;

extern "C" {

int mypbr_guide_reset(mypbr_gpu_scene* scene) {
    if (!scene) {
        set_error_message("mypbr_guide_reset: null scene");
        return MYPBR_ERR_INVALID_ARGUMENT;
    }
    GuideState& g = scene->guide;
    if (g.hidden == 0)
        return MYPBR_OK;
    std::vector<float> w0 = initial_weights(g.hidden, 0x9d2c5680ull);
    size_t P = size_t(g.params);
    MYPBR_CUDA(cudaMemcpy(g.master, w0.data(), P * 4, cudaMemcpyHostToDevice));
    MYPBR_CUDA(cudaMemset(g.m, 0, P * 4));
    MYPBR_CUDA(cudaMemset(g.v, 0, P * 4));
    MYPBR_CUDA(cudaMemset(g.grad, 0, P * 4));
    k_guide_adam<<<64, 256>>>(g.master, g.m, g.v, nullptr, 0, g.w, g.wt, g.params, 0.0f, 0.0f, 0.0f);
    MYPBR_CUDA(cudaGetLastError());
    MYPBR_CUDA(cudaDeviceSynchronize());
    g.steps = 0;
    set_scene_box(scene);
    return MYPBR_OK;
}

int mypbr_guide_configure(mypbr_gpu_scene* scene, float alpha, int32_t depths, float alpha_deep) {
    if (!scene) {
        set_error_message("mypbr_guide_configure: null scene");
        return MYPBR_ERR_INVALID_ARGUMENT;
    }
    if (!(alpha > 0.0f && alpha < 1.0f) || depths < 1 || depths > 4096 || !(alpha_deep < 1.0f)) {
        set_error_message("mypbr_guide_configure: alpha must lie in (0, 1), alpha_deep below 1 and depths in "
                          "[1, 4096]");
        return MYPBR_ERR_INVALID_ARGUMENT;
    }
    scene->guide.alpha = alpha;
    scene->guide.alpha_deep = alpha_deep < 0.0f ? -1.0f : alpha_deep;
    scene->guide.depths = depths;
    return MYPBR_OK;
}

int mypbr_guide_schedule(mypbr_gpu_scene* scene, int32_t steps_early, int32_t steps_late, int32_t max_steps,
                         int32_t use_after, float weight_cap) {
    if (!scene) {
        set_error_message("mypbr_guide_schedule: null scene");
        return MYPBR_ERR_INVALID_ARGUMENT;
    }
    if (steps_early < 0 || steps_late < 0 || max_steps < 0 || steps_early > 4096 || steps_late > 4096 ||
        use_after < 0) {
        set_error_message("mypbr_guide_schedule: steps must lie in [0, 4096], max_steps and use_after be "
                          "non-negative");
        return MYPBR_ERR_INVALID_ARGUMENT;
    }
    if (!(weight_cap == 0.0f || (weight_cap >= 1.0f && weight_cap <= 1.0e6f))) {
        set_error_message("mypbr_guide_schedule: weight_cap must be 0 (no cap) or lie in [1, 1e6]");
        return MYPBR_ERR_INVALID_ARGUMENT;
    }
    scene->guide.steps_early = steps_early;
    scene->guide.steps_late = steps_late;
    scene->guide.max_steps = max_steps;
    scene->guide.use_after = use_after;
    scene->guide.weight_cap = weight_cap;
    return MYPBR_OK;
}

int mypbr_guide_test_forward(int hidden, const float* weights, const float* inputs, int64_t n, float* out) {
    if (!weights || !inputs || !out || n < 0)
        return MYPBR_ERR_INVALID_ARGUMENT;
    TempNet T;
    int rc = temp_net(T, hidden, weights);
    if (rc != MYPBR_OK)
        return rc;
    float *d_in = nullptr, *d_out = nullptr;
    if ((rc = dalloc(d_in, size_t(n) * kGuideIn + 1)) || (rc = dalloc(d_out, size_t(n) * kGuideOut + 1)))
        return rc;
    cudaMemcpy(d_in, inputs, size_t(n) * kGuideIn * 4, cudaMemcpyHostToDevice);
    size_t smem = guide_forward_smem(hidden);
    auto k = k_guide_forward<GivenSource, RowSink>;
    rc = set_smem(k, smem);
    if (rc == MYPBR_OK) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        long long tiles = (n + 127) / 128;
        int grid = int(std::min<long long>(std::max<long long>((tiles + kGuideGroups - 1) / kGuideGroups, 1), sms));
        k<<<grid, 128 * kGuideGroups, smem>>>(view_of(T.g, T.err), GivenSource{d_in, nullptr}, RowSink{d_out}, n);
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess)
            rc = cuda_fail(e, "k_guide_forward");
        else
            rc = read_error(T.err);
    }
    if (rc == MYPBR_OK)
        cudaMemcpy(out, d_out, size_t(n) * kGuideOut * 4, cudaMemcpyDeviceToHost);
    cudaFree(d_in);
    cudaFree(d_out);
    return rc;
}

int mypbr_guide_test_backward(int hidden, const float* weights, const float* inputs, const float* dout, int64_t n,
                              float* grads) {
    if (!weights || !inputs || !dout || !grads || n < 0)
        return MYPBR_ERR_INVALID_ARGUMENT;
    TempNet T;
    int rc = temp_net(T, hidden, weights);
    if (rc != MYPBR_OK)
        return rc;
    float *d_in = nullptr, *d_g = nullptr, *partial = nullptr;
    __nv_bfloat16* scratch = nullptr;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long tiles = (n + 127) / 128;
    // fewer CTAs than tiles, so that groups also take several tiles in turn
    int ctas = int(std::min<long long>(std::max<long long>((tiles + 2 * kTrainGroups - 1) / (2 * kTrainGroups), 1),
                                       sms));
    if ((rc = dalloc(d_in, size_t(n) * kGuideIn + 1)) || (rc = dalloc(d_g, size_t(n) * kGuideOut + 1)) ||
        (rc = dalloc(scratch, size_t(ctas) * kTrainGroups * train_scratch_per_group(hidden))) ||
        (rc = dalloc(partial, size_t(ctas) * kTrainGroups * T.g.params)))
        return rc;
    cudaMemcpy(d_in, inputs, size_t(n) * kGuideIn * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(d_g, dout, size_t(n) * kGuideOut * 4, cudaMemcpyHostToDevice);
    rc = train_dispatch(hidden, view_of(T.g, T.err), GivenSource{d_in, d_g}, n, ctas, scratch, partial, nullptr, 0);
    if (rc == MYPBR_OK) {
        k_guide_sum_partials<<<(T.g.params + 255) / 256, 256>>>(partial, ctas * kTrainGroups, T.g.params,
                                                                T.g.grad);
        cudaError_t e = cudaDeviceSynchronize();
        rc = e != cudaSuccess ? cuda_fail(e, "k_guide_train") : read_error(T.err);
    }
    if (rc == MYPBR_OK)
        cudaMemcpy(grads, T.g.grad, size_t(T.g.params) * 4, cudaMemcpyDeviceToHost);
    cudaFree(d_in);
    cudaFree(d_g);
    cudaFree(partial);
    cudaFree(scratch);
    return rc;
}

}  // extern "C"

namespace mypbr_dev {
// Encodes n rows of 7 scalars into a shared 128-row canonical tile per CTA
// (guide_encode_row, as the forward kernels do) and copies the BF16 features
// out as floats.
__global__ void k_encode_test(const float* scalars, long long n, float* out) {
    __shared__ __align__(16) __nv_bfloat16 tile[128 * kGuideIn];
    for (long long base = (long long)blockIdx.x * 128; base < n; base += (long long)gridDim.x * 128) {
        long long i = base + threadIdx.x;
        float s[kGuideScalars];
        for (int k = 0; k < kGuideScalars; k++)
            s[k] = i < n ? scalars[i * kGuideScalars + k] : 0.0f;
        guide_encode_row(i < n ? s : nullptr, tile, threadIdx.x);
        __syncwarp();
        if (i < n)
            for (int k = 0; k < kGuideIn; k++)
                out[i * kGuideIn + k] = __bfloat162float(tile[canon(threadIdx.x, k, kGuideIn)]);
        __syncthreads();
    }
}
}  // namespace mypbr_dev

extern "C" {

int mypbr_guide_test_encode(const float* scalars, int64_t n, float* out) {
    if (!scalars || !out || n < 0)
        return MYPBR_ERR_INVALID_ARGUMENT;
    float *d_s, *d_out;
    int rc;
    if ((rc = dalloc(d_s, size_t(n) * kGuideScalars + 1)) || (rc = dalloc(d_out, size_t(n) * kGuideIn + 1)))
        return rc;
    cudaMemcpy(d_s, scalars, size_t(n) * kGuideScalars * 4, cudaMemcpyHostToDevice);
    k_encode_test<<<64, 128>>>(d_s, n, d_out);
    cudaError_t e = cudaDeviceSynchronize();
    rc = e != cudaSuccess ? cuda_fail(e, "k_encode_test") : MYPBR_OK;
    if (rc == MYPBR_OK)
        cudaMemcpy(out, d_out, size_t(n) * kGuideIn * 4, cudaMemcpyDeviceToHost);
    cudaFree(d_s);
    cudaFree(d_out);
    return rc;
}

int mypbr_guide_test_loss(const float* raw, const float* dirs, const float* c, int64_t n, float* grad, float* loss) {
    if (!raw || !dirs || !c || !grad || !loss || n < 0)
        return MYPBR_ERR_INVALID_ARGUMENT;
    float *d_raw, *d_dirs, *d_c, *d_grad, *d_loss;
    int rc;
    if ((rc = dalloc(d_raw, size_t(n) * kGuideOut + 1)) || (rc = dalloc(d_dirs, size_t(n) * 3 + 1)) ||
        (rc = dalloc(d_c, size_t(n) + 1)) || (rc = dalloc(d_grad, size_t(n) * kGuideOut + 1)) ||
        (rc = dalloc(d_loss, size_t(n) + 1)))
        return rc;
    cudaMemcpy(d_raw, raw, size_t(n) * kGuideOut * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(d_dirs, dirs, size_t(n) * 12, cudaMemcpyHostToDevice);
    cudaMemcpy(d_c, c, size_t(n) * 4, cudaMemcpyHostToDevice);
    k_loss_test<<<64, 128>>>(d_raw, d_dirs, d_c, n, d_grad, d_loss);
    cudaError_t e = cudaDeviceSynchronize();
    rc = e != cudaSuccess ? cuda_fail(e, "k_loss_test") : MYPBR_OK;
    if (rc == MYPBR_OK) {
        cudaMemcpy(grad, d_grad, size_t(n) * kGuideOut * 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(loss, d_loss, size_t(n) * 4, cudaMemcpyDeviceToHost);
    }
    for (void* p : {(void*)d_raw, (void*)d_dirs, (void*)d_c, (void*)d_grad, (void*)d_loss})
        cudaFree(p);
    return rc;
}

int mypbr_guide_test_mixture(const float* raw, const float* u, const float* dirs, int64_t n, float* samples,
                             float* pdf_sample, float* pdf_dir) {
    if (!raw || !u || !dirs || !samples || !pdf_sample || !pdf_dir || n < 0)
        return MYPBR_ERR_INVALID_ARGUMENT;
    float *d_raw, *d_u, *d_dirs, *d_s, *d_ps, *d_pd;
    int rc;
    if ((rc = dalloc(d_raw, size_t(n) * kGuideOut + 1)) || (rc = dalloc(d_u, size_t(n) * 3 + 1)) ||
        (rc = dalloc(d_dirs, size_t(n) * 3 + 1)) || (rc = dalloc(d_s, size_t(n) * 3 + 1)) ||
        (rc = dalloc(d_ps, size_t(n) + 1)) || (rc = dalloc(d_pd, size_t(n) + 1)))
        return rc;
    cudaMemcpy(d_raw, raw, size_t(n) * kGuideOut * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(d_u, u, size_t(n) * 12, cudaMemcpyHostToDevice);
    cudaMemcpy(d_dirs, dirs, size_t(n) * 12, cudaMemcpyHostToDevice);
    k_mixture_test<<<64, 128>>>(d_raw, d_u, d_dirs, n, d_s, d_ps, d_pd);
    cudaError_t e = cudaDeviceSynchronize();
    rc = e != cudaSuccess ? cuda_fail(e, "k_mixture_test") : MYPBR_OK;
    if (rc == MYPBR_OK) {
        cudaMemcpy(samples, d_s, size_t(n) * 12, cudaMemcpyDeviceToHost);
        cudaMemcpy(pdf_sample, d_ps, size_t(n) * 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(pdf_dir, d_pd, size_t(n) * 4, cudaMemcpyDeviceToHost);
    }
    for (void* p : {(void*)d_raw, (void*)d_u, (void*)d_dirs, (void*)d_s, (void*)d_ps, (void*)d_pd})
        cudaFree(p);
    return rc;
}

}  // extern "C"

// The failure path of the bounded device waits, exercised without a fault:
// a wait that nothing ends gives up, the host reads MYPBR_ERR_DEVICE_TIMEOUT,
// and the context stays usable.
extern "C" int mypbr_gpu_test_wait_timeout(void) {
    using namespace mypbr_dev;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        set_error_message("mypbr_gpu_test_wait_timeout: no CUDA device");
        return MYPBR_ERR_NO_DEVICE;
    }
    int* err = nullptr;
    MYPBR_CUDA(cudaMalloc(&err, sizeof(int)));
    int rc = MYPBR_OK;
    if (cudaMemset(err, 0, sizeof(int)) != cudaSuccess)
        rc = cuda_fail(cudaGetLastError(), "mypbr_gpu_test_wait_timeout");
    if (rc == MYPBR_OK) {
        k_wait_probe<<<1, 32>>>(err);
        cudaError_t e = cudaDeviceSynchronize();
        rc = e != cudaSuccess ? cuda_fail(e, "k_wait_probe") : read_error(err);
    }
    cudaFree(err);
    return rc;
}
