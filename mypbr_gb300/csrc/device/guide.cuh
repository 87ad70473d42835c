// Path guiding: a small MLP maps (position, normal, outgoing direction) at a
// surface vertex to a mixture of 8 von Mises-Fisher lobes over incident
// directions. The renderer samples it as one more MIS proposal beside the
// BSDF (one-sample MIS with probability alpha) and next-event estimation, so
// the estimator stays unbiased whatever the network has learned.
//
// Network: input one-blob encoding (7 scalars in [0, 1]: position 3 x 32
// Gaussian bins, normal and outgoing direction angles 4 x 6; a constant 1 as
// bias, zero padding to 128) -> `hidden` layers of 64
// ReLU units -> 64 outputs, of which 40 are used: per lobe (mu_x, mu_y, mu_z,
// log kappa, logit). BF16 weights and activations, FP32 accumulation on the
// tensor cores (tcgen05.mma, accumulators in TMEM).
//
// Weight storage: matrix l is [64 out][K in] (K = 128 for l = 0, else 64),
// BF16 in the tensor cores' canonical K-major layout without swizzle: 8x8
// core matrices of 128 contiguous bytes, element (r, k) at
//   ((r / 8) * (K / 8) + k / 8) * 64 + (r % 8) * 8 + k % 8
// so the leading (K) byte offset between core matrices is 128 and the stride
// (row-group) byte offset is K * 16.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cstring>

#include "dev_scene.cuh"

namespace mypbr_dev {

constexpr int kGuideIn = 128;
constexpr int kGuideWidth = 64;
constexpr int kGuideOut = 64;
constexpr int kGuideLobes = 8;
constexpr int kGuideUsed = 5 * kGuideLobes;  // raw outputs in use
constexpr int kGuideScalars = 7;
constexpr int kGuideMaxHidden = 8;
constexpr int kGuideRecordDepth = 4;  // vertices of a path recorded for training
constexpr float kGuideLogKappaMin = -4.0f, kGuideLogKappaMax = 9.0f;

// Elements of matrix l and where it starts in the concatenated weights.
MYPBR_HD int guide_in(int l) { return l == 0 ? kGuideIn : kGuideWidth; }
MYPBR_HD int guide_offset(int l) { return l == 0 ? 0 : kGuideWidth * kGuideIn + (l - 1) * kGuideWidth * kGuideWidth; }
MYPBR_HD int guide_params(int hidden) { return guide_offset(hidden + 1); }

// Element offset of (r, k) in a canonical K-major tile with K columns.
MYPBR_HD int canon(int r, int k, int K) { return ((r >> 3) * (K >> 3) + (k >> 3)) * 64 + (r & 7) * 8 + (k & 7); }

// ------------------------------------------------------------- encoding

// The 7 scalars of a vertex, each in [0, 1]: position in the scene box,
// the normal's and the outgoing direction's (theta / pi, phi / 2 pi).
MYPBR_DEV void guide_scalars(float3 p, float3 n, float3 wo, float3 box_lo, float3 box_inv, float s[7]) {
    s[0] = clampf((p.x - box_lo.x) * box_inv.x, 0.0f, 1.0f);
    s[1] = clampf((p.y - box_lo.y) * box_inv.y, 0.0f, 1.0f);
    s[2] = clampf((p.z - box_lo.z) * box_inv.z, 0.0f, 1.0f);
    s[3] = acosf(clampf(n.y, -1.0f, 1.0f)) * kInvPi;
    s[4] = (atan2f(n.z, n.x) + kPi) * (0.5f * kInvPi);
    s[5] = acosf(clampf(wo.y, -1.0f, 1.0f)) * kInvPi;
    s[6] = (atan2f(wo.z, wo.x) + kPi) * (0.5f * kInvPi);
}

// One-blob encoding (Mueller et al., "Neural Importance Sampling", 2019):
// scalar i gets guide_bins_of(i) bins, each a Gaussian of width one bin centred
// on it. Position gets the finer grid (32 bins per axis), the four angles 6
// bins each; then a constant 1 (the first layer's bias) and zero padding:
// 3 x 32 + 4 x 6 + 1 = 121 of the 128 inputs.
MYPBR_HD constexpr int guide_bins_of(int i) { return i < 3 ? 32 : 6; }
MYPBR_HD constexpr int guide_first_bin(int i) { return i < 3 ? 32 * i : 96 + 6 * (i - 3); }
constexpr int kGuideEncoded = 3 * 32 + 4 * 6;  // 120 one-blob features

MYPBR_DEV float one_blob(float s, int b, int bins) {
    float x = (s - (float(b) + 0.5f) / float(bins)) * float(bins);
    return __expf(-0.5f * x * x);
}

// Input feature k (0..127) of the encoded vertex.
MYPBR_DEV float guide_feature(const float s[7], int k) {
    if (k < kGuideEncoded) {
        int i = k < 96 ? k / 32 : 3 + (k - 96) / 6;
        int b = k - guide_first_bin(i);
        return one_blob(s[i], b, guide_bins_of(i));
    }
    return k == kGuideEncoded ? 1.0f : 0.0f;
}

// ------------------------------------------------------------- mixture

// A decoded mixture: unit mean directions, concentrations and weights.
struct GuideMix {
    float3 mu[kGuideLobes];
    float kappa[kGuideLobes];
    float w[kGuideLobes];
};

// Raw network outputs -> mixture (normalised means, kappa = exp(clamped), softmax weights).
MYPBR_DEV void guide_decode(const float* o, GuideMix& m) {
    float mx = -3.0e38f;
#pragma unroll
    for (int j = 0; j < kGuideLobes; j++)
        mx = fmaxf(mx, o[5 * j + 4]);
    float sum = 0.0f;
#pragma unroll
    for (int j = 0; j < kGuideLobes; j++) {
        float3 v = f3(o[5 * j], o[5 * j + 1], o[5 * j + 2]);
        float l2 = dot(v, v);
        m.mu[j] = l2 > 1e-20f ? v * rsqrtf(l2) : f3(0.0f, 1.0f, 0.0f);
        m.kappa[j] = __expf(clampf(o[5 * j + 3], kGuideLogKappaMin, kGuideLogKappaMax));
        m.w[j] = __expf(o[5 * j + 4] - mx);
        sum += m.w[j];
    }
    float inv = 1.0f / sum;
#pragma unroll
    for (int j = 0; j < kGuideLobes; j++)
        m.w[j] *= inv;
}

// vMF density on the unit sphere: kappa / (2 pi (1 - e^{-2 kappa})) e^{kappa (mu.w - 1)}.
MYPBR_DEV float vmf_pdf(float3 mu, float kappa, float3 w) {
    float norm = kappa / (2.0f * kPi * -expm1f(-2.0f * kappa));
    return norm * __expf(kappa * (dot(mu, w) - 1.0f));
}

MYPBR_DEV float guide_pdf(const GuideMix& m, float3 w) {
    float p = 0.0f;
#pragma unroll
    for (int j = 0; j < kGuideLobes; j++)
        p += m.w[j] * vmf_pdf(m.mu[j], m.kappa[j], w);
    return p;
}

// Sampling a vMF lobe by inverting the cosine's distribution in the form of
// Jakob, "Numerically stable sampling of the von Mises Fisher distribution
// on S^2" (2012): cos = 1 + log(u + (1 - u) e^{-2 kappa}) / kappa.
MYPBR_DEV float3 vmf_sample(float3 mu, float kappa, float u1, float u2) {
    float c = 1.0f + __logf(u1 + (1.0f - u1) * __expf(-2.0f * kappa)) / kappa;
    c = clampf(c, -1.0f, 1.0f);
    float s = sqrtf(fmaxf(0.0f, 1.0f - c * c));
    float phi = 2.0f * kPi * u2;
    // branchless orthonormal basis around mu (Duff et al., JCGT 2017)
    float sign = copysignf(1.0f, mu.z);
    float a = -1.0f / (sign + mu.z);
    float b = mu.x * mu.y * a;
    float3 t1 = f3(1.0f + sign * mu.x * mu.x * a, sign * b, -sign * mu.x);
    float3 t2 = f3(b, sign + mu.y * mu.y * a, -mu.y);
    return normalize(c * mu + s * (__cosf(phi) * t1 + __sinf(phi) * t2));
}

MYPBR_DEV float3 guide_sample(const GuideMix& m, float u0, float u1, float u2) {
    int j = kGuideLobes - 1;
    float acc = 0.0f;
#pragma unroll
    for (int k = 0; k < kGuideLobes; k++) {
        acc += m.w[k];
        if (u0 < acc) {
            j = k;
            break;
        }
    }
    float3 mu = m.mu[0];
    float kappa = m.kappa[0];
#pragma unroll
    for (int k = 1; k < kGuideLobes; k++)
        if (k == j) {
            mu = m.mu[k];
            kappa = m.kappa[k];
        }
    return vmf_sample(mu, kappa, u1, u2);
}

// d(-c log q(w)) / d(raw outputs) for the mixture q decoded from o: the
// gradient of the KL divergence between the target density (estimated by
// samples w with weight c = contribution / pdf) and q.
MYPBR_DEV float guide_loss_grad(const float* o, float3 w, float c, float* g) {
    GuideMix m;
    guide_decode(o, m);
    float v[kGuideLobes];
    float q = 0.0f;
#pragma unroll
    for (int j = 0; j < kGuideLobes; j++) {
        v[j] = vmf_pdf(m.mu[j], m.kappa[j], w);
        q += m.w[j] * v[j];
    }
    q = fmaxf(q, 1e-30f);
    float iq = 1.0f / q;
#pragma unroll
    for (int j = 0; j < kGuideLobes; j++) {
        float r = m.w[j] * v[j] * iq;  // responsibility of lobe j
        float3 raw = f3(o[5 * j], o[5 * j + 1], o[5 * j + 2]);
        float len = sqrtf(fmaxf(dot(raw, raw), 1e-20f));
        float k = m.kappa[j];
        float mw = dot(m.mu[j], w);
        // d log v / d mu_raw = kappa (w - (mu.w) mu) / |mu_raw|
        float3 dmu = (k / len) * (w - mw * m.mu[j]);
        // d log v / d log kappa = 1 - 2 kappa / (e^{2 kappa} - 1) + kappa (mu.w - 1)
        float ls = o[5 * j + 3];
        float dls = (ls > kGuideLogKappaMin && ls < kGuideLogKappaMax)
                        ? 1.0f - 2.0f * k / expm1f(2.0f * k) + k * (mw - 1.0f) : 0.0f;
        g[5 * j] = -c * r * dmu.x;
        g[5 * j + 1] = -c * r * dmu.y;
        g[5 * j + 2] = -c * r * dmu.z;
        g[5 * j + 3] = -c * r * dls;
        g[5 * j + 4] = -c * (r - m.w[j]);
    }
    return -c * __logf(q);
}

// ------------------------------------------------------------- tcgen05

namespace tc {

MYPBR_DEV uint32_t smem_u32(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }

// Shared-memory matrix descriptor, K-major, no swizzle: start address, leading
// (K-direction) and stride (row-group) byte offsets, all in 16-byte units;
// bits 46-47 hold the descriptor version 1.
MYPBR_DEV uint64_t desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return uint64_t((saddr >> 4) & 0x3fff) | (uint64_t((lbo >> 4) & 0x3fff) << 16) |
           (uint64_t((sbo >> 4) & 0x3fff) << 32) | (uint64_t(1) << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
MYPBR_HD uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

// The same with A (bit 15) and / or B (bit 16) read MN-major: the operand's
// M (or N) index runs along the 16-byte rows of its core matrices. A tile
// stored K-major as [rows][K] is, read MN-major, its own transpose. For the
// no-swizzle MN-major layout the descriptor's leading byte offset is the
// core-matrix stride along K and the stride byte offset the one along M/N:
// element (mn, k) sits at (mn % 8) * 2 B + (mn / 8) * SBO + (k % 8) * 16 B +
// (k / 8) * LBO.
MYPBR_HD uint32_t idesc_bf16_mn(int M, int N, bool a_mn, bool b_mn) {
    return idesc_bf16(M, N) | (a_mn ? (1u << 15) : 0u) | (b_mn ? (1u << 16) : 0u);
}

MYPBR_DEV void mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

MYPBR_DEV void commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

MYPBR_DEV void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
MYPBR_DEV void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Generic-proxy writes to shared memory made visible to the tensor cores' async proxy.
MYPBR_DEV void fence_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

MYPBR_DEV void bar_init(uint64_t* bar, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

MYPBR_DEV bool bar_try(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the phase with the given parity to complete, for about a second
// at most; false if it never did.
MYPBR_DEV bool bar_wait(uint64_t* bar, uint32_t parity) {
    long long deadline = clock64() + (1ll << 31);
    while (!bar_try(bar, parity))
        if (clock64() > deadline)
            return false;
    return true;
}

// TMEM allocation by one whole warp; the address lands in *slot.
MYPBR_DEV void tmem_alloc(uint32_t* slot, uint32_t cols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
MYPBR_DEV void tmem_free(uint32_t taddr, uint32_t cols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}

// 16 consecutive 32-bit columns of this thread's TMEM lane (32x32b shape: warp
// w of the CTA reads lanes 32 (w % 4) .. + 31, one lane per thread).
MYPBR_DEV void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int k = 0; k < 16; k++)
        v[k] = __uint_as_float(r[k]);
}
MYPBR_DEV void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 64 consecutive 32-bit columns of this thread's lane in one load.
MYPBR_DEV void tmem_ld64(uint32_t taddr, float* v) {
    uint32_t r[64];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
        : "r"(taddr));
#pragma unroll
    for (int k = 0; k < 64; k++)
        v[k] = __uint_as_float(r[k]);
}

// 64 columns starting at `col` of this thread's lane.
MYPBR_DEV void tmem_row64(uint32_t tmem, int col, float* v) {
    uint32_t lane = uint32_t((threadIdx.x >> 5) & 3) * 32u;
    tmem_ld64(tmem + (lane << 16) + uint32_t(col), v);
    tmem_wait_ld();
}

}  // namespace tc

MYPBR_DEV uint32_t pack_bf16(float a, float b) {
    __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
}

// max(a, 0), max(b, 0) rounded to BF16 and packed (a in the low half), one
// instruction.
MYPBR_DEV uint32_t pack_bf16_relu(float a, float b) {
    uint32_t d;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(b), "f"(a));
    return d;
}

// Writes ReLU of 64 values of row r as BF16 into a canonical K-major tile
// with K = 64 columns.
MYPBR_DEV void store_row_bf16_relu(__nv_bfloat16* tile, int r, const float* v) {
#pragma unroll
    for (int b = 0; b < 8; b++) {
        uint4 u;
        u.x = pack_bf16_relu(v[8 * b], v[8 * b + 1]);
        u.y = pack_bf16_relu(v[8 * b + 2], v[8 * b + 3]);
        u.z = pack_bf16_relu(v[8 * b + 4], v[8 * b + 5]);
        u.w = pack_bf16_relu(v[8 * b + 6], v[8 * b + 7]);
        *reinterpret_cast<uint4*>(tile + canon(r, 8 * b, 64)) = u;
    }
}

// Writes 64 values of row r as BF16 into a canonical K-major tile with K
// columns (k from k0), eight 16-byte stores.
MYPBR_DEV void store_row_bf16(__nv_bfloat16* tile, int r, int K, int k0, const float* v) {
#pragma unroll
    for (int b = 0; b < 8; b++) {
        uint4 u;
        u.x = pack_bf16(v[8 * b], v[8 * b + 1]);
        u.y = pack_bf16(v[8 * b + 2], v[8 * b + 3]);
        u.z = pack_bf16(v[8 * b + 4], v[8 * b + 5]);
        u.w = pack_bf16(v[8 * b + 6], v[8 * b + 7]);
        *reinterpret_cast<uint4*>(tile + canon(r, k0 + 8 * b, K)) = u;
    }
}

}  // namespace mypbr_dev

namespace mypbr_dev {

// The network as the kernels see it.
struct GuideNetView {
    int hidden;                    // hidden layers; matrices 0..hidden
    const __nv_bfloat16* w;        // forward weights, canonical [64 out][in] per matrix
    const __nv_bfloat16* wt;       // transposed copies, canonical [in][64 out]
    float* grad;                   // FP32 [out][in] per matrix, accumulated by training
    int* error;                    // sticky error word: 3 = a tensor-core wait timed out
};

// Tiles of 128 rows a forward CTA works on at once: one group of 4 warps
// (128 threads, a thread per row) per tile, all groups sharing one copy of
// the weights in shared memory and each with its own activation tile,
// mbarrier and 64 TMEM columns, synchronising with its own named barrier.
constexpr int kGuideGroups = 4;

// Shared memory of the forward kernel: every weight matrix, then one
// 128 x 128 activation tile per group, then the barriers and the TMEM address.
MYPBR_HD size_t guide_forward_smem(int hidden) {
    return size_t(guide_params(hidden)) * 2 + size_t(kGuideGroups) * 128 * kGuideIn * 2 + 64;
}

namespace tc {
// Named barrier of `count` threads; returns whether any thread passed `pred`.
MYPBR_DEV bool group_sync_or(int id, int count, bool pred) {
    uint32_t out;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.or.pred q, %2, %3, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}\n"
        : "=r"(out)
        : "r"(uint32_t(pred)), "r"(id), "r"(count)
        : "memory");
    return out != 0;
}
MYPBR_DEV void group_sync(int id, int count) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory"); }
}  // namespace tc

// Batched MLP forward on the tensor cores: each CTA (kGuideGroups groups of
// 128 threads, one thread per row) walks tiles of 128 rows, a tile per group
// at a time. Src::count(rows) gives the number of rows (it may read a device
// counter). A row is staged in three steps, so that the memory reads behind
// the next tile's rows are in flight while the current tile's layers run:
// Src::load(i, r) starts the reads of row i into the thread's Src::Row (i =
// -1 for padding rows), Src::finish(r) completes the row's inputs two layers
// later, Src::encode(r, tile, row) writes the encoded input row (BF16,
// canonical, K = 128) when its tile begins. Sink::put(i, r, v) takes the 64
// FP32 outputs of row i.
template <class Src, class Sink>
__global__ void __launch_bounds__(128 * kGuideGroups) k_guide_forward(GuideNetView net, Src src, Sink sink,
                                                                      long long rows) {
    extern __shared__ __align__(1024) uint8_t smem[];
    rows = src.count(rows);
    const long long tiles = (rows + 127) / 128;
    if ((long long)blockIdx.x * kGuideGroups >= tiles)
        return;  // no tile for this CTA: nothing loaded, nothing allocated
    const int P = guide_params(net.hidden);
    const int group = threadIdx.x >> 7, row = threadIdx.x & 127, warp = threadIdx.x >> 5;
    __nv_bfloat16* W = reinterpret_cast<__nv_bfloat16*>(smem);
    __nv_bfloat16* A = W + P + size_t(group) * 128 * kGuideIn;
    uint64_t* bars = reinterpret_cast<uint64_t*>(W + P + size_t(kGuideGroups) * 128 * kGuideIn);
    uint64_t* bar = bars + group;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + kGuideGroups);
    {  // the weights stay resident for every tile this CTA handles
        const uint4* g = reinterpret_cast<const uint4*>(net.w);
        uint4* s = reinterpret_cast<uint4*>(W);
        for (int k = threadIdx.x; k < P / 8; k += blockDim.x)
            s[k] = g[k];
    }
    if (warp == 0)
        tc::tmem_alloc(tmem_slot, 64 * kGuideGroups);
    if (row == 0)
        tc::bar_init(bar, 1);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *tmem_slot + uint32_t(64 * group);
    const int bar_id = 1 + group;  // named barrier 0 is __syncthreads
    uint32_t phase = 0;
    const uint32_t idesc = tc::idesc_bf16(128, 64);
    bool failed = false;
    const long long stride = (long long)gridDim.x * kGuideGroups;
    auto row_of = [&](long long t) { return t < tiles && t * 128 + row < rows ? t * 128 + row : -1LL; };
    // the layer at which the next tile's rows are completed (their reads were
    // started at layer 0)
    const int finish_at = net.hidden < 2 ? net.hidden : 2;
    typename Src::Row cur, next;
    src.load(row_of((long long)blockIdx.x * kGuideGroups + group), cur);
    src.finish(cur);
    for (long long tile = (long long)blockIdx.x * kGuideGroups + group; tile < tiles && !failed; tile += stride) {
        const long long i = tile * 128 + row;
        src.encode(cur, A, row);
        const long long i_next = row_of(tile + stride);
        for (int l = 0; l <= net.hidden; l++) {
            int K = guide_in(l);
            tc::fence_smem();
            tc::group_sync(bar_id, 128);
            if (row == 0) {
                tc::fence_after();
                uint32_t a0 = tc::smem_u32(A), b0 = tc::smem_u32(W + guide_offset(l));
                for (int s = 0; s < K / 16; s++)
                    tc::mma(tmem, tc::desc(a0 + 256 * s, 128, K * 16), tc::desc(b0 + 256 * s, 128, K * 16), idesc,
                            s > 0);
                tc::commit(bar);
            }
            // while the layer's MMAs run: the next tile's rows
            if (l == 0)
                src.load(i_next, next);
            if (l == finish_at)
                src.finish(next);
            bool ok = tc::bar_wait(bar, phase);
            phase ^= 1;
            if (tc::group_sync_or(bar_id, 128, !ok)) {
                if (row == 0)
                    atomicCAS(net.error, 0, 3);
                tc::bar_wait(bar, phase ^ 1);  // once more, bounded, for the MMAs in flight
                failed = true;
                break;
            }
            tc::fence_after();
            float v[64];
            tc::tmem_row64(tmem, 0, v);
            tc::fence_before();
            if (l < net.hidden) {
                store_row_bf16_relu(A, row, v);
            } else if (i < rows) {
                sink.put(i, cur, v);
            }
        }
        cur = next;
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after();
        tc::tmem_free(*tmem_slot, 64 * kGuideGroups);
    }
}

// The one-blob bins of one scalar, out[b] = exp(-0.5 (u - b)^2) with
// u = s * BINS - 0.5 (guide_feature's values), in blocks of up to 8 bins:
// one exponential at the block's middle bin m, then outwards by the ratio of
// neighbouring Gaussians (g[b+1] = g[b] exp(u - b - 0.5) going up, g[b-1] =
// g[b] exp(b - u - 0.5) going down), each ratio shrinking by 1/e per bin.
// Three exponentials per block instead of one per bin. Every bin is within 4
// of m, so a middle value that underflows FP32 (|u - m| > 13) leaves only
// values below 1e-18 (then 0).
template <int BINS>
MYPBR_DEV void one_blob_bins(float s, float* out) {
    constexpr float kInvE = 0.36787944117144233f;
    const float u = s * float(BINS) - 0.5f;
#pragma unroll
    for (int a = 0; a < BINS; a += 8) {
        constexpr int kBlock = BINS < 8 ? BINS : 8;
        const int m = a + kBlock / 2;
        const float x = u - float(m);
        const float gm = __expf(-0.5f * x * x);
        float g = gm, up = __expf(x - 0.5f);
#pragma unroll
        for (int b = m; b < a + kBlock; b++) {
            out[b] = g;
            g *= up;
            up *= kInvE;
        }
        g = gm;
        float down = __expf(-x - 0.5f);
#pragma unroll
        for (int b = m - 1; b >= a; b--) {
            g *= down;
            down *= kInvE;
            out[b] = g;
        }
    }
}

// Packs 8 floats as BF16 into the 16 bytes at `dst`.
MYPBR_DEV void store8_bf16(__nv_bfloat16* dst, const float* v) {
    uint4 u;
    u.x = pack_bf16(v[0], v[1]);
    u.y = pack_bf16(v[2], v[3]);
    u.z = pack_bf16(v[4], v[5]);
    u.w = pack_bf16(v[6], v[7]);
    *reinterpret_cast<uint4*>(dst) = u;
}

// Encodes scalars s into row `row` of a canonical K = 128 tile (zeros if s
// is null): the one-blob features of guide_feature, k = 0..127.
MYPBR_DEV void guide_encode_row(const float* s, __nv_bfloat16* tile, int row) {
    float v[kGuideIn];
    if (s) {
#pragma unroll
        for (int i = 0; i < 3; i++)
            one_blob_bins<32>(s[i], v + 32 * i);
#pragma unroll
        for (int i = 3; i < 7; i++)
            one_blob_bins<6>(s[i], v + 96 + 6 * (i - 3));
        v[kGuideEncoded] = 1.0f;
#pragma unroll
        for (int k = kGuideEncoded + 1; k < kGuideIn; k++)
            v[k] = 0.0f;
    } else {
#pragma unroll
        for (int k = 0; k < kGuideIn; k++)
            v[k] = 0.0f;
    }
#pragma unroll
    for (int b = 0; b < kGuideIn / 8; b++)
        store8_bf16(tile + canon(row, 8 * b, kGuideIn), v + 8 * b);
}

// The decoded mixture of a vertex as the shading kernels read it: per lobe
// (mu xyz, kappa, weight) in FP16, 80 bytes.
struct GuidePacked {
    uint4 q[5];
};

MYPBR_DEV void guide_pack(const float* raw, GuidePacked& out) {
    GuideMix m;
    guide_decode(raw, m);
    __half h[40];
#pragma unroll
    for (int j = 0; j < kGuideLobes; j++) {
        h[5 * j] = __float2half_rn(m.mu[j].x);
        h[5 * j + 1] = __float2half_rn(m.mu[j].y);
        h[5 * j + 2] = __float2half_rn(m.mu[j].z);
        h[5 * j + 3] = __float2half_rn(fminf(m.kappa[j], 60000.0f));
        h[5 * j + 4] = __float2half_rn(m.w[j]);
    }
    memcpy(&out, h, sizeof(out));
}

// Unpacks a mixture; means are renormalised and weights summed again so that
// the pdf used for sampling and for evaluation is one and the same density.
MYPBR_DEV void guide_unpack(const GuidePacked& in, GuideMix& m) {
    __half h[40];
    memcpy(h, &in, sizeof(in));
    float sum = 0.0f;
#pragma unroll
    for (int j = 0; j < kGuideLobes; j++) {
        float3 mu = f3(__half2float(h[5 * j]), __half2float(h[5 * j + 1]), __half2float(h[5 * j + 2]));
        float l2 = dot(mu, mu);
        m.mu[j] = l2 > 1e-12f ? mu * rsqrtf(l2) : f3(0.0f, 1.0f, 0.0f);
        m.kappa[j] = fmaxf(__half2float(h[5 * j + 3]), 1e-4f);
        m.w[j] = fmaxf(__half2float(h[5 * j + 4]), 0.0f);
        sum += m.w[j];
    }
    float inv = sum > 0.0f ? 1.0f / sum : 0.0f;
#pragma unroll
    for (int j = 0; j < kGuideLobes; j++)
        m.w[j] = sum > 0.0f ? m.w[j] * inv : 1.0f / kGuideLobes;
}

// Training records: one per recorded vertex (slot, k < depth), written by the
// shading kernels; `list` holds the indices of the written ones.
struct GuideRecords {
    float4* in0;    // scalars 0-3
    float4* in1;    // scalars 4-6, -
    float4* dir;    // sampled direction, -
    float4* fac;    // f cos / pdf of the sample (what the throughput was multiplied by)
    float4* mark;   // path radiance when the next vertex was reached
    float4* bnext;  // throughput at the next vertex
    float4* fin;    // per slot: the path's final radiance
    uint32_t* list;
    uint32_t* count;
    int depth;      // vertices recorded per path
    uint32_t capacity;  // slots * depth
};

}  // namespace mypbr_dev
