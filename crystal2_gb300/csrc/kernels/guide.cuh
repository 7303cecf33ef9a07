// Learned path-guiding proposal: the network's shapes and the directional mixture it
// parameterises.
//
// Network: 80 inputs (position p in the scene box, normalised to [0, 1]^3 and encoded as
// sin/cos(pi 2^f p) for f = 0..11 per axis = 72; shading normal 3; outgoing direction 3; 2 zeros),
// three hidden ReLU layers of 64, 40 outputs = 8 lobes x (mean direction 3, concentration 1,
// weight logit 1) and the technique-selection logit.  The mixture is a sum of von Mises-Fisher
// lobes on the sphere, which has a closed-form pdf and an exact sampling routine, so the guided
// estimator can use exactly evaluated pdfs.
//
// Matrix products run on the fifth-generation tensor cores (tcgen05.mma, BF16 operands in shared
// memory, FP32 accumulators in tensor memory; guide.cu).  Weight layout per layer l (K_l inputs,
// N_l outputs): `wt` = N_l x K_l row-major BF16 (staged K-major for x @ W, and read MN-major for
// delta @ W^T), `wn` = K_l x N_l row-major BF16, bias FP32.
#pragma once
#include <cuda_bf16.h>

#include "dev_common.cuh"
#include "guide.h"

namespace c2g {

// ---- BF16 packing --------------------------------------------------------------------------
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}
// ReLU and BF16 rounding of two values in one conversion (negative values become +0; a NaN stays
// a NaN, so a non-finite layer still marks the mixture invalid).
__device__ __forceinline__ uint32_t pack_bf16_relu(float lo, float hi) {
    uint32_t r;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}

// ---- the directional mixture -----------------------------------------------------------------
struct Lobe {
    float3 mu;
    float kappa;
    float w;       // mixture weight (softmax)
};

__device__ __forceinline__ float softplusf(float x) { return x > 15.f ? x : log1pf(__expf(x)); }

// Raw outputs (mx, my, mz, kraw, logit) x 8 -> lobes.  kappa = min(softplus(kraw) + 0.05, kappa_max).
__device__ __forceinline__ void guide_lobes(const float* out, Lobe* L, float kappa_max) {
    float mx = -INFINITY;
#pragma unroll
    for (int k = 0; k < kGuideLobes; k++) mx = fmaxf(mx, out[5 * k + 4]);
    float sum = 0.f;
#pragma unroll
    for (int k = 0; k < kGuideLobes; k++) {
        float3 m = f3(out[5 * k], out[5 * k + 1], out[5 * k + 2]);
        float len = sqrtf(dot(m, m));
        L[k].mu = len > 1e-12f ? m * (1.f / len) : f3(0.f, 1.f, 0.f);
        L[k].kappa = fminf(softplusf(out[5 * k + 3]) + 0.05f, kappa_max);
        L[k].w = __expf(out[5 * k + 4] - mx);
        sum += L[k].w;
    }
    float inv = 1.f / sum;
#pragma unroll
    for (int k = 0; k < kGuideLobes; k++) L[k].w *= inv;
}

// vMF density on the unit sphere: kappa / (2 pi (1 - e^-2kappa)) * exp(kappa (mu.w - 1)).
__device__ __forceinline__ float vmf_pdf(const Lobe& l, float3 w) {
    float c = dot(l.mu, w);
    return l.kappa / (2.f * kPiF * (-expm1f(-2.f * l.kappa))) * __expf(l.kappa * (c - 1.f));
}

// Bucket ids whose hits are guided: the non-specular materials whose BSDF sampling routine returns
// the exact density of the directions it draws (the mixture pdf needs it at guide-drawn directions).
__host__ __device__ constexpr bool bucket_guided(int b) {
    return b == MAT_DIFFUSE || b == MAT_MICRO_GGX || b == MAT_MICRO_BECKMANN || b == MAT_PLASTIC_GGX ||
           b == MAT_PLASTIC_BECKMANN || b == MAT_ORENNAYAR;
}

// Work item of the guided vertices that sits at position `pos` of bucket MT's list: the guided
// buckets' lists back to back in bucket order (the order inference runs over them).
template <int MT>
__device__ __forceinline__ int guided_item(const int* bucket_cnt, int pos) {
    int base = 0;
#pragma unroll
    for (int b = 0; b < MT; b++)
        if (bucket_guided(b)) base += __ldg(bucket_cnt + b);
    return base + pos;
}

// ---- packed mixture (inference output, read by the shading kernels) ---------------------------
// Per guided work item kGuidePacked floats as 13 float4 fields: 8 (mean direction, concentration),
// the 8 lobe weights (fields 8-9), the 8 products weight x vMF normaliser (10-11), and the
// probability c of drawing from the mixture rather than the BSDF (12.x).  A non-finite network
// output is flagged by a NaN first weight.  Field-major: field f of item j is float4 f * stride + j
// (stride: the wave's path capacity), so a warp's 32 consecutive items read and write each field
// as one contiguous 512-byte run.
constexpr int kGuidePacked = 52;
constexpr int kGuideFields = kGuidePacked / 4;
struct PackedMix {
    const float4* p;   // field 0 of this item
    int s;             // field stride in float4
    __device__ __forceinline__ float4 f(int k) const { return __ldg(p + (size_t)k * s); }
};

// Technique selection: c = 0.05 + 0.75 sigmoid(s) keeps both techniques in use; at least a fifth
// of the continuations follow the BSDF (a defensive mixture: a mixture that trained onto a few
// sharp lobes cannot make the weights larger than 5x the BSDF-only ones).
__host__ __device__ __forceinline__ float guide_select(float s) { return kGuideSelMin + kGuideSelSpan / (1.f + expf(-s)); }

// d4: field 0 of the item; stride: the field stride in float4.
__device__ __forceinline__ void pack_lobes(const float* out, float4* d4, int stride, float kappa_max) {
    bool finite = true;
#pragma unroll
    for (int k = 0; k < kGuideOut; k++) finite = finite && isfinite(out[k]);
    Lobe L[kGuideLobes];
    guide_lobes(out, L, kappa_max);
    const size_t s = (size_t)stride;
#pragma unroll
    for (int k = 0; k < kGuideLobes; k++) d4[k * s] = make_float4(L[k].mu.x, L[k].mu.y, L[k].mu.z, L[k].kappa);
    float w[kGuideLobes], wc[kGuideLobes];
#pragma unroll
    for (int k = 0; k < kGuideLobes; k++) {
        w[k] = L[k].w;
        wc[k] = L[k].w * L[k].kappa / (2.f * kPiF * (-expm1f(-2.f * L[k].kappa)));
    }
    if (!finite) w[0] = __int_as_float(0x7fc00000);
    d4[8 * s] = make_float4(w[0], w[1], w[2], w[3]);
    d4[9 * s] = make_float4(w[4], w[5], w[6], w[7]);
    d4[10 * s] = make_float4(wc[0], wc[1], wc[2], wc[3]);
    d4[11 * s] = make_float4(wc[4], wc[5], wc[6], wc[7]);
    d4[12 * s] = make_float4(guide_select(out[40]), 0.f, 0.f, 0.f);
}

__device__ __forceinline__ float f4_at(const float4& v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w)); }

// Probability of drawing the continuation from the mixture (vs the BSDF).
__device__ __forceinline__ float packed_select(const PackedMix& p) { return p.f(12).x; }

__device__ __forceinline__ bool packed_valid(const PackedMix& p) { return isfinite(p.f(8).x); }

// Mixture density at the unit direction w.  Kept out of line: the shading kernel calls it per
// light and per continuation, and one copy keeps its instruction footprint small.
static __device__ __noinline__ float packed_pdf(const PackedMix p, float3 w) {
    const float4 wc0 = p.f(10), wc1 = p.f(11);
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < kGuideLobes; k++) {
        const float4 m = p.f(k);
        const float wc = k < 4 ? f4_at(wc0, k) : f4_at(wc1, k - 4);
        s += wc * __expf(m.w * (m.x * w.x + m.y * w.y + m.z * w.z - 1.f));
    }
    return s;
}

// Sample: lobe by weight with u0, then the vMF around its mean (w = cos theta by inversion).
static __device__ __noinline__ float3 packed_sample(const PackedMix p, float u0, float u1, float u2) {
    const float4 w0 = p.f(8), w1 = p.f(9);
    int k = kGuideLobes - 1;
    float acc = 0.f;
#pragma unroll
    for (int i = 0; i < kGuideLobes; i++) {
        acc += i < 4 ? f4_at(w0, i) : f4_at(w1, i - 4);
        if (u0 < acc) { k = i; break; }
    }
    const float4 l = p.f(k);
    const float kappa = l.w;
    const float e = __expf(-2.f * kappa);
    float cw = 1.f + __logf(fmaxf(u1 + (1.f - u1) * e, 1e-30f)) / kappa;
    cw = fminf(fmaxf(cw, -1.f), 1.f);
    const float sw = sqrtf(fmaxf(0.f, 1.f - cw * cw));
    float s, c;
    __sincosf(kTwoPiF * u2, &s, &c);
    // orthonormal basis around mu (Duff et al. 2017, "Building an Orthonormal Basis, Revisited")
    const float3 m = f3(l.x, l.y, l.z);
    const float sign = copysignf(1.f, m.z);
    const float a = -1.f / (sign + m.z);
    const float b = m.x * m.y * a;
    const float3 t1 = f3(1.f + sign * m.x * m.x * a, sign * b, -sign * m.x);
    const float3 t2 = f3(b, sign + m.y * m.y * a, -m.y);
    return normalize(t1 * (sw * c) + t2 * (sw * s) + m * cw);
}

}  // namespace c2g
