// Learned path-guiding proposal: input encoding, the BF16 tensor-core MLP, and the directional
// mixture it parameterises.
//
// Network: 80 inputs (position p in the scene box, normalised to [0, 1]^3 and encoded as
// sin/cos(pi 2^f p) for f = 0..11 per axis = 72; shading normal 3; outgoing direction 3; 2 zeros),
// three hidden ReLU layers of 64, 40 outputs = 8 lobes x (mean direction 3, concentration 1,
// weight logit 1).  The mixture is a sum of
// von Mises-Fisher lobes on the sphere, which has a closed-form pdf and an exact sampling routine,
// so the guided estimator can use exactly evaluated pdfs.
//
// Matrix products use the warp-level tensor-core instruction mma.sync.m16n8k16 (BF16 inputs, FP32
// accumulators) on 16-row tiles held in shared memory (guide.cu).  Weight layout per layer l (K_l inputs,
// N_l outputs): `wt` = N_l x K_l row-major BF16 (the B operand of x @ W), `wn` = K_l x N_l row-major
// BF16 (the B operand of delta @ W^T), bias FP32.
#pragma once
#include <cuda_bf16.h>

#include "dev_common.cuh"
#include "guide.h"

namespace c2g {

// ---- input encoding ------------------------------------------------------------------------
__device__ __forceinline__ void guide_encode(const GuideNet& g, float3 x, float3 n, float3 wo, float* in) {
    float p[3] = {(x.x - g.box_lo[0]) * g.box_inv[0], (x.y - g.box_lo[1]) * g.box_inv[1], (x.z - g.box_lo[2]) * g.box_inv[2]};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        float v = fminf(fmaxf(p[a], 0.f), 1.f);
        // sin/cos(pi v) with exact argument reduction, then the double-angle recurrence
        // sin 2u = 2 sin u cos u, cos 2u = (cos u - sin u)(cos u + sin u) for the higher frequencies
        // (the absolute error grows about 2x per octave: ~1e-4 at 2^11, far below BF16 resolution)
        float s, c;
        sincospif(v, &s, &c);
#pragma unroll
        for (int f = 0; f < kGuideFreqs; f++) {
            in[a * 2 * kGuideFreqs + 2 * f] = s;
            in[a * 2 * kGuideFreqs + 2 * f + 1] = c;
            const float s2 = 2.f * s * c, c2 = (c - s) * (c + s);
            s = s2;
            c = c2;
        }
    }
    in[72] = n.x; in[73] = n.y; in[74] = n.z;
    in[75] = wo.x; in[76] = wo.y; in[77] = wo.z;
    in[78] = 0.f; in[79] = 0.f;
}

// ---- tensor-core tile helpers ----------------------------------------------------------------
__device__ __forceinline__ void mma16816(float* d, const uint32_t* a, const uint32_t* b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

// ---- the directional mixture -----------------------------------------------------------------
struct Lobe {
    float3 mu;
    float kappa;
    float w;       // mixture weight (softmax)
};

__device__ __forceinline__ float softplusf(float x) { return x > 15.f ? x : log1pf(__expf(x)); }

// Raw outputs (mx, my, mz, kraw, logit) x 8 -> lobes.  kappa = softplus(kraw) + 0.05.
__device__ __forceinline__ void guide_lobes(const float* out, Lobe* L) {
    float mx = -INFINITY;
#pragma unroll
    for (int k = 0; k < kGuideLobes; k++) mx = fmaxf(mx, out[5 * k + 4]);
    float sum = 0.f;
#pragma unroll
    for (int k = 0; k < kGuideLobes; k++) {
        float3 m = f3(out[5 * k], out[5 * k + 1], out[5 * k + 2]);
        float len = sqrtf(dot(m, m));
        L[k].mu = len > 1e-12f ? m * (1.f / len) : f3(0.f, 1.f, 0.f);
        L[k].kappa = fminf(softplusf(out[5 * k + 3]) + 0.05f, 2000.f);
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

__device__ __forceinline__ float guide_pdf(const Lobe* L, float3 w) {
    float p = 0.f;
#pragma unroll
    for (int k = 0; k < kGuideLobes; k++) p += L[k].w * vmf_pdf(L[k], w);
    return p;
}

// Sample: lobe by weight with u0 (rescaled), then the vMF around its mean (w = cos theta).
__device__ __forceinline__ float3 guide_sample(const Lobe* L, float u0, float u1, float u2) {
    int k = kGuideLobes - 1;
    float acc = 0.f;
#pragma unroll
    for (int i = 0; i < kGuideLobes; i++) {
        if (u0 < acc + L[i].w) { k = i; break; }
        acc += L[i].w;
    }
    // select the chosen lobe without dynamic register indexing
    Lobe l = L[0];
#pragma unroll
    for (int i = 1; i < kGuideLobes; i++)
        if (i == k) l = L[i];
    float e = __expf(-2.f * l.kappa);
    float cw = 1.f + __logf(fmaxf(u1 + (1.f - u1) * e, 1e-30f)) / l.kappa;
    cw = fminf(fmaxf(cw, -1.f), 1.f);
    float sw = sqrtf(fmaxf(0.f, 1.f - cw * cw));
    float s, c;
    __sincosf(kTwoPiF * u2, &s, &c);
    // orthonormal basis around mu (Duff et al. 2017, "Building an Orthonormal Basis, Revisited")
    float3 m = l.mu;
    float sign = copysignf(1.f, m.z);
    float a = -1.f / (sign + m.z);
    float b = m.x * m.y * a;
    float3 t1 = f3(1.f + sign * m.x * m.x * a, sign * b, -sign * m.x);
    float3 t2 = f3(b, sign + m.y * m.y * a, -m.y);
    return normalize(t1 * (sw * c) + t2 * (sw * s) + m * cw);
}

}  // namespace c2g
