// Device-side helpers shared by the kernels: the device scene view, float3 arithmetic,
// exact-rounding helpers, the Halton sampler and the hash RNG.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../c2g_types.h"
#include "dev_scene.h"

namespace c2g {

__device__ __forceinline__ void dev_flag_error(int* err, int code) {
    if (err) atomicOr(err, code);
}

// ---- float3 ------------------------------------------------------------------------------
__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 f3(const float4& v) { return make_float3(v.x, v.y, v.z); }
__device__ __forceinline__ float3 f3(const float* p) { return make_float3(p[0], p[1], p[2]); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3 operator/(float3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross(float3 a, float3 b) {
    return f3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
__device__ __forceinline__ float3 normalize(float3 v) { return v * (1.0f / sqrtf(dot(v, v))); }
__device__ __forceinline__ float length(float3 v) { return sqrtf(dot(v, v)); }
__device__ __forceinline__ bool is_zero(float3 v) { return v.x == 0.f && v.y == 0.f && v.z == 0.f; }
__device__ __forceinline__ float3 clamp1(float3 v) {  // fixVector (Utils.h:163-166)
    return f3(fminf(fmaxf(v.x, -1.f), 1.f), fminf(fmaxf(v.y, -1.f), 1.f), fminf(fmaxf(v.z, -1.f), 1.f));
}
__device__ __forceinline__ bool any_nan_inf(float3 v) {
    return !isfinite(v.x) || !isfinite(v.y) || !isfinite(v.z);
}
// std::max / std::min as the reference uses them: max(a, b) = a < b ? b : a
__device__ __forceinline__ float smax(float a, float b) { return a < b ? b : a; }
__device__ __forceinline__ float smin(float a, float b) { return b < a ? b : a; }

// Exact-rounding vector helpers (no FMA contraction), for the arithmetic whose bits matter.
__device__ __forceinline__ float3 sub_rn(float3 a, float3 b) {
    return f3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
}
__device__ __forceinline__ float dot_rn(float3 a, float3 b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ float3 normalize_rn(float3 v) {
    float inv = __frcp_rn(__fsqrt_rn(dot_rn(v, v)));
    return f3(__fmul_rn(v.x, inv), __fmul_rn(v.y, inv), __fmul_rn(v.z, inv));
}

constexpr float kPiF = 3.14159265358979323846f;
constexpr float kTwoPiF = 6.28318530717958647692f;
constexpr float kHalfPiF = 1.57079632679489661923f;

// ---- hash RNG for Halton dims >= 100 -----------------------------------------------------
// The reference draws those dims from a shared, unsynchronised std::mt19937
// (HaltonSampler.cpp:285-288), which is not reproducible; here they come from a counter-based
// hash of (pixel, sample, dim, seed), uniform on [0, 1) with 24-bit resolution.
__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}
__device__ __forceinline__ float hash_uniform(uint32_t pixel, uint32_t sample, uint32_t dim, uint64_t seed) {
    uint32_t h = hash32(pixel ^ hash32(sample * 0x9E3779B9U ^ hash32(dim + 0x632BE5ABU * (uint32_t)seed) ^ (uint32_t)(seed >> 32)));
    float u = (float)(h >> 8) * 0x1p-24f;
    return fminf(u, kOneMinusEps);
}

// ---- Halton sampler (HaltonSampler.cpp:118-291) -----------------------------------------
__constant__ int c_primes[kHaltonDims];
__constant__ uint64_t c_divmagic[kHaltonDims];   // floor(2^64 / p) + 1: n / p == umul64hi(n, magic) for n < 2^32

__device__ __forceinline__ uint32_t div_prime(uint32_t n, int dim) {
    return (uint32_t)__umul64hi((uint64_t)n, c_divmagic[dim]);
}

// dim 0: ReverseBits64(v) * 2^-64 in double, narrowed to float (no clamp, :152-157)
__device__ __forceinline__ float halton_dim0(int vidx, const HaltonParams& hp) {
    uint64_t v = (uint64_t)(int64_t)(vidx >> hp.baseExponents[0]);
    double r = __dmul_rn(__ull2double_rn(__brevll(v)), 0x1p-64);
    return __double2float_rn(r);
}
// dim 1: base-3 radical inverse of vidx / scale1 (:118-132), float arithmetic in order
__device__ __forceinline__ float halton_dim1(int vidx, const HaltonParams& hp) {
    uint32_t v = (uint32_t)(vidx / hp.baseScales[1]);
    const float invBase = __frcp_rn(3.0f);
    float result = 0.f, invN = 1.0f;
    while (v) {
        uint32_t q = div_prime(v, 1);
        uint32_t digit = v - q * 3u;
        result = __fadd_rn(__fmul_rn(result, 3.0f), (float)digit);
        invN = __fmul_rn(invN, invBase);
        v = q;
    }
    return fminf(__fmul_rn(result, invN), kOneMinusEps);
}
// dims 2..99: permuted radical inverse (:134-149)
__device__ __forceinline__ float halton_scrambled(int vidx, int dim, const uint16_t* perm, const int* perm_off) {
    const int base = c_primes[dim];
    const uint16_t* tab = perm + __ldg(perm_off + dim);
    const float fb = (float)base;
    const float invBase = __frcp_rn(fb);
    float result = 0.f, invN = 1.0f;
    uint32_t v = (uint32_t)vidx;
    while (v) {
        uint32_t q = div_prime(v, dim);
        uint32_t r = v - q * (uint32_t)base;
        float digit = (float)__ldg(tab + r);
        result = __fadd_rn(__fmul_rn(result, fb), digit);
        invN = __fmul_rn(invN, invBase);
        v = q;
    }
    float p0 = (float)__ldg(tab);
    float tail = __fdiv_rn(__fmul_rn(invBase, p0), __fsub_rn(1.0f, invBase));
    return fminf(__fmul_rn(__fadd_rn(result, tail), invN), kOneMinusEps);
}

__device__ __forceinline__ float halton_sample(const DevScene& S, int vidx, int dim, uint32_t pixel, uint32_t sample) {
    if (dim == 0) return halton_dim0(vidx, S.hp);
    if (dim == 1) return halton_dim1(vidx, S.hp);
    if (dim < kHaltonDims) return halton_scrambled(vidx, dim, S.perm, S.perm_off);
    return hash_uniform(pixel, sample, (uint32_t)dim, S.seed);
}

// ---- Default and Stratified samplers (DefaultSampler.cpp, StratifiedSampler.cpp) -------------
// The reference draws both from one std::mt19937 per 32 x 32 tile that every path of the tile
// advances in turn, so a value depends on how many draws all earlier paths of the tile made: a
// sequential stream.  Here every (pixel, sample, dimension) has its own counter-based value, which
// keeps each draw uniform and independent like the reference's (Default), or stratified over the
// pixel's samples (Stratified), with no order between paths.
//
// Stratified: for each pixel and dimension the samples 0..spp-1 visit the spp strata (1D) or the
// side x side cells (2D) in a keyed random order and jitter uniformly inside them, as the
// reference's StratifiedSample1D/2D + std::shuffle tables do.  Every dimension is stratified (the
// reference stratifies the first 18 one- and two-dimensional requests of a sample and draws the
// rest plainly).  Sample indices past spp start a fresh stratified set per block of spp.

// A keyed bijection of [0, n): a four-round Feistel network (hash32 round function) on the
// smallest even bit width holding n, repeated while the value falls outside [0, n) (cycle
// walking; the cycle through i re-enters [0, n) within 2^bits rounds).  Different keys give
// statistically independent permutations, so the strata orders of two dimensions are unrelated
// and every sample stays jointly uniform over the dimensions.
__device__ __forceinline__ uint32_t permute_index(uint32_t i, uint32_t n, uint32_t key) {
    if (n <= 1) return 0;
    int bits = 32 - __clz(n - 1);
    bits = bits < 2 ? 2 : bits + (bits & 1);
    if (bits > 30) return i;  // sample counts beyond 2^30 are not stratified
    const int half = bits >> 1;
    const uint32_t hmask = (1u << half) - 1u;
    uint32_t rk[4];
#pragma unroll
    for (uint32_t r = 0; r < 4; r++) rk[r] = hash32(key ^ r);
    uint32_t x = i;
    for (uint32_t it = 0; it < (1u << bits); it++) {
        uint32_t L = x >> half, R = x & hmask;
#pragma unroll
        for (uint32_t r = 0; r < 4; r++) {
            const uint32_t F = hash32(R * 0x27d4eb2dU ^ rk[r]) & hmask;
            const uint32_t t = L ^ F;
            L = R;
            R = t;
        }
        x = (L << half) | R;
        if (x < n) break;
    }
    return x;
}
__device__ __forceinline__ uint32_t strata_key(uint32_t pixel, uint32_t block, uint32_t dim, uint64_t seed) {
    return hash32(pixel * 0x9E3779B9U ^ hash32(dim * 0x632BE5ABU ^ hash32(block ^ (uint32_t)seed)));
}
__device__ __forceinline__ float path_sample1(const DevScene& S, int vidx, int dim, uint32_t pixel, uint32_t sample) {
    if (S.sampler == SAMPLER_HALTON) return halton_sample(S, vidx, dim, pixel, sample);
    const float j = hash_uniform(pixel, sample, (uint32_t)dim, S.seed);
    if (S.sampler == SAMPLER_DEFAULT) return j;
    const uint32_t n = (uint32_t)S.spp, s = sample % n;
    const uint32_t cell = permute_index(s, n, strata_key(pixel, sample / n, (uint32_t)dim, S.seed));
    return fminf(__fmul_rn(__frcp_rn((float)n), __fadd_rn((float)cell, j)), kOneMinusEps);
}
__device__ __forceinline__ float2 path_sample2(const DevScene& S, int vidx, int dim, uint32_t pixel, uint32_t sample) {
    if (S.sampler == SAMPLER_HALTON) {
        if (dim == 0) return make_float2(halton_dim0(vidx, S.hp), halton_dim1(vidx, S.hp));
        return make_float2(halton_sample(S, vidx, dim, pixel, sample), halton_sample(S, vidx, dim + 1, pixel, sample));
    }
    const float jx = hash_uniform(pixel, sample, (uint32_t)dim, S.seed);
    const float jy = hash_uniform(pixel, sample, (uint32_t)dim + 1u, S.seed);
    if (S.sampler == SAMPLER_DEFAULT) return make_float2(jx, jy);
    const uint32_t n = (uint32_t)S.spp, s = sample % n, side = (uint32_t)S.strata_side;
    const uint32_t cell = permute_index(s, n, strata_key(pixel, sample / n, (uint32_t)dim, S.seed));
    const uint32_t row = cell / side, col = cell - row * side;
    const float inv = __frcp_rn((float)side);
    return make_float2(fminf(__fmul_rn(inv, __fadd_rn((float)col, jx)), kOneMinusEps),
                       fminf(__fmul_rn(inv, __fadd_rn((float)row, jy)), kOneMinusEps));
}

// GetVectorIndexForSample (HaltonSampler.cpp:251-270), integer arithmetic as the reference.
__device__ __forceinline__ int halton_vector_index(const HaltonParams& hp, int px, int py, int sample) {
    long long off = 0;
    if (hp.sampleStride > 1) {
        int pm[2] = {px % kMaxResolution, py % kMaxResolution};
        for (int i = 0; i < 2; i++) {
            int base = i == 0 ? 2 : 3;
            unsigned long long v = (unsigned long long)(long long)pm[i], rem = 0;
            for (int k = 0; k < hp.baseExponents[i]; k++) { rem = rem * base + (v % base); v /= base; }
            off += (long long)(rem * (unsigned long long)(long long)hp.baseScales[!i] *
                               (unsigned long long)(long long)hp.multInverse[i]);
        }
    }
    return (int)(off + (long long)(sample * hp.sampleStride));
}

// PerspCamera::GenerateRay (PerspCamera.cpp:23-29) with the reference's float rounding.
__device__ __forceinline__ void camera_ray(const Camera& c, float px, float py, float3& o, float3& d) {
    px = __fsub_rn(__fmul_rn(px, 2.0f), 1.0f);
    py = __fsub_rn(__fmul_rn(py, 2.0f), 1.0f);
    px = __fmul_rn(px, c.W);
    py = __fmul_rn(py, c.H);
    float3 r = f3(c.right), u = f3(c.up), l = f3(c.look);
    // _right * x + _up * y + _look * zNear, left to right
    float3 v = f3(__fadd_rn(__fadd_rn(__fmul_rn(r.x, px), __fmul_rn(u.x, py)), __fmul_rn(l.x, c.zNear)),
                  __fadd_rn(__fadd_rn(__fmul_rn(r.y, px), __fmul_rn(u.y, py)), __fmul_rn(l.y, c.zNear)),
                  __fadd_rn(__fadd_rn(__fmul_rn(r.z, px), __fmul_rn(u.z, py)), __fmul_rn(l.z, c.zNear)));
    d = normalize_rn(v);
    o = f3(c.eye);
}

// Film-position of sample s of pixel (x, y): (x + s.x) / W, (y + s.y) / H (SamplerIntegrator.cpp:49-53)
__device__ __forceinline__ void pixel_ndc(int x, int y, float sx, float sy, int W, int H, float& nx, float& ny) {
    nx = __fdiv_rn(__fadd_rn((float)x, sx), (float)W);
    ny = __fdiv_rn(__fadd_rn((float)y, sy), (float)H);
}

}  // namespace c2g
