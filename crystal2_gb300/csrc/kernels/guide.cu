// Learned guiding proposal: inference over shading buckets, online training (fused forward +
// backward on tensor-core tiles, FP32 weight-gradient reduction) and the Adam update.
//
// Training target (neural importance sampling, Mueller et al. 2019): minimise the KL divergence
// from the product f(wo, wi) cos(wi) Li(wi) to the mixture q(wi | x, n, wo).  Its gradient is
// estimated from the path tracer's own vertices as  sum_j w_j * grad(-log q(wi_j)) / sum_j w_j  with
// w_j = f cos Li / p(wi_j), the Monte Carlo weight of the continuation direction the tracer
// sampled; w_j is recovered after the path ends as (luminance of the radiance gathered beyond the
// vertex) / (luminance of the vertex throughput).
#include <cuda_bf16.h>

#include <cmath>
#include <random>
#include <vector>

#include "guide.cuh"
#include "render.h"
#include "shade.cuh"

namespace c2g {

namespace {

constexpr int kLdA0 = 88;    // 80 + 8 (bank-conflict-free rows)
constexpr int kLdH = 72;     // 64 + 8
constexpr int kLdO = 56;     // 48 + 8 (BF16 output gradients)
constexpr int kLdF = 48;     // FP32 outputs (forward)
constexpr int kLdG = 68;     // FP32 scratch of the training kernel (64 columns + 4)

__device__ __forceinline__ float luminance(float3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

// Bucket ids whose hits are guided: the non-specular materials whose BSDF sampling routine returns
// the exact density of the directions it draws (the mixture pdf needs it at guide-drawn directions).
__host__ __device__ constexpr bool bucket_guided(int b) {
    return b == MAT_DIFFUSE || b == MAT_MICRO_GGX || b == MAT_MICRO_BECKMANN || b == MAT_PLASTIC_GGX ||
           b == MAT_PLASTIC_BECKMANN;
}

// Forward pass of one warp's 32 samples: `in` (per lane, FP32) -> F (32 x kLdF FP32 outputs).
// `wts` = the four wt_l matrices back to back (shared memory); A, Bb = two per-warp BF16 tiles.
// F aliases A.
__device__ __forceinline__ void warp_forward(const GuideNet& net, const __nv_bfloat16* wts, const float* in,
                                             __nv_bfloat16* A, __nv_bfloat16* Bb, float* F) {
    const int lane = threadIdx.x & 31;
    constexpr int o1 = kGuideIn * kGuideHidden, o2 = o1 + kGuideHidden * kGuideHidden, o3 = o2 + kGuideHidden * kGuideHidden;
#pragma unroll
    for (int k = 0; k < kGuideIn; k += 2)
        *reinterpret_cast<uint32_t*>(A + lane * kLdA0 + k) = pack_bf16(in[k], in[k + 1]);
    __syncwarp();
    for (int m = 0; m < 2; m++)
        tile_layer<80, 64>(A + m * 16 * kLdA0, kLdA0, wts, net.params + guide_b_off(0), Bb + m * 16 * kLdH, kLdH, true, nullptr, 0);
    __syncwarp();
    for (int m = 0; m < 2; m++)
        tile_layer<64, 64>(Bb + m * 16 * kLdH, kLdH, wts + o1, net.params + guide_b_off(1), A + m * 16 * kLdH, kLdH, true, nullptr, 0);
    __syncwarp();
    for (int m = 0; m < 2; m++)
        tile_layer<64, 64>(A + m * 16 * kLdH, kLdH, wts + o2, net.params + guide_b_off(2), Bb + m * 16 * kLdH, kLdH, true, nullptr, 0);
    __syncwarp();
    for (int m = 0; m < 2; m++)
        tile_layer<64, 48>(Bb + m * 16 * kLdH, kLdH, wts + o3, net.params + guide_b_off(3), nullptr, 0, false, F + m * 16 * kLdF, kLdF);
    __syncwarp();
}

// Copy the forward weights (wt_0..wt_3) into shared memory.
__device__ __forceinline__ void stage_forward_weights(const GuideNet& net, __nv_bfloat16* wts) {
    constexpr int o1 = kGuideIn * kGuideHidden, o2 = o1 + kGuideHidden * kGuideHidden, o3 = o2 + kGuideHidden * kGuideHidden;
    constexpr int total = o3 + kGuideHidden * kGuideOutPad;
    for (int i = threadIdx.x; i < total; i += blockDim.x) {
        int l = i >= o3 ? 3 : i >= o2 ? 2 : i >= o1 ? 1 : 0;
        int base = l == 3 ? o3 : l == 2 ? o2 : l == 1 ? o1 : 0;
        wts[i] = net.bf[guide_bf_off(l) + (i - base)];
    }
    __syncthreads();
}

// ---- inference ---------------------------------------------------------------------------------
// 128 threads; dynamic shared memory: forward weights (32 KB) + two per-warp tiles.
constexpr int kInferWarps = 4;
constexpr int kTileBytes = 32 * kLdF * 4;  // 6144: holds 32 x 88 BF16 rows or 32 x 48 FP32 rows

__global__ void __launch_bounds__(128) k_guide_infer(DevScene S, GuideNet net, const float4* __restrict__ ray_o,
                                                     const float4* __restrict__ ray_d, const float4* __restrict__ hits,
                                                     const int* bucket_cnt, const int* __restrict__ bucket_list, int cap,
                                                     int mask, float* out) {
    extern __shared__ __align__(16) unsigned char smem[];
    __nv_bfloat16* wts = reinterpret_cast<__nv_bfloat16*>(smem);  // wt_0 .. wt_3 back to back
    stage_forward_weights(net, wts);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* wbase = smem + 2 * 16384 + warp * 2 * kTileBytes;
    __nv_bfloat16* A = reinterpret_cast<__nv_bfloat16*>(wbase);
    __nv_bfloat16* Bb = reinterpret_cast<__nv_bfloat16*>(wbase + kTileBytes);
    float* F = reinterpret_cast<float*>(wbase);
    // work list = the guided buckets back to back
    int total = 0;
    int bstart[10], bcnt[10];
    for (int b = 0; b < 10; b++) {
        bstart[b] = total;
        bcnt[b] = ((mask >> b) & 1) ? bucket_cnt[b] : 0;
        total += bcnt[b];
    }
    const int gwarp = blockIdx.x * kInferWarps + warp, nwarps = gridDim.x * kInferWarps;
    for (int base = gwarp * 32; base < total; base += nwarps * 32) {
        int item = base + lane;
        int slot = -1;
        if (item < total) {
            int b = 0;
            while (b < 9 && item >= bstart[b] + bcnt[b]) b++;
            slot = bucket_list[(size_t)b * cap + (item - bstart[b])];
        }
        float in[kGuideIn];
        if (slot >= 0) {
            float4 o4 = ray_o[slot], d4 = ray_d[slot], h4 = hits[slot];
            Hit h{h4.x, h4.y, h4.z, __float_as_int(h4.w)};
            Surface s;
            make_surface(S, f3(o4), f3(d4), h, s);
            guide_encode(net, s.pos, s.N, -f3(d4), in);
        } else {
#pragma unroll
            for (int k = 0; k < kGuideIn; k++) in[k] = 0.f;
        }
        warp_forward(net, wts, in, A, Bb, F);
        if (slot >= 0) {
            float* dst = out + (size_t)slot * kGuideOut;
#pragma unroll
            for (int k = 0; k < kGuideOut; k++) dst[k] = F[lane * kLdF + k];
        }
        __syncwarp();
    }
}

// Forward pass over explicit inputs (x, n, wo as 9 floats per sample): the same tiles as
// k_guide_infer, used to check the network against the oracle.
__global__ void __launch_bounds__(128) k_guide_eval(GuideNet net, const float* __restrict__ xnw, int n, float* out) {
    extern __shared__ __align__(16) unsigned char smem[];
    __nv_bfloat16* wts = reinterpret_cast<__nv_bfloat16*>(smem);
    stage_forward_weights(net, wts);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* wbase = smem + 2 * 16384 + warp * 2 * kTileBytes;
    __nv_bfloat16* A = reinterpret_cast<__nv_bfloat16*>(wbase);
    __nv_bfloat16* Bb = reinterpret_cast<__nv_bfloat16*>(wbase + kTileBytes);
    float* F = reinterpret_cast<float*>(wbase);
    const int gwarp = blockIdx.x * kInferWarps + warp, nwarps = gridDim.x * kInferWarps;
    for (int base = gwarp * 32; base < n; base += nwarps * 32) {
        const int j = base + lane;
        float in[kGuideIn];
        if (j < n) {
            const float* v = xnw + (size_t)9 * j;
            guide_encode(net, f3(v[0], v[1], v[2]), f3(v[3], v[4], v[5]), f3(v[6], v[7], v[8]), in);
        } else {
#pragma unroll
            for (int k = 0; k < kGuideIn; k++) in[k] = 0.f;
        }
        warp_forward(net, wts, in, A, Bb, F);
        if (j < n) {
#pragma unroll
            for (int k = 0; k < kGuideOut; k++) out[(size_t)j * kGuideOut + k] = F[lane * kLdF + k];
        }
        __syncwarp();
    }
}

// ---- records -> weighted training samples ------------------------------------------------------
// Record (4 float4): (x, valid), (n, lum L at the vertex after its direct light), (wo, lum beta at
// the vertex), (wi, 0).  Sample (4 float4): (x, w), (n, 0), (wo, 0), (wi, 0).
__global__ void k_guide_batch(float4* rec, int rec_cap, int rec_depth, int rec_stride, const float4* __restrict__ out_L,
                              int wave_paths, float4* batch, int* batch_count, float* stats, int batch_cap) {
    const int stride = gridDim.x * blockDim.x;
    for (int base = blockIdx.x * blockDim.x; base < rec_cap; base += stride) {
        int r = base + threadIdx.x;
        bool ok = false;
        float4 r0, r1, r2, r3;
        float w = 0.f;
        if (r < rec_cap) {
            r0 = rec[4 * r];
            if (r0.w != 0.f) {
                r1 = rec[4 * r + 1];
                r2 = rec[4 * r + 2];
                r3 = rec[4 * r + 3];
                rec[4 * r] = make_float4(0.f, 0.f, 0.f, 0.f);  // consumed
                int pid = (r / rec_depth) * rec_stride;
                if (pid < wave_paths) {
                    float Lend = luminance(f3(out_L[pid]));
                    w = (Lend - r1.w) / fmaxf(r2.w, 1e-8f);
                    ok = isfinite(w) && w > 0.f;
                }
            }
        }
        unsigned m = __ballot_sync(0xffffffffu, ok);
        int basei = 0;
        if ((threadIdx.x & 31) == 0 && m) basei = atomicAdd(batch_count, __popc(m));
        basei = __shfl_sync(0xffffffffu, basei, 0);
        int j = basei + __popc(m & ((1u << (threadIdx.x & 31)) - 1u));
        if (ok && j < batch_cap) {
            batch[4 * j] = make_float4(r0.x, r0.y, r0.z, w);
            batch[4 * j + 1] = make_float4(r1.x, r1.y, r1.z, 0.f);
            batch[4 * j + 2] = make_float4(r2.x, r2.y, r2.z, 0.f);
            batch[4 * j + 3] = make_float4(r3.x, r3.y, r3.z, 0.f);
            atomicAdd(stats + 2, w);
        }
    }
}

// ---- fused training step: forward + backward on tensor-core tiles, weight gradients in FP32 ----
constexpr int kTrainWarps = 2;
constexpr int kWarpTrainBytes = 32 * kLdA0 * 2 + 6 * 32 * kLdH * 2 + 32 * kLdG * 4 + 32 * kLdO * 2;

__device__ __forceinline__ float bf(const __nv_bfloat16* p) { return __bfloat162float(*p); }

__global__ void __launch_bounds__(64) k_guide_train(GuideNet net, const float4* __restrict__ batch, const int* batch_count,
                                                    int batch_cap, float* grad, float* stats) {
    extern __shared__ __align__(16) unsigned char smem[];
    float* gacc = reinterpret_cast<float*>(smem);  // kGuideParams block-local gradient sums
    for (int i = threadIdx.x; i < kGuideParams; i += blockDim.x) gacc[i] = 0.f;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* wb = smem + kGuideParams * 4 + warp * kWarpTrainBytes;
    __nv_bfloat16* a0 = reinterpret_cast<__nv_bfloat16*>(wb);
    __nv_bfloat16* h1 = a0 + 32 * kLdA0;
    __nv_bfloat16* h2 = h1 + 32 * kLdH;
    __nv_bfloat16* h3 = h2 + 32 * kLdH;
    __nv_bfloat16* d1 = h3 + 32 * kLdH;   // gradient at the input of layer 1 (masked by h1)
    __nv_bfloat16* d2 = d1 + 32 * kLdH;
    __nv_bfloat16* d3 = d2 + 32 * kLdH;
    float* of = reinterpret_cast<float*>(d3 + 32 * kLdH);
    __nv_bfloat16* dout = reinterpret_cast<__nv_bfloat16*>(of + 32 * kLdG);
    __syncthreads();
    const int n = min(*batch_count, batch_cap);
    const float mean_w = stats[2] / fmaxf(1.f, (float)n);
    const __nv_bfloat16* wt[4];
    const __nv_bfloat16* wn[4];
    for (int l = 0; l < 4; l++) {
        wt[l] = net.bf + guide_bf_off(l);
        wn[l] = wt[l] + guide_k(l) * guide_n(l);
    }
    float loss = 0.f, wsum = 0.f;
    const int per_iter = kTrainWarps * 32;
    for (int base = blockIdx.x * per_iter; base < n; base += gridDim.x * per_iter) {
        const int j = base + warp * 32 + lane;
        const bool valid = j < n;
        float in[kGuideIn];
        float3 wi = f3(0.f, 0.f, 1.f);
        float w = 0.f;
        if (valid) {
            float4 b0 = batch[4 * j], b1 = batch[4 * j + 1], b2 = batch[4 * j + 2], b3 = batch[4 * j + 3];
            guide_encode(net, f3(b0), f3(b1), f3(b2), in);
            wi = f3(b3);
            w = fminf(b0.w / fmaxf(mean_w, 1e-12f), 100.f);  // normalised, firefly-clamped weight
        } else {
#pragma unroll
            for (int k = 0; k < kGuideIn; k++) in[k] = 0.f;
        }
#pragma unroll
        for (int k = 0; k < kGuideIn; k += 2) *reinterpret_cast<uint32_t*>(a0 + lane * kLdA0 + k) = pack_bf16(in[k], in[k + 1]);
        __syncwarp();
        for (int m = 0; m < 2; m++) tile_layer<80, 64>(a0 + m * 16 * kLdA0, kLdA0, wt[0], net.params + guide_b_off(0), h1 + m * 16 * kLdH, kLdH, true, nullptr, 0);
        __syncwarp();
        for (int m = 0; m < 2; m++) tile_layer<64, 64>(h1 + m * 16 * kLdH, kLdH, wt[1], net.params + guide_b_off(1), h2 + m * 16 * kLdH, kLdH, true, nullptr, 0);
        __syncwarp();
        for (int m = 0; m < 2; m++) tile_layer<64, 64>(h2 + m * 16 * kLdH, kLdH, wt[2], net.params + guide_b_off(2), h3 + m * 16 * kLdH, kLdH, true, nullptr, 0);
        __syncwarp();
        for (int m = 0; m < 2; m++) tile_layer<64, 48>(h3 + m * 16 * kLdH, kLdH, wt[3], net.params + guide_b_off(3), nullptr, 0, false, of + m * 16 * kLdG, kLdG);
        __syncwarp();
        // loss gradient at the 40 outputs (per lane, FP32)
        float g[kGuideOutPad];
#pragma unroll
        for (int k = 0; k < kGuideOutPad; k++) g[k] = 0.f;
        if (valid && w > 0.f) {
            float o[kGuideOut];
#pragma unroll
            for (int k = 0; k < kGuideOut; k++) o[k] = of[lane * kLdG + k];
            Lobe L[kGuideLobes];
            guide_lobes(o, L);
            float p[kGuideLobes], q = 0.f;
#pragma unroll
            for (int k = 0; k < kGuideLobes; k++) { p[k] = L[k].w * vmf_pdf(L[k], wi); q += p[k]; }
            q = fmaxf(q, 1e-20f);
            loss += w * -__logf(q);
            wsum += w;
#pragma unroll
            for (int k = 0; k < kGuideLobes; k++) {
                float r = p[k] / q;
                float kap = L[k].kappa;
                float c = dot(L[k].mu, wi);
                // d log vMF / d kappa = 1/kappa - 2 e^-2k / (1 - e^-2k) + (mu.wi - 1)
                float e2 = __expf(-2.f * kap);
                float dk = 1.f / kap - 2.f * e2 / fmaxf(-expm1f(-2.f * kap), 1e-20f) + (c - 1.f);
                float kraw = o[5 * k + 3];
                float sig = 1.f / (1.f + __expf(-kraw));
                if (kap >= 2000.f) sig = 0.f;
                float3 m = f3(o[5 * k], o[5 * k + 1], o[5 * k + 2]);
                float len = fmaxf(sqrtf(dot(m, m)), 1e-12f);
                float3 dm = (wi - L[k].mu * c) * (kap / len);
                g[5 * k + 0] = -w * r * dm.x;
                g[5 * k + 1] = -w * r * dm.y;
                g[5 * k + 2] = -w * r * dm.z;
                g[5 * k + 3] = -w * r * dk * sig;
                g[5 * k + 4] = -w * (r - L[k].w);
            }
#pragma unroll
            for (int k = 0; k < kGuideOut; k++) {
                float v = g[k];
                g[k] = isfinite(v) ? fminf(fmaxf(v, -1e3f), 1e3f) : 0.f;
            }
        }
#pragma unroll
        for (int k = 0; k < kGuideOutPad; k += 2) *reinterpret_cast<uint32_t*>(dout + lane * kLdO + k) = pack_bf16(g[k], g[k + 1]);
        __syncwarp();
        // backward through the hidden layers: d_in = (d_out @ W^T) masked by relu'(h_in)
        for (int m = 0; m < 2; m++) tile_layer<48, 64>(dout + m * 16 * kLdO, kLdO, wn[3], nullptr, nullptr, 0, false, of + m * 16 * kLdG, kLdG);
        __syncwarp();
        for (int c = 0; c < 64; c += 2) {
            float v0 = bf(h3 + lane * kLdH + c) > 0.f ? of[lane * kLdG + c] : 0.f;
            float v1 = bf(h3 + lane * kLdH + c + 1) > 0.f ? of[lane * kLdG + c + 1] : 0.f;
            *reinterpret_cast<uint32_t*>(d3 + lane * kLdH + c) = pack_bf16(v0, v1);
        }
        __syncwarp();
        for (int m = 0; m < 2; m++) tile_layer<64, 64>(d3 + m * 16 * kLdH, kLdH, wn[2], nullptr, nullptr, 0, false, of + m * 16 * kLdG, kLdG);
        __syncwarp();
        for (int c = 0; c < 64; c += 2) {
            float v0 = bf(h2 + lane * kLdH + c) > 0.f ? of[lane * kLdG + c] : 0.f;
            float v1 = bf(h2 + lane * kLdH + c + 1) > 0.f ? of[lane * kLdG + c + 1] : 0.f;
            *reinterpret_cast<uint32_t*>(d2 + lane * kLdH + c) = pack_bf16(v0, v1);
        }
        __syncwarp();
        for (int m = 0; m < 2; m++) tile_layer<64, 64>(d2 + m * 16 * kLdH, kLdH, wn[1], nullptr, nullptr, 0, false, of + m * 16 * kLdG, kLdG);
        __syncwarp();
        for (int c = 0; c < 64; c += 2) {
            float v0 = bf(h1 + lane * kLdH + c) > 0.f ? of[lane * kLdG + c] : 0.f;
            float v1 = bf(h1 + lane * kLdH + c + 1) > 0.f ? of[lane * kLdG + c + 1] : 0.f;
            *reinterpret_cast<uint32_t*>(d1 + lane * kLdH + c) = pack_bf16(v0, v1);
        }
        __syncthreads();
        // weight and bias gradients of this block's 64 samples: dW_l = a_in^T d_out (FP32 sums)
        for (int pidx = threadIdx.x; pidx < kGuideParams; pidx += blockDim.x) {
            int l = 3;
            while (l > 0 && pidx < guide_w_off(l)) l--;
            int K = guide_k(l), N = guide_n(l);
            int rel = pidx - guide_w_off(l);
            bool is_bias = rel >= K * N;
            int kk = is_bias ? 0 : rel / N, nn = is_bias ? rel - K * N : rel % N;
            float acc = 0.f;
            for (int wv = 0; wv < kTrainWarps; wv++) {
                unsigned char* wbw = smem + kGuideParams * 4 + wv * kWarpTrainBytes;
                const __nv_bfloat16* A0 = reinterpret_cast<const __nv_bfloat16*>(wbw);
                const __nv_bfloat16* H1 = A0 + 32 * kLdA0;
                const __nv_bfloat16* H2 = H1 + 32 * kLdH;
                const __nv_bfloat16* H3 = H2 + 32 * kLdH;
                const __nv_bfloat16* D1 = H3 + 32 * kLdH;
                const __nv_bfloat16* D2 = D1 + 32 * kLdH;
                const __nv_bfloat16* D3 = D2 + 32 * kLdH;
                const float* OF = reinterpret_cast<const float*>(D3 + 32 * kLdH);
                const __nv_bfloat16* DO = reinterpret_cast<const __nv_bfloat16*>(OF + 32 * kLdG);
                const __nv_bfloat16* ain = l == 0 ? A0 : (l == 1 ? H1 : (l == 2 ? H2 : H3));
                const int lda = l == 0 ? kLdA0 : kLdH;
                const __nv_bfloat16* dlt = l == 0 ? D1 : (l == 1 ? D2 : (l == 2 ? D3 : DO));
                const int ldd = l == 3 ? kLdO : kLdH;
                for (int r = 0; r < 32; r++) {
                    float dv = __bfloat162float(dlt[r * ldd + nn]);
                    acc += is_bias ? dv : __bfloat162float(ain[r * lda + kk]) * dv;
                }
            }
            gacc[pidx] += acc;
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < kGuideParams; i += blockDim.x) {
        float v = gacc[i];
        if (v != 0.f) atomicAdd(grad + i, v);
    }
    // loss bookkeeping
    for (int o = 16; o > 0; o >>= 1) {
        loss += __shfl_down_sync(0xffffffffu, loss, o);
        wsum += __shfl_down_sync(0xffffffffu, wsum, o);
    }
    if (lane == 0) {
        atomicAdd(stats + 0, loss);
        atomicAdd(stats + 1, wsum);
    }
}

// Adam on the FP32 master weights (gradients normalised by the batch weight sum), then the two
// BF16 layouts the kernels read.  The padded output columns stay zero.
__global__ void k_guide_adam(float* params, float* grad, float* m, float* v, __nv_bfloat16* bfw, const float* stats,
                             float lr, float b1, float b2, float eps, float c1, float c2) {
    const float norm = 1.f / fmaxf(stats[1], 1e-12f);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < kGuideParams; p += gridDim.x * blockDim.x) {
        int l = 3;
        while (l > 0 && p < guide_w_off(l)) l--;
        int K = guide_k(l), N = guide_n(l);
        int rel = p - guide_w_off(l);
        bool is_bias = rel >= K * N;
        int kk = is_bias ? 0 : rel / N, nn = is_bias ? rel - K * N : rel % N;
        bool pad = (l == 3) && (nn >= kGuideOut);
        float g = pad ? 0.f : grad[p] * norm;
        if (!isfinite(g)) g = 0.f;  // a non-finite batch leaves the weights unchanged
        grad[p] = 0.f;
        float mm = b1 * m[p] + (1.f - b1) * g;
        float vv = b2 * v[p] + (1.f - b2) * g * g;
        m[p] = mm;
        v[p] = vv;
        float w = params[p] - lr * (mm / c1) / (sqrtf(vv / c2) + eps);
        if (pad) w = 0.f;
        params[p] = w;
        if (!is_bias) {
            __nv_bfloat16 h = __float2bfloat16_rn(w);
            bfw[guide_bf_off(l) + nn * K + kk] = h;           // wt: N x K
            bfw[guide_bf_off(l) + K * N + kk * N + nn] = h;   // wn: K x N
        }
    }
}

__global__ void k_guide_bf16_from_params(const float* params, __nv_bfloat16* bfw) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < kGuideParams; p += gridDim.x * blockDim.x) {
        int l = 3;
        while (l > 0 && p < guide_w_off(l)) l--;
        int K = guide_k(l), N = guide_n(l);
        int rel = p - guide_w_off(l);
        if (rel >= K * N) continue;
        int kk = rel / N, nn = rel % N;
        __nv_bfloat16 h = __float2bfloat16_rn(params[p]);
        bfw[guide_bf_off(l) + nn * K + kk] = h;
        bfw[guide_bf_off(l) + K * N + kk * N + nn] = h;
    }
}

constexpr size_t kInferSmem = 2 * 16384 + kInferWarps * 2 * kTileBytes;
constexpr size_t kTrainSmem = kGuideParams * 4 + kTrainWarps * kWarpTrainBytes;

}  // namespace

// ---- host -------------------------------------------------------------------------------------------
GuideTrainer::~GuideTrainer() = default;

void GuideTrainer::release(DeviceArena& arena) {
    void* ps[] = {params_, grad_, adam_m_, adam_v_, bf_, out_, rec_, batch_, batch_count_, loss_acc_};
    for (void* p : ps)
        if (p) arena.free(p);
    params_ = grad_ = adam_m_ = adam_v_ = nullptr;
    bf_ = nullptr;
    out_ = nullptr;
    rec_ = batch_ = nullptr;
    batch_count_ = nullptr;
    loss_acc_ = nullptr;
    cap_ = 0;
    rec_cap_ = 0;
    rec_depth_ = 1;
    steps_ = 0;
}

int GuideTrainer::init(DeviceArena& arena, size_t paths, int max_depth, const float box_lo[3], const float box_hi[3],
                       unsigned long long seed, std::string& err) {
    auto A = [&](size_t bytes) { return arena.alloc(bytes, err); };
    if (!params_) {
        params_ = (float*)A(kGuideParams * 4);
        grad_ = (float*)A(kGuideParams * 4);
        adam_m_ = (float*)A(kGuideParams * 4);
        adam_v_ = (float*)A(kGuideParams * 4);
        bf_ = (__nv_bfloat16*)A(kGuideBf16 * 2);
        loss_acc_ = (float*)A(16);
        batch_count_ = (int*)A(16);
        if (!params_ || !grad_ || !adam_m_ || !adam_v_ || !bf_ || !loss_acc_ || !batch_count_) return C2G_ERR_OOM;
        // He-uniform initialisation (seeded); the output layer starts small so the first mixture is broad
        std::vector<float> h(kGuideParams, 0.f);
        std::mt19937_64 rng(seed ^ 0x9e3779b97f4a7c15ULL);
        std::uniform_real_distribution<float> U(-1.f, 1.f);
        for (int l = 0; l < kGuideLayers; l++) {
            int K = guide_k(l), N = guide_n(l);
            float bound = std::sqrt(6.f / K) * (l == 3 ? 0.1f : 1.f);
            for (int k = 0; k < K; k++)
                for (int n = 0; n < N; n++) {
                    float v = U(rng) * bound;
                    if (l == 3 && n >= kGuideOut) v = 0.f;
                    h[guide_w_off(l) + k * N + n] = v;
                }
        }
        cudaMemcpy(params_, h.data(), kGuideParams * 4, cudaMemcpyHostToDevice);
        cudaMemset(grad_, 0, kGuideParams * 4);
        cudaMemset(adam_m_, 0, kGuideParams * 4);
        cudaMemset(adam_v_, 0, kGuideParams * 4);
        k_guide_bf16_from_params<<<64, 256>>>(params_, bf_);
        cudaFuncSetAttribute(k_guide_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInferSmem);
        cudaFuncSetAttribute(k_guide_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmem);
        cudaFuncSetAttribute(k_guide_eval, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInferSmem);
        steps_ = 0;
    }
    for (int a = 0; a < 3; a++) {
        box_lo_[a] = box_lo[a];
        float ext = box_hi[a] - box_lo[a];
        box_inv_[a] = ext > 0.f ? 1.f / ext : 1.f;
    }
    if (paths > cap_ || std::max(1, max_depth) != rec_depth_) {
        if (out_) arena.free(out_);
        if (rec_) arena.free(rec_);
        if (batch_) arena.free(batch_);
        cap_ = paths;
        rec_depth_ = std::max(1, max_depth);
        // about 2^18 recorded vertices per wave: every rec_stride-th path records its bounces
        rec_stride_ = (int)std::max<size_t>(1, paths * 3 / (1u << 18));
        rec_cap_ = (paths / rec_stride_ + 1) * rec_depth_;
        out_ = (float*)A(paths * kGuideOut * 4);
        rec_ = (float4*)A(rec_cap_ * 64);
        batch_ = (float4*)A(rec_cap_ * 64);
        if (!out_ || !rec_ || !batch_) return C2G_ERR_OOM;
        cudaMemset(rec_, 0, rec_cap_ * 64);
    }
    return C2G_OK;
}

void GuideTrainer::infer(cudaStream_t st, const void* Sv, const float4* ray_o, const float4* ray_d, const float4* hits,
                         const int* bucket_cnt, const int* bucket_list, int cap, int bucket_mask) {
    static int grid = 0;
    if (!grid) {
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_guide_infer, 128, kInferSmem);
        grid = std::max(1, sms * std::max(1, per));
    }
    int mask = 0;
    for (int b = 0; b < kBuckets; b++)
        if (((bucket_mask >> b) & 1) && bucket_guided(b)) mask |= 1 << b;
    if (!mask) return;
    k_guide_infer<<<grid, 128, kInferSmem, st>>>(*static_cast<const DevScene*>(Sv), view(false, false).net, ray_o, ray_d, hits,
                                                bucket_cnt, bucket_list, cap, mask, out_);
}

void GuideTrainer::train(cudaStream_t st, const float4* out_L, int wave_paths, int steps) {
    cudaMemsetAsync(batch_count_, 0, 16, st);
    cudaMemsetAsync(loss_acc_, 0, 16, st);
    k_guide_batch<<<(int)std::min<size_t>(4096, (rec_cap_ + 255) / 256), 256, 0, st>>>(
        rec_, (int)rec_cap_, rec_depth_, rec_stride_, out_L, wave_paths, batch_, batch_count_, loss_acc_, (int)rec_cap_);
    static int grid = 0;
    if (!grid) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        grid = sms;
    }
    GuideNet net = view(false, false).net;
    for (int s = 0; s < steps; s++) {
        k_guide_train<<<grid, 64, kTrainSmem, st>>>(net, batch_, batch_count_, (int)rec_cap_, grad_, loss_acc_);
        steps_++;
        const float b1 = 0.9f, b2 = 0.99f;
        float c1 = 1.f - std::pow(b1, (float)steps_), c2 = 1.f - std::pow(b2, (float)steps_);
        k_guide_adam<<<64, 256, 0, st>>>(params_, grad_, adam_m_, adam_v_, bf_, loss_acc_, lr_, b1, b2, 1e-8f, c1, c2);
    }
}

GuideView GuideTrainer::view(bool record, bool sample) const {
    GuideView v{};
    v.net.bf = bf_;
    v.net.params = params_;
    for (int a = 0; a < 3; a++) { v.net.box_lo[a] = box_lo_[a]; v.net.box_inv[a] = box_inv_[a]; }
    v.net.alpha = alpha_;
    v.net.enabled = sample ? 1 : 0;
    v.out = out_;
    v.rec = rec_;
    v.rec_stride = rec_stride_;
    v.rec_depth = rec_depth_;
    v.record = record ? 1 : 0;
    v.sample = sample ? 1 : 0;
    return v;
}

int GuideTrainer::set_params(const float* host, std::string& err) {
    if (!params_) { err = "guide network not initialised"; return C2G_ERR_STATE; }
    if (cudaMemcpy(params_, host, kGuideParams * 4, cudaMemcpyHostToDevice) != cudaSuccess) { err = "copy failed"; return C2G_ERR_CUDA; }
    cudaMemset(grad_, 0, kGuideParams * 4);
    cudaMemset(adam_m_, 0, kGuideParams * 4);
    cudaMemset(adam_v_, 0, kGuideParams * 4);
    k_guide_bf16_from_params<<<64, 256>>>(params_, bf_);
    steps_ = 0;
    if (cudaDeviceSynchronize() != cudaSuccess) { err = cudaGetErrorString(cudaGetLastError()); return C2G_ERR_CUDA; }
    return C2G_OK;
}

int GuideTrainer::get_params(float* host, std::string& err) {
    if (!params_) { err = "guide network not initialised"; return C2G_ERR_STATE; }
    if (cudaMemcpy(host, params_, kGuideParams * 4, cudaMemcpyDeviceToHost) != cudaSuccess) { err = "copy failed"; return C2G_ERR_CUDA; }
    return C2G_OK;
}

int GuideTrainer::eval(DeviceArena& arena, const float* host_xnw, int n, float* host_out, std::string& err) {
    if (!params_) { err = "guide network not initialised"; return C2G_ERR_STATE; }
    if (n <= 0) return C2G_OK;
    float* din = (float*)arena.alloc((size_t)n * 9 * 4, err);
    float* dout = (float*)arena.alloc((size_t)n * kGuideOut * 4, err);
    int rc = C2G_OK;
    if (!din || !dout) rc = C2G_ERR_OOM;
    if (!rc) {
        cudaMemcpy(din, host_xnw, (size_t)n * 9 * 4, cudaMemcpyHostToDevice);
        int blocks = std::min(1024, (n + 127) / 128);
        k_guide_eval<<<blocks, 128, kInferSmem>>>(view(false, false).net, din, n, dout);
        if (cudaDeviceSynchronize() != cudaSuccess) { err = cudaGetErrorString(cudaGetLastError()); rc = C2G_ERR_CUDA; }
        else cudaMemcpy(host_out, dout, (size_t)n * kGuideOut * 4, cudaMemcpyDeviceToHost);
    }
    if (din) arena.free(din);
    if (dout) arena.free(dout);
    return rc;
}

int GuideTrainer::gradient(DeviceArena& arena, const float* host_samples, int n, float* host_grad, double* loss, std::string& err) {
    if (!params_) { err = "guide network not initialised"; return C2G_ERR_STATE; }
    if (n <= 0) { err = "empty batch"; return C2G_ERR_INVALID; }
    std::vector<float4> b((size_t)n * 4);
    for (int j = 0; j < n; j++) {
        const float* v = host_samples + (size_t)13 * j;
        b[4 * j] = make_float4(v[0], v[1], v[2], v[12]);
        b[4 * j + 1] = make_float4(v[3], v[4], v[5], 0.f);
        b[4 * j + 2] = make_float4(v[6], v[7], v[8], 0.f);
        b[4 * j + 3] = make_float4(v[9], v[10], v[11], 0.f);
    }
    float4* db = (float4*)arena.alloc(b.size() * 16, err);
    if (!db) return C2G_ERR_OOM;
    // stats[2] = n makes the kernel's weight normaliser (mean weight) exactly 1
    float st[4] = {0.f, 0.f, (float)n, 0.f};
    cudaMemcpy(db, b.data(), b.size() * 16, cudaMemcpyHostToDevice);
    cudaMemcpy(batch_count_, &n, 4, cudaMemcpyHostToDevice);
    cudaMemcpy(loss_acc_, st, 16, cudaMemcpyHostToDevice);
    cudaMemset(grad_, 0, kGuideParams * 4);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    k_guide_train<<<sms, 64, kTrainSmem>>>(view(false, false).net, db, batch_count_, n, grad_, loss_acc_);
    int rc = C2G_OK;
    if (cudaDeviceSynchronize() != cudaSuccess) { err = cudaGetErrorString(cudaGetLastError()); rc = C2G_ERR_CUDA; }
    else {
        cudaMemcpy(host_grad, grad_, kGuideParams * 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(st, loss_acc_, 16, cudaMemcpyDeviceToHost);
        if (loss) *loss = st[1] > 0 ? (double)st[0] / st[1] : 0.0;
    }
    cudaMemset(grad_, 0, kGuideParams * 4);
    arena.free(db);
    return rc;
}

GuideStats GuideTrainer::stats() {
    float h[4] = {0, 0, 0, 0};
    int n = 0;
    if (loss_acc_) cudaMemcpy(h, loss_acc_, 16, cudaMemcpyDeviceToHost);
    if (batch_count_) cudaMemcpy(&n, batch_count_, 4, cudaMemcpyDeviceToHost);
    last_.loss = h[1] > 0 ? h[0] / h[1] : 0.0;
    last_.records = n;
    last_.steps = steps_;
    return last_;
}

}  // namespace c2g
