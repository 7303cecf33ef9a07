// Learned guiding proposal: inference over shading buckets, online training (fused forward +
// backward + weight gradients on tensor-core tiles) and the Adam update.
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
#include "umma.cuh"

namespace c2g {

namespace {

// Shared-memory tile strides (elements): rows padded by 8 so that the eight row groups of an MMA
// fragment load fall in distinct banks.
constexpr int kLdA0 = 88;    // encoded inputs (80)
constexpr int kLdH = 72;     // hidden activations / deltas (64)
constexpr int kLdO = 56;     // output-layer gradient (48)
constexpr int kLdOF = 52;    // FP32 outputs (training)

// Padded weight copies in shared memory.  Forward: wt_l (N_l rows of K_l + 8).  Backward: wn_l
// (K_l rows of N_l + 8), layers 1..3 (the input gradient of layer 0 is never needed).
__host__ __device__ constexpr int fw_ld(int l) { return guide_k(l) + 8; }
__host__ __device__ constexpr int fw_off(int l) { return l == 0 ? 0 : fw_off(l - 1) + guide_n(l - 1) * fw_ld(l - 1); }
constexpr int kFwElems = fw_off(4);
__host__ __device__ constexpr int bw_ld(int l) { return guide_n(l) + 8; }
__host__ __device__ constexpr int bw_off(int l) { return l <= 1 ? 0 : bw_off(l - 1) + guide_k(l - 1) * bw_ld(l - 1); }
constexpr int kBwElems = bw_off(4);

__device__ __forceinline__ float luminance(float3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

// Bucket ids whose hits are guided: the non-specular materials whose BSDF sampling routine returns
// the exact density of the directions it draws (the mixture pdf needs it at guide-drawn directions).
__host__ __device__ constexpr bool bucket_guided(int b) {
    return b == MAT_DIFFUSE || b == MAT_MICRO_GGX || b == MAT_MICRO_BECKMANN || b == MAT_PLASTIC_GGX ||
           b == MAT_PLASTIC_BECKMANN || b == MAT_ORENNAYAR;
}

__device__ __forceinline__ void stage_forward_weights(const GuideNet& net, __nv_bfloat16* wts) {
#pragma unroll
    for (int l = 0; l < kGuideLayers; l++) {
        const int K = guide_k(l), N = guide_n(l), vpr = K / 8;
        const uint4* src = reinterpret_cast<const uint4*>(net.bf + guide_bf_off(l));
        for (int i = threadIdx.x; i < N * vpr; i += blockDim.x) {
            int n = i / vpr, c = i - n * vpr;
            *reinterpret_cast<uint4*>(wts + fw_off(l) + n * fw_ld(l) + c * 8) = src[i];
        }
    }
}

__device__ __forceinline__ void stage_backward_weights(const GuideNet& net, __nv_bfloat16* wns) {
#pragma unroll
    for (int l = 1; l < kGuideLayers; l++) {
        const int K = guide_k(l), N = guide_n(l), vpr = N / 8;
        const uint4* src = reinterpret_cast<const uint4*>(net.bf + guide_bf_off(l) + K * N);
        for (int i = threadIdx.x; i < K * vpr; i += blockDim.x) {
            int k = i / vpr, c = i - k * vpr;
            *reinterpret_cast<uint4*>(wns + bw_off(l) + k * bw_ld(l) + c * 8) = src[i];
        }
    }
}

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

// MT 16-row tiles through one layer: out[16 MT x N] = epilogue(in[16 MT x K] @ W + bias), W given
// as w = N x K (row stride ldw).  A fragments are loaded once and reused across the N columns;
// each B fragment serves all MT row tiles.  Epilogue: FP32 store to outf when non-null; else
// optional ReLU, optional mask (value kept where mask > 0, the ReLU derivative) and a BF16 store.
template <int MT, int K, int N>
__device__ __forceinline__ void mma_rows(const __nv_bfloat16* in, int ldi, const __nv_bfloat16* w, int ldw,
                                         const float* bias, __nv_bfloat16* out, int ldo, bool relu, float* outf, int ldf,
                                         const __nv_bfloat16* mask, int ldm) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    uint32_t a[MT][K / 16][4];
#pragma unroll
    for (int m = 0; m < MT; m++)
#pragma unroll
        for (int kk = 0; kk < K / 16; kk++) {
            const __nv_bfloat16* r0 = in + (m * 16 + g) * ldi + kk * 16 + 2 * t;
            a[m][kk][0] = ld32(r0);
            a[m][kk][1] = ld32(r0 + 8 * ldi);
            a[m][kk][2] = ld32(r0 + 8);
            a[m][kk][3] = ld32(r0 + 8 * ldi + 8);
        }
#pragma unroll
    for (int n0 = 0; n0 < N; n0 += 8) {
        float d[MT][4];
        const float b0 = bias ? bias[n0 + 2 * t] : 0.f, b1 = bias ? bias[n0 + 2 * t + 1] : 0.f;
#pragma unroll
        for (int m = 0; m < MT; m++) { d[m][0] = b0; d[m][1] = b1; d[m][2] = b0; d[m][3] = b1; }
#pragma unroll
        for (int kk = 0; kk < K / 16; kk++) {
            uint32_t b[2];
            const __nv_bfloat16* wr = w + (n0 + g) * ldw + kk * 16 + 2 * t;
            b[0] = ld32(wr);
            b[1] = ld32(wr + 8);
#pragma unroll
            for (int m = 0; m < MT; m++) mma16816(d[m], a[m][kk], b);
        }
#pragma unroll
        for (int m = 0; m < MT; m++) {
            const int r0 = m * 16 + g, r1 = r0 + 8, c = n0 + 2 * t;
            if (outf) {
                outf[r0 * ldf + c] = d[m][0];
                outf[r0 * ldf + c + 1] = d[m][1];
                outf[r1 * ldf + c] = d[m][2];
                outf[r1 * ldf + c + 1] = d[m][3];
                continue;
            }
            if (relu) {
#pragma unroll
                for (int q = 0; q < 4; q++) d[m][q] = fmaxf(d[m][q], 0.f);
            }
            if (mask) {
                __nv_bfloat162 k0 = *reinterpret_cast<const __nv_bfloat162*>(mask + r0 * ldm + c);
                __nv_bfloat162 k1 = *reinterpret_cast<const __nv_bfloat162*>(mask + r1 * ldm + c);
                if (!(__low2float(k0) > 0.f)) d[m][0] = 0.f;
                if (!(__high2float(k0) > 0.f)) d[m][1] = 0.f;
                if (!(__low2float(k1) > 0.f)) d[m][2] = 0.f;
                if (!(__high2float(k1) > 0.f)) d[m][3] = 0.f;
            }
            *reinterpret_cast<uint32_t*>(out + r0 * ldo + c) = pack_bf16(d[m][0], d[m][1]);
            *reinterpret_cast<uint32_t*>(out + r1 * ldo + c) = pack_bf16(d[m][2], d[m][3]);
        }
    }
}

__device__ __forceinline__ void store_inputs(__nv_bfloat16* row, const float* in) {
#pragma unroll
    for (int k = 0; k < kGuideIn; k += 2) *reinterpret_cast<uint32_t*>(row + k) = pack_bf16(in[k], in[k + 1]);
}

// ---- inference on the fifth-generation tensor cores (tcgen05) -----------------------------------
// Two kernels.  k_guide_encode (one thread per guided vertex, full occupancy) reconstructs the
// surface, encodes (x, n, wo) and writes the row as BF16 into 128-row operand tiles in global
// memory, already in the tensor core's shared-memory layout.  k_guide_mlp_tc streams those tiles
// into shared memory with the bulk-copy engine and runs the four layers: two warpgroups per CTA
// share the staged weights; per warpgroup and tile one thread issues K/16 tcgen05.mma (M = 128,
// N = 64 or 48, BF16 operands from shared-memory descriptors, FP32 accumulator in 64 tensor-memory
// columns) and commits them to an mbarrier; every thread then reads its row (tcgen05.ld), adds the
// bias, applies ReLU and writes BF16 for the next layer, or packs the mixture after the last.  The
// next tile's copy starts as soon as layer 0 has consumed the input buffer.
// Operand layout: K-major 8-row x 16-byte core matrices without swizzle; element (r, k) of a
// K-column operand sits at (r / 8) * 16K + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2 bytes, so one
// K=16 step spans two core matrices 128 B apart (descriptor LBO), 8-row groups 16K bytes apart (SBO).
constexpr int kTcRows = 128;
constexpr int kTcGroups = 2;                            // warpgroups per CTA
constexpr int kTcThreads = kTcRows * kTcGroups;
constexpr int kTcTileBytes = kTcRows * kGuideIn * 2;    // one staged input tile: 20480 B
// staging bytes for n vertices: whole 128-row tiles
constexpr size_t stage_bytes(size_t n) { return (n + kTcRows - 1) / kTcRows * (size_t)kTcTileBytes; }
__host__ __device__ constexpr int tc_w_off(int l) { return l == 0 ? 0 : tc_w_off(l - 1) + guide_n(l - 1) * guide_k(l - 1) * 2; }
constexpr int kTcActBytes = kTcRows * kGuideHidden * 2;
constexpr int kTcGroupBytes = kTcTileBytes + kTcActBytes;  // input tile + hidden activations
__host__ __device__ constexpr int tc_in(int g) { return tc_w_off(4) + g * kTcGroupBytes; }
__host__ __device__ constexpr int tc_act(int g) { return tc_in(g) + kTcTileBytes; }
constexpr int kTcBias = tc_w_off(4) + kTcGroups * kTcGroupBytes;
constexpr int kTcBiasN = 3 * kGuideHidden + kGuideOutPad;
constexpr int kTcBar = kTcBias + kTcBiasN * 4;          // per warpgroup: MMA-done and input-full mbarriers
constexpr int kTcTmemSlot = kTcBar + 16 * kTcGroups;
constexpr size_t kTcSmem = (size_t)kTcTmemSlot + 8;
constexpr uint32_t kTcColsPerGroup = 64;
constexpr uint32_t kTcCols = kTcColsPerGroup * kTcGroups;  // tensor-memory columns per CTA (power of 2)
constexpr uint32_t kTcWaitPolls = 1u << 22;
static_assert(tc_in(0) % 128 == 0 && tc_act(0) % 128 == 0 && kTcGroupBytes % 128 == 0 && kTcBar % 8 == 0,
              "operand and barrier alignment");

__device__ __forceinline__ int tc_cm(int r, int k, int K) { return (r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2; }

// Eight consecutive columns [k0, k0 + 8) of operand row r, rounded to BF16.
__device__ __forceinline__ void tc_store8(unsigned char* base, int r, int k0, int K, const float* v) {
    uint4 q;
    q.x = pack_bf16(v[0], v[1]);
    q.y = pack_bf16(v[2], v[3]);
    q.z = pack_bf16(v[4], v[5]);
    q.w = pack_bf16(v[6], v[7]);
    *reinterpret_cast<uint4*>(base + tc_cm(r, k0, K)) = q;
}

// guide_encode written straight into row r of a K = 80 operand tile, eight values at a time (the
// same arithmetic in the same order, with eight values live instead of eighty).
__device__ __forceinline__ void tc_encode_row(const GuideNet& g, float3 x, float3 n, float3 wo, unsigned char* base, int r) {
    const float p[3] = {(x.x - g.box_lo[0]) * g.box_inv[0], (x.y - g.box_lo[1]) * g.box_inv[1], (x.z - g.box_lo[2]) * g.box_inv[2]};
    float chunk[8];
    int fill = 0, col = 0;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        float v = fminf(fmaxf(p[a], 0.f), 1.f);
        float s, c;
        sincospif(v, &s, &c);
#pragma unroll
        for (int f = 0; f < kGuideFreqs; f++) {
            chunk[fill++] = s;
            chunk[fill++] = c;
            if (fill == 8) {
                tc_store8(base, r, col, kGuideIn, chunk);
                col += 8;
                fill = 0;
            }
            const float s2 = 2.f * s * c, c2 = (c - s) * (c + s);
            s = s2;
            c = c2;
        }
    }
    const float tail[8] = {n.x, n.y, n.z, wo.x, wo.y, wo.z, 0.f, 0.f};
    tc_store8(base, r, 72, kGuideIn, tail);
}

// Work list of the guided buckets back to back: item -> queue slot.
__device__ __forceinline__ int guided_slot(const int* bend, const int* bucket_list, int cap, int item) {
    int b = 0;
    while (b < kBuckets - 1 && item >= bend[b]) b++;
    return bucket_list[(size_t)b * cap + (item - (b ? bend[b - 1] : 0))];
}
__device__ __forceinline__ void guided_bucket_ends(const int* bucket_cnt, int mask, int* bend) {
    int total = 0;
    for (int b = 0; b < kBuckets; b++) {
        total += ((mask >> b) & 1) ? bucket_cnt[b] : 0;
        bend[b] = total;
    }
}

// MODE 0: the guided buckets' vertices; MODE 1: explicit inputs xnw (9 floats each).  Rows past the
// last item of the last tile are zero.
template <int MODE>
__global__ void __launch_bounds__(256) k_guide_encode(DevScene S, GuideNet net, const float4* __restrict__ ray_o,
                                                     const float4* __restrict__ ray_d, const float4* __restrict__ hits,
                                                     const int* bucket_cnt, const int* __restrict__ bucket_list, int cap,
                                                     int mask, const float* __restrict__ xnw, int n_in,
                                                     unsigned char* stage) {
    __shared__ int bend[kBuckets];
    if (MODE == 0 && threadIdx.x == 0) guided_bucket_ends(bucket_cnt, mask, bend);
    __syncthreads();
    const int total = MODE == 0 ? bend[kBuckets - 1] : n_in;
    const int padded = (total + kTcRows - 1) / kTcRows * kTcRows;
    for (int item = blockIdx.x * blockDim.x + threadIdx.x; item < padded; item += gridDim.x * blockDim.x) {
        unsigned char* tile = stage + (size_t)(item / kTcRows) * kTcTileBytes;
        const int r = item % kTcRows;
        if (item < total) {
            if (MODE == 0) {
                const int slot = guided_slot(bend, bucket_list, cap, item);
                const float4 o4 = ray_o[slot], d4 = ray_d[slot], h4 = hits[slot];
                Hit h{h4.x, h4.y, h4.z, __float_as_int(h4.w)};
                Surface sf;
                make_surface(S, f3(o4), f3(d4), h, sf);
                tc_encode_row(net, sf.pos, sf.N, -f3(d4), tile, r);
            } else {
                const float* v = xnw + (size_t)9 * item;
                tc_encode_row(net, f3(v[0], v[1], v[2]), f3(v[3], v[4], v[5]), f3(v[6], v[7], v[8]), tile, r);
            }
        } else {
            const float z[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int k = 0; k < kGuideIn; k += 8) tc_store8(tile, r, k, kGuideIn, z);
        }
    }
}

// MODE 0: packed mixtures per queue slot; MODE 1: raw outputs (kGuideOut floats per input).
template <int MODE>
__global__ void __launch_bounds__(kTcThreads, 2) k_guide_mlp_tc(GuideNet net, const unsigned char* __restrict__ stage,
                                                               const int* bucket_cnt, const int* __restrict__ bucket_list,
                                                               int cap, int mask, int n_in, float* out, int* err) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int grp = threadIdx.x / kTcRows, row = threadIdx.x - grp * kTcRows, warp = threadIdx.x >> 5;
    float* bias = reinterpret_cast<float*>(smem + kTcBias);
    const uint32_t bar_mma = smem_u32(smem + kTcBar + 16 * grp), bar_in = bar_mma + 8;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + kTcTmemSlot);
    // weights -> core-matrix layout; biases
#pragma unroll
    for (int l = 0; l < kGuideLayers; l++) {
        const int K = guide_k(l), N = guide_n(l), vpr = K / 8;
        const uint4* src = reinterpret_cast<const uint4*>(net.bf + guide_bf_off(l));  // wt: N x K, K contiguous
        for (int i = threadIdx.x; i < N * vpr; i += kTcThreads) {
            const int nn = i / vpr, c = i - nn * vpr;
            *reinterpret_cast<uint4*>(smem + tc_w_off(l) + tc_cm(nn, 8 * c, K)) = src[i];
        }
    }
    for (int i = threadIdx.x; i < kTcBiasN; i += kTcThreads) {
        const int l = i < 3 * kGuideHidden ? i / kGuideHidden : 3;
        const int j = i - l * kGuideHidden;
        bias[i] = net.params[guide_b_off(l) + j];
    }
    __shared__ int bend[kBuckets];
    if (threadIdx.x == 0) {
        for (int g = 0; g < kTcGroups; g++) {
            mbar_init(smem_u32(smem + kTcBar + 16 * g), 1);
            mbar_init(smem_u32(smem + kTcBar + 16 * g + 8), 1);
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        if (MODE == 0) guided_bucket_ends(bucket_cnt, mask, bend);
    }
    if (warp == 0) tmem_alloc(smem_u32(tslot), kTcCols);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot + grp * kTcColsPerGroup;             // this warpgroup's columns
    const uint32_t trow = tmem + ((uint32_t)((warp & 3) * 32) << 16);  // this warp's 32 lanes
    unsigned char* IN = smem + tc_in(grp);
    unsigned char* ACT = smem + tc_act(grp);
    const int bar_id = 1 + grp;
    const int total = MODE == 0 ? bend[kBuckets - 1] : n_in;
    const int tiles = (total + kTcRows - 1) / kTcRows;
    const int tstride = gridDim.x * kTcGroups;
    int tile = blockIdx.x * kTcGroups + grp;
    // phases of the two barriers, and whether a tile copy / an MMA group is outstanding (the same
    // in every thread of the warpgroup: issue decisions are uniform)
    uint32_t ph_mma = 0, ph_in = 0;
    bool copy_pending = false, mma_pending = false, failed = false;
    if (tile < tiles) {
        if (row == 0) {
            mbar_arrive_expect_tx(bar_in, kTcTileBytes);
            bulk_g2s(smem_u32(IN), stage + (size_t)tile * kTcTileBytes, kTcTileBytes, bar_in);
        }
        copy_pending = true;
    }
    for (; tile < tiles && !failed; tile += tstride) {
        bool ok = mbar_wait(bar_in, ph_in, kTcWaitPolls);
        if (ok) { ph_in ^= 1u; copy_pending = false; }
        float o[kGuideOutPad];
#pragma unroll
        for (int l = 0; l < kGuideLayers; l++) {
            const int K = guide_k(l), N = guide_n(l);
            fence_async_smem();
            tc_fence_before();
            if (wg_sync_or(bar_id, !ok)) { failed = true; break; }
            if (row == 0) {
                tc_fence_after();
                const uint32_t a0 = smem_u32(l == 0 ? IN : ACT), b0 = smem_u32(smem + tc_w_off(l));
                const uint32_t idesc = umma_idesc_bf16(kTcRows, N);
                for (int kk = 0; kk < K / 16; kk++)
                    umma_bf16(tmem, umma_desc(a0 + kk * 256, 128, K * 16), umma_desc(b0 + kk * 256, 128, K * 16), idesc, kk > 0);
                umma_commit(bar_mma);
            }
            mma_pending = true;
            ok = mbar_wait(bar_mma, ph_mma, kTcWaitPolls);
            if (ok) { ph_mma ^= 1u; mma_pending = false; }
            if (wg_sync_or(bar_id, !ok)) { failed = true; break; }
            tc_fence_after();
            if (l == 0 && tile + tstride < tiles) {
                // layer 0 has consumed the input tile: fetch the next one behind layers 1-3
                if (row == 0) {
                    mbar_arrive_expect_tx(bar_in, kTcTileBytes);
                    bulk_g2s(smem_u32(IN), stage + (size_t)(tile + tstride) * kTcTileBytes, kTcTileBytes, bar_in);
                }
                copy_pending = true;
            }
            if (l < kGuideLayers - 1) {
#pragma unroll
                for (int c = 0; c < kGuideHidden; c += 32) {
                    uint32_t r[32];
                    tmem_ld16(trow + c, r);
                    tmem_ld16(trow + c + 16, r + 16);
                    tmem_wait();
#pragma unroll
                    for (int q = 0; q < 32; q += 8) {
                        float v[8];
#pragma unroll
                        for (int j = 0; j < 8; j++) v[j] = fmaxf(__uint_as_float(r[q + j]) + bias[l * kGuideHidden + c + q + j], 0.f);
                        tc_store8(ACT, row, c + q, kGuideHidden, v);
                    }
                }
            } else {
                uint32_t r[kGuideOutPad];
#pragma unroll
                for (int c = 0; c < kGuideOutPad; c += 16) tmem_ld16(trow + c, r + c);
                tmem_wait();
#pragma unroll
                for (int j = 0; j < kGuideOutPad; j++) o[j] = __uint_as_float(r[j]) + bias[3 * kGuideHidden + j];
            }
        }
        if (failed) break;
        const int item = tile * kTcRows + row;
        if (item < total) {
            if (MODE == 0) pack_lobes(o, out + (size_t)guided_slot(bend, bucket_list, cap, item) * kGuidePacked);
            else {
#pragma unroll
                for (int k = 0; k < kGuideOut; k++) out[(size_t)item * kGuideOut + k] = o[k];
            }
        }
    }
    if (failed) {
        if (row == 0) dev_flag_error(err, DEVERR_WAIT);
        // let what is still in flight finish (bounded) before the tensor memory is freed and the
        // CTA's shared memory is released
        if (mma_pending) mbar_wait(bar_mma, ph_mma, kTcWaitPolls);
        if (copy_pending) mbar_wait(bar_in, ph_in, kTcWaitPolls);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_free(*tslot, kTcCols);
    }
}

// ---- records -> weighted training samples ------------------------------------------------------
// Record (4 float4): (x, valid), (n, lum L at the vertex after its direct light), (wo, lum beta at
// the vertex), (wi, BSDF density at wi).  Sample (4 float4): (x, w), (n, 0), (wo, 0), (wi, p_bsdf).
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
        bool keep = ok && j < batch_cap;
        if (keep) {
            batch[4 * j] = make_float4(r0.x, r0.y, r0.z, w);
            batch[4 * j + 1] = make_float4(r1.x, r1.y, r1.z, 0.f);
            batch[4 * j + 2] = make_float4(r2.x, r2.y, r2.z, 0.f);
            batch[4 * j + 3] = r3;  // wi, BSDF density
        }
        float ws = keep ? w : 0.f;
        for (int o = 16; o > 0; o >>= 1) ws += __shfl_xor_sync(0xffffffffu, ws, o);
        if ((threadIdx.x & 31) == 0 && ws != 0.f) atomicAdd(stats + 2, ws);
    }
}

// ---- fused training step ------------------------------------------------------------------------
// 256 threads = 8 warps; a block takes 128 samples per iteration, 16 per warp.  Each warp runs the
// forward and backward passes of its samples on tensor-core tiles (weights staged in shared memory,
// activations and deltas kept as BF16 tiles).  The weight gradients dW_l = A_l^T D_l are then
// tensor-core products over the block's 128 samples: the 124 (16 x 8) output tiles of the four
// layers are split over the warps, each accumulating its tiles in FP32 registers for the whole
// sweep (A^T and D fragments come from ldmatrix.trans); they reach global memory once per block.
constexpr int kTrainWarps = 8;
// A wave's batch is split into at most this many minibatch windows, taken in turn by its Adam
// steps: smaller windows made the mixture collapse onto a few sharp lobes in some runs.
constexpr int kTrainWindows = 4;
constexpr int kTrainRows = 16;
// per-warp tile offsets (elements)
constexpr int kTA0 = 0;
constexpr int kTH1 = kTA0 + kTrainRows * kLdA0;
constexpr int kTH2 = kTH1 + kTrainRows * kLdH;
constexpr int kTH3 = kTH2 + kTrainRows * kLdH;
constexpr int kTD1 = kTH3 + kTrainRows * kLdH;
constexpr int kTD2 = kTD1 + kTrainRows * kLdH;
constexpr int kTD3 = kTD2 + kTrainRows * kLdH;
constexpr int kTDO = kTD3 + kTrainRows * kLdH;
constexpr int kTWarpElems = kTDO + kTrainRows * kLdO;
static_assert(kTrainRows * kLdOF * 4 <= 2 * kTrainRows * kLdH * 2, "FP32 outputs alias the d1/d2 tiles");
constexpr size_t kTrainSmem = (size_t)(kFwElems + kBwElems + kTrainWarps * kTWarpElems) * 2;
// dW tiles: layer 0 5 x 8, layers 1-2 4 x 8, layer 3 4 x 6 (outputs 40..47: selection + padding)
constexpr int kDwTiles = 40 + 32 + 32 + 24;
constexpr int kDwPerWarp = (kDwTiles + kTrainWarps - 1) / kTrainWarps;

__device__ __forceinline__ void ldsm_x4_trans(uint32_t* r, const void* p) {
    uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(a));
}
__device__ __forceinline__ void ldsm_x2_trans(uint32_t* r, const void* p) {
    uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n" : "=r"(r[0]), "=r"(r[1]) : "r"(a));
}

__device__ __forceinline__ void dw_tile(int idx, int& l, int& mt, int& nt) {
    if (idx < 40) { l = 0; mt = idx >> 3; nt = idx & 7; }
    else if (idx < 72) { l = 1; mt = (idx - 40) >> 3; nt = (idx - 40) & 7; }
    else if (idx < 104) { l = 2; mt = (idx - 72) >> 3; nt = (idx - 72) & 7; }
    else { l = 3; mt = (idx - 104) / 6; nt = (idx - 104) % 6; }
}

// Gradient of w * -log q_mix(wi), q_mix = (1 - c) p_bsdf + c q_guide, with respect to the 41 raw
// outputs o (see the oracle for the formulas); returns -log q_mix.  g[41..47] (padding) are left
// to the caller.
__device__ __forceinline__ float nll_output_grad(const float* o, float3 wi, float w, float pb, float* g) {
    Lobe L[kGuideLobes];
    guide_lobes(o, L);
    float p[kGuideLobes], q = 0.f;
#pragma unroll
    for (int k = 0; k < kGuideLobes; k++) { p[k] = L[k].w * vmf_pdf(L[k], wi); q += p[k]; }
    q = fmaxf(q, 1e-20f);
    const float inv_q = 1.f / q;
    // the mixture with the BSDF: lobe gradients scale by c q / q_mix; the selection logit s gets
    // -w (q - p_bsdf) dc/ds / q_mix
    const float sg = 1.f / (1.f + __expf(-o[40]));
    const float csel = kGuideSelMin + kGuideSelSpan * sg;
    const float qmix = fmaxf((1.f - csel) * pb + csel * q, 1e-20f);
    const float rho = csel * q / qmix;
#pragma unroll
    for (int k = 0; k < kGuideLobes; k++) {
        const float r = p[k] * inv_q;
        const float kap = L[k].kappa;
        const float c = dot(L[k].mu, wi);
        // d log vMF / d kappa = 1/kappa - 2 e^-2k / (1 - e^-2k) + (mu.wi - 1)
        const float e2 = __expf(-2.f * kap);
        const float dk = 1.f / kap - 2.f * e2 / fmaxf(-expm1f(-2.f * kap), 1e-20f) + (c - 1.f);
        const float kraw = o[5 * k + 3];
        float sig = 1.f / (1.f + __expf(-kraw));
        if (kap >= kGuideKappaMax) sig = 0.f;
        const float3 m = f3(o[5 * k], o[5 * k + 1], o[5 * k + 2]);
        const float len = fmaxf(sqrtf(dot(m, m)), 1e-12f);
        const float3 dm = (wi - L[k].mu * c) * (kap / len);
        g[5 * k + 0] = -w * rho * r * dm.x;
        g[5 * k + 1] = -w * rho * r * dm.y;
        g[5 * k + 2] = -w * rho * r * dm.z;
        g[5 * k + 3] = -w * rho * r * dk * sig;
        g[5 * k + 4] = -w * rho * (r - L[k].w);
    }
    g[40] = -w * (q - pb) * kGuideSelSpan * sg * (1.f - sg) / qmix;
#pragma unroll
    for (int k = 0; k < kGuideOut; k++) {
        const float v = g[k];
        g[k] = isfinite(v) ? fminf(fmaxf(v, -1e3f), 1e3f) : 0.f;
    }
    return -__logf(qmix);
}

__global__ void __launch_bounds__(256, 1) k_guide_train(GuideNet net, const float4* __restrict__ batch, const int* batch_count,
                                                        int batch_cap, float* grad, float* stats, int splits,
                                                        const int* __restrict__ step) {
    extern __shared__ __align__(128) unsigned char smem[];
    __nv_bfloat16* wts = reinterpret_cast<__nv_bfloat16*>(smem);
    __nv_bfloat16* wns = wts + kFwElems;
    __nv_bfloat16* tiles = wns + kBwElems;
    stage_forward_weights(net, wts);
    stage_backward_weights(net, wns);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __nv_bfloat16* T = tiles + warp * kTWarpElems;
    float* OF = reinterpret_cast<float*>(T + kTD1);
    const int n = min(*batch_count, batch_cap);
    const float mean_w = stats[2] / fmaxf(1.f, (float)n);
    // minibatch of this Adam step: the batch split into `splits` windows, taken in turn, so the
    // steps of one wave pass over the batch once
    const int per = (n + splits - 1) / splits;
    const int lo = min(n, (*step % splits) * per), hi = min(n, lo + per);

    float acc[kDwPerWarp][4];
#pragma unroll
    for (int q = 0; q < kDwPerWarp; q++) acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = 0.f;
    // bias gradients: thread -> one of the 64 + 64 + 64 + 40 bias columns
    float bacc = 0.f;
    int bl = -1, bc = 0;
    if (threadIdx.x < 192) { bl = threadIdx.x >> 6; bc = threadIdx.x & 63; }
    else if (threadIdx.x < 192 + kGuideOut) { bl = 3; bc = threadIdx.x - 192; }
    float loss = 0.f, wsum = 0.f;

    const int chunk = kTrainWarps * kTrainRows;
    for (int base = lo + blockIdx.x * chunk; base < hi; base += gridDim.x * chunk) {
        const int s = lane & 15;
        const int j = base + warp * kTrainRows + s;
        const bool valid = j < hi;
        float3 wi = f3(0.f, 0.f, 1.f);
        float w = 0.f, pb = 0.f;
        if (lane < 16) {
            float in[kGuideIn];
            if (valid) {
                const float4 b0 = batch[4 * j], b1 = batch[4 * j + 1], b2 = batch[4 * j + 2], b3 = batch[4 * j + 3];
                guide_encode(net, f3(b0), f3(b1), f3(b2), in);
                wi = f3(b3);
                pb = b3.w;
                w = fminf(b0.w / fmaxf(mean_w, 1e-12f), 20.f);  // normalised, firefly-clamped weight
            } else {
#pragma unroll
                for (int k = 0; k < kGuideIn; k++) in[k] = 0.f;
            }
            store_inputs(T + kTA0 + s * kLdA0, in);
        }
        __syncwarp();
        mma_rows<1, 80, 64>(T + kTA0, kLdA0, wts + fw_off(0), fw_ld(0), net.params + guide_b_off(0), T + kTH1, kLdH, true, nullptr, 0, nullptr, 0);
        __syncwarp();
        mma_rows<1, 64, 64>(T + kTH1, kLdH, wts + fw_off(1), fw_ld(1), net.params + guide_b_off(1), T + kTH2, kLdH, true, nullptr, 0, nullptr, 0);
        __syncwarp();
        mma_rows<1, 64, 64>(T + kTH2, kLdH, wts + fw_off(2), fw_ld(2), net.params + guide_b_off(2), T + kTH3, kLdH, true, nullptr, 0, nullptr, 0);
        __syncwarp();
        mma_rows<1, 64, 48>(T + kTH3, kLdH, wts + fw_off(3), fw_ld(3), net.params + guide_b_off(3), nullptr, 0, false, OF, kLdOF, nullptr, 0);
        __syncwarp();
        // loss gradient at the outputs: one lane per sample
        float g[kGuideOutPad];
#pragma unroll
        for (int k = 0; k < kGuideOutPad; k++) g[k] = 0.f;
        if (lane < 16 && valid && w > 0.f) {
            float o[kGuideOut];
#pragma unroll
            for (int k = 0; k < kGuideOut; k++) o[k] = OF[s * kLdOF + k];
            loss += w * nll_output_grad(o, wi, w, pb, g);
            wsum += w;
        }
        __syncwarp();  // OF (aliasing d1/d2) fully read before the deltas are written
        if (lane < 16) {
#pragma unroll
            for (int k = 0; k < kGuideOutPad; k += 2) *reinterpret_cast<uint32_t*>(T + kTDO + s * kLdO + k) = pack_bf16(g[k], g[k + 1]);
        }
        __syncwarp();
        // backward: d_l = (d_{l+1} @ W_{l+1}^T) masked by relu'(h)
        mma_rows<1, 48, 64>(T + kTDO, kLdO, wns + bw_off(3), bw_ld(3), nullptr, T + kTD3, kLdH, false, nullptr, 0, T + kTH3, kLdH);
        __syncwarp();
        mma_rows<1, 64, 64>(T + kTD3, kLdH, wns + bw_off(2), bw_ld(2), nullptr, T + kTD2, kLdH, false, nullptr, 0, T + kTH2, kLdH);
        __syncwarp();
        mma_rows<1, 64, 64>(T + kTD2, kLdH, wns + bw_off(1), bw_ld(1), nullptr, T + kTD1, kLdH, false, nullptr, 0, T + kTH1, kLdH);
        __syncthreads();
        // weight gradients over the block's 128 samples
        {
            const int jm = lane >> 3, qr = lane & 7;
#pragma unroll
            for (int q = 0; q < kDwPerWarp; q++) {
                const int idx = warp + kTrainWarps * q;
                if (idx < kDwTiles) {
                    int l, mt, nt;
                    dw_tile(idx, l, mt, nt);
                    const int ain = l == 0 ? kTA0 : (l == 1 ? kTH1 : (l == 2 ? kTH2 : kTH3));
                    const int lda = l == 0 ? kLdA0 : kLdH;
                    const int dlt = l == 0 ? kTD1 : (l == 1 ? kTD2 : (l == 2 ? kTD3 : kTDO));
                    const int ldd = l == 3 ? kLdO : kLdH;
                    const int arow = qr + (jm >> 1) * 8, acol = mt * 16 + (jm & 1) * 8;
                    const int brow = qr + (jm & 1) * 8, bcol = nt * 8;
#pragma unroll
                    for (int wv = 0; wv < kTrainWarps; wv++) {
                        const __nv_bfloat16* Tw = tiles + wv * kTWarpElems;
                        uint32_t a[4], b[2];
                        ldsm_x4_trans(a, Tw + ain + arow * lda + acol);
                        ldsm_x2_trans(b, Tw + dlt + brow * ldd + bcol);
                        mma16816(acc[q], a, b);
                    }
                }
            }
        }
        if (bl >= 0) {
            const int dlt = bl == 0 ? kTD1 : (bl == 1 ? kTD2 : (bl == 2 ? kTD3 : kTDO));
            const int ldd = bl == 3 ? kLdO : kLdH;
            for (int wv = 0; wv < kTrainWarps; wv++) {
                const __nv_bfloat16* D = tiles + wv * kTWarpElems + dlt;
#pragma unroll
                for (int r = 0; r < kTrainRows; r++) bacc += __bfloat162float(D[r * ldd + bc]);
            }
        }
        __syncthreads();
    }
    // flush: dW_l[k][n] with k = mt*16 + g (+8), n = nt*8 + 2t (+1)
    {
        const int g = lane >> 2, t = lane & 3;
#pragma unroll
        for (int q = 0; q < kDwPerWarp; q++) {
            const int idx = warp + kTrainWarps * q;
            if (idx < kDwTiles) {
                int l, mt, nt;
                dw_tile(idx, l, mt, nt);
                const int N = guide_n(l);
                float* G = grad + guide_w_off(l);
                const int k0 = mt * 16 + g, c = nt * 8 + 2 * t;
                if (acc[q][0] != 0.f) atomicAdd(G + k0 * N + c, acc[q][0]);
                if (acc[q][1] != 0.f) atomicAdd(G + k0 * N + c + 1, acc[q][1]);
                if (acc[q][2] != 0.f) atomicAdd(G + (k0 + 8) * N + c, acc[q][2]);
                if (acc[q][3] != 0.f) atomicAdd(G + (k0 + 8) * N + c + 1, acc[q][3]);
            }
        }
    }
    if (bl >= 0 && bacc != 0.f) atomicAdd(grad + guide_b_off(bl) + bc, bacc);
    for (int o = 16; o > 0; o >>= 1) {
        loss += __shfl_down_sync(0xffffffffu, loss, o);
        wsum += __shfl_down_sync(0xffffffffu, wsum, o);
    }
    if (lane == 0 && wsum != 0.f) {
        atomicAdd(stats + 0, loss);
        atomicAdd(stats + 1, wsum);
    }
}

// Adam on the FP32 master weights (gradients normalised by the batch weight sum), then the two
// BF16 layouts the kernels read.  The padded output columns stay zero.
__global__ void k_guide_adam(float* params, float* grad, float* m, float* v, __nv_bfloat16* bfw, const float* stats,
                             float lr, float b1, float b2, float eps, const int* step) {
    const float norm = 1.f / fmaxf(stats[1], 1e-12f);
    // bias corrections of Adam step t = *step + 1 (the counter lives on the device so that captured
    // graphs replay correctly; k_guide_tick advances it)
    const float t = (float)(*step + 1);
    const float c1 = 1.f - powf(b1, t), c2 = 1.f - powf(b2, t);
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

__global__ void k_guide_tick(int* step) { *step += 1; }

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

}  // namespace

// ---- host -------------------------------------------------------------------------------------------
GuideTrainer::~GuideTrainer() = default;

void GuideTrainer::release(DeviceArena& arena) {
    void* ps[] = {params_, grad_, adam_m_, adam_v_, bf_, out_, stage_, rec_, batch_, batch_count_, loss_acc_, step_dev_};
    for (void* p : ps)
        if (p) arena.free(p);
    params_ = grad_ = adam_m_ = adam_v_ = nullptr;
    bf_ = nullptr;
    out_ = nullptr;
    stage_ = nullptr;
    rec_ = batch_ = nullptr;
    batch_count_ = nullptr;
    loss_acc_ = nullptr;
    step_dev_ = nullptr;
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
        step_dev_ = (int*)A(16);
        if (!params_ || !grad_ || !adam_m_ || !adam_v_ || !bf_ || !loss_acc_ || !batch_count_ || !step_dev_) return C2G_ERR_OOM;
        cudaMemset(step_dev_, 0, 16);
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
        // selection bias: the untrained network draws from the mixture with probability
        // 1 - alpha (the configured BSDF fraction), c = 0.05 + 0.75 sigmoid(s)
        const float c0 = std::min(kGuideSelMin + 0.99f * kGuideSelSpan, std::max(kGuideSelMin + 0.01f * kGuideSelSpan, 1.f - alpha_));
        const float sg = (c0 - kGuideSelMin) / kGuideSelSpan;
        h[guide_b_off(3) + 40] = std::log(sg / (1.f - sg));
        cudaMemcpy(params_, h.data(), kGuideParams * 4, cudaMemcpyHostToDevice);
        cudaMemset(grad_, 0, kGuideParams * 4);
        cudaMemset(adam_m_, 0, kGuideParams * 4);
        cudaMemset(adam_v_, 0, kGuideParams * 4);
        k_guide_bf16_from_params<<<64, 256>>>(params_, bf_);
        cudaFuncSetAttribute(k_guide_mlp_tc<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
        cudaFuncSetAttribute(k_guide_mlp_tc<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
        cudaFuncSetAttribute(k_guide_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmem);
        steps_ = 0;
    }
    for (int a = 0; a < 3; a++) {
        box_lo_[a] = box_lo[a];
        float ext = box_hi[a] - box_lo[a];
        box_inv_[a] = ext > 0.f ? 1.f / ext : 1.f;
    }
    if (paths > cap_ || std::max(1, max_depth) != rec_depth_) {
        if (out_) arena.free(out_);
        if (stage_) arena.free(stage_);
        if (rec_) arena.free(rec_);
        if (batch_) arena.free(batch_);
        cap_ = paths;
        rec_depth_ = std::max(1, max_depth);
        // about 2^18 recorded vertices per wave: every rec_stride-th path records its bounces
        rec_stride_ = (int)std::max<size_t>(1, paths * 3 / (1u << 18));
        rec_cap_ = (paths / rec_stride_ + 1) * rec_depth_;
        out_ = (float*)A(paths * kGuidePacked * 4);
        stage_ = (unsigned char*)A(stage_bytes(paths));
        rec_ = (float4*)A(rec_cap_ * 64);
        batch_ = (float4*)A(rec_cap_ * 64);
        if (!out_ || !stage_ || !rec_ || !batch_) return C2G_ERR_OOM;
        cudaMemset(rec_, 0, rec_cap_ * 64);
    }
    return C2G_OK;
}

namespace {
int g_infer_grid = 0, g_train_grid = 0, g_encode_grid = 0;
}  // namespace

void GuideTrainer::prepare_launch() {
    if (g_infer_grid) return;
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaFuncSetAttribute(k_guide_mlp_tc<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
    cudaFuncSetAttribute(k_guide_mlp_tc<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_guide_mlp_tc<0>, kTcThreads, kTcSmem);
    // resident CTAs per SM as shared memory allows (1 KB reserved per CTA), in case the query
    // under-reports; extra CTAs of a persistent grid only wait for a slot
    int smem_sm = 0;
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    const int per_smem = smem_sm / (int)(kTcSmem + 1024);
    per = std::max(per, std::min(2, per_smem));
    g_infer_grid = std::max(1, sms * std::max(1, per));
    g_train_grid = std::max(1, sms);
    int per_enc = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_enc, k_guide_encode<0>, 256, 0);
    g_encode_grid = std::max(1, sms * std::max(1, per_enc));
}

int GuideTrainer::infer(cudaStream_t st, const void* Sv, const float4* ray_o, const float4* ray_d, const float4* hits,
                        const int* bucket_cnt, const int* bucket_list, int cap, int bucket_mask) {
    prepare_launch();
    const int grid = g_infer_grid;
    int mask = 0;
    for (int b = 0; b < kBuckets; b++)
        if (((bucket_mask >> b) & 1) && bucket_guided(b)) mask |= 1 << b;
    if (!mask) return 0;
    const DevScene& S = *static_cast<const DevScene*>(Sv);
    const GuideNet net = view(false, false).net;
    k_guide_encode<0><<<g_encode_grid, 256, 0, st>>>(S, net, ray_o, ray_d, hits, bucket_cnt, bucket_list, cap, mask, nullptr, 0,
                                                     stage_);
    k_guide_mlp_tc<0><<<grid, kTcThreads, kTcSmem, st>>>(net, stage_, bucket_cnt, bucket_list, cap, mask, 0, out_, S.err);
    return 2;
}

void GuideTrainer::train(cudaStream_t st, const float4* out_L, int wave_paths, int steps) {
    cudaMemsetAsync(batch_count_, 0, 16, st);
    cudaMemsetAsync(loss_acc_, 0, 16, st);
    k_guide_batch<<<(int)std::min<size_t>(4096, (rec_cap_ + 255) / 256), 256, 0, st>>>(
        rec_, (int)rec_cap_, rec_depth_, rec_stride_, out_L, wave_paths, batch_, batch_count_, loss_acc_, (int)rec_cap_);
    prepare_launch();
    const int grid = g_train_grid;
    GuideNet net = view(false, false).net;
    for (int s = 0; s < steps; s++) {
        cudaMemsetAsync(loss_acc_, 0, 8, st);  // this step's loss and weight sum (Adam normalises by it)
        k_guide_train<<<grid, 256, kTrainSmem, st>>>(net, batch_, batch_count_, (int)rec_cap_, grad_, loss_acc_,
                                                     std::min(steps, kTrainWindows), step_dev_);
        steps_++;
        k_guide_adam<<<64, 256, 0, st>>>(params_, grad_, adam_m_, adam_v_, bf_, loss_acc_, lr_, 0.9f, 0.99f, 1e-8f, step_dev_);
        k_guide_tick<<<1, 1, 0, st>>>(step_dev_);
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
    cudaMemset(step_dev_, 0, 16);
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
    unsigned char* dstage = (unsigned char*)arena.alloc(stage_bytes((size_t)n), err);
    int* derr = (int*)arena.alloc(16, err);
    int rc = C2G_OK;
    if (!din || !dout || !dstage || !derr) rc = C2G_ERR_OOM;
    if (!rc) {
        cudaMemcpy(din, host_xnw, (size_t)n * 9 * 4, cudaMemcpyHostToDevice);
        cudaMemset(derr, 0, 16);
        prepare_launch();
        const GuideNet net = view(false, false).net;
        k_guide_encode<1><<<std::min(g_encode_grid, (n + 255) / 256), 256>>>(DevScene{}, net, nullptr, nullptr, nullptr, nullptr,
                                                                           nullptr, 0, 0, din, n, dstage);
        const int blocks = std::min(g_infer_grid, (n + kTcThreads - 1) / kTcThreads);
        k_guide_mlp_tc<1><<<blocks, kTcThreads, kTcSmem>>>(net, dstage, nullptr, nullptr, 0, 0, n, dout, derr);
        int h = 0;
        if (cudaDeviceSynchronize() != cudaSuccess) { err = cudaGetErrorString(cudaGetLastError()); rc = C2G_ERR_CUDA; }
        else if (cudaMemcpy(&h, derr, 4, cudaMemcpyDeviceToHost) == cudaSuccess && h) {
            err = "guide inference: tensor-core completion wait timed out";
            rc = C2G_ERR_DEVICE;
        } else cudaMemcpy(host_out, dout, (size_t)n * kGuideOut * 4, cudaMemcpyDeviceToHost);
    }
    if (din) arena.free(din);
    if (dout) arena.free(dout);
    if (dstage) arena.free(dstage);
    if (derr) arena.free(derr);
    return rc;
}

int GuideTrainer::gradient(DeviceArena& arena, const float* host_samples, int n, float* host_grad, double* loss, std::string& err) {
    if (!params_) { err = "guide network not initialised"; return C2G_ERR_STATE; }
    if (n <= 0) { err = "empty batch"; return C2G_ERR_INVALID; }
    std::vector<float4> b((size_t)n * 4);
    for (int j = 0; j < n; j++) {
        const float* v = host_samples + (size_t)14 * j;
        b[4 * j] = make_float4(v[0], v[1], v[2], v[12]);
        b[4 * j + 1] = make_float4(v[3], v[4], v[5], 0.f);
        b[4 * j + 2] = make_float4(v[6], v[7], v[8], 0.f);
        b[4 * j + 3] = make_float4(v[9], v[10], v[11], v[13]);
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
    k_guide_train<<<sms, 256, kTrainSmem>>>(view(false, false).net, db, batch_count_, n, grad_, loss_acc_, 1, step_dev_);
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
    int t = steps_;
    if (step_dev_) cudaMemcpy(&t, step_dev_, 4, cudaMemcpyDeviceToHost);
    last_.loss = h[1] > 0 ? h[0] / h[1] : 0.0;
    last_.records = n;
    last_.steps = t;
    return last_;
}

}  // namespace c2g
