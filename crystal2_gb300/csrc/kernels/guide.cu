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
__device__ __forceinline__ float luminance(float3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }


// ---- inference on the fifth-generation tensor cores (tcgen05) -----------------------------------
// Two kernels.  k_guide_record (one thread per guided vertex, full occupancy) reconstructs the
// surface and writes the vertex's network input as a compact record of 9 floats (x, n, wo), 36 B,
// records of consecutive work items back to back.  k_guide_mlp_tc streams 128-record tiles into
// shared memory with the bulk-copy engine; every thread frequency-encodes its own row into the
// BF16 operand tile, already in the tensor core's shared-memory layout, and the warpgroup runs the
// four layers: two warpgroups per CTA share the staged weights; per warpgroup and tile one thread
// issues K/16 tcgen05.mma (M = 128, N = 64 or 48, K = 80 with the bias folded in below, BF16
// operands from shared-memory descriptors, FP32 accumulator in 64 tensor-memory columns) and
// commits them to an mbarrier; every thread then reads its row (tcgen05.ld), applies ReLU and
// writes BF16 for the next layer over the operand tile (the layer that read it has completed), or
// packs the mixture after the last.
// The next tile's record copy starts as soon as the current tile is encoded.
// Operand layout: K-major 8-row x 16-byte core matrices without swizzle; element (r, k) of a
// K-column operand sits at (r / 8) * 16K + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2 bytes, so one
// K=16 step spans two core matrices 128 B apart (descriptor LBO), 8-row groups 16K bytes apart (SBO).
constexpr int kTcRows = 128;
constexpr int kTcGroups = 2;                            // warpgroups per CTA
constexpr int kTcThreads = kTcRows * kTcGroups;
constexpr int kTcRecFloats = 9;                         // network input record: x, n, wo
constexpr int kTcRecBytes = kTcRows * kTcRecFloats * 4;   // one tile of records: 4608 B
// Every layer runs with K = 80: the 80 inputs of layer 0, or a layer's 64 inputs then 16 more
// columns.  Two columns of every operand row hold 1.0 (inputs 78-79 of layer 0, whose features are
// the encoding's two zeros; columns 64-65 of the hidden activations) and the matching weight
// columns the bias split into two BF16 halves (hi = bf16(b), lo = bf16(b - hi)), so the MMA adds
// the bias to within FP32 rounding and the epilogues only apply ReLU.
constexpr int kTcK = kGuideIn;
static_assert(kTcK >= kGuideHidden + 2 && kTcK % 16 == 0, "room for the bias columns");
__host__ __device__ constexpr int tc_bias_col(int l) { return l == 0 ? kGuideIn - 2 : kGuideHidden; }
constexpr int kTcTileBytes = kTcRows * kTcK * 2;        // one BF16 operand tile: 20480 B
// record bytes for n vertices: whole 128-row tiles
constexpr size_t stage_bytes(size_t n) { return (n + kTcRows - 1) / kTcRows * (size_t)kTcRecBytes; }
// weights of layer l, K-major: K = guide_k(l) (training kernel) or kTcK (inference kernel)
__host__ __device__ constexpr int tc_w_off(int l) { return l == 0 ? 0 : tc_w_off(l - 1) + guide_n(l - 1) * guide_k(l - 1) * 2; }
__host__ __device__ constexpr int tc_wi_off(int l) { return l == 0 ? 0 : tc_wi_off(l - 1) + guide_n(l - 1) * kTcK * 2; }
constexpr int kTcGroupBytes = kTcTileBytes + kTcRecBytes;  // operand tile (input, then hidden activations) + records
__host__ __device__ constexpr int tc_in(int g) { return tc_wi_off(4) + g * kTcGroupBytes; }
__host__ __device__ constexpr int tc_rec(int g) { return tc_in(g) + kTcTileBytes; }
constexpr int kTcBiasN = 3 * kGuideHidden + kGuideOutPad;   // (the training kernel's bias table)
constexpr int kTcBar = tc_wi_off(4) + kTcGroups * kTcGroupBytes;  // per warpgroup: MMA-done and input-full mbarriers
constexpr int kTcTmemSlot = kTcBar + 16 * kTcGroups;
constexpr size_t kTcSmem = (size_t)kTcTmemSlot + 8;
constexpr uint32_t kTcColsPerGroup = 64;
constexpr uint32_t kTcCols = kTcColsPerGroup * kTcGroups;  // tensor-memory columns per CTA (power of 2)
constexpr uint32_t kTcWaitPolls = 1u << 22;
static_assert(tc_in(0) % 128 == 0 && tc_rec(0) % 16 == 0 && kTcGroupBytes % 128 == 0 && kTcBar % 8 == 0,
              "operand, bulk-copy and barrier alignment");
static_assert(kTcRecBytes % 16 == 0 && (32 * kTcRecFloats * 4) % 16 == 0, "record tiles and warp chunks are 16-byte multiples");

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

// The encoded inputs of one vertex straight into row r of a W-wide operand tile (columns 0..79),
// eight values at a time: position p in the scene box as sin/cos(pi 2^f p), f = 0..11 per axis
// (one exactly reduced sincospif, then the double-angle recurrence sin 2u = 2 sin u cos u,
// cos 2u = (cos u - sin u)(cos u + sin u), whose absolute error grows about 2x per octave: ~1e-4 at
// 2^11, far below BF16 resolution), the shading normal, the outgoing direction, two zeros (two
// ones with BIAS_COLS: the inference kernel's bias columns).
template <int W = kGuideIn, bool BIAS_COLS = false>
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
                tc_store8(base, r, col, W, chunk);
                col += 8;
                fill = 0;
            }
            const float s2 = 2.f * s * c, c2 = (c - s) * (c + s);
            s = s2;
            c = c2;
        }
    }
    const float one = BIAS_COLS ? 1.f : 0.f;
    const float tail[8] = {n.x, n.y, n.z, wo.x, wo.y, wo.z, one, one};
    tc_store8(base, r, 72, W, tail);
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

// The guided buckets' vertices -> network input records (x, n, wo; kTcRecFloats floats each, work
// item i at floats [9 i, 9 i + 9)).  Each warp assembles its 32 consecutive records in shared
// memory and writes them as one contiguous 1152-byte run of float4 stores.
__global__ void __launch_bounds__(256) k_guide_record(DevScene S, const float4* __restrict__ ray_o,
                                                     const float4* __restrict__ ray_d, const float4* __restrict__ hits,
                                                     const int* bucket_cnt, const int* __restrict__ bucket_list, int cap,
                                                     int mask, float* rec) {
    __shared__ int bend[kBuckets];
    __shared__ __align__(16) float chunk[8][32 * kTcRecFloats];
    if (threadIdx.x == 0) guided_bucket_ends(bucket_cnt, mask, bend);
    __syncthreads();
    const int total = bend[kBuckets - 1];
    const int padded = (total + 31) & ~31;  // whole warps (the record buffer holds whole tiles)
    const int lane = threadIdx.x & 31;
    float* mine = chunk[threadIdx.x >> 5];
    for (int item = blockIdx.x * blockDim.x + threadIdx.x; item < padded; item += gridDim.x * blockDim.x) {
        float v[kTcRecFloats] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (item < total) {
            const int slot = guided_slot(bend, bucket_list, cap, item);
            const float4 o4 = ray_o[slot], d4 = ray_d[slot], h4 = hits[slot];
            Hit h{h4.x, h4.y, h4.z, __float_as_int(h4.w)};
            Surface sf;
            make_surface(S, f3(o4), f3(d4), h, sf);
            v[0] = sf.pos.x; v[1] = sf.pos.y; v[2] = sf.pos.z;
            v[3] = sf.N.x; v[4] = sf.N.y; v[5] = sf.N.z;
            v[6] = -d4.x; v[7] = -d4.y; v[8] = -d4.z;
        }
#pragma unroll
        for (int k = 0; k < kTcRecFloats; k++) mine[lane * kTcRecFloats + k] = v[k];
        __syncwarp();
        // the warp's items are item - lane .. item - lane + 31 (32-aligned): one contiguous run
        float4* dst = reinterpret_cast<float4*>(rec + (size_t)(item - lane) * kTcRecFloats);
        const float4* src = reinterpret_cast<const float4*>(mine);
        for (int q = lane; q < 32 * kTcRecFloats / 4; q += 32) dst[q] = src[q];
        __syncwarp();
    }
}

// Input: records (kTcRecFloats floats per work item, whole 128-row tiles; rows past the last item
// are not read).  MODE 0: the guided buckets' vertices, packed mixtures per work item (field-major,
// out_stride float4 per field); MODE 1: n_in explicit inputs, raw outputs (kGuideOut floats each).
template <int MODE>
__global__ void __launch_bounds__(kTcThreads, 2) k_guide_mlp_tc(GuideNet net, const unsigned char* __restrict__ stage,
                                                               const int* bucket_cnt, int mask, int n_in, float* out,
                                                               int out_stride, int* err) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int grp = threadIdx.x / kTcRows, row = threadIdx.x - grp * kTcRows, warp = threadIdx.x >> 5;
    const uint32_t bar_mma = smem_u32(smem + kTcBar + 16 * grp), bar_in = bar_mma + 8;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + kTcTmemSlot);
    // weights -> core-matrix layout with K = kTcK: the layer's weights (wt: N x K, K contiguous),
    // the two bias halves in the bias columns, zeros after them
#pragma unroll
    for (int l = 0; l < kGuideLayers; l++) {
        const int K = guide_k(l), N = guide_n(l), bc = tc_bias_col(l);
        const __nv_bfloat16* wt = net.bf + guide_bf_off(l);
        for (int i = threadIdx.x; i < N * (kTcK / 8); i += kTcThreads) {
            const int nn = i / (kTcK / 8), c = i - nn * (kTcK / 8);
            const float b = net.params[guide_b_off(l) + nn];
            const __nv_bfloat16 bh = __float2bfloat16_rn(b);
            const __nv_bfloat16 bl = __float2bfloat16_rn(b - __bfloat162float(bh));
            __align__(16) __nv_bfloat16 v[8];
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const int k = 8 * c + j;
                v[j] = k < bc ? wt[nn * K + k] : (k == bc ? bh : (k == bc + 1 ? bl : __float2bfloat16_rn(0.f)));
            }
            *reinterpret_cast<uint4*>(smem + tc_wi_off(l) + tc_cm(nn, 8 * c, kTcK)) = *reinterpret_cast<const uint4*>(v);
        }
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
    const float* REC = reinterpret_cast<const float*>(smem + tc_rec(grp));
    const int bar_id = 1 + grp;
    const int total = MODE == 0 ? bend[kBuckets - 1] : n_in;
    const int tiles = (total + kTcRows - 1) / kTcRows;
    const int tstride = gridDim.x * kTcGroups;
    int tile = blockIdx.x * kTcGroups + grp;
    // phases of the two barriers, and whether a record copy / an MMA group is outstanding (the same
    // in every thread of the warpgroup: issue decisions are uniform)
    uint32_t ph_mma = 0, ph_in = 0;
    bool copy_pending = false, mma_pending = false, failed = false;
    if (tile < tiles) {
        if (row == 0) {
            mbar_arrive_expect_tx(bar_in, kTcRecBytes);
            bulk_g2s(smem_u32(REC), stage + (size_t)tile * kTcRecBytes, kTcRecBytes, bar_in);
        }
        copy_pending = true;
    }
    for (; tile < tiles && !failed; tile += tstride) {
        bool ok = mbar_wait(bar_in, ph_in, kTcWaitPolls);
        if (ok) { ph_in ^= 1u; copy_pending = false; }
        const int item = tile * kTcRows + row;
        // this thread's row of the operand tile (the previous tile's last layer has completed)
        if (ok) {
            if (item < total) {
                const float* v = REC + row * kTcRecFloats;  // 9-float stride: conflict-free
                tc_encode_row<kTcK, true>(net, f3(v[0], v[1], v[2]), f3(v[3], v[4], v[5]), f3(v[6], v[7], v[8]), IN, row);
            } else {
                const float z[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
                for (int k = 0; k < kTcK; k += 8) tc_store8(IN, row, k, kTcK, z);
            }
        }
        float o[kGuideOutPad];
#pragma unroll
        for (int l = 0; l < kGuideLayers; l++) {
            const int N = guide_n(l);
            fence_async_smem();
            tc_fence_before();
            if (wg_sync_or(bar_id, !ok)) { failed = true; break; }
            if (row == 0) {
                tc_fence_after();
                const uint32_t a0 = smem_u32(IN), b0 = smem_u32(smem + tc_wi_off(l));
                const uint32_t idesc = umma_idesc_bf16(kTcRows, N);
                for (int kk = 0; kk < kTcK / 16; kk++)
                    umma_bf16(tmem, umma_desc(a0 + kk * 256, 128, kTcK * 16), umma_desc(b0 + kk * 256, 128, kTcK * 16), idesc,
                              kk > 0);
                umma_commit(bar_mma);
                if (l == 0 && tile + tstride < tiles) {
                    // every row of this tile is encoded: fetch the next tile's records behind the layers
                    mbar_arrive_expect_tx(bar_in, kTcRecBytes);
                    bulk_g2s(smem_u32(REC), stage + (size_t)(tile + tstride) * kTcRecBytes, kTcRecBytes, bar_in);
                }
            }
            if (l == 0 && tile + tstride < tiles) copy_pending = true;
            mma_pending = true;
            ok = mbar_wait(bar_mma, ph_mma, kTcWaitPolls);
            if (ok) { ph_mma ^= 1u; mma_pending = false; }
            if (wg_sync_or(bar_id, !ok)) { failed = true; break; }
            tc_fence_after();
            if (l < kGuideLayers - 1) {
                // the next layer's operand over this one's (its MMAs have completed): ReLU, BF16
#pragma unroll
                for (int c = 0; c < kGuideHidden; c += 32) {
                    uint32_t r[32];
                    tmem_ld16(trow + c, r);
                    tmem_ld16(trow + c + 16, r + 16);
                    tmem_wait();
#pragma unroll
                    for (int q = 0; q < 32; q += 8) {
                        uint4 u;
                        u.x = pack_bf16_relu(__uint_as_float(r[q + 0]), __uint_as_float(r[q + 1]));
                        u.y = pack_bf16_relu(__uint_as_float(r[q + 2]), __uint_as_float(r[q + 3]));
                        u.z = pack_bf16_relu(__uint_as_float(r[q + 4]), __uint_as_float(r[q + 5]));
                        u.w = pack_bf16_relu(__uint_as_float(r[q + 6]), __uint_as_float(r[q + 7]));
                        *reinterpret_cast<uint4*>(IN + tc_cm(row, c + q, kTcK)) = u;
                    }
                }
                if (l == 0) {
                    // the hidden layers' bias columns (1, 1) and zeros over the rest of the input
                    const float t0[8] = {1.f, 1.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                    const float t1[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                    tc_store8(IN, row, kGuideHidden, kTcK, t0);
                    tc_store8(IN, row, kGuideHidden + 8, kTcK, t1);
                }
            } else {
                uint32_t r[kGuideOutPad];
#pragma unroll
                for (int c = 0; c < kGuideOutPad; c += 16) tmem_ld16(trow + c, r + c);
                tmem_wait();
#pragma unroll
                for (int j = 0; j < kGuideOutPad; j++) o[j] = __uint_as_float(r[j]);
            }
        }
        if (failed) break;
        if (item < total) {
            if (MODE == 0) pack_lobes(o, reinterpret_cast<float4*>(out) + item, out_stride, net.kappa_max);
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

// ---- fused training step on the fifth-generation tensor cores (tcgen05) -------------------------
// One CTA per SM with two warpgroups, each working through its own 128-sample tiles; thread r of a
// warpgroup owns row r of its tiles.  Per tile:
//  * the thread encodes its sample into the input tile (BF16, the inference kernel's K-major core
//    layout);
//  * four forward layers: one thread issues tcgen05.mma (M = 128, BF16 operands from shared-memory
//    descriptors) into a 64-column tensor-memory scratch and commits to the warpgroup's mbarrier;
//    every thread reads its row back (tcgen05.ld), adds the bias, applies ReLU and writes the next
//    activation tile;
//  * the loss gradient at the 41 outputs, one row per thread, stored as the output-delta tile;
//  * per layer j = 3, 2, 1 one commit group with the input gradient G = delta_j W_j^T (A: the delta
//    tile; B: the forward weight copy read MN-major) and the weight gradient
//    dW_j += [a_j | 1]^T delta_j over the tile's 128 samples (both operands read MN-major from the
//    activation and delta tiles, so no transposed copies are written); then delta_{j-1} =
//    G * relu'(a_j) replaces a_j in place (the MMA that read a_j has completed);
//  * dW_0 = [a_0 | 1]^T delta_0 into the scratch, added row by row (81 rows) into the warpgroup's
//    partial gradient in global memory (a region only this warpgroup touches).
// Every activation tile carries a constant-one column behind its features, so row K_j of dW_j is
// the bias gradient.  dW_1..dW_3 accumulate in tensor memory over all tiles of the launch.  Each
// warpgroup finally writes its partial gradient of every parameter; k_guide_adam sums them.
// MN-major operands (no swizzle) are 8 K-rows x 16-byte (8 element) core matrices; the descriptor's
// SBO is the byte stride between 8-element groups along M or N, its LBO the stride between 8-row
// groups along K.  An M = 128 weight-gradient operand covers 128 features of a narrower tile: rows
// past the tile's features read other rows' values (finite BF16 numbers inside the allocation) and
// land in tensor-memory rows that are never read.
constexpr int kTgGroups = 2;                             // warpgroups per CTA
constexpr int kTgThreads = 128 * kTgGroups;
constexpr int kTgW0 = kGuideIn + 8;                      // input tile: 80 encoded inputs, the one column
constexpr int kTgWH = kGuideHidden + 8;                  // hidden tiles: 64 activations, the one column
constexpr int kTgWO = kGuideOutPad;                      // output-delta tile
constexpr int kTgA0 = 128 * kTgW0 * 2;
constexpr int kTgH = 128 * kTgWH * 2;
constexpr int kTgD = 128 * kTgWO * 2;
constexpr int kTgGroupBytes = kTgA0 + 3 * kTgH + kTgD;
// weights sit behind both warpgroups' tiles, so every operand read stays inside the allocation
constexpr int kTgWts = kTgGroups * kTgGroupBytes;
constexpr int kTgBias = kTgWts + tc_w_off(4);
constexpr int kTgBar = kTgBias + kTcBiasN * 4;
constexpr int kTgSlot = kTgBar + 8 * kTgGroups;
// Slack behind the last buffer: the MN-major weight operand of G = delta_3 W_3^T would reach up to
// 5.4 KB past the weights if the descriptor's two strides were read the other way round, and the
// allocation covers that reach too.
constexpr int kTgSlack = 8192;
constexpr size_t kTgSmem = (size_t)kTgSlot + 8 + kTgSlack;
constexpr uint32_t kTgColsPerGroup = 256;                // scratch 64 | dW_1 64 | dW_2 64 | dW_3 48
constexpr uint32_t kTgCols = kTgColsPerGroup * kTgGroups;
static_assert(kTgA0 % 128 == 0 && kTgH % 128 == 0 && kTgD % 128 == 0 && kTgWts % 128 == 0 && kTgBar % 8 == 0,
              "operand and barrier alignment");
static_assert(kTgSmem <= 232448, "training tiles fit one CTA's shared memory");
static_assert(64 + 2 * kGuideHidden + kGuideOutPad <= (int)kTgColsPerGroup, "tensor-memory columns per warpgroup");

// Instruction descriptor with the A and / or B operand read MN-major.
__host__ __device__ constexpr uint32_t umma_idesc_mn(int N, bool a_mn, bool b_mn) {
    return umma_idesc_bf16(128, N) | (a_mn ? 1u << 15 : 0u) | (b_mn ? 1u << 16 : 0u);
}
static_assert(umma_idesc_mn(64, true, true) == (umma_idesc_bf16(128, 64) | (3u << 15)), "transpose bits");

// Gradient of w * -log q_mix(wi), q_mix = (1 - c) p_bsdf + c q_guide, with respect to the 41 raw
// outputs o (see the oracle for the formulas), each handed to put(k, g_k) as soon as it is known
// (clamped to [-1e3, 1e3], a non-finite value as 0); returns -log q_mix.
template <class Put>
__device__ __forceinline__ float nll_output_grad(const float* o, float3 wi, float w, float pb, float kappa_max, Put put) {
    auto clamped = [](float v) { return isfinite(v) ? fminf(fmaxf(v, -1e3f), 1e3f) : 0.f; };
    Lobe L[kGuideLobes];
    guide_lobes(o, L, kappa_max);
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
        if (kap >= kappa_max) sig = 0.f;
        const float3 m = f3(o[5 * k], o[5 * k + 1], o[5 * k + 2]);
        const float len = fmaxf(sqrtf(dot(m, m)), 1e-12f);
        const float3 dm = (wi - L[k].mu * c) * (kap / len);
        put(5 * k + 0, clamped(-w * rho * r * dm.x));
        put(5 * k + 1, clamped(-w * rho * r * dm.y));
        put(5 * k + 2, clamped(-w * rho * r * dm.z));
        put(5 * k + 3, clamped(-w * rho * r * dk * sig));
        put(5 * k + 4, clamped(-w * rho * (r - L[k].w)));
    }
    put(40, clamped(-w * (q - pb) * kGuideSelSpan * sg * (1.f - sg) / qmix));
    return -__logf(qmix);
}

__global__ void __launch_bounds__(kTgThreads, 1) k_guide_train_tc(GuideNet net, const float4* __restrict__ batch,
                                                                 const int* batch_count, int batch_cap, float* part,
                                                                 float* stats, int splits, const int* __restrict__ step,
                                                                 int* err) {
    extern __shared__ __align__(128) unsigned char smem[];
    const int grp = threadIdx.x >> 7, row = threadIdx.x & 127, warp = threadIdx.x >> 5;
    unsigned char* const A0 = smem + grp * kTgGroupBytes;
    unsigned char* const H1 = A0 + kTgA0;
    unsigned char* const H2 = H1 + kTgH;
    unsigned char* const H3 = H2 + kTgH;
    unsigned char* const DO = H3 + kTgH;
    unsigned char* const WT = smem + kTgWts;
    float* bias = reinterpret_cast<float*>(smem + kTgBias);
    const uint32_t bar = smem_u32(smem + kTgBar + 8 * grp);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + kTgSlot);
    // forward weights in the K-major core layout (as inference), biases
#pragma unroll
    for (int l = 0; l < kGuideLayers; l++) {
        const int K = guide_k(l), N = guide_n(l), vpr = K / 8;
        const uint4* src = reinterpret_cast<const uint4*>(net.bf + guide_bf_off(l));
        for (int i = threadIdx.x; i < N * vpr; i += kTgThreads) {
            const int nn = i / vpr, c = i - nn * vpr;
            *reinterpret_cast<uint4*>(WT + tc_w_off(l) + tc_cm(nn, 8 * c, K)) = src[i];
        }
    }
    for (int i = threadIdx.x; i < kTcBiasN; i += kTgThreads) {
        const int l = i < 3 * kGuideHidden ? i / kGuideHidden : 3;
        bias[i] = net.params[guide_b_off(l) + (i - l * kGuideHidden)];
    }
    // the constant-one columns (then seven zeros) of this thread's rows and the padding outputs of
    // its delta row; the epilogues never write them
    {
        const float one[8] = {1.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        const float z[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        tc_store8(A0, row, kGuideIn, kTgW0, one);
        tc_store8(H1, row, kGuideHidden, kTgWH, one);
        tc_store8(H2, row, kGuideHidden, kTgWH, one);
        tc_store8(H3, row, kGuideHidden, kTgWH, one);
        tc_store8(DO, row, kGuideOutPad - 8, kTgWO, z);
    }
    if (threadIdx.x == 0) {
        for (int g = 0; g < kTgGroups; g++) mbar_init(smem_u32(smem + kTgBar + 8 * g), 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) tmem_alloc(smem_u32(tslot), kTgCols);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tS = *tslot + grp * kTgColsPerGroup;            // scratch (lane 0, column base)
    const uint32_t tW1 = tS + 64, tW2 = tS + 128, tW3 = tS + 192;   // weight-gradient accumulators
    const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;    // this warp's 32 lanes
    const int bar_id = 1 + grp;

    const int n = min(*batch_count, batch_cap);
    const float mean_w = stats[2] / fmaxf(1.f, (float)n);
    // minibatch of this Adam step: the batch split into `splits` windows, taken in turn
    const int per = (n + splits - 1) / splits;
    const int lo = min(n, (*step % splits) * per), hi = min(n, lo + per);
    const int tiles = (hi - lo + 127) / 128;

    float loss = 0.f, wsum = 0.f;
    float* P = part + (size_t)(blockIdx.x * kTgGroups + grp) * kGuideParams;
    // row K_0 of dW_0 is the bias gradient b_0
    float* dw0_row = row < kGuideIn ? P + guide_w_off(0) + row * kGuideHidden : P + guide_b_off(0);
    uint32_t ph = 0;
    bool failed = false, pending = false, have = false;

    // Make this warpgroup's shared-memory writes visible to the tensor core, let one thread issue
    // `mma` and commit it, and wait (bounded) for completion.  Returns false once a wait timed out.
    auto run = [&](auto&& mma) -> bool {
        fence_async_smem();
        tc_fence_before();
        if (wg_sync_or(bar_id, failed)) { failed = true; return false; }
        if (row == 0) {
            tc_fence_after();
            mma();
            umma_commit(bar);
        }
        pending = true;
        const bool ok = mbar_wait(bar, ph, kTcWaitPolls);
        if (ok) { ph ^= 1u; pending = false; }
        if (wg_sync_or(bar_id, !ok)) { failed = true; return false; }
        tc_fence_after();
        return true;
    };
    // forward layer l: scratch = a_l W_l (a_l: W-wide tile, K-major; W_l: K-major)
    auto fwd = [&](int l, const unsigned char* a, int W) {
        const int K = guide_k(l), N = guide_n(l);
        const uint32_t a0 = smem_u32(a), b0 = smem_u32(WT + tc_w_off(l));
        for (int kk = 0; kk < K / 16; kk++)
            umma_bf16(tS, umma_desc(a0 + kk * 256, 128, 16 * W), umma_desc(b0 + kk * 256, 128, 16 * K),
                      umma_idesc_bf16(128, N), kk > 0);
    };
    // input gradient of layer j: scratch = delta_j W_j^T (K = layer j's outputs, N = its 64 inputs)
    auto grad_in = [&](int j, const unsigned char* d, int W) {
        const int K = guide_n(j), N = guide_k(j);
        const uint32_t a0 = smem_u32(d), b0 = smem_u32(WT + tc_w_off(j));
        for (int kk = 0; kk < K / 16; kk++)
            umma_bf16(tS, umma_desc(a0 + kk * 256, 128, 16 * W), umma_desc(b0 + kk * 32 * N, 16 * N, 128),
                      umma_idesc_mn(N, false, true), kk > 0);
    };
    // weight gradient of layer j: D (+)= [a_j | 1]^T delta_j over the tile's 128 samples
    auto grad_w = [&](int j, uint32_t dst, const unsigned char* a, int Wa, const unsigned char* d, int Wd, bool acc) {
        const uint32_t a0 = smem_u32(a), b0 = smem_u32(d);
        for (int kk = 0; kk < 8; kk++)
            umma_bf16(dst, umma_desc(a0 + kk * 32 * Wa, 16 * Wa, 128), umma_desc(b0 + kk * 32 * Wd, 16 * Wd, 128),
                      umma_idesc_mn(guide_n(j), true, true), acc || kk > 0);
    };
    // delta_{j-1} = G * relu'(a_j), written over a_j (this thread's row)
    auto delta = [&](unsigned char* a) {
#pragma unroll
        for (int c = 0; c < kGuideHidden; c += 32) {
            uint32_t r[32];
            tmem_ld16(tS + lane_off + c, r);
            tmem_ld16(tS + lane_off + c + 16, r + 16);
            tmem_wait();
#pragma unroll
            for (int q = 0; q < 32; q += 8) {
                const uint4 hv = *reinterpret_cast<const uint4*>(a + tc_cm(row, c + q, kTgWH));
                const __nv_bfloat16* h = reinterpret_cast<const __nv_bfloat16*>(&hv);
                float v[8];
#pragma unroll
                for (int e = 0; e < 8; e++) v[e] = __bfloat162float(h[e]) > 0.f ? __uint_as_float(r[q + e]) : 0.f;
                tc_store8(a, row, c + q, kTgWH, v);
            }
        }
    };

    for (int t = blockIdx.x * kTgGroups + grp; t < tiles && !failed; t += gridDim.x * kTgGroups) {
        const int j = lo + t * 128 + row;
        const bool valid = j < hi;
        float3 wi = f3(0.f, 0.f, 1.f);
        float w = 0.f, pb = 0.f;
        if (valid) {
            const float4 b0 = batch[4 * j], b1 = batch[4 * j + 1], b2 = batch[4 * j + 2], b3 = batch[4 * j + 3];
            tc_encode_row<kTgW0>(net, f3(b0), f3(b1), f3(b2), A0, row);
            wi = f3(b3);
            pb = b3.w;
            w = fminf(b0.w / fmaxf(mean_w, 1e-12f), net.weight_clamp);  // normalised, firefly-clamped weight
        } else {
            const float z[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int k = 0; k < kGuideIn; k += 8) tc_store8(A0, row, k, kTgW0, z);
        }
        // ---- forward
        float o[kGuideOutPad];
        unsigned char* act[4] = {A0, H1, H2, H3};
#pragma unroll
        for (int l = 0; l < kGuideLayers; l++) {
            if (!run([&] { fwd(l, act[l], l == 0 ? kTgW0 : kTgWH); })) break;
            if (l < kGuideLayers - 1) {
#pragma unroll
                for (int c = 0; c < kGuideHidden; c += 32) {
                    uint32_t r[32];
                    tmem_ld16(tS + lane_off + c, r);
                    tmem_ld16(tS + lane_off + c + 16, r + 16);
                    tmem_wait();
#pragma unroll
                    for (int q = 0; q < 32; q += 8) {
                        float v[8];
#pragma unroll
                        for (int e = 0; e < 8; e++) v[e] = fmaxf(__uint_as_float(r[q + e]) + bias[l * kGuideHidden + c + q + e], 0.f);
                        tc_store8(act[l + 1], row, c + q, kTgWH, v);
                    }
                }
            } else {
                uint32_t r[kGuideOutPad];
#pragma unroll
                for (int c = 0; c < kGuideOutPad; c += 16) tmem_ld16(tS + lane_off + c, r + c);
                tmem_wait();
#pragma unroll
                for (int k = 0; k < kGuideOutPad; k++) o[k] = __uint_as_float(r[k]) + bias[3 * kGuideHidden + k];
            }
        }
        if (failed) break;
        // ---- loss gradient at the outputs (BF16, straight into this row of the delta tile; its
        // padding columns 41..47 stay zero)
        if (valid && w > 0.f) {
            loss += w * nll_output_grad(o, wi, w, pb, net.kappa_max, [&](int k, float v) {
                *reinterpret_cast<__nv_bfloat16*>(DO + tc_cm(row, k, kTgWO)) = __float2bfloat16_rn(v);
            });
            wsum += w;
        } else {
            const float z[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int k = 0; k < kGuideOutPad; k += 8) tc_store8(DO, row, k, kTgWO, z);
        }
        // ---- backward
        if (!run([&] { grad_in(3, DO, kTgWO); grad_w(3, tW3, H3, kTgWH, DO, kTgWO, have); })) break;
        delta(H3);
        if (!run([&] { grad_in(2, H3, kTgWH); grad_w(2, tW2, H2, kTgWH, H3, kTgWH, have); })) break;
        delta(H2);
        if (!run([&] { grad_in(1, H2, kTgWH); grad_w(1, tW1, H1, kTgWH, H2, kTgWH, have); })) break;
        delta(H1);
        if (!run([&] { grad_w(0, tS, A0, kTgW0, H1, kTgWH, false); })) break;
#pragma unroll
        for (int c = 0; c < kGuideHidden; c += 32) {
            uint32_t r[32];
            tmem_ld16(tS + lane_off + c, r);
            tmem_ld16(tS + lane_off + c + 16, r + 16);
            tmem_wait();
            if (row <= kGuideIn) {
                float4* d4 = reinterpret_cast<float4*>(dw0_row + c);
#pragma unroll
                for (int q = 0; q < 8; q++) {
                    float4 v = make_float4(__uint_as_float(r[4 * q]), __uint_as_float(r[4 * q + 1]), __uint_as_float(r[4 * q + 2]),
                                           __uint_as_float(r[4 * q + 3]));
                    if (have) {
                        const float4 u = d4[q];
                        v.x += u.x; v.y += u.y; v.z += u.z; v.w += u.w;
                    }
                    d4[q] = v;
                }
            }
        }
        have = true;
    }
    if (failed) {
        if (row == 0) dev_flag_error(err, DEVERR_WAIT);
        if (pending) mbar_wait(bar, ph, kTcWaitPolls);  // the MMAs still in flight finish (bounded)
    }
    // ---- this warpgroup's partial gradient: rows 0..K-1 of dW_l are weights, row K the bias
    tc_fence_before();
    wg_sync(bar_id);
    tc_fence_after();
    const bool use = have && !failed;
    if (!use && row <= kGuideIn) {
#pragma unroll
        for (int k = 0; k < kGuideHidden; k++) dw0_row[k] = 0.f;
    }
    const uint32_t tW[4] = {0u, tW1, tW2, tW3};
    for (int l = 1; l < kGuideLayers; l++) {
        const int N = guide_n(l);
        float* dst = row < kGuideHidden ? P + guide_w_off(l) + row * N : P + guide_b_off(l);
        for (int c = 0; c < N; c += 16) {
            uint32_t r[16];
            if (use) {
                tmem_ld16(tW[l] + lane_off + c, r);
                tmem_wait();
            } else {
#pragma unroll
                for (int k = 0; k < 16; k++) r[k] = 0u;
            }
            if (row <= kGuideHidden) {
                float4* d4 = reinterpret_cast<float4*>(dst + c);
#pragma unroll
                for (int k = 0; k < 4; k++)
                    d4[k] = make_float4(__uint_as_float(r[4 * k]), __uint_as_float(r[4 * k + 1]), __uint_as_float(r[4 * k + 2]),
                                        __uint_as_float(r[4 * k + 3]));
            }
        }
    }
    for (int s = 16; s > 0; s >>= 1) {
        loss += __shfl_down_sync(0xffffffffu, loss, s);
        wsum += __shfl_down_sync(0xffffffffu, wsum, s);
    }
    if ((threadIdx.x & 31) == 0 && wsum != 0.f) {
        atomicAdd(stats + 0, loss);
        atomicAdd(stats + 1, wsum);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_free(*tslot, kTgCols);
    }
}

// Adam on the FP32 master weights: the gradient is the sum of the training kernel's per-warpgroup
// partials, normalised by the batch weight sum; then the two BF16 layouts the kernels read.  The
// padded output columns stay zero.
__global__ void k_guide_adam(float* params, const float* __restrict__ part, int nparts, float* m, float* v,
                             __nv_bfloat16* bfw, const float* stats, float lr, float b1, float b2, float eps,
                             const int* step, float decay_steps) {
    const float norm = 1.f / fmaxf(stats[1], 1e-12f);
    // bias corrections of Adam step t = *step + 1 (the counter lives on the device so that captured
    // graphs replay correctly; k_guide_tick advances it)
    const float t = (float)(*step + 1);
    const float c1 = 1.f - powf(b1, t), c2 = 1.f - powf(b2, t);
    // learning rate lr / (1 + t / decay_steps) (decay_steps 0: constant)
    if (decay_steps > 0.f) lr = lr / (1.f + t / decay_steps);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < kGuideParams; p += gridDim.x * blockDim.x) {
        int l = 3;
        while (l > 0 && p < guide_w_off(l)) l--;
        int K = guide_k(l), N = guide_n(l);
        int rel = p - guide_w_off(l);
        bool is_bias = rel >= K * N;
        int kk = is_bias ? 0 : rel / N, nn = is_bias ? rel - K * N : rel % N;
        bool pad = (l == 3) && (nn >= kGuideOut);
        float sum = 0.f;
        for (int q = 0; q < nparts; q++) sum += part[(size_t)q * kGuideParams + p];
        float g = pad ? 0.f : sum * norm;
        if (!isfinite(g)) g = 0.f;  // a non-finite batch leaves the weights unchanged
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

// Sum of the per-warpgroup partial gradients (the explicit-batch gradient entry point).
__global__ void k_guide_reduce(const float* __restrict__ part, int nparts, float* grad) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < kGuideParams; p += gridDim.x * blockDim.x) {
        float sum = 0.f;
        for (int q = 0; q < nparts; q++) sum += part[(size_t)q * kGuideParams + p];
        grad[p] = sum;
    }
}

// After an Adam step: advance the step counter, keep the step's loss and weight sum for reporting
// (stats[4..5]) and clear the accumulators for the next step.
__global__ void k_guide_tick(int* step, float* stats) {
    *step += 1;
    stats[4] = stats[0];
    stats[5] = stats[1];
    stats[0] = 0.f;
    stats[1] = 0.f;
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

}  // namespace

// ---- host -------------------------------------------------------------------------------------------
GuideTrainer::~GuideTrainer() = default;

void GuideTrainer::release(DeviceArena& arena) {
    void* ps[] = {params_, grad_, part_, adam_m_, adam_v_, bf_, out_, stage_, rec_, batch_, batch_count_, loss_acc_, step_dev_};
    for (void* p : ps)
        if (p) arena.free(p);
    params_ = grad_ = part_ = adam_m_ = adam_v_ = nullptr;
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
        prepare_launch();
        nparts_ = train_parts();
        params_ = (float*)A(kGuideParams * 4);
        grad_ = (float*)A(kGuideParams * 4);
        part_ = (float*)A((size_t)nparts_ * kGuideParams * 4);
        adam_m_ = (float*)A(kGuideParams * 4);
        adam_v_ = (float*)A(kGuideParams * 4);
        bf_ = (__nv_bfloat16*)A(kGuideBf16 * 2);
        loss_acc_ = (float*)A(32);
        batch_count_ = (int*)A(16);
        step_dev_ = (int*)A(16);
        if (!params_ || !grad_ || !part_ || !adam_m_ || !adam_v_ || !bf_ || !loss_acc_ || !batch_count_ || !step_dev_)
            return C2G_ERR_OOM;
        cudaMemset(step_dev_, 0, 16);
        cudaMemset(loss_acc_, 0, 32);
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
        cudaFuncSetAttribute(k_guide_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTgSmem);
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
        // about rec_target_ recorded vertices per wave: every rec_stride-th path records its bounces
        rec_stride_ = (int)std::max<size_t>(1, paths * 3 / (size_t)rec_target_);
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
    cudaFuncSetAttribute(k_guide_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTgSmem);
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
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_enc, k_guide_record, 256, 0);
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
    k_guide_record<<<g_encode_grid, 256, 0, st>>>(S, ray_o, ray_d, hits, bucket_cnt, bucket_list, cap, mask, (float*)stage_);
    k_guide_mlp_tc<0><<<grid, kTcThreads, kTcSmem, st>>>(net, stage_, bucket_cnt, mask, 0, out_, (int)cap_, S.err);
    return 2;
}

int GuideTrainer::train_parts() {
    prepare_launch();
    return g_train_grid * kTgGroups;
}

void GuideTrainer::train(cudaStream_t st, const float4* out_L, int wave_paths, int steps, int* err) {
    cudaMemsetAsync(batch_count_, 0, 16, st);
    cudaMemsetAsync(loss_acc_, 0, 32, st);
    k_guide_batch<<<(int)std::min<size_t>(4096, (rec_cap_ + 255) / 256), 256, 0, st>>>(
        rec_, (int)rec_cap_, rec_depth_, rec_stride_, out_L, wave_paths, batch_, batch_count_, loss_acc_, (int)rec_cap_);
    prepare_launch();
    GuideNet net = view(false, false).net;
    // per Adam step: the fused tensor-core forward/backward over one minibatch window (partial
    // gradients per warpgroup), Adam over their sum, and the step counter; k_guide_tick clears the
    // loss accumulators for the next step
    for (int s = 0; s < steps; s++) {
        k_guide_train_tc<<<g_train_grid, kTgThreads, kTgSmem, st>>>(net, batch_, batch_count_, (int)rec_cap_, part_, loss_acc_,
                                                                   std::min(steps, windows_), step_dev_, err);
        steps_++;
        k_guide_adam<<<64, 256, 0, st>>>(params_, part_, nparts_, adam_m_, adam_v_, bf_, loss_acc_, lr_, 0.9f, 0.99f, 1e-8f,
                                         step_dev_, lr_decay_);
        k_guide_tick<<<1, 1, 0, st>>>(step_dev_, loss_acc_);
    }
}

GuideView GuideTrainer::view(bool record, bool sample) const {
    GuideView v{};
    v.net.bf = bf_;
    v.net.params = params_;
    for (int a = 0; a < 3; a++) { v.net.box_lo[a] = box_lo_[a]; v.net.box_inv[a] = box_inv_[a]; }
    v.net.alpha = alpha_;
    v.net.enabled = sample ? 1 : 0;
    v.net.kappa_max = kappa_max_;
    v.net.weight_clamp = weight_clamp_;
    v.out = out_;
    v.out_stride = (int)cap_;
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
    // the inputs are already records (9 floats each); the buffer holds whole tiles
    float* din = (float*)arena.alloc(stage_bytes((size_t)n), err);
    float* dout = (float*)arena.alloc((size_t)n * kGuideOut * 4, err);
    int* derr = (int*)arena.alloc(16, err);
    int rc = C2G_OK;
    if (!din || !dout || !derr) rc = C2G_ERR_OOM;
    if (!rc) {
        cudaMemcpy(din, host_xnw, (size_t)n * 9 * 4, cudaMemcpyHostToDevice);
        cudaMemset(derr, 0, 16);
        prepare_launch();
        const GuideNet net = view(false, false).net;
        const int blocks = std::min(g_infer_grid, (n + kTcThreads - 1) / kTcThreads);
        k_guide_mlp_tc<1><<<blocks, kTcThreads, kTcSmem>>>(net, (const unsigned char*)din, nullptr, 0, n, dout, 0, derr);
        int h = 0;
        if (cudaDeviceSynchronize() != cudaSuccess) { err = cudaGetErrorString(cudaGetLastError()); rc = C2G_ERR_CUDA; }
        else if (cudaMemcpy(&h, derr, 4, cudaMemcpyDeviceToHost) == cudaSuccess && h) {
            err = "guide inference: tensor-core completion wait timed out";
            rc = C2G_ERR_DEVICE;
        } else cudaMemcpy(host_out, dout, (size_t)n * kGuideOut * 4, cudaMemcpyDeviceToHost);
    }
    if (din) arena.free(din);
    if (dout) arena.free(dout);
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
    int* derr = (int*)arena.alloc(16, err);
    if (!db || !derr) {
        if (db) arena.free(db);
        if (derr) arena.free(derr);
        return C2G_ERR_OOM;
    }
    // stats[2] = n makes the kernel's weight normaliser (mean weight) exactly 1
    float st[8] = {0.f, 0.f, (float)n, 0.f, 0.f, 0.f, 0.f, 0.f};
    cudaMemcpy(db, b.data(), b.size() * 16, cudaMemcpyHostToDevice);
    cudaMemcpy(batch_count_, &n, 4, cudaMemcpyHostToDevice);
    cudaMemcpy(loss_acc_, st, 32, cudaMemcpyHostToDevice);
    cudaMemset(derr, 0, 16);
    prepare_launch();
    k_guide_train_tc<<<g_train_grid, kTgThreads, kTgSmem>>>(view(false, false).net, db, batch_count_, n, part_, loss_acc_, 1,
                                                           step_dev_, derr);
    k_guide_reduce<<<64, 256>>>(part_, nparts_, grad_);
    int rc = C2G_OK, h = 0;
    if (cudaDeviceSynchronize() != cudaSuccess) { err = cudaGetErrorString(cudaGetLastError()); rc = C2G_ERR_CUDA; }
    else if (cudaMemcpy(&h, derr, 4, cudaMemcpyDeviceToHost) == cudaSuccess && h) {
        err = "guide training: tensor-core completion wait timed out";
        rc = C2G_ERR_DEVICE;
    } else {
        cudaMemcpy(host_grad, grad_, kGuideParams * 4, cudaMemcpyDeviceToHost);
        cudaMemcpy(st, loss_acc_, 32, cudaMemcpyDeviceToHost);
        if (loss) *loss = st[1] > 0 ? (double)st[0] / st[1] : 0.0;
    }
    cudaMemset(loss_acc_, 0, 32);
    arena.free(db);
    arena.free(derr);
    return rc;
}

GuideStats GuideTrainer::stats() {
    float h[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int n = 0;
    if (loss_acc_) cudaMemcpy(h, loss_acc_, 32, cudaMemcpyDeviceToHost);
    if (batch_count_) cudaMemcpy(&n, batch_count_, 4, cudaMemcpyDeviceToHost);
    int t = steps_;
    if (step_dev_) cudaMemcpy(&t, step_dev_, 4, cudaMemcpyDeviceToHost);
    last_.loss = h[5] > 0 ? h[4] / h[5] : 0.0;  // the last Adam step's batch
    last_.records = n;
    last_.steps = t;
    return last_;
}

}  // namespace c2g
