// Wavefront path tracer for sm_103a: kernels and their host orchestration.
//
// One wave = a fixed set of camera paths (all pixels x a range of samples).  Per bounce:
//   extend     closest hit of every queued path ray                      (BVH::Intersect)
//   shade      hit record -> emission, NEE rays, BSDF continuation, RR   (Evaluate + EsimateDirect)
//   shadow     any-hit of the NEE light-sample rays                      (BVH::IntersectTest)
//   mis        closest hit of the NEE BSDF-sample rays + emitter check   (EsimateDirect, BSDF half)
//   accumulate direct lighting added to the path radiance; finished paths written out
// and at the end of the wave `film` adds every sample to its pixel in sample order
// (FrameBuffer::AddSample).  Path state is SoA in float4 arrays and is compacted into the
// next queue with warp ballot/popc appends, so every kernel reads its inputs coalesced.
#include <algorithm>
#include <functional>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../host/bvh.h"
#include "../host/scene.h"
#include "guide.cuh"
#include "render.h"
#include "shade.cuh"

namespace c2g {

// ---- arena -----------------------------------------------------------------------------------
DeviceArena::~DeviceArena() { free_all(); }

void* DeviceArena::alloc(size_t bytes, std::string& err) {
    if (bytes == 0) bytes = 16;
    bytes = (bytes + 255) & ~size_t(255);
    if (cap_ && used_ + bytes > cap_) {
        err = "device memory cap exceeded (" + std::to_string(used_) + " in use + " + std::to_string(bytes) + " requested > " +
              std::to_string(cap_) + " bytes)";
        return nullptr;
    }
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        err = std::string("cudaMalloc failed: ") + cudaGetErrorString(e);
        return nullptr;
    }
    blocks_.push_back({p, bytes});
    used_ += bytes;
    return p;
}

void DeviceArena::free(void* p) {
    if (!p) return;
    for (size_t i = 0; i < blocks_.size(); i++) {
        if (blocks_[i].p == p) {
            cudaFree(p);
            used_ -= blocks_[i].n;
            blocks_.erase(blocks_.begin() + i);
            return;
        }
    }
}

void DeviceArena::free_all() {
    for (auto& b : blocks_) cudaFree(b.p);
    blocks_.clear();
    used_ = 0;
}

// ---- buffers -----------------------------------------------------------------------------------
struct DeviceSceneBuffers {
    DevScene S{};
    std::vector<void*> owned;
    int* err = nullptr;
    unsigned long long* counts = nullptr;  // nodes/prims counters (closest, any)
    int* fetch = nullptr;                  // ray-query fetch counter
    float4* film = nullptr;                // rgb sum, weight
    float4* film_m2 = nullptr;             // rgb sum of squares
    float* film_pack = nullptr;            // downloads: rgb (3 floats per pixel) then weights
    int n_lights = 0;
};

struct WaveBuffers {
    size_t P = 0;     // path capacity
    int K = 0;        // NEE slots per path
    float4* o[2] = {nullptr, nullptr};
    float4* d[2] = {nullptr, nullptr};
    float4* beta[2] = {nullptr, nullptr};
    float4* L[2] = {nullptr, nullptr};
    float4* hit = nullptr;
    int2* acc = nullptr;
    float4* out_L = nullptr;
    float4* sh_o = nullptr;
    float4* sh_d = nullptr;
    float4* sh_c = nullptr;
    float4* mis_o = nullptr;
    float4* mis_d = nullptr;
    float4* mis_c = nullptr;
    float4* mis_hit = nullptr;
    int* sh_list = nullptr;
    int* mis_list = nullptr;
    int* bucket_list = nullptr;  // kBuckets lists of P slots
    int* counters = nullptr;  // [0],[1] path queues, [2] shadow, [3] mis, [8..20) material buckets
    int* levels = nullptr;    // statistics: paths entering each bounce level (C2G_LEVELS)
    std::vector<void*> owned;
};

GpuScene::GpuScene() : sb_(new DeviceSceneBuffers()), wb_(new WaveBuffers()) {}
GpuScene::~GpuScene() {
    if (side_) cudaStreamDestroy(side_);
    if (ahead_) cudaStreamDestroy(ahead_);
    for (int k = 0; k < 4; k++) {
        if (fork_ev_[k]) cudaEventDestroy(fork_ev_[k]);
        if (join_ev_[k]) cudaEventDestroy(join_ev_[k]);
    }
    delete sb_;
    delete wb_;
}

int GpuScene::side_stream(std::string& err) {
    if (side_) return C2G_OK;
    if (cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking) != cudaSuccess) {
        err = "cannot create the side stream";
        side_ = nullptr;
        return C2G_ERR_CUDA;
    }
    if (cudaStreamCreateWithFlags(&ahead_, cudaStreamNonBlocking) != cudaSuccess) {
        err = "cannot create the look-ahead stream";
        ahead_ = nullptr;
        return C2G_ERR_CUDA;
    }
    for (int k = 0; k < 4; k++)
        if (cudaEventCreateWithFlags(&fork_ev_[k], cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&join_ev_[k], cudaEventDisableTiming) != cudaSuccess) {
            err = "cannot create stream events";
            return C2G_ERR_CUDA;
        }
    return C2G_OK;
}

// ---- small device helpers ------------------------------------------------------------------------
__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

// Warp-aggregated append: one atomic per warp, lanes with pred get consecutive slots in lane order.
// Must be called by all 32 lanes of the warp.
__device__ __forceinline__ int warp_append(int* counter, bool pred) {
    unsigned m = __ballot_sync(0xffffffffu, pred);
    int base = 0;
    if (lane_id() == 0 && m) base = atomicAdd(counter, __popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    return pred ? base + __popc(m & ((1u << lane_id()) - 1u)) : -1;
}

__device__ __forceinline__ void warp_count(unsigned long long* dst, unsigned v) {
    unsigned long long s = v;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane_id() == 0 && s) atomicAdd(dst, s);
}


__device__ __forceinline__ int wave_sample0(const WaveArgs& a) { return a.sample0_dev ? *a.sample0_dev : a.sample0; }

__device__ __forceinline__ void slot_pixel(const WaveArgs& a, int slot, int& x, int& y) {
    int tile = slot >> 6, w = slot & 63;
    x = (tile % a.tiles_x) * 8 + (w & 7);
    y = (tile / a.tiles_x) * 8 + (w >> 3);
}

// Path state word: Halton dimension (16 bits), bounce (8), light_path (1), mis_emit (1).
// mis_emit: the ray was drawn by the guided integrator's mixture; an emitter it reaches adds its
// radiance with the MIS weight against light sampling, the mixture pdf riding in L.w.
__device__ __forceinline__ int pack_state(int dim, int bounce, int light_path, int mis_emit = 0) {
    return (dim & 0xffff) | ((bounce & 0xff) << 16) | (light_path << 24) | (mis_emit << 25);
}

struct PathRefs {
    float4 *o, *d, *beta, *L;
};

// Hits are shaded per material bucket: 0..7 = MatType of the hit's material, 8 = no material
// (pass-through), 9 = miss.  k_extend appends each queue slot to its bucket; one specialised
// k_shade<bucket> per bucket then runs without material divergence.
constexpr int kCntBucket = 8;  // counters[8 .. 8 + kBuckets): bucket sizes

// Warp-aggregated append into per-key lists (lanes with equal keys share one atomic).
// Must be called by all 32 lanes; key < 0 appends nothing.
__device__ __forceinline__ int warp_append_keyed(int* counters, int key) {
    unsigned peers = __match_any_sync(0xffffffffu, key);
    int leader = __ffs(peers) - 1;
    int base = 0;
    if (key >= 0 && lane_id() == leader) base = atomicAdd(counters + key, __popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    return key >= 0 ? base + __popc(peers & ((1u << lane_id()) - 1u)) : -1;
}

// ---- raygen (SamplerIntegrator.cpp:42-55 + PerspCamera::GenerateRay) -----------------------------
__global__ void k_raygen(DevScene S, WaveArgs a, PathRefs out, float4* out_L, int* qcount) {
    const int total = a.nslots * a.wave_samples;
    const int stride = gridDim.x * blockDim.x;
    for (int base = blockIdx.x * blockDim.x; base < total; base += stride) {
        int pid = base + threadIdx.x;
        bool valid = pid < total;
        int x = 0, y = 0, s_local = 0;
        if (valid) {
            s_local = pid / a.nslots;
            slot_pixel(a, pid - s_local * a.nslots, x, y);
            valid = x < a.W && y < a.H;
            out_L[pid] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        int j = warp_append(qcount, valid);
        if (valid) {
            int sample = wave_sample0(a) + s_local;
            int vidx = S.sampler == SAMPLER_HALTON ? halton_vector_index(S.hp, x, y, sample) : 0;
            const float2 sj = path_sample2(S, vidx, 0, (uint32_t)(y * a.W + x), (uint32_t)sample);
            float sx = sj.x, sy = sj.y;
            float nx, ny;
            pixel_ndc(x, y, sx, sy, a.W, a.H, nx, ny);
            float3 o, d;
            camera_ray(S.cam, nx, ny, o, d);
            out.o[j] = make_float4(o.x, o.y, o.z, __int_as_float(pid));
            out.d[j] = make_float4(d.x, d.y, d.z, __int_as_float(pack_state(2, 0, 1)));
            out.beta[j] = make_float4(1.f, 1.f, 1.f, __int_as_float(vidx));
            out.L[j] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
}

// Minimum resident blocks per SM of the dynamic-fetch traversal kernels (a register budget:
// 65536 / (128 x blocks) registers per thread).  The traversal waits on dependent node loads, so
// more resident warps hide more of that latency, until spills to local memory cost more.
#ifndef C2G_EXTEND_MIN_BLOCKS
#define C2G_EXTEND_MIN_BLOCKS 1
#endif
#ifndef C2G_SHADOW_MIN_BLOCKS
#define C2G_SHADOW_MIN_BLOCKS 1
#endif
// Minimum resident 128-thread blocks per SM of the shading kernels (their register budget).
#ifndef C2G_SHADE_MIN_BLOCKS
#define C2G_SHADE_MIN_BLOCKS 4
#endif

// ---- extend: closest hit of each queued path ray ------------------------------------------------
// Per-kernel-kind traversal counters: cnt[3 * kind + {0: rays, 1: nodes, 2: prims}].
__device__ __forceinline__ void flush_counts(unsigned long long* cnt, int kind, unsigned rays, const TraceCounters& tc) {
    warp_count(cnt + 3 * kind + 0, rays);
    warp_count(cnt + 3 * kind + 1, tc.nodes);
    warp_count(cnt + 3 * kind + 2, tc.prims);
}

template <bool COUNT>
__global__ void k_extend(DevScene S, const float4* __restrict__ qo, const float4* __restrict__ qd, float4* hit,
                         const int* qcount, int* zero_a, int* zero_b, int* zero_c, int* bucket_cnt, int* bucket_list,
                         int cap, unsigned long long* cnt) {
    if (blockIdx.x == 0 && threadIdx.x == 0) { *zero_a = 0; *zero_b = 0; *zero_c = 0; zero_b[2] = 0; }  // + shadow fetch counter
    const int n = *qcount;
    const int stride = gridDim.x * blockDim.x;
    TraceCounters tc{0, 0};
    unsigned rays = 0;
    for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const int i = base + threadIdx.x;
        int key = -1;
        if (i < n) {
            float4 o = qo[i], d = qd[i];
            Hit h = trace_closest<COUNT>(S, f3(o), f3(d), &tc);
            hit[i] = make_float4(h.t, h.u, h.v, __int_as_float(h.obj));
            rays++;
            if (h.obj < 0) key = kBucketMiss;
            else {
                int m = S.objs[h.obj].material;
                key = m < 0 ? kBucketNone : S.mats[m].type;
            }
        }
        int j = warp_append_keyed(bucket_cnt, key);
        if (key >= 0) bucket_list[key * cap + j] = i;
    }
    if (COUNT) flush_counts(cnt, C2G_K_EXTEND, rays, tc);
}

// Four-wide closest-hit extension with dynamic ray fetch (see k_shadow_fetch).  A lane whose ray
// is finished writes its hit, appends the slot to its material bucket (all lanes join the keyed
// append of every round; idle lanes with no key) and takes the next ray.
template <bool COUNT>
__global__ void __launch_bounds__(256, C2G_EXTEND_MIN_BLOCKS) k_extend_fetch(DevScene S, const float4* __restrict__ qo, const float4* __restrict__ qd,
                                                      float4* hit, const int* qcount, int* zero_a, int* zero_b, int* zero_c,
                                                      int* bucket_cnt, int* bucket_list, int cap, int* fetch,
                                                      unsigned long long* cnt) {
    if (blockIdx.x == 0 && threadIdx.x == 0) { *zero_a = 0; *zero_b = 0; *zero_c = 0; zero_b[2] = 0; }  // + shadow fetch counter
    const int n = *qcount;
    TraceCounters tc{0, 0};
    unsigned rays = 0;
    int ray = -1;
    bool exhausted = false;
    RayQ r;
    Hit h{INFINITY, 0.f, 0.f, -1};
    Bvh4State st;
    while (true) {
        const bool need = ray < 0 && !exhausted;
        const int idx = warp_fetch(fetch, need, n);
        if (need) {
            if (idx >= 0) {
                const float4 o = qo[idx], d = qd[idx];
                r = make_rayq(f3(o), f3(d));
                h = Hit{INFINITY, 0.f, 0.f, -1};
                ray = idx;
                bvh4_begin(st);
                rays++;
            } else {
                exhausted = true;
            }
        }
        if (__ballot_sync(0xffffffffu, ray >= 0) == 0) break;
        int key = -1, done_ray = -1;
        if (ray >= 0 && bvh4_closest_round<COUNT>(S, r, INFINITY, h, st, &tc)) {
            hit[ray] = make_float4(h.t, h.u, h.v, __int_as_float(h.obj));
            if (h.obj < 0) key = kBucketMiss;
            else {
                const int mt = S.objs[h.obj].material;
                key = mt < 0 ? kBucketNone : S.mats[mt].type;
            }
            done_ray = ray;
            ray = -1;
        }
        const int j = warp_append_keyed(bucket_cnt, key);
        if (key >= 0) bucket_list[key * cap + j] = done_ray;
    }
    if (COUNT) flush_counts(cnt, C2G_K_EXTEND, rays, tc);
}

// ---- shade ---------------------------------------------------------------------------------------
struct ShadeOut {
    PathRefs nxt;
    int* nxt_count;
    float4 *sh_o, *sh_d, *sh_c;
    float4 *mis_o, *mis_d, *mis_c;
    int *sh_list, *mis_list;
    int *sh_count, *mis_count;
    int2* acc;
    float4* mis_hit;   // per path slot: emitted radiance reaching the MIS ray, light index in w
};

template <int MT, bool G>
__global__ void __launch_bounds__(128, C2G_SHADE_MIN_BLOCKS) k_shade(DevScene S, WaveArgs a, PathRefs cur, const float4* __restrict__ hits,
                                                const int* bucket_cnt, const int* __restrict__ bucket_list, int cap, ShadeOut out,
                                                GuideView gv) {
    const int n = bucket_cnt[MT];
    const int* list = bucket_list + (size_t)MT * cap;
    const int stride = gridDim.x * blockDim.x;
    const int K = a.K;
    for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const bool valid = base + (int)threadIdx.x < n;
        const int i = valid ? __ldg(list + base + threadIdx.x) : 0;
        // ---- load path state
        float4 o4 = make_float4(0, 0, 0, 0), d4 = o4, b4 = o4, L4 = o4, h4 = make_float4(0, 0, 0, __int_as_float(-1));
        if (valid) { o4 = cur.o[i]; d4 = cur.d[i]; b4 = cur.beta[i]; L4 = cur.L[i]; h4 = hits[i]; }
        const int pid = __float_as_int(o4.w);
        const int packed = __float_as_int(d4.w);
        int dim = packed & 0xffff;
        int bounce = (packed >> 16) & 0xff;
        int light_path = (packed >> 24) & 1;
        const bool mis_emit = (packed >> 25) & 1;
        const float prev_pdf = L4.w;
        const int vidx = __float_as_int(b4.w);
        int s_local = valid ? pid / a.nslots : 0;
        int px = 0, py = 0;
        if (valid) slot_pixel(a, pid - s_local * a.nslots, px, py);
        const uint32_t pixel = (uint32_t)(py * a.W + px);
        const uint32_t sample = (uint32_t)(wave_sample0(a) + s_local);
        float3 ro = f3(o4), rd = f3(d4);
        float3 beta = f3(b4), L = f3(L4);
        Hit h{h4.x, h4.y, h4.z, __float_as_int(h4.w)};

        bool alive = valid && MT != kBucketMiss;  // miss: the path ends
        // a miss adds the skybox, if any (PathTracingIntegrator.cpp:39-46, DirectLightingIntegrator.cpp:34-38);
        // not for a guided vertex's ray traced past the depth only for emitter MIS
        if (MT == kBucketMiss && valid && S.sky[0] >= 0 && bounce < a.max_depth) L = L + beta * sky_lookup(S, rd);
        // a guided path's ray past the depth limit only collects the emission it reaches
        const bool emit_only = mis_emit && bounce >= a.max_depth;
        bool do_nee = false;
        bool cont = false;
        int next_mis = 0;       // guided continuation: MIS-weighted emission at the next hit
        float next_pdf = 0.f;   // its mixture pdf
        float3 next_o = ro, next_d = rd;
        Surface s;
        BxDF bx;
        Frame fr;
        float3 wo = -rd;
        const bool direct = a.integrator == C2G_INTEGRATOR_DIRECT;
        if (alive) {
            make_surface(S, ro, rd, h, s);
            // DirectLightingIntegrator adds emission at every hit (DirectLightingIntegrator.cpp:40-41)
            if ((light_path || direct) && s.light >= 0) {
                const Light& Lg = S.lights[s.light];
                float3 n_actual = s.front ? s.N : -s.N;
                L = L + beta * area_Le(Lg, n_actual, -rd);
            } else if (mis_emit && s.light >= 0) {
                // mixture-sampled ray reaching an emitter: power heuristic against that light's
                // sampling pdf (solid angle at the previous vertex); lights NEE skips weigh 1
                const Light& Lg = S.lights[s.light];
                float3 n_actual = s.front ? s.N : -s.N;
                float3 Le = area_Le(Lg, n_actual, -rd);
                if (!is_zero(Le)) {
                    float wgt = 1.f;
                    if (Lg.flux_zero == 0.f) {
                        float3 dv = s.pos - ro;
                        float cl = fabsf(dot(normalize(rd), n_actual));
                        float pdf_light = cl > 0.f ? dot(dv, dv) / (cl * Lg.area) : 0.f;
                        wgt = pdf_light > 0.f ? power_heuristic(prev_pdf, pdf_light) : 1.f;
                    }
                    L = L + beta * (Le * wgt);
                }
            }
            if (emit_only) {
                // nothing more on this path
            } else if (MT == kBucketNone) {
                // no BSDF: continue straight through (PathTracingIntegrator.cpp:64-68); the direct
                // lighting integrator stops at an emitter instead (DirectLightingIntegrator.cpp:48-55)
                if (!(direct && s.light >= 0)) {
                    next_o = spawn_origin(s, rd);
                    next_d = rd;
                    cont = true;
                }
            } else {
                bx = make_bxdf(S.mats[s.mat], s.front);
                const int tex = S.mats[s.mat].tex;
                if (tex >= 0) bx.R = tex_lookup(S, tex, surface_uv(S, ro, rd, h));  // Kd texture
                bx.mtype = MT;  // compile-time material: the BxDF switches fold away
                bx.flags = material_flags(MT);
                fr.T = s.dpdu; fr.N = s.N; fr.B = s.dpdv;
                do_nee = true;
            }
        }
        // ---- next-event estimation: UniformSampleAllLights (PathTracingIntegrator.cpp:175-186)
        // Every material builds one BxDF, so the BSDF sample of EsimateDirect's second half
        // (:229-238) ignores its 1D sample and uses the 2D sample shared by all lights: it is the
        // same direction for every light.  It is drawn once here and its ray traced once (k_mis);
        // the per-light MIS weights and the "hit entity carries this light" test are unchanged.
        // Specular BxDFs give f = 0 and match no non-specular sample, so they skip the light loop.
        float2 uL = make_float2(0, 0), uB = make_float2(0, 0);
        const int nsflags = BXDF_ALL & ~BXDF_SPECULAR;
        // Guided vertex: the continuation is drawn from alpha * BSDF + (1 - alpha) * learned mixture
        // (1 - alpha: the network's selection probability at this vertex) and doubles as the BSDF
        // technique of direct lighting (no separate MIS ray); light samples are weighted against the
        // mixture pdf.  Before the network is trained alpha = 1.
        const bool gvert = G && do_nee && !direct && (bx.flags & BXDF_SPECULAR) == 0;
        const PackedMix lobes{reinterpret_cast<const float4*>(gv.out) + (G ? guided_item<MT>(bucket_cnt, base + (int)threadIdx.x) : 0),
                              gv.out_stride};
        float alpha = 1.f;
        const float detM = gvert ? fabsf(dot(fr.T, cross(fr.N, fr.B))) : 1.f;
        if (gvert && gv.sample) {
            // a non-finite network output or a degenerate shading frame leaves this vertex to
            // plain BSDF sampling
            alpha = (packed_valid(lobes) && detM > 1e-6f) ? 1.f - packed_select(lobes) : 1.f;
        }
        bool nee_work = false, mis_ok = false, any_mis = false;
        float3 f2 = f3(0.f, 0.f, 0.f), wi2 = f3(0.f, 0.f, 0.f);
        float pdf_b2 = 0.f;
        if (do_nee) {
            uL = path_sample2(S, vidx, dim, pixel, sample);
            uB = path_sample2(S, vidx, dim + 2, pixel, sample);
            dim += 4;
            int n_area = 0;
            for (int l = 0; l < S.n_lights; l++) {
                const Light& Lg = S.lights[l];
                if (Lg.flux_zero == 0.f && (direct || l != s.light) && Lg.type != LIGHT_POINT) n_area++;
            }
            dim += n_area;  // one (unused) 1D sample per eligible non-delta light
            nee_work = (bx.flags & BXDF_SPECULAR) == 0;
            if (nee_work && n_area > 0 && !gvert) {
                int stype = 0;
                f2 = bsdf_sample(bx, fr, 0.f, uB, wo, wi2, pdf_b2, nsflags, stype, mis_ok);
                if (mis_ok) f2 = f2 * fmaxf(0.f, dot(s.N, wi2));
            }
        }
        for (int l = 0; l < K; l++) {
            bool sh_valid = false;
            float4 sh_o4, sh_d4, sh_c4 = make_float4(0, 0, 0, 0), mis_c4 = make_float4(0, 0, 0, 0);
            if (nee_work && l < S.n_lights) {
                const Light Lg = S.lights[l];
                // the path tracer skips the hit's own light (PathTracingIntegrator.cpp:182), the direct
                // lighting integrator does not (DirectLightingIntegrator.cpp:71)
                bool eligible = !(Lg.flux_zero != 0.f) && (direct || l != s.light);
                if (eligible) {
                    // light-sampling half (EsimateDirect, :195-227)
                    float3 lpos;
                    float pdf_l;
                    float3 Li = light_sample_li(S, Lg, s.pos, s.N, uL, lpos, pdf_l);
                    float3 wi = normalize(lpos - s.pos);
                    if (pdf_l != 0.f && !is_zero(Li)) {
                        float pdf_b;
                        float3 f = bsdf_f_pdf(bx, fr, wo, wi, nsflags, pdf_b) * fmaxf(0.f, dot(s.N, wi));
                        if (gvert && alpha < 1.f) pdf_b = alpha * pdf_b + (1.f - alpha) * packed_pdf(lobes, wi);
                        if (!is_zero(f)) {
                            bool back = dot(lpos - s.pos, s.N) < 0;
                            float3 org = s.pos + (back ? -s.N : s.N) * kSpawnEps;
                            float3 dir = lpos - org;
                            float3 c;
                            if (Lg.type == LIGHT_POINT) c = f * Li / pdf_l;
                            else c = f * Li * power_heuristic(pdf_l, pdf_b) / pdf_l;
                            c = beta * c;
                            sh_valid = true;
                            sh_o4 = make_float4(org.x, org.y, org.z, __int_as_float(Lg.type == LIGHT_AREA ? Lg.obj : -1));
                            sh_d4 = make_float4(dir.x, dir.y, dir.z, 1.f - kEpsTri);
                            sh_c4 = make_float4(c.x, c.y, c.z, 0.f);
                        }
                    }
                    // BSDF-sampling half (:229-270): weight for this light of the shared sample
                    if (mis_ok && Lg.type != LIGHT_POINT) {
                        float pdf_l2 = light_pdf(S, Lg, s.pos, s.N, wi2);
                        if (pdf_l2 != 0.f) {
                            float3 m = beta * (f2 * power_heuristic(pdf_b2, pdf_l2) / pdf_b2);
                            mis_c4 = make_float4(m.x, m.y, m.z, 0.f);
                            any_mis = true;
                        }
                    }
                }
            }
            const int e = i * K + l;
            if (do_nee) {
                out.sh_c[e] = sh_c4;
                out.mis_c[e] = mis_c4;
            }
            // shadow rays are stored densely in append order (coalesced reads in k_shadow); the
            // list keeps the (slot, light) entry the result belongs to
            int js = warp_append(out.sh_count, sh_valid);
            if (sh_valid) { out.sh_list[js] = e; out.sh_o[js] = sh_o4; out.sh_d[js] = sh_d4; }
        }
        {
            // one MIS ray per path (closest hit; k_mis records which light, if any, it reaches)
            int jm = warp_append(out.mis_count, any_mis);
            if (any_mis) {
                float3 org = spawn_origin(s, wi2);
                out.mis_list[jm] = i;
                out.mis_o[jm] = make_float4(org.x, org.y, org.z, 0.f);
                out.mis_d[jm] = make_float4(wi2.x, wi2.y, wi2.z, 0.f);
            }
            if (do_nee) out.mis_hit[i] = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
        }
        // ---- continuation: BSDF sample (PathTracingIntegrator.cpp:73-102); none for direct lighting
        if (do_nee && !direct) {
            // GCC evaluates SampleDirection(Get1D(), Get2D(), ...) right to left: Get2D first.
            float2 u2 = path_sample2(S, vidx, dim, pixel, sample);
            float u1 = path_sample1(S, vidx, dim + 2, pixel, sample);
            dim += 3;
            float3 wi = f3(0.f, 0.f, 0.f);
            float pdf = 0.f;
            int stype = 0;
            bool ok = false;
            // a guided vertex picks its technique first: the mixture's draws need no BSDF sample
            const bool mix = gvert && alpha < 1.f;
            const bool use_guide = mix && hash_uniform(pixel, sample, 0x4000u + 4u * bounce, S.seed) >= alpha;
            float3 f = f3(0.f, 0.f, 0.f);
            if (!use_guide) f = bsdf_sample(bx, fr, u1, u2, wo, wi, pdf, BXDF_ALL, stype, ok);
            float pb_rec = pdf;  // BSDF density of the continuation (local measure), for training
            if (mix) {
                // One-sample MIS over {BSDF, learned mixture}: q = alpha p_bsdf + (1 - alpha) p_guide,
                // both exactly evaluated, so the estimator stays unbiased.  The BSDF technique draws
                // a local direction l and traces M l (M = [dpdu N dpdv], not orthonormal under
                // interpolated normals), so q is kept in that local measure: the guide's world pdf
                // times the Jacobian of l -> M l / |M l|, |det M| / |M l|^3.  The extra random
                // numbers come from hashed dimensions far above the plain path's.
                const float3 c0 = cross(fr.N, fr.B), c1 = cross(fr.B, fr.T), c2 = cross(fr.T, fr.N);
                const float3 wol = to_local(fr, wo);
                if (use_guide) {
                    float3 wg = packed_sample(lobes, hash_uniform(pixel, sample, 0x4001u + 4u * bounce, S.seed),
                                             hash_uniform(pixel, sample, 0x4002u + 4u * bounce, S.seed),
                                             hash_uniform(pixel, sample, 0x4003u + 4u * bounce, S.seed));
                    // l = M^-1 wg (rows of the inverse: the cross products over det M; the frame
                    // [dpdu N N x dpdu] is left-handed, det M < 0), normalised
                    const float sgn = dot(fr.T, c0) < 0.f ? -1.f : 1.f;
                    float3 l = normalize(f3(dot(c0, wg), dot(c1, wg), dot(c2, wg)) * sgn);
                    float pb = 0.f;
                    f = f3(0.f, 0.f, 0.f);
                    if (l.y * wol.y > 0.f) f = bxdf_f_pdf(bx, wol, l, pb);  // reflection-only BxDFs
                    wi = to_world(fr, l);
                    const float lm = length(wi);
                    stype = (bx.flags & ~(BXDF_REFLECTION | BXDF_TRANSMISSION)) | BXDF_REFLECTION;
                    pdf = alpha * pb + (1.f - alpha) * packed_pdf(lobes, wg) * detM / (lm * lm * lm);
                    pb_rec = pb;
                    ok = !is_zero(f) && pdf > 0.f;
                } else if (ok) {
                    const float lm = length(wi);
                    pdf = alpha * pdf + (1.f - alpha) * packed_pdf(lobes, wi * (1.f / lm)) * detM / (lm * lm * lm);
                }
            }
            if (ok && fabsf(pdf) != 0.f) {
                bool specular = (stype & BXDF_SPECULAR) != 0;
                float cosine = specular ? 1.0f : fmaxf(0.f, (stype & BXDF_TRANSMISSION) ? dot(-s.N, wi) : dot(s.N, wi));
                light_path = (specular || (stype & BXDF_TRANSMISSION)) ? 1 : 0;
                next_o = spawn_origin(s, wi);
                next_d = wi;
                if (gvert) { next_mis = 1; next_pdf = pdf; }
                if (G && gv.record && !specular && (pid % gv.rec_stride) == 0 && bounce < gv.rec_depth) {
                    // training record: vertex, throughput and radiance so far (direct light added later)
                    float4* r = gv.rec + 4 * ((size_t)(pid / gv.rec_stride) * gv.rec_depth + bounce);
                    r[1] = make_float4(s.N.x, s.N.y, s.N.z, 0.2126f * L.x + 0.7152f * L.y + 0.0722f * L.z);
                    r[2] = make_float4(wo.x, wo.y, wo.z, 0.2126f * beta.x + 0.7152f * beta.y + 0.0722f * beta.z);
                    // wi and the BSDF density in the world measure the network's mixture lives in
                    const float lm = length(wi);
                    const float3 wn = wi * (1.f / lm);
                    r[3] = make_float4(wn.x, wn.y, wn.z, pb_rec * lm * lm * lm / fmaxf(detM, 1e-6f));
                    r[0] = make_float4(s.pos.x, s.pos.y, s.pos.z, 1.f);
                }
                beta = beta * (f * cosine / pdf);
                cont = true;
                if (bounce > 3) {
                    float q = fmaxf(.05f, 1.f - length(beta));
                    float u = path_sample1(S, vidx, dim, pixel, sample);
                    dim += 1;
                    if (u < q) cont = false;
                    else beta = beta / (1 - q);
                }
            }
        }
        // Depth limit.  Direct lighting only re-enters at the same level through pass-through
        // surfaces (DirectLightingIntegrator.cpp:54); the 8-bit hop counter bounds that walk.  A
        // guided vertex's ray is traced one level past the limit for the emission it reaches (its
        // light-sampling partner was counted at this vertex).
        if (cont && (direct ? bounce + 1 >= 255 : bounce + 1 >= a.max_depth + next_mis)) cont = false;
        // ---- enqueue the continuation; finished paths keep L in place for `accumulate`
        int j = warp_append(out.nxt_count, cont);
        if (valid) {
            if (cont) {
                out.nxt.o[j] = make_float4(next_o.x, next_o.y, next_o.z, __int_as_float(pid));
                out.nxt.d[j] = make_float4(next_d.x, next_d.y, next_d.z, __int_as_float(pack_state(dim, bounce + 1, light_path, next_mis)));
                out.nxt.beta[j] = make_float4(beta.x, beta.y, beta.z, __int_as_float(vidx));
                out.nxt.L[j] = make_float4(L.x, L.y, L.z, next_pdf);
            } else {
                cur.L[i] = make_float4(L.x, L.y, L.z, 0.f);
            }
            out.acc[i] = make_int2(cont ? j : -1, do_nee ? 1 : 0);
        }
    }
}

// ---- shadow: any-hit of NEE light samples (BVH::IntersectTest) ------------------------------------
template <bool COUNT>
__global__ void k_shadow(DevScene S, const int* __restrict__ list, const int* count, const float4* __restrict__ so,
                         const float4* __restrict__ sd, float4* sc, unsigned long long* cnt) {
    const int n = *count;
    const int stride = gridDim.x * blockDim.x;
    TraceCounters tc{0, 0};
    unsigned rays = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float4 o = so[i], d = sd[i];
        bool occ = trace_any<COUNT>(S, f3(o), f3(d), 0.f, d.w, __float_as_int(o.w), &tc);
        if (occ) sc[list[i]] = make_float4(0.f, 0.f, 0.f, 0.f);
        rays++;
    }
    if (COUNT) flush_counts(cnt, C2G_K_SHADOW, rays, tc);
}

// Four-wide any-hit traversal with dynamic ray fetch: a lane whose ray is finished takes the next
// ray from a global counter at the end of every while-while round, instead of idling until the
// slowest ray of its warp ends (persistent threads with ray replacement).  Same per-ray traversal
// as trace_any_bvh4, so the same rays are occluded.
template <bool COUNT>
__global__ void __launch_bounds__(256, C2G_SHADOW_MIN_BLOCKS) k_shadow_fetch(DevScene S, const int* __restrict__ list, const int* count,
                                                      const float4* __restrict__ so, const float4* __restrict__ sd,
                                                      float4* sc, int* fetch, unsigned long long* cnt) {
    const int n = *count;
    TraceCounters tc{0, 0};
    unsigned rays = 0;
    int ray = -1;
    bool exhausted = false;
    RayQ r;
    float tmax = 0.f;
    int ign = -1;
    Bvh4AnyState st;
    while (true) {
        const bool need = ray < 0 && !exhausted;
        const int idx = warp_fetch(fetch, need, n);
        if (need) {
            if (idx >= 0) {
                const float4 o = so[idx], d = sd[idx];
                r = make_rayq(f3(o), f3(d));
                tmax = d.w;
                ign = __float_as_int(o.w);
                ray = idx;
                bvh4_begin(st);
                rays++;
            } else {
                exhausted = true;
            }
        }
        if (__ballot_sync(0xffffffffu, ray >= 0) == 0) break;
        if (ray < 0) continue;
        bool occluded;
        if (bvh4_any_round<COUNT>(S, r, 0.f, tmax, ign, st, &tc, occluded)) {
            if (occluded) sc[list[ray]] = make_float4(0.f, 0.f, 0.f, 0.f);
            ray = -1;
        }
    }
    if (COUNT) flush_counts(cnt, C2G_K_SHADOW, rays, tc);
}

// ---- mis: closest hit of the NEE BSDF sample; records the emitter it reaches ---------------------
template <bool COUNT>
__global__ void k_mis(DevScene S, const int* __restrict__ list, const int* count, const float4* __restrict__ mo,
                      const float4* __restrict__ md, float4* mis_hit, unsigned long long* cnt) {
    const int n = *count;
    const int stride = gridDim.x * blockDim.x;
    TraceCounters tc{0, 0};
    unsigned rays = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        int slot = list[i];
        float4 o = mo[i], d = md[i];
        Hit h = trace_closest<COUNT>(S, f3(o), f3(d), &tc);
        rays++;
        float3 Le = f3(0.f, 0.f, 0.f);
        int light = -1;
        if (h.obj >= 0) {
            const ObjInfo oi = S.objs[h.obj];
            if (oi.light >= 0) {
                Surface s;
                make_surface(S, f3(o), f3(d), h, s);
                float3 n_actual = s.front ? s.N : -s.N;
                Le = area_Le(S.lights[oi.light], n_actual, -f3(d));
                light = oi.light;
            }
        }
        // no hit: Light::Le of an area light is zero (Light.h:52)
        mis_hit[slot] = make_float4(Le.x, Le.y, Le.z, __int_as_float(light));
    }
    if (COUNT) flush_counts(cnt, C2G_K_MIS, rays, tc);
}

// ---- accumulate ------------------------------------------------------------------------------------
__global__ void k_accumulate(WaveArgs a, PathRefs cur, PathRefs nxt, const int2* __restrict__ acc, const float4* __restrict__ sc,
                             const float4* __restrict__ mc, const float4* __restrict__ mis_hit, float4* out_L, const int* qcount,
                             GuideView gv) {
    const int n = *qcount;
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        int2 ac = acc[i];
        float3 direct = f3(0.f, 0.f, 0.f);
        if (ac.y) {
            float4 mh = mis_hit[i];
            int hl = __float_as_int(mh.w);
            for (int l = 0; l < a.K; l++) {
                float4 s = sc[i * a.K + l];
                float3 m = f3(0.f, 0.f, 0.f);
                if (l == hl) m = f3(mc[i * a.K + l]) * f3(mh);
                direct = direct + (f3(s) + m);
            }
        }
        if (gv.record && ac.y) {
            int pid = __float_as_int(cur.o[i].w);
            int bounce = (__float_as_int(cur.d[i].w) >> 16) & 0xff;
            if ((pid % gv.rec_stride) == 0 && bounce < gv.rec_depth) {
                float4* r = gv.rec + 4 * ((size_t)(pid / gv.rec_stride) * gv.rec_depth + bounce);
                if (r[0].w != 0.f) r[1].w += 0.2126f * direct.x + 0.7152f * direct.y + 0.0722f * direct.z;
            }
        }
        if (ac.x >= 0) {
            if (ac.y) {
                float4 L = nxt.L[ac.x];
                nxt.L[ac.x] = make_float4(L.x + direct.x, L.y + direct.y, L.z + direct.z, L.w);  // w: mixture pdf
            }
        } else {
            float4 L = cur.L[i];
            int pid = __float_as_int(cur.o[i].w);
            out_L[pid] = make_float4(L.x + direct.x, L.y + direct.y, L.z + direct.z, 0.f);
        }
    }
}

// ---- film download: float4 (rgb, w) per pixel -> rgb triples and weights ----------------------------
__global__ void k_film_pack(const float4* __restrict__ film, size_t npx, float* rgb, float* w) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < npx; i += (size_t)gridDim.x * blockDim.x) {
        const float4 f = film[i];
        rgb[3 * i] = f.x;
        rgb[3 * i + 1] = f.y;
        rgb[3 * i + 2] = f.z;
        w[i] = f.w;
    }
}

// ---- film: FrameBuffer::AddSample for every sample of the wave, in sample order ------------------
__global__ void k_film(WaveArgs a, const float4* __restrict__ out_L, float4* film, float4* film_m2) {
    const int stride = gridDim.x * blockDim.x;
    for (int slot = blockIdx.x * blockDim.x + threadIdx.x; slot < a.nslots; slot += stride) {
        int x, y;
        slot_pixel(a, slot, x, y);
        if (x >= a.W || y >= a.H) continue;
        int p = y * a.W + x;
        float4 f = film[p];
        float4 m2 = film_m2[p];
        for (int s = 0; s < a.wave_samples; s++) {
            float4 c = out_L[(size_t)s * a.nslots + slot];
            if (!isfinite(c.x) || !isfinite(c.y) || !isfinite(c.z)) c = make_float4(0.f, 0.f, 0.f, 0.f);
            f.x += c.x; f.y += c.y; f.z += c.z; f.w += 1.f;
            m2.x += c.x * c.x; m2.y += c.y * c.y; m2.z += c.z * c.z;
        }
        film[p] = f;
        film_m2[p] = m2;
    }
}

// ---- ray queries ----------------------------------------------------------------------------------
__global__ void k_trace_rays(DevScene S, int n, const float* o, const float* d, const float* tmin, const float* tmax,
                             const int* ignore, int any_hit, int* obj, float* t) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float3 ro = f3(o[3 * i], o[3 * i + 1], o[3 * i + 2]);
    float3 rd = f3(d[3 * i], d[3 * i + 1], d[3 * i + 2]);
    if (any_hit) {
        float a = tmin ? tmin[i] : 0.f, b = tmax ? tmax[i] : INFINITY;
        int ig = ignore ? ignore[i] : -1;
        obj[i] = trace_any<false>(S, ro, rd, a, b, ig, nullptr) ? 1 : 0;
    } else {
        Hit h = trace_closest<false>(S, ro, rd, nullptr);
        obj[i] = h.obj;
        if (t) t[i] = h.obj >= 0 ? h.t : INFINITY;
    }
}

// Ray queries on four-wide nodes with dynamic fetch (same results as k_trace_rays).
__global__ void __launch_bounds__(128) k_trace_rays_fetch(DevScene S, int n, const float* o, const float* d, const float* tmin,
                                                          const float* tmax, const int* ignore, int any_hit, int* obj,
                                                          float* t, int* fetch) {
    int ray = -1;
    bool exhausted = false;
    RayQ r;
    float a = 0.f, b = INFINITY;
    int ig = -1;
    Hit h{INFINITY, 0.f, 0.f, -1};
    Bvh4State st;
    Bvh4AnyState sa;
    while (true) {
        const bool need = ray < 0 && !exhausted;
        const int idx = warp_fetch(fetch, need, n);
        if (need) {
            if (idx >= 0) {
                r = make_rayq(f3(o[3 * idx], o[3 * idx + 1], o[3 * idx + 2]), f3(d[3 * idx], d[3 * idx + 1], d[3 * idx + 2]));
                a = tmin ? tmin[idx] : 0.f;
                b = tmax ? tmax[idx] : INFINITY;
                ig = ignore ? ignore[idx] : -1;
                h = Hit{INFINITY, 0.f, 0.f, -1};
                ray = idx;
                if (any_hit) bvh4_begin(sa);
                else bvh4_begin(st);
            } else {
                exhausted = true;
            }
        }
        if (__ballot_sync(0xffffffffu, ray >= 0) == 0) break;
        if (ray < 0) continue;
        if (any_hit) {
            bool occ;
            if (bvh4_any_round<false>(S, r, a, b, ig, sa, nullptr, occ)) {
                obj[ray] = occ ? 1 : 0;
                ray = -1;
            }
        } else if (bvh4_closest_round<false>(S, r, INFINITY, h, st, nullptr)) {
            obj[ray] = h.obj;
            if (t) t[ray] = h.obj >= 0 ? h.t : INFINITY;
            ray = -1;
        }
    }
}

__global__ void k_halton(DevScene S, HaltonParams hp, int W, int n, const int* px, const int* py, const int* sample, int ndim, float* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int vidx = halton_vector_index(hp, px[i], py[i], sample[i]);
    for (int dd = 0; dd < ndim; dd++) {
        float v;
        if (dd == 0) v = halton_dim0(vidx, hp);
        else if (dd == 1) v = halton_dim1(vidx, hp);
        else v = halton_sample(S, vidx, dd, (uint32_t)(py[i] * W + px[i]), (uint32_t)sample[i]);
        out[(size_t)i * ndim + dd] = v;
    }
}

// Values of the scene's sampler: the camera pair (dim 0) and the integrator's draws use the same
// path_sample1/2 calls.  out: n * (1 + two_d) floats.
__global__ void k_sampler_values(DevScene S, int W, int n, const int* px, const int* py, const int* sample, int dim, int two_d,
                                 float* out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int vidx = S.sampler == SAMPLER_HALTON ? halton_vector_index(S.hp, px[i], py[i], sample[i]) : 0;
    const uint32_t pixel = (uint32_t)(py[i] * W + px[i]);
    if (two_d) {
        const float2 v = path_sample2(S, vidx, dim, pixel, (uint32_t)sample[i]);
        out[2 * i] = v.x;
        out[2 * i + 1] = v.y;
    } else {
        out[i] = path_sample1(S, vidx, dim, pixel, (uint32_t)sample[i]);
    }
}

__global__ void k_camera(Camera c, int n, const float* pos2, float* o, float* d) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float3 ro, rd;
    camera_ray(c, pos2[2 * i], pos2[2 * i + 1], ro, rd);
    o[3 * i] = ro.x; o[3 * i + 1] = ro.y; o[3 * i + 2] = ro.z;
    d[3 * i] = rd.x; d[3 * i + 1] = rd.y; d[3 * i + 2] = rd.z;
}

// ---- host side -------------------------------------------------------------------------------------
namespace {

#define C2G_CUDA(call)                                                                       \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            err = std::string(#call) + ": " + cudaGetErrorString(e_);                       \
            return C2G_ERR_CUDA;                                                             \
        }                                                                                    \
    } while (0)

template <typename T>
T* upload_vec(const std::vector<T>& v, DeviceArena& arena, std::vector<void*>& owned, std::string& err, int& rc) {
    size_t bytes = std::max<size_t>(sizeof(T), v.size() * sizeof(T));
    T* p = (T*)arena.alloc(bytes, err);
    if (!p) { rc = C2G_ERR_OOM; return nullptr; }
    owned.push_back(p);
    if (!v.empty()) {
        cudaError_t e = cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) { err = cudaGetErrorString(e); rc = C2G_ERR_CUDA; return nullptr; }
    }
    return p;
}

int grid_for(const void* kernel, int block, size_t smem = 0) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, block, smem);
    if (per <= 0) per = 1;
    return sms * per;
}

}  // namespace

void launch_shade(int bk, int grid, cudaStream_t st, const DevScene& S, const WaveArgs& a, const PathRefs& cur, const float4* hits,
                  const int* bcnt, const int* blist, int cap, const ShadeOut& so, const GuideView& gv, bool guided) {
    if (guided) {
        switch (bk) {
#define C2G_SHADE_G(B) case B: k_shade<B, true><<<grid, 128, 0, st>>>(S, a, cur, hits, bcnt, blist, cap, so, gv); return;
            // guided buckets: diffuse, GGX/Beckmann reflection, plastic, Oren-Nayar (exact sampling densities)
            C2G_SHADE_G(0) C2G_SHADE_G(4) C2G_SHADE_G(5) C2G_SHADE_G(6) C2G_SHADE_G(7) C2G_SHADE_G(8)
#undef C2G_SHADE_G
        }
    }
    switch (bk) {
#define C2G_SHADE_CASE(B) case B: k_shade<B, false><<<grid, 128, 0, st>>>(S, a, cur, hits, bcnt, blist, cap, so, gv); break;
        C2G_SHADE_CASE(0) C2G_SHADE_CASE(1) C2G_SHADE_CASE(2) C2G_SHADE_CASE(3) C2G_SHADE_CASE(4)
        C2G_SHADE_CASE(5) C2G_SHADE_CASE(6) C2G_SHADE_CASE(7) C2G_SHADE_CASE(8) C2G_SHADE_CASE(9)
        C2G_SHADE_CASE(10) C2G_SHADE_CASE(11)
#undef C2G_SHADE_CASE
    }
}

int GpuScene::upload(const HostScene& s, int tree, const RefTree* ref, const SahTree* sah, DeviceArena& arena, std::string& err) {
    // release previous scene buffers
    for (void* p : sb_->owned) arena.free(p);
    sb_->owned.clear();
    int rc = C2G_OK;
    DevScene& S = sb_->S;
    S = DevScene{};
    S.objs = upload_vec(s.objs, arena, sb_->owned, err, rc);
    if (rc) return rc;
    S.tri_shade = upload_vec(s.tri_shade, arena, sb_->owned, err, rc);
    if (rc) return rc;
    std::vector<float4> tp(s.tri_pos.size());
    for (size_t i = 0; i < tp.size(); i++) tp[i] = make_float4(s.tri_pos[i].x, s.tri_pos[i].y, s.tri_pos[i].z, 0.f);
    S.tri_pos = upload_vec(tp, arena, sb_->owned, err, rc);
    if (rc) return rc;
    S.quads = upload_vec(s.quads, arena, sb_->owned, err, rc);
    if (rc) return rc;
    S.mats = upload_vec(s.mats, arena, sb_->owned, err, rc);
    if (rc) return rc;
    {
        std::vector<float2> uv(s.tri_uv.size() / 2);
        for (size_t k = 0; k < uv.size(); k++) uv[k] = make_float2(s.tri_uv[2 * k], s.tri_uv[2 * k + 1]);
        S.tri_uv = upload_vec(uv, arena, sb_->owned, err, rc);
        if (rc) return rc;
        S.texels = upload_vec(s.texels, arena, sb_->owned, err, rc);
        if (rc) return rc;
        std::vector<int4> ti(s.tex_info.size() / 4);
        for (size_t k = 0; k < ti.size(); k++)
            ti[k] = make_int4(s.tex_info[4 * k], s.tex_info[4 * k + 1], s.tex_info[4 * k + 2], 0);
        S.tex_info = upload_vec(ti, arena, sb_->owned, err, rc);
        for (int k = 0; k < 6; k++) S.sky[k] = s.sky[k];
    }
    if (rc) return rc;
    S.lights = upload_vec(s.lights, arena, sb_->owned, err, rc);
    if (rc) return rc;
    S.n_lights = (int)s.lights.size();
    S.n_objs = (int)s.objs.size();
    std::vector<Prim> prims;
    S.tree = tree;
    if (tree == C2G_TREE_SAH) {
        make_prims(s, sah->order, prims);
        S.wide_nodes = upload_vec(sah->nodes, arena, sb_->owned, err, rc);
        if (rc) return rc;
        if (!sah->nodes4.empty()) {
            S.nodes4 = upload_vec(sah->nodes4, arena, sb_->owned, err, rc);
            if (rc) return rc;
        }
        S.sah_width = S.nodes4 ? sah_width_ : 2;
    } else {
        make_prims(s, ref->order, prims);
        S.ref_nodes = upload_vec(ref->nodes, arena, sb_->owned, err, rc);
        if (rc) return rc;
    }
    S.prims = upload_vec(prims, arena, sb_->owned, err, rc);
    if (rc) return rc;
    S.n_prims = (int)prims.size();
    S.anyhit_clip = s.cfg.accel == "BVH" ? 1 : 0;
    S.closest_box = s.cfg.accel == "Brute" ? 0 : 1;
    S.cam = s.cam;
    S.hp = halton_params(s.cfg.width, s.cfg.height);
    std::vector<uint16_t> perm;
    std::vector<int> off;
    halton_perm_tables(perm, off);
    S.perm = upload_vec(perm, arena, sb_->owned, err, rc);
    if (rc) return rc;
    S.perm_off = upload_vec(off, arena, sb_->owned, err, rc);
    if (rc) return rc;
    S.seed = (uint64_t)s.cfg.seed;
    S.sampler = s.cfg.sampler == "Default" ? SAMPLER_DEFAULT : s.cfg.sampler == "Stratified" ? SAMPLER_STRATIFIED : SAMPLER_HALTON;
    S.spp = std::max(1, s.cfg.spp);
    S.strata_side = 1;
    while ((S.strata_side + 1) * (S.strata_side + 1) <= S.spp) S.strata_side++;
    const int* primes = halton_primes();
    uint64_t magic[kHaltonDims];
    for (int i = 0; i < kHaltonDims; i++) magic[i] = UINT64_MAX / (uint64_t)primes[i] + 1;
    C2G_CUDA(cudaMemcpyToSymbol(c_primes, primes, sizeof(int) * kHaltonDims));
    C2G_CUDA(cudaMemcpyToSymbol(c_divmagic, magic, sizeof(magic)));
    sb_->err = (int*)arena.alloc(sizeof(int) * 4, err);
    if (!sb_->err) return C2G_ERR_OOM;
    sb_->owned.push_back(sb_->err);
    C2G_CUDA(cudaMemset(sb_->err, 0, sizeof(int) * 4));
    S.err = sb_->err;
    sb_->counts = (unsigned long long*)arena.alloc(sizeof(unsigned long long) * 3 * C2G_K_KINDS, err);
    if (!sb_->counts) return C2G_ERR_OOM;
    sb_->owned.push_back(sb_->counts);
    sb_->fetch = (int*)arena.alloc(256, err);
    if (!sb_->fetch) return C2G_ERR_OOM;
    sb_->owned.push_back(sb_->fetch);
    C2G_CUDA(cudaMemset(sb_->counts, 0, sizeof(unsigned long long) * 3 * C2G_K_KINDS));
    // film
    film_w_ = s.cfg.width;
    film_h_ = s.cfg.height;
    size_t npx = (size_t)film_w_ * film_h_;
    sb_->film = (float4*)arena.alloc(npx * sizeof(float4), err);
    if (!sb_->film) return C2G_ERR_OOM;
    sb_->owned.push_back(sb_->film);
    sb_->film_m2 = (float4*)arena.alloc(npx * sizeof(float4), err);
    if (!sb_->film_m2) return C2G_ERR_OOM;
    sb_->owned.push_back(sb_->film_m2);
    sb_->film_pack = (float*)arena.alloc(npx * 4 * sizeof(float), err);
    if (!sb_->film_pack) return C2G_ERR_OOM;
    sb_->owned.push_back(sb_->film_pack);
    C2G_CUDA(cudaMemset(sb_->film, 0, npx * sizeof(float4)));
    C2G_CUDA(cudaMemset(sb_->film_m2, 0, npx * sizeof(float4)));
    sb_->n_lights = S.n_lights;
    for (int k = 0; k < 3; k++) { box_lo_[k] = INFINITY; box_hi_[k] = -INFINITY; }
    for (size_t o = 0; o < s.objs.size(); o++) {
        float b[6];
        s.object_box((int)o, b);
        for (int k = 0; k < 3; k++) { box_lo_[k] = std::min(box_lo_[k], b[k]); box_hi_[k] = std::max(box_hi_[k], b[3 + k]); }
    }
    guide_steps_ = 0;
    wave_counter_ = nullptr;  // freed with the previous scene's buffers
    guide_.release(arena);  // a new scene trains a new network
    present_buckets_ = 1 << kBucketMiss;
    for (const ObjInfo& o : s.objs) present_buckets_ |= 1 << (o.material < 0 ? kBucketNone : s.mats[o.material].type);
    // wave buffers depend on the light count: drop them
    for (void* p : wb_->owned) arena.free(p);
    wb_->owned.clear();
    *wb_ = WaveBuffers();
    return C2G_OK;
}

int GpuScene::film_clear(cudaStream_t st) {
    size_t npx = (size_t)film_w_ * film_h_;
    if (!sb_->film) return C2G_ERR_STATE;
    if (cudaMemsetAsync(sb_->film, 0, npx * sizeof(float4), st) != cudaSuccess) return C2G_ERR_CUDA;
    if (cudaMemsetAsync(sb_->film_m2, 0, npx * sizeof(float4), st) != cudaSuccess) return C2G_ERR_CUDA;
    return C2G_OK;
}

int GpuScene::check_device_error(std::string& err) {
    int h[4] = {0, 0, 0, 0};
    if (!sb_->err) return C2G_OK;
    C2G_CUDA(cudaMemcpy(h, sb_->err, sizeof(h), cudaMemcpyDeviceToHost));
    if (h[0]) {
        err = "device error word " + std::to_string(h[0]) + ((h[0] & DEVERR_STACK) ? " (traversal stack overflow)" : "") +
              ((h[0] & DEVERR_QUEUE) ? " (queue overflow)" : "") +
              ((h[0] & DEVERR_WAIT) ? " (tensor-core completion wait timed out)" : "");
        cudaMemset(sb_->err, 0, sizeof(int));
        return C2G_ERR_DEVICE;
    }
    return C2G_OK;
}

// The film in the caller's layout: a kernel packs rgb (and weights) into one device buffer, then
// one copy per array goes straight into the caller's memory (no host-side repacking).
int GpuScene::film_download(float* rgb_sum, float* weight, float* rgb_sumsq, std::string& err) {
    const size_t npx = (size_t)film_w_ * film_h_;
    if (!sb_->film) { err = "no scene loaded"; return C2G_ERR_STATE; }
    if (!npx) return C2G_OK;
    const int grid = (int)std::min<size_t>(4096, (npx + 255) / 256);
    float* rgb = sb_->film_pack;
    float* w = sb_->film_pack + 3 * npx;
    if (rgb_sum || weight) {
        k_film_pack<<<grid, 256>>>(sb_->film, npx, rgb, w);
        C2G_CUDA(cudaGetLastError());
        if (rgb_sum) C2G_CUDA(cudaMemcpy(rgb_sum, rgb, 3 * npx * sizeof(float), cudaMemcpyDeviceToHost));
        if (weight) C2G_CUDA(cudaMemcpy(weight, w, npx * sizeof(float), cudaMemcpyDeviceToHost));
    }
    if (rgb_sumsq) {
        k_film_pack<<<grid, 256>>>(sb_->film_m2, npx, rgb, w);
        C2G_CUDA(cudaGetLastError());
        C2G_CUDA(cudaMemcpy(rgb_sumsq, rgb, 3 * npx * sizeof(float), cudaMemcpyDeviceToHost));
    }
    return C2G_OK;
}

namespace {
int g_raygen = 0, g_shade = 0, g_acc = 0, g_film = 0;
// Persistent grids of the traversal kernels for one block size (64, 128 or 256 threads).
struct TraceGrids {
    int ext, ext_c, sh, sh_c, shf, shf_c, exf, exf_c, mis, mis_c;
};
TraceGrids g_trace[3] = {};
int trace_block_index(int threads) { return threads <= 64 ? 0 : (threads <= 128 ? 1 : 2); }
void ensure_grids() {
    if (g_raygen) return;
    g_raygen = grid_for((const void*)k_raygen, 256);
    g_shade = grid_for((const void*)k_shade<MAT_DIFFUSE, false>, 128);
    g_acc = grid_for((const void*)k_accumulate, 256);
    g_film = grid_for((const void*)k_film, 256);
    for (int i = 0; i < 3; i++) {
        const int tb = 64 << i;
        TraceGrids& g = g_trace[i];
        g.ext = grid_for((const void*)k_extend<false>, tb);
        g.ext_c = grid_for((const void*)k_extend<true>, tb);
        g.sh = grid_for((const void*)k_shadow<false>, tb);
        g.sh_c = grid_for((const void*)k_shadow<true>, tb);
        g.shf = grid_for((const void*)k_shadow_fetch<false>, tb);
        g.shf_c = grid_for((const void*)k_shadow_fetch<true>, tb);
        g.exf = grid_for((const void*)k_extend_fetch<false>, tb);
        g.exf_c = grid_for((const void*)k_extend_fetch<true>, tb);
        g.mis = grid_for((const void*)k_mis<false>, tb);
        g.mis_c = grid_for((const void*)k_mis<true>, tb);
    }
}

__global__ void k_advance(int* sample0, int by) { *sample0 += by; }
__global__ void k_set_int(int* dst, int v) { *dst = v; }
// The last kernel of a device-side wave loop: advance the sample counter and keep looping while
// samples of the job remain.
__global__ void k_advance_loop(int* sample0, int by, int end, cudaGraphConditionalHandle h) {
    *sample0 += by;
    cudaGraphSetConditional(h, *sample0 < end ? 1u : 0u);
}
// statistics: *total += *count (paths entering a bounce level)
__global__ void k_level_add(int* total, const int* count) { *total += *count; }
}  // namespace

size_t GpuScene::default_wave_paths(int K, const DeviceArena& arena) const {
    const size_t per_path = 260 + 68 * (size_t)K + kGuidePacked * 4;  // wave buffers (+ guide slots)
    size_t budget = arena.cap() ? arena.cap() : 0;
    if (!budget) {
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) free_b = (size_t)1 << 32;
        budget = free_b;
    }
    size_t n = budget / 4 / per_path;
    return std::max<size_t>(1u << 16, std::min<size_t>(n, (size_t)1 << 25));
}

// Validate p, size the wave buffers and (guided) the network for it; fills the wave plan.
int GpuScene::prepare(const c2g_render_params& p, DeviceArena& arena, WavePlan& plan, std::string& err) {
    if (!sb_->film) { err = "no scene loaded"; return C2G_ERR_STATE; }
    if (p.width != film_w_ || p.height != film_h_) { err = "render size differs from the loaded film size"; return C2G_ERR_INVALID; }
    if (p.max_depth < 0 || p.sample_count < 0 || p.sample_begin < 0) { err = "invalid render parameters"; return C2G_ERR_INVALID; }
    if (p.integrator != C2G_INTEGRATOR_PATH && p.integrator != C2G_INTEGRATOR_DIRECT && p.integrator != C2G_INTEGRATOR_GUIDED) {
        err = "unknown integrator";
        return C2G_ERR_INVALID;
    }
    if (p.max_depth > 255) { err = "max_depth above 255"; return C2G_ERR_INVALID; }
    plan.guided = p.integrator == C2G_INTEGRATOR_GUIDED;
    DevScene& S = plan.S;
    S = sb_->S;
    S.anyhit_clip = p.accel == C2G_ACCEL_BVH ? 1 : 0;
    S.closest_box = p.accel == C2G_ACCEL_BVH ? 1 : 0;
    S.seed = p.seed;
    WaveArgs& a = plan.a;
    a = WaveArgs{};
    a.W = p.width;
    a.H = p.height;
    a.tiles_x = (p.width + 7) / 8;
    int tiles_y = (p.height + 7) / 8;
    a.nslots = a.tiles_x * tiles_y * 64;
    a.max_depth = p.max_depth;
    a.K = std::max(1, S.n_lights);
    a.integrator = p.integrator;
    // Wave capacity: the caller's, else the default - up to 2^25 paths, within a quarter of the free
    // device memory (or of the context's memory cap).  Larger waves keep the deep bounce levels
    // busy: on the 1080p many-material scene 2^21 paths run at 231 Mpaths/s, 2^25 at 513.
    size_t want = p.wave_paths > 0 ? (size_t)p.wave_paths : default_wave_paths(a.K, arena);
    int spw = (int)std::max<size_t>(1, want / (size_t)a.nslots);
    spw = std::min(spw, std::max(1, p.sample_count));
    plan.spw = spw;
    // Bounce levels per wave.  A guided vertex's ray is traced one level past the depth for the
    // emission it reaches; direct lighting walks pass-through surfaces up to 255 hops.
    plan.levels = p.integrator == C2G_INTEGRATOR_DIRECT ? 255 : p.max_depth + (plan.guided ? 1 : 0);
    size_t P = (size_t)spw * a.nslots;
    if (wb_->P < P || wb_->K != a.K) {
        for (void* q : wb_->owned) arena.free(q);
        wb_->owned.clear();
        *wb_ = WaveBuffers();
        auto A = [&](size_t bytes) -> void* {
            void* q = arena.alloc(bytes, err);
            if (q) wb_->owned.push_back(q);
            return q;
        };
        size_t PK = P * (size_t)a.K;
        bool ok = true;
        for (int b = 0; b < 2 && ok; b++) {
            ok = ok && (wb_->o[b] = (float4*)A(P * 16)) && (wb_->d[b] = (float4*)A(P * 16)) &&
                 (wb_->beta[b] = (float4*)A(P * 16)) && (wb_->L[b] = (float4*)A(P * 16));
        }
        ok = ok && (wb_->hit = (float4*)A(P * 16)) && (wb_->acc = (int2*)A(P * 8)) && (wb_->out_L = (float4*)A(P * 16)) &&
             (wb_->sh_o = (float4*)A(PK * 16)) && (wb_->sh_d = (float4*)A(PK * 16)) && (wb_->sh_c = (float4*)A(PK * 16)) &&
             (wb_->mis_o = (float4*)A(P * 16)) && (wb_->mis_d = (float4*)A(P * 16)) && (wb_->mis_c = (float4*)A(PK * 16)) &&
             (wb_->mis_hit = (float4*)A(P * 16)) && (wb_->sh_list = (int*)A(PK * 4)) && (wb_->mis_list = (int*)A(P * 4)) &&
             (wb_->bucket_list = (int*)A(P * 4 * kBuckets)) && (wb_->counters = (int*)A(256)) &&
             (wb_->levels = (int*)A(4 * C2G_LEVELS));
        if (!ok) {
            for (void* q : wb_->owned) arena.free(q);
            wb_->owned.clear();
            *wb_ = WaveBuffers();
            return C2G_ERR_OOM;
        }
        wb_->P = P;
        wb_->K = a.K;
    }
    if (plan.guided) {
        int rc = guide_.init(arena, wb_->P, p.max_depth, box_lo_, box_hi_, p.seed, err);
        if (rc) return rc;
    }
    ensure_grids();
    return C2G_OK;
}

// Enqueue one wave (a.wave_samples samples of every pixel slot) on st: raygen, the bounce levels,
// the film and (guided) a training step.  begin/end bracket every launch (timing hooks).
int GpuScene::enqueue_wave(const WavePlan& plan, const WaveArgs& a, const GuideView& gv, bool count, cudaStream_t st,
                           const std::function<void(int, cudaStream_t)>& begin, const std::function<void(cudaStream_t)>& end,
                           int& launches, std::string& err, bool advance) {
    const DevScene& S = plan.S;
    const bool guided = plan.guided;
    WaveBuffers& w = *wb_;
    unsigned long long* cnt = sb_->counts;
    launches = 0;
    const int tb = 64 << trace_block_index(trace_block_);
    const TraceGrids& TG = g_trace[trace_block_index(trace_block_)];
    const bool overlap = overlap_ && side_stream(err) == C2G_OK;
    // fork: the side stream waits for everything enqueued on st so far; join: st waits for the side
    auto fork = [&](int k) {
        cudaEventRecord(fork_ev_[k], st);
        cudaStreamWaitEvent(side_, fork_ev_[k], 0);
    };
    auto join = [&](int k) {
        cudaEventRecord(join_ev_[k], side_);
        cudaStreamWaitEvent(st, join_ev_[k], 0);
    };
    int* C = w.counters;
    C2G_CUDA(cudaMemsetAsync(C, 0, 256, st));
    PathRefs buf[2] = {{w.o[0], w.d[0], w.beta[0], w.L[0]}, {w.o[1], w.d[1], w.beta[1], w.L[1]}};
    begin(C2G_K_RAYGEN, st);
    k_raygen<<<g_raygen, 256, 0, st>>>(S, a, buf[0], w.out_L, C + 0);
    end(st);
    // Extension of the paths in queue q on stream es: closest hits, appended to the material buckets.
    // Block 0 zeroes *za (the count of the queue this level's shading fills), *zb and zb[2] (the
    // shadow queue and its fetch counter) and *zc (the MIS queue): the live counters when it runs in
    // order, spare slots when it runs ahead beside the previous level's shadow rays (the live ones
    // are then zeroed on st after that level's accumulation).
    auto extend = [&](int q, int* za, int* zb, int* zc, cudaStream_t es) {
        begin(C2G_K_EXTEND, es);
        // bucket sizes and the extension fetch counter C[5] start at zero on every level
        cudaMemsetAsync(C + 5, 0, sizeof(int) * (kCntBucket - 5 + kBuckets), es);
        if (S.tree == C2G_TREE_SAH && S.sah_width == 4) {
            if (count)
                k_extend_fetch<true><<<TG.exf_c, tb, 0, es>>>(S, buf[q].o, buf[q].d, w.hit, C + q, za, zb, zc, C + kCntBucket,
                                                              w.bucket_list, (int)w.P, C + 5, cnt);
            else
                k_extend_fetch<false><<<TG.exf, tb, 0, es>>>(S, buf[q].o, buf[q].d, w.hit, C + q, za, zb, zc, C + kCntBucket,
                                                               w.bucket_list, (int)w.P, C + 5, cnt);
        } else if (count) {
            k_extend<true><<<TG.ext_c, tb, 0, es>>>(S, buf[q].o, buf[q].d, w.hit, C + q, za, zb, zc, C + kCntBucket,
                                                    w.bucket_list, (int)w.P, cnt);
        } else {
            k_extend<false><<<TG.ext, tb, 0, es>>>(S, buf[q].o, buf[q].d, w.hit, C + q, za, zb, zc, C + kCntBucket,
                                                     w.bucket_list, (int)w.P, cnt);
        }
        end(es);
    };
    int* const spare = C + 56;  // counter slots no kernel reads
    static_assert(kCntBucket + kBuckets <= 56, "counter layout");
    bool ahead_done = false;    // this level's extension was launched during the previous level
    int cur = 0;
    for (int b = 0; b < plan.levels; b++) {
        int nxt = cur ^ 1;
        if (b >= a.max_depth && a.integrator == C2G_INTEGRATOR_DIRECT) {
            // pass-through hops past the depth: stop once the queue is empty
            int qn = 0;
            C2G_CUDA(cudaMemcpyAsync(&qn, C + cur, sizeof(int), cudaMemcpyDeviceToHost, st));
            C2G_CUDA(cudaStreamSynchronize(st));
            if (qn == 0) break;
        }
        // statistics: the paths entering this level
        if (count) k_level_add<<<1, 1, 0, st>>>(w.levels + std::min(b, C2G_LEVELS - 1), C + cur);
        const bool pre = ahead_done;
        if (pre) cudaStreamWaitEvent(st, join_ev_[2], 0);
        else extend(cur, C + nxt, C + 2, C + 3, st);
        // the guide serves the first guide_levels_ bounce levels; deeper vertices shade plainly
        const bool glevel = guided && (guide_levels_ <= 0 || b < guide_levels_);
        if (gv.sample && glevel && !pre) {
            begin(C2G_K_GUIDE, st);
            launches += guide_.infer(st, &S, buf[cur].o, buf[cur].d, w.hit, C + kCntBucket, w.bucket_list, (int)w.P,
                                     present_buckets_);
            end(st);
        }
        ShadeOut so{buf[nxt], C + nxt, w.sh_o, w.sh_d, w.sh_c, w.mis_o, w.mis_d, w.mis_c, w.sh_list, w.mis_list, C + 2, C + 3, w.acc, w.mis_hit};
        // the material buckets are independent (they append to the shared queues with atomics):
        // with overlap the present buckets take the three streams in turn
        if (overlap) {
            fork(0);
            cudaEventRecord(fork_ev_[3], st);
            cudaStreamWaitEvent(ahead_, fork_ev_[3], 0);
        }
        int nb = 0;
        for (int bk = 0; bk < kBuckets; bk++) {
            if (!(present_buckets_ & (1 << bk))) continue;
            const cudaStream_t ss = !overlap ? st : (nb % 3 == 1 ? side_ : (nb % 3 == 2 ? ahead_ : st));
            begin(C2G_K_SHADE, ss);
            launch_shade(bk, g_shade, ss, S, a, buf[cur], w.hit, C + kCntBucket, w.bucket_list, (int)w.P, so, gv, glevel);
            end(ss);
            launches++;
            nb++;
        }
        if (overlap) {
            join(0);
            cudaEventRecord(join_ev_[3], ahead_);
            cudaStreamWaitEvent(st, join_ev_[3], 0);
        }
        // The next level's queue is complete: its extension runs ahead on the third stream, beside
        // this level's shadow and MIS rays and accumulation (none of which reads the hits or the
        // buckets it writes).  Not for direct lighting, whose walk checks the queue on the host.
        ahead_done = false;
        if (overlap && a.integrator != C2G_INTEGRATOR_DIRECT && b + 1 < plan.levels) {
            cudaEventRecord(fork_ev_[2], st);
            cudaStreamWaitEvent(ahead_, fork_ev_[2], 0);
            extend(nxt, spare, spare + 1, spare + 4, ahead_);
            launches++;
            // the next level's guide inference needs only its rays and hits: it follows on the
            // same stream (this level's shading has read its mixtures already)
            if (gv.sample && guided && (guide_levels_ <= 0 || b + 1 < guide_levels_)) {
                begin(C2G_K_GUIDE, ahead_);
                launches += guide_.infer(ahead_, &S, buf[nxt].o, buf[nxt].d, w.hit, C + kCntBucket, w.bucket_list, (int)w.P,
                                         present_buckets_);
                end(ahead_);
            }
            cudaEventRecord(join_ev_[2], ahead_);
            ahead_done = true;
        }
        // MIS rays (closest hit + emitter test) beside the shadow rays (any hit): disjoint inputs
        // and outputs; both must finish before k_accumulate
        if (overlap) {
            fork(1);
            begin(C2G_K_MIS, side_);
            if (count) k_mis<true><<<TG.mis_c, tb, 0, side_>>>(S, w.mis_list, C + 3, w.mis_o, w.mis_d, w.mis_hit, cnt);
            else k_mis<false><<<TG.mis, tb, 0, side_>>>(S, w.mis_list, C + 3, w.mis_o, w.mis_d, w.mis_hit, cnt);
            end(side_);
        }
        begin(C2G_K_SHADOW, st);
        if (S.tree == C2G_TREE_SAH && S.sah_width == 4) {
            // four-wide nodes: the dynamic-fetch kernel (fetch counter C[4], zeroed by k_extend)
            if (count) k_shadow_fetch<true><<<TG.shf_c, tb, 0, st>>>(S, w.sh_list, C + 2, w.sh_o, w.sh_d, w.sh_c, C + 4, cnt);
            else k_shadow_fetch<false><<<TG.shf, tb, 0, st>>>(S, w.sh_list, C + 2, w.sh_o, w.sh_d, w.sh_c, C + 4, cnt);
        } else if (count) {
            k_shadow<true><<<TG.sh_c, tb, 0, st>>>(S, w.sh_list, C + 2, w.sh_o, w.sh_d, w.sh_c, cnt);
        } else {
            k_shadow<false><<<TG.sh, tb, 0, st>>>(S, w.sh_list, C + 2, w.sh_o, w.sh_d, w.sh_c, cnt);
        }
        end(st);
        if (overlap) {
            join(1);
        } else {
            begin(C2G_K_MIS, st);
            if (count) k_mis<true><<<TG.mis_c, tb, 0, st>>>(S, w.mis_list, C + 3, w.mis_o, w.mis_d, w.mis_hit, cnt);
            else k_mis<false><<<TG.mis, tb, 0, st>>>(S, w.mis_list, C + 3, w.mis_o, w.mis_d, w.mis_hit, cnt);
            end(st);
        }
        begin(C2G_K_ACCUM, st);
        k_accumulate<<<g_acc, 256, 0, st>>>(a, buf[cur], buf[nxt], w.acc, w.sh_c, w.mis_c, w.mis_hit, w.out_L, C + cur, gv);
        end(st);
        if (ahead_done) {
            // the counters the look-ahead extension left alone: the queue after the next level, the
            // shadow and MIS queues and the shadow fetch counter
            cudaMemsetAsync(C + cur, 0, sizeof(int), st);
            cudaMemsetAsync(C + 2, 0, 3 * sizeof(int), st);
        }
        launches += pre ? 3 : 4;
        cur = nxt;
    }
    begin(C2G_K_FILM, st);
    k_film<<<g_film, 256, 0, st>>>(a, w.out_L, sb_->film, sb_->film_m2);
    end(st);
    launches += 2;
    if (guided) {
        // online training on this wave's recorded vertices (batch build, fused fwd/bwd, Adam)
        begin(C2G_K_TRAIN, st);
        guide_.train(st, w.out_L, a.nslots * a.wave_samples, guide_train_steps_, S.err);
        end(st);
        launches += 1 + 3 * guide_train_steps_;
    }
    if (a.sample0_dev && advance) {
        k_advance<<<1, 1, 0, st>>>(const_cast<int*>(a.sample0_dev), a.wave_samples);
        launches++;
    }
    return C2G_OK;
}

void GpuScene::set_sah_width(int w) {
    sah_width_ = w == 2 ? 2 : 4;
    if (sb_->S.tree == C2G_TREE_SAH) sb_->S.sah_width = sb_->S.nodes4 ? sah_width_ : 2;
}

void GpuScene::release_wave_buffers(DeviceArena& arena) {
    cudaDeviceSynchronize();
    for (void* q : wb_->owned) arena.free(q);
    wb_->owned.clear();
    *wb_ = WaveBuffers();
}

int GpuScene::set_wave_counter(int sample, cudaStream_t st, DeviceArena& arena, std::string& err) {
    if (!wave_counter_) {
        wave_counter_ = (int*)arena.alloc(256, err);
        if (!wave_counter_) return C2G_ERR_OOM;
        sb_->owned.push_back(wave_counter_);
    }
    C2G_CUDA(cudaMemcpyAsync(wave_counter_, &sample, sizeof(int), cudaMemcpyHostToDevice, st));
    C2G_CUDA(cudaStreamSynchronize(st));
    return C2G_OK;
}

// Shared set-up of the captured waves: plan, device sample counter, guide view; one stream.
int GpuScene::capture_plan(const c2g_render_params& p, bool guide_sample, cudaStream_t st, DeviceArena& arena, WavePlan& plan,
                           GuideView& gv, std::string& err) {
    if (p.integrator == C2G_INTEGRATOR_DIRECT) {
        err = "batched rendering runs the path tracers (the direct lighting walk synchronises)";
        return C2G_ERR_UNSUPPORTED;
    }
    int rc = prepare(p, arena, plan, err);
    if (rc) return rc;
    rc = set_wave_counter(p.sample_begin, st, arena, err);
    if (rc) return rc;
    guide_.prepare_launch();
    plan.a.wave_samples = plan.spw;
    plan.a.sample0 = 0;
    plan.a.sample0_dev = wave_counter_;
    gv = plan.guided ? guide_.view(true, guide_sample) : GuideView{};
    // batched jobs already overlap each other; the side-stream branches inside each graph measured
    // slower there (64-job batch: 770 vs 872 Mpaths/s), so graphs keep one stream
    overlap_ = false;
    return C2G_OK;
}

int GpuScene::capture_wave(const c2g_render_params& p, bool guide_sample, cudaStream_t st, DeviceArena& arena,
                           cudaGraphExec_t* exec, int* wave_samples, std::string& err) {
    WavePlan plan;
    GuideView gv;
    int rc = capture_plan(p, guide_sample, st, arena, plan, gv, err);
    if (rc) return rc;
    auto no_begin = [](int, cudaStream_t) {};
    auto no_end = [](cudaStream_t) {};
    C2G_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
    int launches = 0;
    rc = enqueue_wave(plan, plan.a, gv, false, st, no_begin, no_end, launches, err);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    if (rc || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        if (!rc) { err = std::string("stream capture: ") + cudaGetErrorString(e); rc = C2G_ERR_CUDA; }
        return rc;
    }
    e = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) { err = std::string("graph instantiation: ") + cudaGetErrorString(e); return C2G_ERR_CUDA; }
    *wave_samples = plan.spw;
    return C2G_OK;
}

int GpuScene::capture_wave_loop(const c2g_render_params& p, bool guide_sample, cudaGraph_t body, cudaGraphConditionalHandle h,
                                int end_sample, cudaStream_t st, DeviceArena& arena, int* wave_samples, std::string& err) {
    WavePlan plan;
    GuideView gv;
    int rc = capture_plan(p, guide_sample, st, arena, plan, gv, err);
    if (rc) return rc;
    auto no_begin = [](int, cudaStream_t) {};
    auto no_end = [](cudaStream_t) {};
    C2G_CUDA(cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    int launches = 0;
    rc = enqueue_wave(plan, plan.a, gv, false, st, no_begin, no_end, launches, err, false);
    if (!rc) k_advance_loop<<<1, 1, 0, st>>>(wave_counter_, plan.spw, end_sample, h);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (rc) return rc;
    if (e != cudaSuccess) { err = std::string("stream capture: ") + cudaGetErrorString(e); return C2G_ERR_CUDA; }
    *wave_samples = plan.spw;
    return C2G_OK;
}

void GpuScene::set_trace_block(int threads) { trace_block_ = 64 << trace_block_index(threads); }

int GpuScene::append_job(cudaGraph_t G, const cudaGraphNode_t* deps, int ndeps, const c2g_render_params& p, int wave_paths,
                         cudaEvent_t done, cudaStream_t st, DeviceArena& arena, cudaGraphNode_t* last, int* spw, int* waves,
                         std::string& err) {
    const int nslots = ((p.width + 7) / 8) * ((p.height + 7) / 8) * 64;
    // samples per wave: as many as the wave size holds, dividing the job's sample count
    int s = std::max(1, std::min(p.sample_count, wave_paths / nslots));
    while (p.sample_count % s) s--;
    c2g_render_params q = p;
    q.wave_paths = s * nslots;
    const bool guided = q.integrator == C2G_INTEGRATOR_GUIDED;
    const int n_waves = p.sample_count / s;
    const int warm = guided ? std::min(n_waves, guide_warmup_) : 0;
    // the counter reset (its address exists once the plan is prepared)
    {
        WavePlan plan;
        int rc = prepare(q, arena, plan, err);
        if (rc) return rc;
        rc = set_wave_counter(p.sample_begin, st, arena, err);
        if (rc) return rc;
    }
    cudaGraphNode_t prev = nullptr;
    {
        int* counter = wave_counter_;
        int value = p.sample_begin;
        void* args[] = {&counter, &value};
        cudaKernelNodeParams kp{};
        kp.func = (void*)k_set_int;
        kp.gridDim = dim3(1);
        kp.blockDim = dim3(1);
        kp.kernelParams = args;
        C2G_CUDA(cudaGraphAddKernelNode(&prev, G, deps, ndeps, &kp));
    }
    // one while loop per wave kind: the guided integrator's first waves only train
    for (int part = 0; part < 2; part++) {
        const int loop_waves = part == 0 ? warm : n_waves - warm;
        if (loop_waves <= 0) continue;
        cudaGraphConditionalHandle h;
        C2G_CUDA(cudaGraphConditionalHandleCreate(&h, G, 1, cudaGraphCondAssignDefault));
        cudaGraphNodeParams np{};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node;
        C2G_CUDA(cudaGraphAddNode(&node, G, &prev, nullptr, 1, &np));
        const int end = p.sample_begin + (part == 0 ? warm : n_waves) * s;
        int got = 0;
        int rc = capture_wave_loop(q, part == 1, np.conditional.phGraph_out[0], h, end, st, arena, &got, err);
        if (rc) return rc;
        prev = node;
    }
    cudaGraphNode_t ev;
    C2G_CUDA(cudaGraphAddEventRecordNode(&ev, G, &prev, 1, done));
    *last = ev;
    *spw = s;
    *waves = n_waves;
    return C2G_OK;
}

int GpuScene::render(const HostScene& s, const c2g_render_params& p, cudaStream_t st, DeviceArena& arena, std::string& err) {
    (void)s;
    WavePlan plan;
    int rc = prepare(p, arena, plan, err);
    if (rc) return rc;
    const bool guided = plan.guided;
    const bool count = (counting_ & C2G_COUNT_TRAVERSAL) != 0;
    const bool timing = (counting_ & C2G_COUNT_TIMING) != 0;
    // timing events are recorded on the stream each kernel runs on; C2G_COUNT_SERIAL keeps every
    // kernel on st, so that their times are exclusive
    overlap_ = (counting_ & C2G_COUNT_SERIAL) == 0;
    unsigned long long* cnt = sb_->counts;
    if (count) {
        C2G_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * 3 * C2G_K_KINDS, st));
        C2G_CUDA(cudaMemsetAsync(wb_->levels, 0, sizeof(int) * C2G_LEVELS, st));
    }
    // per-launch events (timing mode): a pool reused across calls
    struct Ev { cudaEvent_t a, b; int kind; };
    static std::vector<Ev> pool;
    size_t used = 0;
    int kcount[C2G_K_KINDS] = {};
    // per-level time: from one extension launch's begin event to the next one (or to the film)
    std::vector<std::pair<size_t, int>> level_marks;  // (pool index, level)
    int level = 0;
    auto begin = [&](int kind, cudaStream_t ks) {
        kcount[kind]++;
        if (!timing) return;
        if (kind == C2G_K_EXTEND) level_marks.push_back({used, level++});
        else if (kind == C2G_K_FILM || kind == C2G_K_RAYGEN) {
            if (kind == C2G_K_FILM) level_marks.push_back({used, -1});  // end of the wave's levels
            level = 0;
        }
        if (used == pool.size()) {
            Ev e{};
            cudaEventCreate(&e.a);
            cudaEventCreate(&e.b);
            pool.push_back(e);
        }
        pool[used].kind = kind;
        cudaEventRecord(pool[used].a, ks);
    };
    auto end = [&](cudaStream_t ks) {
        if (!timing) return;
        cudaEventRecord(pool[used].b, ks);
        used++;
    };
    cudaEvent_t ev0, ev1;
    cudaEventCreate(&ev0);
    cudaEventCreate(&ev1);
    cudaEventRecord(ev0, st);
    int launches = 0, waves = 0;
    WaveArgs a = plan.a;
    for (int s0 = 0; s0 < p.sample_count; s0 += plan.spw) {
        a.wave_samples = std::min(plan.spw, p.sample_count - s0);
        a.sample0 = p.sample_begin + s0;
        // guided waves record training vertices; they sample the mixture once the network has trained
        const GuideView gv = guided ? guide_.view(true, guide_steps_ >= guide_warmup_) : GuideView{};
        int n = 0;
        rc = enqueue_wave(plan, a, gv, count, st, begin, end, n, err);
        if (rc) return rc;
        launches += n;
        waves++;
        if (guided) guide_steps_++;
    }
    cudaEventRecord(ev1, st);
    C2G_CUDA(cudaGetLastError());
    C2G_CUDA(cudaStreamSynchronize(st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev0, ev1);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    stats_ = c2g_stats{};
    stats_.seconds = ms * 1e-3;
    stats_.paths = (double)p.width * p.height * p.sample_count;
    stats_.kernel_launches = launches;
    stats_.waves = waves;
    for (int k = 0; k < C2G_K_KINDS; k++) stats_.kernel_count[k] = kcount[k];
    for (size_t i = 0; i < used; i++) {
        float t = 0.f;
        cudaEventElapsedTime(&t, pool[i].a, pool[i].b);
        stats_.kernel_ms[pool[i].kind] += t;
    }
    for (size_t i = 0; i + 1 < level_marks.size(); i++) {
        if (level_marks[i].second < 0) continue;
        float t = 0.f;
        cudaEventElapsedTime(&t, pool[level_marks[i].first].a, pool[level_marks[i + 1].first].a);
        stats_.level_ms[std::min(level_marks[i].second, C2G_LEVELS - 1)] += t;
        stats_.levels = std::max(stats_.levels, level_marks[i].second + 1);
    }
    if (count) {
        int lv[C2G_LEVELS];
        C2G_CUDA(cudaMemcpy(lv, wb_->levels, sizeof(lv), cudaMemcpyDeviceToHost));
        for (int l = 0; l < C2G_LEVELS; l++) stats_.level_paths[l] = lv[l];
        unsigned long long h[3 * C2G_K_KINDS];
        C2G_CUDA(cudaMemcpy(h, cnt, sizeof(h), cudaMemcpyDeviceToHost));
        for (int k = 0; k < C2G_K_KINDS; k++) {
            stats_.rays[k] = (double)h[3 * k];
            stats_.nodes[k] = (double)h[3 * k + 1];
            stats_.prims[k] = (double)h[3 * k + 2];
        }
    }
    return check_device_error(err);
}

int GpuScene::trace_rays_dev(int n, const float* o, const float* d, const float* tmin, const float* tmax, const int* ignore,
                             int any_hit, int* obj, float* t, cudaStream_t st, std::string& err) {
    if (!sb_->film) { err = "no scene loaded"; return C2G_ERR_STATE; }
    if (n <= 0) return C2G_OK;
    const DevScene& S = sb_->S;
    if (S.tree == C2G_TREE_SAH && S.sah_width == 4 && sb_->fetch) {
        static int grid = 0;
        if (!grid) grid = grid_for((const void*)k_trace_rays_fetch, 128);
        C2G_CUDA(cudaMemsetAsync(sb_->fetch, 0, sizeof(int), st));
        k_trace_rays_fetch<<<grid, 128, 0, st>>>(S, n, o, d, tmin, tmax, ignore, any_hit, obj, t, sb_->fetch);
    } else {
        k_trace_rays<<<(n + 127) / 128, 128, 0, st>>>(S, n, o, d, tmin, tmax, ignore, any_hit, obj, t);
    }
    C2G_CUDA(cudaGetLastError());
    return C2G_OK;
}

int GpuScene::halton(int width, int height, int n, const int* px, const int* py, const int* sample, int ndim, float* out,
                     DeviceArena& arena, std::string& err) {
    if (!sb_->S.perm) { err = "no scene loaded"; return C2G_ERR_STATE; }
    if (n <= 0 || ndim <= 0) return C2G_OK;
    HaltonParams hp = halton_params(width, height);
    size_t bytes_i = (size_t)n * 4, bytes_o = (size_t)n * ndim * 4;
    int* dpx = (int*)arena.alloc(bytes_i * 3, err);
    float* dout = (float*)arena.alloc(bytes_o, err);
    if (!dpx || !dout) { arena.free(dpx); arena.free(dout); return C2G_ERR_OOM; }
    int rc = C2G_OK;
    do {
        if (cudaMemcpy(dpx, px, bytes_i, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(dpx + n, py, bytes_i, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(dpx + 2 * n, sample, bytes_i, cudaMemcpyHostToDevice) != cudaSuccess) { rc = C2G_ERR_CUDA; break; }
        k_halton<<<(n + 127) / 128, 128>>>(sb_->S, hp, width, n, dpx, dpx + n, dpx + 2 * n, ndim, dout);
        if (cudaGetLastError() != cudaSuccess || cudaMemcpy(out, dout, bytes_o, cudaMemcpyDeviceToHost) != cudaSuccess) rc = C2G_ERR_CUDA;
    } while (0);
    if (rc) err = "halton query failed";
    arena.free(dpx);
    arena.free(dout);
    return rc;
}

int GpuScene::sampler_values(int width, int n, const int* px, const int* py, const int* sample, int dim, int two_d, float* out,
                             DeviceArena& arena, std::string& err) {
    if (!sb_->S.perm) { err = "no scene loaded"; return C2G_ERR_STATE; }
    if (n <= 0) return C2G_OK;
    size_t bytes_i = (size_t)n * 4, bytes_o = (size_t)n * (two_d ? 2 : 1) * 4;
    int* dpx = (int*)arena.alloc(bytes_i * 3, err);
    float* dout = (float*)arena.alloc(bytes_o, err);
    if (!dpx || !dout) { arena.free(dpx); arena.free(dout); return C2G_ERR_OOM; }
    int rc = C2G_OK;
    do {
        if (cudaMemcpy(dpx, px, bytes_i, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(dpx + n, py, bytes_i, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(dpx + 2 * n, sample, bytes_i, cudaMemcpyHostToDevice) != cudaSuccess) { rc = C2G_ERR_CUDA; break; }
        k_sampler_values<<<(n + 127) / 128, 128>>>(sb_->S, width, n, dpx, dpx + n, dpx + 2 * n, dim, two_d, dout);
        if (cudaGetLastError() != cudaSuccess || cudaMemcpy(out, dout, bytes_o, cudaMemcpyDeviceToHost) != cudaSuccess) rc = C2G_ERR_CUDA;
    } while (0);
    if (rc) err = "sampler query failed";
    arena.free(dpx);
    arena.free(dout);
    return rc;
}

int GpuScene::camera_rays(int n, const float* pos2, float* o, float* d, DeviceArena& arena, std::string& err) {
    if (!sb_->film) { err = "no scene loaded"; return C2G_ERR_STATE; }
    if (n <= 0) return C2G_OK;
    float* buf = (float*)arena.alloc((size_t)n * 8 * 4, err);
    if (!buf) return C2G_ERR_OOM;
    int rc = C2G_OK;
    if (cudaMemcpy(buf, pos2, (size_t)n * 8, cudaMemcpyHostToDevice) != cudaSuccess) rc = C2G_ERR_CUDA;
    if (!rc) {
        k_camera<<<(n + 127) / 128, 128>>>(sb_->S.cam, n, buf, buf + 2 * n, buf + 5 * n);
        if (cudaGetLastError() != cudaSuccess || cudaMemcpy(o, buf + 2 * n, (size_t)n * 12, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(d, buf + 5 * n, (size_t)n * 12, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = C2G_ERR_CUDA;
    }
    if (rc) err = "camera query failed";
    arena.free(buf);
    return rc;
}


// ---- allocation-free rendering ------------------------------------------------------------------
// Some callers cannot call cudaMalloc while they render: a host application that owns all device
// memory through its own pool and forbids plug-ins to allocate, or a frame loop that must not
// pay cudaMalloc's implicit device synchronisation.  render_noalloc() renders with the same
// kernels as render(), but the wave's working memory (path state, queues, NEE entries, counters)
// lives in the file-scope array below instead of context allocations, and the film is a buffer
// the caller provides.  The array is part of the library image: every GPU that loads the library
// holds it until the process exits.
//
// Limits: a frame of at most kNoAllocSlots pixel slots (width and height rounded up to multiples
// of 8; 16384 slots = 128 x 128 pixels) and at most kNoAllocLights lights; larger requests are
// rejected with C2G_ERR_INVALID.  One sample per pixel per wave.  The first call on a device looks up
// the array's device address (cudaGetSymbolAddress, with that device current), so that first call
// should come before any stream capture.  Every call shares the array and overwrites what the
// previous call left there; calls that overlap on the GPU (two streams, two threads) race on it.
constexpr int kNoAllocSlots = 16384;
constexpr int kNoAllocLights = 8;
constexpr size_t kNoAllocPathBytes = 2 * 4 * 16   // o, d, beta, L (ping-pong)
                                   + 16 + 8 + 16  // hit, acc, out_L
                                   + 16           // per-pixel sums of squares (film_m2; not returned)
                                   + 3 * 16 + 4   // mis_o, mis_d, mis_hit, mis_list
                                   + 4 * kBuckets // bucket lists
                                   + (size_t)kNoAllocLights * (4 * 16 + 4);  // sh_o, sh_d, sh_c, mis_c, sh_list
constexpr size_t kNoAllocBytes = (size_t)kNoAllocSlots * kNoAllocPathBytes + 256;
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {
constexpr int kMaxDevices = 64;
void* g_noalloc_ptr[kMaxDevices] = {nullptr};
}  // namespace

int GpuScene::render_noalloc(const c2g_render_params& p, float4* film_dev, cudaStream_t st, std::string& err) {
    if (!sb_->film) { err = "no scene loaded"; return C2G_ERR_STATE; }
    if (!film_dev) { err = "film buffer is null"; return C2G_ERR_INVALID; }
    if (p.width != film_w_ || p.height != film_h_) { err = "render size differs from the loaded film size"; return C2G_ERR_INVALID; }
    if (p.max_depth < 0 || p.sample_count < 0 || p.sample_begin < 0) { err = "invalid render parameters"; return C2G_ERR_INVALID; }
    if (p.integrator != C2G_INTEGRATOR_PATH && p.integrator != C2G_INTEGRATOR_DIRECT) { err = "the allocation-free entry point runs the path tracer and direct lighting only"; return C2G_ERR_UNSUPPORTED; }
    if (p.max_depth > 255) { err = "max_depth above 255"; return C2G_ERR_INVALID; }
    WaveArgs a{};
    a.W = p.width;
    a.H = p.height;
    a.tiles_x = (p.width + 7) / 8;
    a.nslots = a.tiles_x * ((p.height + 7) / 8) * 64;
    a.max_depth = p.max_depth;
    a.K = std::max(1, sb_->S.n_lights);
    a.integrator = p.integrator;
    if (a.nslots > kNoAllocSlots) {
        err = "allocation-free render: frame of " + std::to_string(a.nslots) + " pixel slots exceeds the maximum of " +
              std::to_string(kNoAllocSlots) + " (128 x 128 pixels)";
        return C2G_ERR_INVALID;
    }
    if (a.K > kNoAllocLights) {
        err = "allocation-free render: " + std::to_string(a.K) + " lights exceed the maximum of " + std::to_string(kNoAllocLights);
        return C2G_ERR_INVALID;
    }
    // set-up, once per device with that device current: the device address of the scratch array
    int dev = 0;
    C2G_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) { err = "device ordinal out of range"; return C2G_ERR_INVALID; }
    if (!g_noalloc_ptr[dev]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
            return C2G_ERR_CUDA;
        }
        g_noalloc_ptr[dev] = ptr;
    }
    // carve the scratch array (slot-sized pieces first, then K-sized ones)
    const size_t P = (size_t)a.nslots, PK = P * (size_t)a.K;
    unsigned char* q = (unsigned char*)g_noalloc_ptr[dev];
    auto take = [&](size_t bytes) { unsigned char* r = q; q += (bytes + 255) & ~size_t(255); return r; };
    WaveBuffers w;
    for (int b = 0; b < 2; b++) {
        w.o[b] = (float4*)take(P * 16); w.d[b] = (float4*)take(P * 16);
        w.beta[b] = (float4*)take(P * 16); w.L[b] = (float4*)take(P * 16);
    }
    w.hit = (float4*)take(P * 16);
    w.acc = (int2*)take(P * 8);
    w.out_L = (float4*)take(P * 16);
    w.mis_o = (float4*)take(P * 16);
    w.mis_d = (float4*)take(P * 16);
    w.mis_hit = (float4*)take(P * 16);
    w.mis_list = (int*)take(P * 4);
    w.bucket_list = (int*)take(P * 4 * kBuckets);
    w.sh_o = (float4*)take(PK * 16);
    w.sh_d = (float4*)take(PK * 16);
    w.sh_c = (float4*)take(PK * 16);
    w.mis_c = (float4*)take(PK * 16);
    w.sh_list = (int*)take(PK * 4);
    float4* m2 = (float4*)take(P * 16);
    w.counters = (int*)take(256);
    if ((size_t)(q - (unsigned char*)g_noalloc_ptr[dev]) > kNoAllocBytes) { err = "allocation-free render: scratch layout overflow"; return C2G_ERR_INVALID; }
    w.P = P;
    w.K = a.K;
    DevScene S = sb_->S;
    S.anyhit_clip = p.accel == C2G_ACCEL_BVH ? 1 : 0;
    S.closest_box = p.accel == C2G_ACCEL_BVH ? 1 : 0;
    S.seed = p.seed;
    const int g_raygen = grid_for((const void*)k_raygen, 256), g_ext = grid_for((const void*)k_extend<false>, 128);
    const int g_shade = grid_for((const void*)k_shade<MAT_DIFFUSE, false>, 128), g_sh = grid_for((const void*)k_shadow<false>, 128);
    const int g_mis = grid_for((const void*)k_mis<false>, 128), g_acc = grid_for((const void*)k_accumulate, 256);
    const int g_film = grid_for((const void*)k_film, 256);
    int* C = w.counters;
    PathRefs buf[2] = {{w.o[0], w.d[0], w.beta[0], w.L[0]}, {w.o[1], w.d[1], w.beta[1], w.L[1]}};
    C2G_CUDA(cudaMemsetAsync(m2, 0, P * 16, st));
    // Bounce levels: as in render(), direct lighting keeps walking through surfaces without a
    // material past the depth (the reference's DirectLightingIntegrator continues such a path at the
    // same level), up to 255 hops, and stops once its queue is empty.
    const int levels = p.integrator == C2G_INTEGRATOR_DIRECT ? 255 : p.max_depth;
    for (int s0 = 0; s0 < p.sample_count; s0++) {
        a.wave_samples = 1;
        a.sample0 = p.sample_begin + s0;
        C2G_CUDA(cudaMemsetAsync(C, 0, 256, st));  // counters start at zero for every wave
        k_raygen<<<g_raygen, 256, 0, st>>>(S, a, buf[0], w.out_L, C + 0);
        int cur = 0;
        for (int b = 0; b < levels; b++) {
            int nxt = cur ^ 1;
            if (b >= a.max_depth) {
                // the queue count goes to a host stack variable: no allocation
                int qn = 0;
                C2G_CUDA(cudaMemcpyAsync(&qn, C + cur, sizeof(int), cudaMemcpyDeviceToHost, st));
                C2G_CUDA(cudaStreamSynchronize(st));
                if (qn == 0) break;
            }
            C2G_CUDA(cudaMemsetAsync(C + kCntBucket, 0, sizeof(int) * kBuckets, st));
            k_extend<false><<<g_ext, 128, 0, st>>>(S, buf[cur].o, buf[cur].d, w.hit, C + cur, C + nxt, C + 2, C + 3,
                                                     C + kCntBucket, w.bucket_list, (int)w.P, nullptr);
            ShadeOut so{buf[nxt], C + nxt, w.sh_o, w.sh_d, w.sh_c, w.mis_o, w.mis_d, w.mis_c, w.sh_list, w.mis_list, C + 2, C + 3, w.acc, w.mis_hit};
            for (int bk = 0; bk < kBuckets; bk++)
                if (present_buckets_ & (1 << bk))
                    launch_shade(bk, g_shade, st, S, a, buf[cur], w.hit, C + kCntBucket, w.bucket_list, (int)w.P, so, GuideView{}, false);
            k_shadow<false><<<g_sh, 128, 0, st>>>(S, w.sh_list, C + 2, w.sh_o, w.sh_d, w.sh_c, nullptr);
            k_mis<false><<<g_mis, 128, 0, st>>>(S, w.mis_list, C + 3, w.mis_o, w.mis_d, w.mis_hit, nullptr);
            k_accumulate<<<g_acc, 256, 0, st>>>(a, buf[cur], buf[nxt], w.acc, w.sh_c, w.mis_c, w.mis_hit, w.out_L, C + cur, GuideView{});
            cur = nxt;
        }
        // the caller's film gets the radiance sums and weights; the sums of squares stay in scratch
        k_film<<<g_film, 256, 0, st>>>(a, w.out_L, film_dev, m2);
    }
    C2G_CUDA(cudaGetLastError());
    C2G_CUDA(cudaStreamSynchronize(st));
    return check_device_error(err);
}

// ---- L2 read roof ---------------------------------------------------------------------------------
namespace {
__global__ void k_l2_read(const float4* __restrict__ p, size_t n, int reps, float* sink) {
    float acc = 0.f;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (int r = 0; r < reps; r++) {
#pragma unroll 4
        for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += stride) {
            const float4 v = __ldcg(p + i);  // L2 only: every rep after the first is an L2 hit
            acc += (v.x + v.y) + (v.z + v.w);
        }
    }
    if (acc == -1.f) *sink = acc;  // keeps the loads live; the buffer holds no negative values
}
}  // namespace

int probe_l2_read(size_t bytes, int reps, double* gbs, std::string& err) {
    if (bytes < 4096 || reps < 1) { err = "probe size out of range"; return C2G_ERR_INVALID; }
    const size_t n = bytes / 16;
    float4* buf = nullptr;
    float* sink = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = C2G_OK;
    do {
        if (cudaMalloc(&buf, n * 16) != cudaSuccess || cudaMalloc(&sink, sizeof(float)) != cudaSuccess) { rc = C2G_ERR_OOM; break; }
        if (cudaMemset(buf, 0, n * 16) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
            rc = C2G_ERR_CUDA;
            break;
        }
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const int grid = sms * 8;
        k_l2_read<<<grid, 256>>>(buf, n, 2, sink);  // brings the buffer into L2
        cudaEventRecord(e0);
        k_l2_read<<<grid, 256>>>(buf, n, reps, sink);
        cudaEventRecord(e1);
        if (cudaEventSynchronize(e1) != cudaSuccess) { rc = C2G_ERR_CUDA; break; }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        *gbs = (double)n * 16.0 * reps / (ms * 1e-3) / 1e9;
    } while (0);
    if (rc) err = "L2 probe failed";
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(buf);
    cudaFree(sink);
    return rc;
}

}  // namespace c2g
