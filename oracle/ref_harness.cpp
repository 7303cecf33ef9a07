// Harness over the reference renderer (Crystal2), compiled together with the reference's own
// translation units into oracle/_ref/libc2ref.so by oracle/build_ref.py.
//
// TEST INFRASTRUCTURE ONLY: the parity tests, the golden-vector generator and the CPU baseline
// call these entry points to obtain the reference's own answers.  Every computation below is
// done by unmodified reference classes; this file only wires inputs to them and copies results
// out.  It reaches private members (the BVH's reordered object list, the scene's lights, the
// integrator's sampler) by compiling the reference headers with `private`/`protected` opened;
// member layout is unchanged by that.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <random>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>
#include <fstream>
#include <sstream>
#include <iostream>
#include <queue>
#include <condition_variable>
#include <limits>

#define STB_IMAGE_IMPLEMENTATION
#include <stbi/stb_image.h>

#define private public
#define protected public
#include <Crystal2.h>
#include <SJson/SJson.h>
#include <Loaders/JsonLoader.h>
#include <Loaders/ConfigLoader.h>
#include <Core/Scene.h>
#include <Core/Entities.h>
#include <Core/SurfaceInteraction.h>
#include <Core/FrameBuffer.h>
#include <Core/Utils.h>
#include <Cameras/Camera.h>
#include <Accelerators/Accelerator.h>
#include <Accelerators/BVH.h>
#include <Integrators/Integrator.h>
#include <Integrators/SamplerIntegrator.h>
#include <Integrators/PathTracingIntegrator.h>
#include <Integrators/DirectLightingIntegrator.h>
#include <Samplers/HaltonSampler.h>
#include <Materials/Material.h>
#include <BSDFs/BSDF.h>
#include <Lights/Light.h>
#include <Lights/AreaLight.h>
#include <Shapes/Shape.h>
#undef private
#undef protected

namespace {

// Same field layout as the node struct private to BVH.cpp (BVH.cpp:18-33).
struct RefBVHNode {
    Bound3f bound;
    union {
        struct { int entitiesStartOffset; int count; };
        int ch[2];
    };
    int8_t splitAxis;
};

struct RefCtx {
    std::shared_ptr<SJson::SJsonNode> cfgNode, sceneNode;
    config::ConfigInfo info;
    std::unique_ptr<Scene> scene;
    std::unique_ptr<Camera> camera;
    std::unique_ptr<crystal::Integrator> integrator;
    std::vector<const crystal::Entity*> objects;               // scene order (Scene::GetObjects)
    std::unordered_map<const void*, int> objIndex;             // entity -> scene index
    std::unordered_map<const void*, int> shapeIndex;           // shape  -> scene index
    std::unordered_map<const void*, int> lightIndex;           // light  -> index in Scene::_lights
};

// FixedThreadPool's workers are detached and still lock the pool's queue after its destructor has
// returned (FixedThreadPool.cpp:5-43), a use-after-free once the integrator that owns the pool is
// freed.  Before an integrator is destroyed here its workers are told to end, given time to leave,
// and only then is the pool freed.
void retire_integrator(std::unique_ptr<crystal::Integrator>& integ) {
    auto* si = dynamic_cast<crystal::SamplerIntegrator*>(integ.get());
    if (si && si->_threadPool) {
        {
            std::lock_guard<std::mutex> lock(si->_threadPool->_queue.Mutex);
            si->_threadPool->_queue.ShouldEnd = true;
        }
        si->_threadPool->_queue.Condition.notify_all();
        std::this_thread::sleep_for(std::chrono::milliseconds(50));
    }
    integ.reset();
}

void set_err(char* err, int errlen, const char* msg) {
    if (err && errlen > 0) { std::snprintf(err, errlen, "%s", msg); }
}

const Shape* entity_shape(const crystal::Entity* e) {
    return static_cast<const crystal::GeometricEntity*>(e)->_shape;
}

}  // namespace

extern "C" {

void* ref_open(const char* cfg_path, const char* scene_path, char* err, int errlen) {
    try {
        auto ctx = new RefCtx();
        ctx->cfgNode = loader::JsonLoader::LoadJsonFile(cfg_path);
        ctx->sceneNode = loader::JsonLoader::LoadJsonFile(scene_path);
        ctx->info = config::ConfigLoader::LoadConfigInfo(ctx->cfgNode);
        // Same construction order as RayTracer::RayTracer (RayTracer.cpp:11-22).
        ctx->scene = Scene::CreateScene(ctx->sceneNode->GetMember("Scene"), ctx->info);
        ctx->camera = Camera::CreateCamera(ctx->sceneNode->GetMember("Camera"), ctx->info);
        ctx->integrator = crystal::Integrator::LoadIntegrator(ctx->cfgNode.get(), ctx->info);
        ctx->objects = ctx->scene->GetObjects();
        for (int i = 0; i < (int)ctx->objects.size(); i++) {
            ctx->objIndex[ctx->objects[i]] = i;
            ctx->shapeIndex[entity_shape(ctx->objects[i])] = i;
        }
        for (int i = 0; i < (int)ctx->scene->_lights.size(); i++)
            ctx->lightIndex[ctx->scene->_lights[i].get()] = i;
        return ctx;
    } catch (const std::exception& e) {
        set_err(err, errlen, e.what());
    } catch (...) {
        set_err(err, errlen, "unknown exception");
    }
    return nullptr;
}

void ref_close(void* h) {
    auto ctx = static_cast<RefCtx*>(h);
    retire_integrator(ctx->integrator);
    delete ctx;
}

int ref_num_objects(void* h) { return (int)static_cast<RefCtx*>(h)->objects.size(); }
int ref_num_lights(void* h) { return (int)static_cast<RefCtx*>(h)->scene->_lights.size(); }

// Light i: type (0 area, 1 point), the scene index of its shape's entity (-1 for point lights)
// and its Flux() (3 floats).
void ref_light_info(void* h, int i, int* type, int* obj, float* flux) {
    auto ctx = static_cast<RefCtx*>(h);
    const crystal::Light* L = ctx->scene->_lights[i].get();
    auto* area = dynamic_cast<const crystal::AreaLight*>(L);
    *type = area ? 0 : 1;
    *obj = -1;
    if (area) {
        auto it = ctx->shapeIndex.find(area->GetAttachedObject());
        *obj = it == ctx->shapeIndex.end() ? -1 : it->second;
    }
    auto F = L->Flux();
    flux[0] = F.x; flux[1] = F.y; flux[2] = F.z;
}

// BVH::_objects after the build, as scene indices (the "primitive order").
int ref_bvh_order(void* h, int* order) {
    auto ctx = static_cast<RefCtx*>(h);
    auto* bvh = dynamic_cast<BVH*>(ctx->scene->_accelStructure.get());
    if (!bvh) return -1;
    for (size_t i = 0; i < bvh->_objects.size(); i++) order[i] = ctx->objIndex.at(bvh->_objects[i]);
    return (int)bvh->_objects.size();
}

// Node array 1.._tot.  bounds: 6 floats (min, max); a: ch[0], ch[1] (internal) or
// start, count (leaf); axis: splitAxis (-1 leaf).  Returns _tot (0 when not a BVH).
int ref_bvh_nodes(void* h, float* bounds, int* a, int* axis) {
    auto ctx = static_cast<RefCtx*>(h);
    auto* bvh = dynamic_cast<BVH*>(ctx->scene->_accelStructure.get());
    if (!bvh) return 0;
    auto* nodes = reinterpret_cast<const RefBVHNode*>(bvh->_nodes);
    int tot = bvh->_tot;
    if (bounds) {
        for (int i = 1; i <= tot; i++) {
            auto mn = nodes[i].bound.GetMinPos(), mx = nodes[i].bound.GetMaxPos();
            float* b = bounds + 6 * (i - 1);
            b[0] = mn.x; b[1] = mn.y; b[2] = mn.z; b[3] = mx.x; b[4] = mx.y; b[5] = mx.z;
            a[2 * (i - 1)] = nodes[i].ch[0];
            a[2 * (i - 1) + 1] = nodes[i].ch[1];
            axis[i - 1] = nodes[i].splitAxis;
        }
    }
    return tot;
}

// Scene::Intersect per ray: scene index of the hit object (-1 on miss) and its distance.
void ref_intersect(void* h, int n, const float* o, const float* d, int* obj, float* t, int threads) {
    auto ctx = static_cast<RefCtx*>(h);
    auto work = [&](int lo, int hi) {
        for (int i = lo; i < hi; i++) {
            Ray3f ray(glm::vec3(o[3 * i], o[3 * i + 1], o[3 * i + 2]), glm::vec3(d[3 * i], d[3 * i + 1], d[3 * i + 2]));
            SurfaceInteraction isec;
            bool hit = ctx->scene->Intersect(ray, &isec);
            if (hit && isec.GetHitEntity()) {
                obj[i] = ctx->objIndex.at(isec.GetHitEntity());
                t[i] = isec.GetDistance();
            } else {
                obj[i] = -1;
                t[i] = std::numeric_limits<float>::infinity();
            }
        }
    };
    if (threads <= 1) { work(0, n); return; }
    std::vector<std::thread> th;
    int chunk = (n + threads - 1) / threads;
    for (int k = 0; k < threads; k++) th.emplace_back(work, std::min(n, k * chunk), std::min(n, (k + 1) * chunk));
    for (auto& x : th) x.join();
}

// Scene::IntersectTest per ray with [tmin, tmax] and an ignored object (scene index or -1).
void ref_intersect_test(void* h, int n, const float* o, const float* d, const float* tmin, const float* tmax,
                        const int* ignore_obj, int* occluded) {
    auto ctx = static_cast<RefCtx*>(h);
    for (int i = 0; i < n; i++) {
        Ray3f ray(glm::vec3(o[3 * i], o[3 * i + 1], o[3 * i + 2]), glm::vec3(d[3 * i], d[3 * i + 1], d[3 * i + 2]));
        const crystal::IIntersectable* ign = nullptr;
        if (ignore_obj && ignore_obj[i] >= 0) ign = entity_shape(ctx->objects[ignore_obj[i]]);
        occluded[i] = ctx->scene->IntersectTest(ray, tmin[i], tmax[i], ign) ? 1 : 0;
    }
}

// PerspCamera::GenerateRay for NDC positions pos2 = (x, y) in [0,1]^2.
void ref_camera(void* h, int n, const float* pos2, float* o, float* d) {
    auto ctx = static_cast<RefCtx*>(h);
    for (int i = 0; i < n; i++) {
        auto r = ctx->camera->GenerateRay(glm::vec2(pos2[2 * i], pos2[2 * i + 1]));
        o[3 * i] = r.start.x; o[3 * i + 1] = r.start.y; o[3 * i + 2] = r.start.z;
        d[3 * i] = r.dir.x; d[3 * i + 1] = r.dir.y; d[3 * i + 2] = r.dir.z;
    }
}

// The reference renderer itself: Integrator::Render with `threads` workers (<= 16) into a
// FrameBuffer; returns wall seconds (steady_clock) and the raw per-pixel sums and weights
// (row y = pixel y of the sample loop, unflipped).
double ref_render(void* h, int threads, float* rgb_sum, float* weight) {
    auto ctx = static_cast<RefCtx*>(h);
    config::ConfigInfo info = ctx->info;
    if (threads > 0) info.NumOfThreads = std::min(16, threads);
    auto integ = crystal::Integrator::LoadIntegrator(ctx->cfgNode.get(), info);
    FrameBuffer fb(info.Width, info.Height);
    fb.Clear();
    auto t0 = std::chrono::steady_clock::now();
    integ->Render(ctx->scene.get(), ctx->camera.get(), &fb);
    auto t1 = std::chrono::steady_clock::now();
    retire_integrator(integ);
    int W = info.Width, H = info.Height;
    for (int i = 0; i < W * H; i++) {
        auto& p = fb._hdrData[i];
        if (rgb_sum) { rgb_sum[3 * i] = p.color.x; rgb_sum[3 * i + 1] = p.color.y; rgb_sum[3 * i + 2] = p.color.z; }
        if (weight) weight[i] = p.weight;
    }
    return std::chrono::duration<double>(t1 - t0).count();
}

// The reference's Radiance writer (stb_image_write, called by RayTracer.cpp:40) on caller data.
extern "C" int stbi_write_hdr(char const* filename, int w, int h, int comp, const float* data);
int ref_write_hdr(const char* path, int w, int h, const float* rgb) { return stbi_write_hdr(path, w, h, 3, rgb); }

// Per-pixel statistics over the rectangle [x0,x1) x [y0,y1) at `spp` samples: the same loop as
// SamplerIntegrator::Render (SamplerIntegrator.cpp:42-59) calling the integrator's own Evaluate,
// accumulating sum and sum of squares per pixel (after the FrameBuffer's NaN/Inf zeroing,
// FrameBuffer.cpp:21-28).  Rows are split across `threads` workers, each with its own sampler
// clone.  With group > 0 the sums are kept per run of `group` consecutive samples (sample s adds to
// group s / group): sum holds ceil(spp / group) planes of 3 floats per pixel, each plane an
// independent estimate from its own samples.  Returns wall seconds.  sum/sumsq: 3 doubles per pixel
// of the rectangle (row-major) per plane; sumsq covers all samples.
static double render_region_groups(RefCtx* ctx, int threads, int x0, int y0, int x1, int y1, int group, double* sum,
                                   double* sumsq) {
    auto* si = dynamic_cast<crystal::SamplerIntegrator*>(ctx->integrator.get());
    if (!si) return -1.0;
    int W = ctx->info.Width, H = ctx->info.Height;
    const int spp = (int)si->_sampler->GetSamplesPerPixel();
    if (group <= 0) group = spp;
    const int ngroups = (spp + group - 1) / group;
    const int rw = x1 - x0, rh = y1 - y0;
    const size_t plane = (size_t)rw * rh * 3;
    std::atomic<int> nextRow{y0};
    auto worker = [&]() {
        auto sampler = si->_sampler->Clone(0);
        std::vector<double> s(3 * (size_t)ngroups);
        while (true) {
            int yy = nextRow.fetch_add(1);
            if (yy >= y1) break;
            for (int xx = x0; xx < x1; xx++) {
                std::fill(s.begin(), s.end(), 0.0);
                double q[3] = {0, 0, 0};
                int k = 0;
                sampler->StartPixel(Point2i(xx, yy));
                do {
                    auto u = sampler->Get2D();
                    glm::vec2 pos = glm::vec2(xx, yy) + u;
                    pos.x = pos.x / W;
                    pos.y = pos.y / H;
                    auto ray = ctx->camera->GenerateRay(pos);
                    auto c = si->Evaluate(ray, ctx->scene.get(), sampler.get());
                    if (glm::isnan(c) != glm::bvec3(false) || glm::isinf(c) != glm::bvec3(false)) c = glm::vec3(0);
                    const int g = std::min(ngroups - 1, k / group);
                    for (int j = 0; j < 3; j++) { s[3 * g + j] += c[j]; q[j] += (double)c[j] * c[j]; }
                    k++;
                } while (sampler->StartNextSample());
                size_t idx = (size_t)(yy - y0) * rw + (xx - x0);
                for (int g = 0; g < ngroups; g++)
                    for (int j = 0; j < 3; j++) sum[g * plane + 3 * idx + j] = s[3 * g + j];
                for (int j = 0; j < 3; j++) sumsq[3 * idx + j] = q[j];
            }
        }
    };
    auto t0 = std::chrono::steady_clock::now();
    int nt = std::max(1, threads);
    std::vector<std::thread> th;
    for (int k = 0; k < nt; k++) th.emplace_back(worker);
    for (auto& x : th) x.join();
    auto t1 = std::chrono::steady_clock::now();
    (void)H;
    return std::chrono::duration<double>(t1 - t0).count();
}

double ref_render_region(void* h, int threads, int x0, int y0, int x1, int y1, double* sum, double* sumsq) {
    return render_region_groups(static_cast<RefCtx*>(h), threads, x0, y0, x1, y1, 0, sum, sumsq);
}

double ref_render_region_groups(void* h, int threads, int x0, int y0, int x1, int y1, int group, double* sum,
                                double* sumsq) {
    return render_region_groups(static_cast<RefCtx*>(h), threads, x0, y0, x1, y1, group, sum, sumsq);
}

// Scene::IntersectTest on `threads` workers (the same per-ray call as ref_intersect_test).
void ref_intersect_test_mt(void* h, int n, const float* o, const float* d, const float* tmin, const float* tmax,
                           const int* ignore_obj, int* occluded, int threads) {
    auto ctx = static_cast<RefCtx*>(h);
    auto work = [&](int lo, int hi) {
        for (int i = lo; i < hi; i++) {
            Ray3f ray(glm::vec3(o[3 * i], o[3 * i + 1], o[3 * i + 2]), glm::vec3(d[3 * i], d[3 * i + 1], d[3 * i + 2]));
            const crystal::IIntersectable* ign = nullptr;
            if (ignore_obj && ignore_obj[i] >= 0) ign = entity_shape(ctx->objects[ignore_obj[i]]);
            occluded[i] = ctx->scene->IntersectTest(ray, tmin[i], tmax[i], ign) ? 1 : 0;
        }
    };
    int nt = std::max(1, threads);
    std::vector<std::thread> th;
    int chunk = (n + nt - 1) / nt;
    for (int k = 0; k < nt; k++) th.emplace_back(work, std::min(n, k * chunk), std::min(n, (k + 1) * chunk));
    for (auto& x : th) x.join();
}

// Per-sample radiance for a few pixels: out[(p * spp + s) * 3 + c].
void ref_render_samples(void* h, int n, const int* px, const int* py, float* out) {
    auto ctx = static_cast<RefCtx*>(h);
    auto* si = dynamic_cast<crystal::SamplerIntegrator*>(ctx->integrator.get());
    int W = ctx->info.Width, H = ctx->info.Height;
    auto sampler = si->_sampler->Clone(0);
    int spp = (int)sampler->GetSamplesPerPixel();
    for (int p = 0; p < n; p++) {
        sampler->StartPixel(Point2i(px[p], py[p]));
        int s = 0;
        do {
            auto u = sampler->Get2D();
            glm::vec2 pos = glm::vec2(px[p], py[p]) + u;
            pos.x = pos.x / W;
            pos.y = pos.y / H;
            auto ray = ctx->camera->GenerateRay(pos);
            auto c = si->Evaluate(ray, ctx->scene.get(), sampler.get());
            out[((size_t)p * spp + s) * 3 + 0] = c.x;
            out[((size_t)p * spp + s) * 3 + 1] = c.y;
            out[((size_t)p * spp + s) * 3 + 2] = c.z;
            s++;
        } while (sampler->StartNextSample());
    }
}

// HaltonSampler::SampleValue(GetVectorIndexForSample(sample), dim) for dims < 100.
void ref_halton(int W, int H, int spp, int n, const int* px, const int* py, const int* sample, int ndim, float* out) {
    crystal::HaltonSampler hs(spp, Bound2i(Point2i(0, 0), Point2i(W, H)));
    for (int i = 0; i < n; i++) {
        hs.StartPixel(Point2i(px[i], py[i]));
        int idx = hs.GetVectorIndexForSample(sample[i]);
        for (int d = 0; d < ndim; d++) out[(size_t)i * ndim + d] = hs.SampleValue(idx, d);
    }
}

// Vector index of (pixel, sample) (HaltonSampler.cpp:251-270).
void ref_halton_index(int W, int H, int spp, int n, const int* px, const int* py, const int* sample, long long* out) {
    crystal::HaltonSampler hs(spp, Bound2i(Point2i(0, 0), Point2i(W, H)));
    for (int i = 0; i < n; i++) {
        hs.StartPixel(Point2i(px[i], py[i]));
        out[i] = hs.GetVectorIndexForSample(sample[i]);
    }
}

// BSDF of a material on a synthetic hit.  frame = N, dpdu, dpdv (9 floats).  For each i:
// f_eval/pdf_eval = BSDF::DistributionFunction(wo, wi) and BSDF::Pdf(wo, wi, flags);
// f_samp/wi_samp/pdf_samp/type_samp = BSDF::SampleDirection(u[0], (u[1], u[2]), wo, flags).
// Returns the number of BxDFs, or -1 when the material cannot be built.
int ref_bsdf(const char* material_json, int front_face, const float* frame, int n, const float* wo,
             const float* wi, const float* u3, int flags, float* f_eval, float* pdf_eval, float* f_samp,
             float* wi_samp, float* pdf_samp, int* type_samp) {
    std::shared_ptr<Material> mat;
    try {
        auto node = SJson::SJsonParse(std::string(material_json));
        mat = Material::CreateMaterial(node.get(), nullptr);
    } catch (...) {
        return -1;
    }
    glm::vec3 N(frame[0], frame[1], frame[2]), T(frame[3], frame[4], frame[5]), B(frame[6], frame[7], frame[8]);
    int nb = 0;
    for (int i = 0; i < n; i++) {
        SurfaceInteraction isec;
        isec.SetHitInfo(1.f, glm::vec3(0), glm::vec3(0, 0, 1), N, glm::vec2(0), front_face != 0, T, B);
        BSDF bsdf(&isec);
        isec.SetBSDF(&bsdf);
        mat->ComputeScatteringFunctions(isec, true);
        nb = bsdf.NumBxDFs();
        glm::vec3 o(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]), w(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]);
        auto f = bsdf.DistributionFunction(o, w);
        f_eval[3 * i] = f.x; f_eval[3 * i + 1] = f.y; f_eval[3 * i + 2] = f.z;
        pdf_eval[i] = bsdf.Pdf(o, w, (BxDFType)flags);
        glm::vec3 ws(0.f);
        float pdf = 0.f;
        BxDFType st = (BxDFType)0;
        auto fs = bsdf.SampleDirection(u3[3 * i], glm::vec2(u3[3 * i + 1], u3[3 * i + 2]), o, &ws, &pdf, (BxDFType)flags, &st);
        f_samp[3 * i] = fs.x; f_samp[3 * i + 1] = fs.y; f_samp[3 * i + 2] = fs.z;
        wi_samp[3 * i] = ws.x; wi_samp[3 * i + 1] = ws.y; wi_samp[3 * i + 2] = ws.z;
        pdf_samp[i] = pdf;
        type_samp[i] = (int)st;
    }
    return nb;
}

// Light::Sample_Li and Light::Pdf_Li for light `li` at surface points (pos, normal).
void ref_light_sample(void* h, int li, int n, const float* pos, const float* nrm, const float* u2, float* Li,
                      float* endpoint, float* pdf) {
    auto ctx = static_cast<RefCtx*>(h);
    const crystal::Light* L = ctx->scene->_lights[li].get();
    for (int i = 0; i < n; i++) {
        SurfaceInfo s(glm::vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]), glm::vec3(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]));
        glm::vec3 ep(0.f);
        float p = 0.f;
        auto v = L->Sample_Li(s, glm::vec2(u2[2 * i], u2[2 * i + 1]), &ep, &p);
        Li[3 * i] = v.x; Li[3 * i + 1] = v.y; Li[3 * i + 2] = v.z;
        endpoint[3 * i] = ep.x; endpoint[3 * i + 1] = ep.y; endpoint[3 * i + 2] = ep.z;
        pdf[i] = p;
    }
}

void ref_light_pdf(void* h, int li, int n, const float* pos, const float* nrm, const float* wi, float* pdf) {
    auto ctx = static_cast<RefCtx*>(h);
    const crystal::Light* L = ctx->scene->_lights[li].get();
    for (int i = 0; i < n; i++) {
        SurfaceInfo s(glm::vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]), glm::vec3(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]));
        pdf[i] = L->Pdf_Li(s, glm::vec3(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]));
    }
}

}  // extern "C"
