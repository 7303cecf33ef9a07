// C ABI (include/c2g.h) over the host scene, the tree builders and the CUDA renderer.
#include <cuda_runtime.h>

#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/c2g.h"
#include "host/bvh.h"
#include "host/json.h"
#include "host/scene.h"
#include "kernels/render.h"

using namespace c2g;

struct c2g_ctx {
    int device = 0;
    int verbose = 0;
    std::string last_error;
    std::unique_ptr<DeviceArena> arena;
    std::unique_ptr<GpuScene> gpu;
    std::unique_ptr<HostScene> scene;
    RefTree ref;
    SahTree sah;
    int tree = C2G_TREE_REF_EQUAL_COUNT;
    bool loaded = false;       // scene uploaded to the device
    bool host_loaded = false;  // scene parsed and trees built on the host
    bool host_only = false;    // created with device < 0: no CUDA calls at all
    cudaStream_t stream = nullptr;
};

namespace {

int fail(c2g_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    return code;
}

int set_device(c2g_ctx* ctx) {
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return fail(ctx, C2G_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    return C2G_OK;
}

int build_and_upload(c2g_ctx* ctx, int tree) {
    if (tree != C2G_TREE_REF_EQUAL_COUNT && tree != C2G_TREE_SAH) return fail(ctx, C2G_ERR_INVALID, "unknown tree kind");
    // the reference tree is always built: it defines the primitive order the parity checks use
    build_ref_tree(*ctx->scene, ctx->ref);
    if (tree == C2G_TREE_SAH) build_sah_tree(*ctx->scene, ctx->sah, 4);
    ctx->tree = tree;
    ctx->host_loaded = true;
    if (ctx->host_only) return C2G_OK;
    int rc = set_device(ctx);
    if (rc) return rc;
    std::string err;
    rc = ctx->gpu->upload(*ctx->scene, tree, &ctx->ref, tree == C2G_TREE_SAH ? &ctx->sah : nullptr, *ctx->arena, err);
    if (rc) return fail(ctx, rc, err);
    ctx->loaded = true;
    return C2G_OK;
}

int load_texts(c2g_ctx* ctx, const std::string& cfg, const std::string& scn, int tree) {
    ctx->loaded = false;
    ctx->host_loaded = false;
    try {
        auto s = std::make_unique<HostScene>();
        load_scene(*s, cfg, scn);
        ctx->scene = std::move(s);
    } catch (const SceneError& e) {
        return fail(ctx, e.code, e.what());
    } catch (const JsonError& e) {
        return fail(ctx, e.code, e.what());
    } catch (const std::exception& e) {
        return fail(ctx, C2G_ERR_INVALID, e.what());
    }
    return build_and_upload(ctx, tree);
}

cudaStream_t pick_stream(c2g_ctx* ctx, void* s) { return s ? (cudaStream_t)s : ctx->stream; }

}  // namespace

// ---- learned guiding proposal ----------------------------------------------------------------
namespace {
int guide_ready(c2g_ctx* ctx) {
    if (!ctx) return C2G_ERR_INVALID;
    if (ctx->host_only) return fail(ctx, C2G_ERR_STATE, "host-only context");
    if (!ctx->gpu->guide().ready()) return fail(ctx, C2G_ERR_STATE, "no guide network (c2g_guide_reset or a guided render)");
    return set_device(ctx);
}
}  // namespace

extern "C" {

const char* c2g_version(void) { return "crystal2-gb300 0.1 (sm_103a)"; }

int c2g_create(c2g_ctx** out, const c2g_device_opts* opts) {
    if (!out) return C2G_ERR_INVALID;
    *out = nullptr;
    auto ctx = new (std::nothrow) c2g_ctx();
    if (!ctx) return C2G_ERR_OOM;
    if (opts) {
        ctx->device = opts->device;
        ctx->verbose = opts->verbose;
    }
    ctx->arena = std::make_unique<DeviceArena>(opts ? opts->mem_limit_bytes : 0);
    ctx->gpu = std::make_unique<GpuScene>();
    if (ctx->device < 0) {
        // host-only context: scene parsing and tree builds, no device work
        ctx->host_only = true;
        *out = ctx;
        return C2G_OK;
    }
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n <= 0) {
        cudaGetLastError();
        ctx->last_error = "no CUDA device available";
        *out = ctx;
        return C2G_ERR_CUDA;
    }
    if (ctx->device < 0 || ctx->device >= n) {
        ctx->last_error = "device ordinal out of range";
        *out = ctx;
        return C2G_ERR_INVALID;
    }
    cudaSetDevice(ctx->device);
    e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        ctx->last_error = std::string("cudaStreamCreate: ") + cudaGetErrorString(e);
        *out = ctx;
        return C2G_ERR_CUDA;
    }
    *out = ctx;
    return C2G_OK;
}

void c2g_destroy(c2g_ctx* ctx) {
    if (!ctx) return;
    if (ctx->host_only) {
        delete ctx;
        return;
    }
    if (ctx->stream) {
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        cudaStreamDestroy(ctx->stream);
    }
    ctx->gpu.reset();
    ctx->arena.reset();
    delete ctx;
}

const char* c2g_last_error(const c2g_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

int c2g_load_json(c2g_ctx* ctx, const char* config_path, const char* scene_path, int tree) {
    if (!ctx || !config_path || !scene_path) return fail(ctx, C2G_ERR_INVALID, "null argument");
    std::string cfg, scn;
    try {
        cfg = read_text_file(config_path);
        scn = read_text_file(scene_path);
    } catch (const SceneError& e) {
        return fail(ctx, e.code, e.what());
    }
    return load_texts(ctx, cfg, scn, tree);
}

int c2g_load_json_text(c2g_ctx* ctx, const char* config_json, const char* scene_json, int tree) {
    if (!ctx || !config_json || !scene_json) return fail(ctx, C2G_ERR_INVALID, "null argument");
    return load_texts(ctx, config_json, scene_json, tree);
}

int c2g_bvh_build(c2g_ctx* ctx, int tree) {
    if (!ctx) return C2G_ERR_INVALID;
    if (!ctx->scene) return fail(ctx, C2G_ERR_STATE, "no scene loaded");
    return build_and_upload(ctx, tree);
}

int c2g_get_render_params(c2g_ctx* ctx, c2g_render_params* out) {
    if (!ctx || !out) return fail(ctx, C2G_ERR_INVALID, "null argument");
    if (!ctx->scene) return fail(ctx, C2G_ERR_STATE, "no scene loaded");
    const HostConfig& c = ctx->scene->cfg;
    std::memset(out, 0, sizeof(*out));
    out->width = c.width;
    out->height = c.height;
    out->spp = c.spp;
    out->max_depth = c.depth;
    out->integrator = c.integrator == "DirectLight" ? C2G_INTEGRATOR_DIRECT
                      : c.integrator == "GuidedPathTracer" ? C2G_INTEGRATOR_GUIDED : C2G_INTEGRATOR_PATH;
    out->accel = c.accel == "BVH" ? C2G_ACCEL_BVH : C2G_ACCEL_BRUTE;
    out->sample_begin = 0;
    out->sample_count = c.spp;
    out->wave_paths = 0;
    out->seed = (uint64_t)c.seed;
    return C2G_OK;
}

int c2g_num_objects(c2g_ctx* ctx) { return ctx && ctx->scene ? (int)ctx->scene->objs.size() : -1; }
int c2g_num_lights(c2g_ctx* ctx) { return ctx && ctx->scene ? (int)ctx->scene->lights.size() : -1; }

int c2g_bvh_order(c2g_ctx* ctx, int* order, int n) {
    if (!ctx || !order) return fail(ctx, C2G_ERR_INVALID, "null argument");
    if (!ctx->host_loaded) return fail(ctx, C2G_ERR_STATE, "no scene loaded");
    int m = (int)ctx->ref.order.size();
    for (int i = 0; i < m && i < n; i++) order[i] = ctx->ref.order[i];
    return m;
}

int c2g_bvh_nodes(c2g_ctx* ctx, float* bounds, int* a, int* axis, int cap) {
    if (!ctx) return C2G_ERR_INVALID;
    if (!ctx->host_loaded) return fail(ctx, C2G_ERR_STATE, "no scene loaded");
    int tot = ctx->ref.tot;
    if (bounds && a && axis) {
        for (int i = 1; i <= tot && i <= cap; i++) {
            const RefNode& n = ctx->ref.nodes[i];
            float* b = bounds + 6 * (i - 1);
            for (int k = 0; k < 3; k++) { b[k] = n.mn[k]; b[3 + k] = n.mx[k]; }
            int ax = (n.b >> 28) & 3;
            a[2 * (i - 1)] = n.a;
            a[2 * (i - 1) + 1] = n.b & 0x0fffffff;
            axis[i - 1] = ax == 3 ? -1 : ax;
        }
    }
    return tot;
}

int c2g_render(c2g_ctx* ctx, const c2g_render_params* params, void* stream) {
    if (!ctx || !params) return fail(ctx, C2G_ERR_INVALID, "null argument");
    if (!ctx->loaded) return fail(ctx, C2G_ERR_STATE, "no scene loaded");
    int rc = set_device(ctx);
    if (rc) return rc;
    std::string err;
    rc = ctx->gpu->render(*ctx->scene, *params, pick_stream(ctx, stream), *ctx->arena, err);
    if (rc) return fail(ctx, rc, err);
    return C2G_OK;
}

int c2g_render_noalloc(c2g_ctx* ctx, const c2g_render_params* params, float* film_dev, void* stream) {
    if (!ctx || !params || !film_dev) return fail(ctx, C2G_ERR_INVALID, "null argument");
    if (!ctx->loaded) return fail(ctx, C2G_ERR_STATE, "no scene loaded");
    int rc = set_device(ctx);
    if (rc) return rc;
    std::string err;
    rc = ctx->gpu->render_noalloc(*params, (float4*)film_dev, pick_stream(ctx, stream), err);
    if (rc) return fail(ctx, rc, err);
    return C2G_OK;
}

int c2g_film_clear(c2g_ctx* ctx, void* stream) {
    if (!ctx) return C2G_ERR_INVALID;
    if (!ctx->loaded) return fail(ctx, C2G_ERR_STATE, "no scene loaded");
    int rc = set_device(ctx);
    if (rc) return rc;
    rc = ctx->gpu->film_clear(pick_stream(ctx, stream));
    if (rc) return fail(ctx, rc, "film clear failed");
    return C2G_OK;
}

int c2g_film_download(c2g_ctx* ctx, float* rgb_sum, float* weight) {
    if (!ctx) return C2G_ERR_INVALID;
    if (!ctx->loaded) return fail(ctx, C2G_ERR_STATE, "no scene loaded");
    int rc = set_device(ctx);
    if (rc) return rc;
    cudaStreamSynchronize(ctx->stream);
    std::string err;
    rc = ctx->gpu->film_download(rgb_sum, weight, nullptr, err);
    if (rc) return fail(ctx, rc, err);
    return C2G_OK;
}

int c2g_film_download_m2(c2g_ctx* ctx, float* rgb_sumsq) {
    if (!ctx || !rgb_sumsq) return fail(ctx, C2G_ERR_INVALID, "null argument");
    if (!ctx->loaded) return fail(ctx, C2G_ERR_STATE, "no scene loaded");
    int rc = set_device(ctx);
    if (rc) return rc;
    cudaStreamSynchronize(ctx->stream);
    std::string err;
    rc = ctx->gpu->film_download(nullptr, nullptr, rgb_sumsq, err);
    if (rc) return fail(ctx, rc, err);
    return C2G_OK;
}

int c2g_film_image(c2g_ctx* ctx, float* rgb) {
    if (!ctx || !rgb) return fail(ctx, C2G_ERR_INVALID, "null argument");
    if (!ctx->loaded) return fail(ctx, C2G_ERR_STATE, "no scene loaded");
    int W = ctx->scene->cfg.width, H = ctx->scene->cfg.height;
    std::vector<float> sum((size_t)W * H * 3), wgt((size_t)W * H);
    int rc = c2g_film_download(ctx, sum.data(), wgt.data());
    if (rc) return rc;
    // GetImageDataRGB32F (FrameBuffer.cpp:58-75): row i of the image is film row H - 1 - i
    for (int i = 0; i < H; i++)
        for (int j = 0; j < W; j++) {
            size_t orig = (size_t)(H - i - 1) * W + j, dest = (size_t)i * W + j;
            for (int k = 0; k < 3; k++) rgb[3 * dest + k] = sum[3 * orig + k] / wgt[orig];
        }
    return C2G_OK;
}

int c2g_get_stats(c2g_ctx* ctx, c2g_stats* out) {
    if (!ctx || !out) return fail(ctx, C2G_ERR_INVALID, "null argument");
    *out = ctx->gpu->stats();
    return C2G_OK;
}

int c2g_set_counting(c2g_ctx* ctx, int flags) {
    if (!ctx) return C2G_ERR_INVALID;
    ctx->gpu->set_counting(flags);
    return C2G_OK;
}

int c2g_trace_rays_dev(c2g_ctx* ctx, int n, const float* o_dev, const float* d_dev, const float* tmin_dev,
                       const float* tmax_dev, const int* ignore_dev, int any_hit, int* obj_dev, float* t_dev, void* stream) {
    if (!ctx || n < 0 || (n > 0 && (!o_dev || !d_dev || !obj_dev))) return fail(ctx, C2G_ERR_INVALID, "null argument");
    if (!ctx->loaded) return fail(ctx, C2G_ERR_STATE, "no scene loaded");
    int rc = set_device(ctx);
    if (rc) return rc;
    std::string err;
    rc = ctx->gpu->trace_rays_dev(n, o_dev, d_dev, tmin_dev, tmax_dev, ignore_dev, any_hit, obj_dev, t_dev,
                                  pick_stream(ctx, stream), err);
    if (rc) return fail(ctx, rc, err);
    return C2G_OK;
}

int c2g_trace_rays(c2g_ctx* ctx, int n, const float* o, const float* d, const float* tmin, const float* tmax,
                   const int* ignore, int any_hit, int* obj, float* t) {
    if (!ctx || n < 0 || (n > 0 && (!o || !d || !obj))) return fail(ctx, C2G_ERR_INVALID, "null argument");
    if (!ctx->loaded) return fail(ctx, C2G_ERR_STATE, "no scene loaded");
    if (n == 0) return C2G_OK;
    int rc = set_device(ctx);
    if (rc) return rc;
    std::string err;
    size_t n3 = (size_t)n * 12, n1 = (size_t)n * 4;
    size_t total = 2 * n3 + 4 * n1;
    char* buf = (char*)ctx->arena->alloc(total, err);
    if (!buf) return fail(ctx, C2G_ERR_OOM, err);
    float* d_o = (float*)buf;
    float* d_d = (float*)(buf + n3);
    float* d_tmin = (float*)(buf + 2 * n3);
    float* d_tmax = (float*)(buf + 2 * n3 + n1);
    int* d_ign = (int*)(buf + 2 * n3 + 2 * n1);
    int* d_obj = (int*)(buf + 2 * n3 + 3 * n1);
    float* d_t = t ? (float*)ctx->arena->alloc(n1, err) : nullptr;
    cudaStream_t st = ctx->stream;
    rc = C2G_OK;
    do {
        if (t && !d_t) { rc = fail(ctx, C2G_ERR_OOM, err); break; }
        if (cudaMemcpyAsync(d_o, o, n3, cudaMemcpyHostToDevice, st) != cudaSuccess ||
            cudaMemcpyAsync(d_d, d, n3, cudaMemcpyHostToDevice, st) != cudaSuccess) { rc = fail(ctx, C2G_ERR_CUDA, "copy failed"); break; }
        if (tmin && cudaMemcpyAsync(d_tmin, tmin, n1, cudaMemcpyHostToDevice, st) != cudaSuccess) { rc = fail(ctx, C2G_ERR_CUDA, "copy failed"); break; }
        if (tmax && cudaMemcpyAsync(d_tmax, tmax, n1, cudaMemcpyHostToDevice, st) != cudaSuccess) { rc = fail(ctx, C2G_ERR_CUDA, "copy failed"); break; }
        if (ignore && cudaMemcpyAsync(d_ign, ignore, n1, cudaMemcpyHostToDevice, st) != cudaSuccess) { rc = fail(ctx, C2G_ERR_CUDA, "copy failed"); break; }
        rc = ctx->gpu->trace_rays_dev(n, d_o, d_d, tmin ? d_tmin : nullptr, tmax ? d_tmax : nullptr, ignore ? d_ign : nullptr,
                                      any_hit, d_obj, d_t, st, err);
        if (rc) { fail(ctx, rc, err); break; }
        if (cudaMemcpyAsync(obj, d_obj, n1, cudaMemcpyDeviceToHost, st) != cudaSuccess) { rc = fail(ctx, C2G_ERR_CUDA, "copy failed"); break; }
        if (t && cudaMemcpyAsync(t, d_t, n1, cudaMemcpyDeviceToHost, st) != cudaSuccess) { rc = fail(ctx, C2G_ERR_CUDA, "copy failed"); break; }
        if (cudaStreamSynchronize(st) != cudaSuccess) { rc = fail(ctx, C2G_ERR_CUDA, "stream sync failed"); break; }
        rc = ctx->gpu->check_device_error(err);
        if (rc) fail(ctx, rc, err);
    } while (0);
    cudaStreamSynchronize(st);
    ctx->arena->free(buf);
    if (d_t) ctx->arena->free(d_t);
    return rc;
}

int c2g_halton(c2g_ctx* ctx, int width, int height, int n, const int* px, const int* py, const int* sample, int ndim, float* out) {
    if (!ctx || n < 0 || ndim < 0 || (n > 0 && (!px || !py || !sample || !out))) return fail(ctx, C2G_ERR_INVALID, "null argument");
    if (width <= 0 || height <= 0) return fail(ctx, C2G_ERR_INVALID, "film size must be positive");
    if (!ctx->loaded) return fail(ctx, C2G_ERR_STATE, "no scene loaded");
    int rc = set_device(ctx);
    if (rc) return rc;
    std::string err;
    rc = ctx->gpu->halton(width, height, n, px, py, sample, ndim, out, *ctx->arena, err);
    if (rc) return fail(ctx, rc, err);
    return C2G_OK;
}

int c2g_camera_rays(c2g_ctx* ctx, int n, const float* pos2, float* o, float* d) {
    if (!ctx || n < 0 || (n > 0 && (!pos2 || !o || !d))) return fail(ctx, C2G_ERR_INVALID, "null argument");
    if (!ctx->loaded) return fail(ctx, C2G_ERR_STATE, "no scene loaded");
    int rc = set_device(ctx);
    if (rc) return rc;
    std::string err;
    rc = ctx->gpu->camera_rays(n, pos2, o, d, *ctx->arena, err);
    if (rc) return fail(ctx, rc, err);
    return C2G_OK;
}


static_assert(C2G_GUIDE_PARAMS == kGuideParams, "guide parameter count");
static_assert(C2G_GUIDE_OUTPUTS == kGuideOut, "guide output count");

int c2g_guide_reset(c2g_ctx* ctx, const float box_lo[3], const float box_hi[3], unsigned long long seed) {
    if (!ctx || !box_lo || !box_hi) return fail(ctx, C2G_ERR_INVALID, "null argument");
    if (ctx->host_only) return fail(ctx, C2G_ERR_STATE, "host-only context");
    int rc = set_device(ctx);
    if (rc) return rc;
    std::string err;
    ctx->gpu->guide().release(*ctx->arena);
    rc = ctx->gpu->guide().init(*ctx->arena, 64, 1, box_lo, box_hi, seed, err);
    if (!rc && cudaDeviceSynchronize() != cudaSuccess) { rc = C2G_ERR_CUDA; err = cudaGetErrorString(cudaGetLastError()); }
    return rc ? fail(ctx, rc, err) : C2G_OK;
}

int c2g_guide_set_params(c2g_ctx* ctx, const float* params) {
    if (!params) return fail(ctx, C2G_ERR_INVALID, "null argument");
    int rc = guide_ready(ctx);
    if (rc) return rc;
    std::string err;
    rc = ctx->gpu->guide().set_params(params, err);
    return rc ? fail(ctx, rc, err) : C2G_OK;
}

int c2g_guide_get_params(c2g_ctx* ctx, float* params) {
    if (!params) return fail(ctx, C2G_ERR_INVALID, "null argument");
    int rc = guide_ready(ctx);
    if (rc) return rc;
    std::string err;
    rc = ctx->gpu->guide().get_params(params, err);
    return rc ? fail(ctx, rc, err) : C2G_OK;
}

int c2g_guide_eval(c2g_ctx* ctx, int n, const float* xnw, float* out) {
    if (n < 0 || (n > 0 && (!xnw || !out))) return fail(ctx, C2G_ERR_INVALID, "null argument");
    int rc = guide_ready(ctx);
    if (rc) return rc;
    std::string err;
    rc = ctx->gpu->guide().eval(*ctx->arena, xnw, n, out, err);
    return rc ? fail(ctx, rc, err) : C2G_OK;
}

int c2g_guide_gradient(c2g_ctx* ctx, int n, const float* samples, float* grad, double* loss) {
    if (n <= 0 || !samples || !grad) return fail(ctx, C2G_ERR_INVALID, "invalid argument");
    int rc = guide_ready(ctx);
    if (rc) return rc;
    std::string err;
    rc = ctx->gpu->guide().gradient(*ctx->arena, samples, n, grad, loss, err);
    return rc ? fail(ctx, rc, err) : C2G_OK;
}

int c2g_guide_stats(c2g_ctx* ctx, double* loss, int* records, int* steps) {
    int rc = guide_ready(ctx);
    if (rc) return rc;
    GuideStats g = ctx->gpu->guide_stats();
    if (loss) *loss = g.loss;
    if (records) *records = g.records;
    if (steps) *steps = g.steps;
    return C2G_OK;
}

int c2g_guide_config(c2g_ctx* ctx, float learning_rate, float bsdf_fraction, int warmup_waves, int train_steps) {
    if (!ctx) return C2G_ERR_INVALID;
    if (!(learning_rate > 0.f) || !(bsdf_fraction > 0.f && bsdf_fraction <= 1.f) || warmup_waves < 0 || train_steps < 0)
        return fail(ctx, C2G_ERR_INVALID, "invalid guide configuration");
    if (ctx->host_only) return fail(ctx, C2G_ERR_STATE, "host-only context");
    ctx->gpu->guide().set_learning_rate(learning_rate);
    ctx->gpu->guide().set_alpha(bsdf_fraction);
    ctx->gpu->set_guide_schedule(warmup_waves, train_steps);
    return C2G_OK;
}

}  // extern "C"
