// C ABI (include/c2g.h) over the host scene, the tree builders and the CUDA renderer.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
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
    ImageRegistry images;      // decoded images registered by path (textures, skybox faces)
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
    if (tree == C2G_TREE_SAH) {
        // leaves of at most two primitives: on the 2.05M-triangle 1080p scene 10.3 node visits and
        // 1.9 triangle tests per shadow ray against 9.9 and 3.0 with four, 2.8% faster per step
        build_sah_tree(*ctx->scene, ctx->sah, 2);
        collapse_bvh4(ctx->sah);
    }
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
        load_scene(*s, cfg, scn, &ctx->images);
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

int c2g_register_image(c2g_ctx* ctx, const char* path, int width, int height, const unsigned char* rgb8) {
    if (!ctx || !path || !rgb8 || width <= 0 || height <= 0) return fail(ctx, C2G_ERR_INVALID, "invalid image");
    Image im;
    im.width = width;
    im.height = height;
    im.rgb.assign(rgb8, rgb8 + (size_t)width * height * 3);
    ctx->images[path] = std::move(im);
    return C2G_OK;
}

int c2g_film_rgb8(c2g_ctx* ctx, float gamma, unsigned char* rgb8) {
    if (!ctx || !rgb8) return fail(ctx, C2G_ERR_INVALID, "null argument");
    if (!ctx->loaded) return fail(ctx, C2G_ERR_STATE, "no scene loaded");
    int W = ctx->scene->cfg.width, H = ctx->scene->cfg.height;
    std::vector<float> sum((size_t)W * H * 3), wgt((size_t)W * H);
    int rc = c2g_film_download(ctx, sum.data(), wgt.data());
    if (rc) return rc;
    // GetImageDataRGB8 (FrameBuffer.cpp:42-56): flipped rows, pow(mean, gamma), clamp to
    // [0, 0.999], floor(x * 256); a NaN mean (empty pixel) becomes 0
    for (int i = 0; i < H; i++)
        for (int j = 0; j < W; j++) {
            size_t orig = (size_t)(H - i - 1) * W + j, dest = (size_t)i * W + j;
            for (int k = 0; k < 3; k++) {
                float c = std::pow(sum[3 * orig + k] / wgt[orig], gamma);
                if (!(c == c)) c = 0.f;
                c = std::min(std::max(c, 0.f), 0.999f);
                rgb8[3 * dest + k] = (unsigned char)std::floor(c * 256);
            }
        }
    return C2G_OK;
}

// Radiance RGBE (Ward's shared-exponent pixels; the new-style run-length scanlines of the
// Radiance format): what stbi_write_hdr produces for RayTracer.cpp:40.
static void rgbe_pixel(const float* c, unsigned char* out) {
    const float r = std::max(c[0], 0.f), g = std::max(c[1], 0.f), b = std::max(c[2], 0.f);
    const float mx = std::max(r, std::max(g, b));
    if (!(mx >= 1e-32f)) { out[0] = out[1] = out[2] = out[3] = 0; return; }
    int e = 0;
    const float scale = (float)std::frexp(mx, &e) * 256.0f / mx;
    out[0] = (unsigned char)(r * scale);
    out[1] = (unsigned char)(g * scale);
    out[2] = (unsigned char)(b * scale);
    out[3] = (unsigned char)(e + 128);
}
// One channel of a scanline: runs of 4..127 equal bytes as (128 + n, byte), the rest as literal
// blocks of up to 128 bytes (n, bytes...).
static void rle_channel(const unsigned char* v, int n, std::string& out) {
    int i = 0;
    while (i < n) {
        int j = i;
        while (j < n && j - i < 127 && v[j] == v[i]) j++;
        if (j - i >= 4) {
            out.push_back((char)(unsigned char)(128 + (j - i)));
            out.push_back((char)v[i]);
            i = j;
            continue;
        }
        int k = i;
        while (k < n && k - i < 128) {
            int r = k;
            while (r < n && r - k < 4 && v[r] == v[k]) r++;
            if (r - k >= 4) break;
            k++;
        }
        out.push_back((char)(unsigned char)(k - i));
        out.append((const char*)v + i, (size_t)(k - i));
        i = k;
    }
}

int c2g_write_hdr(const char* path, int width, int height, const float* rgb) {
    if (!path || !rgb || width <= 0 || height <= 0) return C2G_ERR_INVALID;
    std::string buf = "#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y " + std::to_string(height) + " +X " +
                      std::to_string(width) + "\n";
    std::vector<unsigned char> px((size_t)width * 4), ch((size_t)width);
    for (int y = 0; y < height; y++) {
        for (int x = 0; x < width; x++) rgbe_pixel(rgb + 3 * ((size_t)y * width + x), &px[4 * (size_t)x]);
        if (width < 8 || width > 32767) {
            buf.append((const char*)px.data(), px.size());
            continue;
        }
        buf.push_back(2);
        buf.push_back(2);
        buf.push_back((char)(unsigned char)(width >> 8));
        buf.push_back((char)(unsigned char)(width & 255));
        for (int c = 0; c < 4; c++) {
            for (int x = 0; x < width; x++) ch[x] = px[4 * (size_t)x + c];
            rle_channel(ch.data(), width, buf);
        }
    }
    FILE* f = std::fopen(path, "wb");
    if (!f) return C2G_ERR_IO;
    const bool ok = std::fwrite(buf.data(), 1, buf.size(), f) == buf.size();
    return (std::fclose(f) == 0 && ok) ? C2G_OK : C2G_ERR_IO;
}

int c2g_film_write_hdr(c2g_ctx* ctx, const char* path) {
    if (!ctx || !path) return fail(ctx, C2G_ERR_INVALID, "null argument");
    if (!ctx->loaded) return fail(ctx, C2G_ERR_STATE, "no scene loaded");
    const int W = ctx->scene->cfg.width, H = ctx->scene->cfg.height;
    std::vector<float> img((size_t)W * H * 3);
    int rc = c2g_film_image(ctx, img.data());
    if (rc) return rc;
    rc = c2g_write_hdr(path, W, H, img.data());
    if (rc) return fail(ctx, rc, std::string("cannot write ") + path);
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

int c2g_set_traversal(c2g_ctx* ctx, int width) {
    if (!ctx) return C2G_ERR_INVALID;
    if (width != 2 && width != 4) return fail(ctx, C2G_ERR_INVALID, "traversal width is 2 or 4");
    ctx->gpu->set_sah_width(width);
    return C2G_OK;
}

int c2g_set_trace_block(c2g_ctx* ctx, int threads) {
    if (!ctx) return C2G_ERR_INVALID;
    if (threads != 64 && threads != 128 && threads != 256) return fail(ctx, C2G_ERR_INVALID, "trace block is 64, 128 or 256");
    if (ctx->host_only) return fail(ctx, C2G_ERR_STATE, "host-only context");
    ctx->gpu->set_trace_block(threads);
    return C2G_OK;
}

int c2g_probe_l2_read(int device, size_t bytes, int reps, double* gbs) {
    if (!gbs) return C2G_ERR_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return C2G_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return C2G_ERR_CUDA;
    std::string err;
    return c2g::probe_l2_read(bytes, reps, gbs, err);
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

int c2g_sampler_values(c2g_ctx* ctx, int n, const int* px, const int* py, const int* sample, int dim, int two_d,
                       float* out) {
    if (!ctx || n < 0 || dim < 0 || (n > 0 && (!px || !py || !sample || !out))) return fail(ctx, C2G_ERR_INVALID, "null argument");
    if (!ctx->loaded) return fail(ctx, C2G_ERR_STATE, "no scene loaded");
    int rc = set_device(ctx);
    if (rc) return rc;
    std::string err;
    rc = ctx->gpu->sampler_values(ctx->scene->cfg.width, n, px, py, sample, dim, two_d ? 1 : 0, out, *ctx->arena, err);
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

int c2g_guide_levels(c2g_ctx* ctx, int levels) {
    if (!ctx) return C2G_ERR_INVALID;
    if (levels < 0) return fail(ctx, C2G_ERR_INVALID, "levels >= 0");
    if (ctx->host_only) return fail(ctx, C2G_ERR_STATE, "host-only context");
    ctx->gpu->set_guide_levels(levels);
    return C2G_OK;
}

int c2g_guide_batch(c2g_ctx* ctx, int records_per_wave, int windows) {
    if (!ctx) return C2G_ERR_INVALID;
    if (records_per_wave < 1024 || windows < 1 || windows > 64) return fail(ctx, C2G_ERR_INVALID, "invalid training batch");
    if (ctx->host_only) return fail(ctx, C2G_ERR_STATE, "host-only context");
    ctx->gpu->guide().set_batch(records_per_wave, windows);
    return C2G_OK;
}

int c2g_guide_regularize(c2g_ctx* ctx, float kappa_max, float weight_clamp, float decay_steps) {
    if (!ctx) return C2G_ERR_INVALID;
    if (!(kappa_max >= 1.f && kappa_max <= c2g::kGuideKappaMax) || !(weight_clamp >= 1.f) || !(decay_steps >= 0.f))
        return fail(ctx, C2G_ERR_INVALID, "kappa_max in [1, 500], weight_clamp >= 1, decay_steps >= 0");
    if (ctx->host_only) return fail(ctx, C2G_ERR_STATE, "host-only context");
    ctx->gpu->guide().set_regularisation(kappa_max, weight_clamp, decay_steps);
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

// ---- batched multi-job rendering ---------------------------------------------------------------
namespace {
struct BatchJob {
    c2g_ctx* ctx = nullptr;
    c2g_render_params p{};
    cudaGraphExec_t g_warm = nullptr;  // guided: waves that only train (mixture not used yet)
    cudaGraphExec_t g_main = nullptr;
    int spw = 0, waves = 0, warm_waves = 0;
    int stream = 0;
    cudaEvent_t done = nullptr;
    double latency_ms = 0.0;
    double paths() const { return (double)p.width * p.height * p.sample_count; }
};
}  // namespace

struct c2g_batch {
    int device = 0;
    std::vector<BatchJob> jobs;
    std::vector<cudaStream_t> streams;
    int wave_paths = 1 << 20;
    int n_streams = 0;          // 0: every job in one graph launch; > 0: per-job graphs on this many streams
    int lanes = 8;              // one-launch mode: chains of jobs that run side by side (0: every job alone)
    int traversal = 4;          // SAH node width of every job's traversal
    int trace_block = 128;      // threads per block of the traversal kernels
    int captured_wave_paths = -1;
    std::string last_error;
};

namespace {
int bfail(c2g_batch* b, int code, const std::string& msg) {
    if (b) b->last_error = msg;
    return code;
}

void drop_graphs(BatchJob& j) {
    if (j.g_warm) cudaGraphExecDestroy(j.g_warm);
    if (j.g_main) cudaGraphExecDestroy(j.g_main);
    j.g_warm = j.g_main = nullptr;
}

// The batch's traversal variant and block size on every job's context (taken by the next capture).
void batch_apply_trace(c2g_batch* b) {
    for (BatchJob& j : b->jobs) {
        j.ctx->gpu->set_sah_width(b->traversal);
        j.ctx->gpu->set_trace_block(b->trace_block);
    }
}

// Capture every job's wave graphs for the batch's wave size.
int batch_capture(c2g_batch* b) {
    if (b->captured_wave_paths == b->wave_paths) return C2G_OK;
    batch_apply_trace(b);
    cudaStream_t st = b->streams.empty() ? nullptr : b->streams[0];
    for (size_t i = 0; i < b->jobs.size(); i++) {
        BatchJob& j = b->jobs[i];
        drop_graphs(j);
        const int nslots = ((j.p.width + 7) / 8) * ((j.p.height + 7) / 8) * 64;
        // samples per wave: as many as the wave size holds, dividing the job's sample count
        int spw = std::max(1, std::min(j.p.sample_count, b->wave_paths / nslots));
        while (j.p.sample_count % spw) spw--;
        c2g_render_params q = j.p;
        q.wave_paths = spw * nslots;
        std::string err;
        int got = 0;
        const bool guided = q.integrator == C2G_INTEGRATOR_GUIDED;
        // g_main: the guided integrator samples its mixture; g_warm: its first waves only train
        int rc = j.ctx->gpu->capture_wave(q, true, st, *j.ctx->arena, &j.g_main, &got, err);
        if (!rc && guided) rc = j.ctx->gpu->capture_wave(q, false, st, *j.ctx->arena, &j.g_warm, &got, err);
        if (rc) return bfail(b, rc, "job " + std::to_string(i) + ": " + err);
        j.spw = got;
        j.waves = j.p.sample_count / got;
        j.warm_waves = guided ? std::min(j.waves, j.ctx->gpu->guide_warmup()) : 0;
    }
    b->captured_wave_paths = b->wave_paths;
    return C2G_OK;
}

int batch_streams(c2g_batch* b) {
    while ((int)b->streams.size() < b->n_streams) {
        cudaStream_t st;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return bfail(b, C2G_ERR_CUDA, "stream creation failed");
        b->streams.push_back(st);
    }
    return C2G_OK;
}

void fill_stats(c2g_batch* b, std::vector<double> lat, double paths, float total_ms, int launches, c2g_batch_stats* out) {
    if (!out) return;
    std::sort(lat.begin(), lat.end());
    auto pct = [&](double q) {
        if (lat.empty()) return 0.0;
        size_t i = (size_t)std::min<double>((double)lat.size() - 1, std::ceil(q * lat.size()) - 1);
        return lat[i];
    };
    double mean = 0.0;
    for (double v : lat) mean += v;
    *out = c2g_batch_stats{};
    out->jobs = (int)b->jobs.size();
    out->paths = paths;
    out->seconds = total_ms * 1e-3;
    out->mpaths_per_s = total_ms > 0 ? paths / (total_ms * 1e-3) / 1e6 : 0.0;
    out->latency_p50_ms = pct(0.5);
    out->latency_p90_ms = pct(0.9);
    out->latency_p99_ms = pct(0.99);
    out->latency_max_ms = lat.empty() ? 0.0 : lat.back();
    out->latency_mean_ms = lat.empty() ? 0.0 : mean / lat.size();
    out->wave_paths = b->wave_paths;
    out->streams = b->n_streams;
    out->graph_launches = launches;
    out->traversal = b->traversal;
    out->trace_block = b->trace_block;
}

// Longest job first onto the least-loaded of n queues, shortest first within a queue (the order of
// the streams mode and of the one-launch mode's lanes).
std::vector<std::vector<int>> batch_queues(c2g_batch* b, int n) {
    std::vector<int> order(b->jobs.size());
    for (size_t i = 0; i < order.size(); i++) order[i] = (int)i;
    std::sort(order.begin(), order.end(), [&](int x, int y) { return b->jobs[x].paths() > b->jobs[y].paths(); });
    std::vector<double> load(n, 0.0);
    std::vector<std::vector<int>> per(n);
    for (int i : order) {
        int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        load[k] += b->jobs[i].paths();
        per[k].push_back(i);
    }
    for (auto& v : per) std::reverse(v.begin(), v.end());
    return per;
}

// Every job in one graph: per job a chain (sample counter reset, device-side while loops over its
// waves, completion event); the jobs of a lane follow each other (shortest first), the lanes run
// side by side (lanes = 0: every job on its own), so one cudaGraphLaunch renders the whole batch
// and the GPU interleaves the lanes' kernels.  `spp_limit` caps every job's samples.
int batch_pass_graph(c2g_batch* b, int spp_limit, c2g_batch_stats* out) {
    if (cudaSetDevice(b->device) != cudaSuccess) return bfail(b, C2G_ERR_CUDA, "cudaSetDevice failed");
    if (cudaDeviceSynchronize() != cudaSuccess) return bfail(b, C2G_ERR_CUDA, "device error before the batch");
    if (b->streams.empty()) {
        cudaStream_t st;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return bfail(b, C2G_ERR_CUDA, "stream creation failed");
        b->streams.push_back(st);
    }
    cudaStream_t st = b->streams[0];
    batch_apply_trace(b);
    cudaGraph_t G = nullptr;
    if (cudaGraphCreate(&G, 0) != cudaSuccess) return bfail(b, C2G_ERR_CUDA, "graph creation failed");
    double paths = 0.0;
    int rc = C2G_OK;
    std::vector<std::vector<int>> lanes;
    if (b->lanes > 0) lanes = batch_queues(b, std::min<int>(b->lanes, (int)b->jobs.size()));
    else
        for (size_t i = 0; i < b->jobs.size(); i++) lanes.push_back({(int)i});
    for (const auto& lane : lanes) {
        cudaGraphNode_t prev = nullptr;
        for (int i : lane) {
            BatchJob& j = b->jobs[i];
            if (!j.done) cudaEventCreate(&j.done);
            c2g_render_params q = j.p;
            if (spp_limit > 0) q.sample_count = std::max(1, std::min(q.sample_count, spp_limit));
            std::string err;
            int spw = 0, waves = 0;
            rc = j.ctx->gpu->append_job(G, prev ? &prev : nullptr, prev ? 1 : 0, q, b->wave_paths, j.done, st, *j.ctx->arena,
                                        &prev, &spw, &waves, err);
            if (rc) {
                bfail(b, rc, "job " + std::to_string(i) + ": " + err);
                break;
            }
            j.spw = spw;
            j.waves = waves;
            paths += (double)q.width * q.height * q.sample_count;
        }
        if (rc) break;
    }
    cudaGraphExec_t exec = nullptr;
    if (!rc) {
        cudaError_t e = cudaGraphInstantiate(&exec, G, 0);
        if (e != cudaSuccess) rc = bfail(b, C2G_ERR_CUDA, std::string("batch graph instantiation: ") + cudaGetErrorString(e));
    }
    cudaGraphDestroy(G);
    if (rc) return rc;
    cudaEvent_t start, stop;
    cudaEventCreate(&start);
    cudaEventCreate(&stop);
    cudaEventRecord(start, st);
    cudaError_t e = cudaGraphLaunch(exec, st);
    cudaEventRecord(stop, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(stop);
    cudaGraphExecDestroy(exec);
    if (e != cudaSuccess) {
        cudaEventDestroy(start);
        cudaEventDestroy(stop);
        return bfail(b, C2G_ERR_CUDA, std::string("batch: ") + cudaGetErrorString(e));
    }
    float total = 0.f;
    cudaEventElapsedTime(&total, start, stop);
    std::vector<double> lat;
    for (BatchJob& j : b->jobs) {
        float t = 0.f;
        cudaEventElapsedTime(&t, start, j.done);
        j.latency_ms = t;
        lat.push_back(t);
    }
    cudaEventDestroy(start);
    cudaEventDestroy(stop);
    for (BatchJob& j : b->jobs) {
        std::string err;
        rc = j.ctx->gpu->check_device_error(err);
        if (rc) return bfail(b, rc, err);
    }
    fill_stats(b, lat, paths, total, 1, out);
    return C2G_OK;
}

// One pass over every job, `spp_limit` samples each (0 = the job's own count).
int batch_pass(c2g_batch* b, int spp_limit, c2g_batch_stats* out) {
    if (b->n_streams == 0) return batch_pass_graph(b, spp_limit, out);
    if (cudaSetDevice(b->device) != cudaSuccess) return bfail(b, C2G_ERR_CUDA, "cudaSetDevice failed");
    // work the jobs' contexts queued on their own streams (film clears, renders) comes first
    if (cudaDeviceSynchronize() != cudaSuccess) return bfail(b, C2G_ERR_CUDA, "device error before the batch");
    int rc = batch_streams(b);
    if (rc) return rc;
    rc = batch_capture(b);
    if (rc) return rc;
    const int ns = b->n_streams;
    // longest job first onto the least-loaded stream; shortest first within a stream
    std::vector<std::vector<int>> per = batch_queues(b, ns);
    for (BatchJob& j : b->jobs) {
        std::string err;
        rc = j.ctx->gpu->set_wave_counter(j.p.sample_begin, b->streams[0], *j.ctx->arena, err);
        if (rc) return bfail(b, rc, err);
        if (!j.done) cudaEventCreate(&j.done);
    }
    cudaEvent_t start, stop;
    cudaEventCreate(&start);
    cudaEventCreate(&stop);
    cudaEventRecord(start, b->streams[0]);
    for (int k = 1; k < ns; k++) cudaStreamWaitEvent(b->streams[k], start, 0);
    int launches = 0;
    double paths = 0.0;
    // enqueue wave by wave across the streams so that no stream's host-side queue runs far ahead
    std::vector<size_t> next_job(ns, 0);
    std::vector<int> next_wave(ns, 0);
    bool any = true;
    while (any) {
        any = false;
        for (int k = 0; k < ns; k++) {
            if (next_job[k] >= per[k].size()) continue;
            any = true;
            BatchJob& j = b->jobs[per[k][next_job[k]]];
            const int waves = spp_limit > 0 ? std::max(1, std::min(j.waves, spp_limit / std::max(1, j.spw))) : j.waves;
            const int w = next_wave[k];
            cudaGraphExec_t g = (w < j.warm_waves && j.g_warm) ? j.g_warm : j.g_main;
            if (cudaGraphLaunch(g, b->streams[k]) != cudaSuccess) return bfail(b, C2G_ERR_CUDA, "graph launch failed");
            launches++;
            if (w + 1 >= waves) {
                cudaEventRecord(j.done, b->streams[k]);
                paths += (double)j.p.width * j.p.height * waves * j.spw;
                next_job[k]++;
                next_wave[k] = 0;
            } else {
                next_wave[k] = w + 1;
            }
        }
    }
    for (int k = 0; k < ns; k++) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        cudaEventRecord(e, b->streams[k]);
        cudaStreamWaitEvent(b->streams[0], e, 0);
        cudaEventDestroy(e);
    }
    cudaEventRecord(stop, b->streams[0]);
    cudaError_t e = cudaEventSynchronize(stop);
    if (e != cudaSuccess) return bfail(b, C2G_ERR_CUDA, std::string("batch: ") + cudaGetErrorString(e));
    float total = 0.f;
    cudaEventElapsedTime(&total, start, stop);
    std::vector<double> lat;
    for (BatchJob& j : b->jobs) {
        float t = 0.f;
        cudaEventElapsedTime(&t, start, j.done);
        j.latency_ms = t;
        lat.push_back(t);
    }
    cudaEventDestroy(start);
    cudaEventDestroy(stop);
    for (BatchJob& j : b->jobs) {
        std::string err;
        rc = j.ctx->gpu->check_device_error(err);
        if (rc) return bfail(b, rc, err);
    }
    fill_stats(b, lat, paths, total, launches, out);
    return C2G_OK;
}
}  // namespace

extern "C" {

int c2g_batch_create(c2g_batch** out, int device) {
    if (!out) return C2G_ERR_INVALID;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return C2G_ERR_DEVICE;
    c2g_batch* b = new c2g_batch();
    b->device = device;
    *out = b;
    return C2G_OK;
}

void c2g_batch_destroy(c2g_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    for (BatchJob& j : b->jobs) {
        drop_graphs(j);
        if (j.done) cudaEventDestroy(j.done);
    }
    for (cudaStream_t st : b->streams) cudaStreamDestroy(st);
    delete b;
}

const char* c2g_batch_last_error(c2g_batch* b) { return b ? b->last_error.c_str() : "null batch"; }

int c2g_batch_add(c2g_batch* b, c2g_ctx* job, const c2g_render_params* params, int* index) {
    if (!b || !job || !params) return bfail(b, C2G_ERR_INVALID, "null argument");
    if (!job->loaded || job->device != b->device) return bfail(b, C2G_ERR_STATE, "job context has no scene on the batch's device");
    if (params->sample_count <= 0) return bfail(b, C2G_ERR_INVALID, "a job renders at least one sample");
    for (const BatchJob& j : b->jobs)
        if (j.ctx == job) return bfail(b, C2G_ERR_INVALID, "context already in the batch");
    BatchJob j;
    j.ctx = job;
    j.p = *params;
    b->jobs.push_back(j);
    b->captured_wave_paths = -1;
    if (index) *index = (int)b->jobs.size() - 1;
    return C2G_OK;
}

int c2g_batch_tune(c2g_batch* b, int wave_paths, int streams) {
    if (!b) return C2G_ERR_INVALID;
    if (wave_paths < 64 || streams < 0 || streams > 32) return bfail(b, C2G_ERR_INVALID, "wave_paths >= 64 and 0 <= streams <= 32");
    if (wave_paths != b->wave_paths) b->captured_wave_paths = -1;
    b->wave_paths = wave_paths;
    b->n_streams = streams;
    return C2G_OK;
}

int c2g_batch_autotune(c2g_batch* b, const int* wave_paths, int n_wave_paths, const int* streams, int n_streams,
                       int trial_spp, double* best_mpaths_per_s) {
    if (!b || !wave_paths || !streams || n_wave_paths <= 0 || n_streams <= 0 || trial_spp <= 0) return bfail(b, C2G_ERR_INVALID, "invalid candidates");
    double best = -1.0;
    int bw = b->wave_paths, bs = b->n_streams;
    for (int i = 0; i < n_wave_paths; i++)
        for (int k = 0; k < n_streams; k++) {
            int rc = c2g_batch_tune(b, wave_paths[i], streams[k]);
            if (rc) return rc;
            c2g_batch_stats st{};
            rc = batch_pass(b, trial_spp, &st);
            if (rc) return rc;
            if (st.mpaths_per_s > best) { best = st.mpaths_per_s; bw = wave_paths[i]; bs = streams[k]; }
        }
    // trials leave samples in the films and train the networks: start the real run clean
    for (BatchJob& j : b->jobs) {
        drop_graphs(j);
        j.ctx->gpu->guide().release(*j.ctx->arena);
        j.ctx->gpu->film_clear(nullptr);
    }
    b->captured_wave_paths = -1;
    c2g_batch_tune(b, bw, bs);
    if (best_mpaths_per_s) *best_mpaths_per_s = best;
    return cudaDeviceSynchronize() == cudaSuccess ? C2G_OK : bfail(b, C2G_ERR_CUDA, "autotune");
}

int c2g_batch_set_trace(c2g_batch* b, int traversal, int trace_block) {
    if (!b) return C2G_ERR_INVALID;
    if ((traversal != 2 && traversal != 4) || (trace_block != 64 && trace_block != 128 && trace_block != 256))
        return bfail(b, C2G_ERR_INVALID, "traversal 2 or 4, trace_block 64, 128 or 256");
    if (traversal != b->traversal || trace_block != b->trace_block) b->captured_wave_paths = -1;
    b->traversal = traversal;
    b->trace_block = trace_block;
    return C2G_OK;
}

int c2g_batch_set_lanes(c2g_batch* b, int lanes) {
    if (!b) return C2G_ERR_INVALID;
    if (lanes < 0 || lanes > 256) return bfail(b, C2G_ERR_INVALID, "0 <= lanes <= 256");
    b->lanes = lanes;
    return C2G_OK;
}

int c2g_batch_search(c2g_batch* b, const c2g_batch_space* space, int trial_spp, double* best_mpaths_per_s) {
    if (!b || !space || trial_spp <= 0) return bfail(b, C2G_ERR_INVALID, "invalid search");
    if (b->jobs.empty()) return bfail(b, C2G_ERR_STATE, "empty batch");
    auto bad = [](const int* v, int n) { return n < 0 || (n > 0 && !v); };
    if (bad(space->wave_paths, space->n_wave_paths) || bad(space->streams, space->n_streams) ||
        bad(space->traversal, space->n_traversal) || bad(space->trace_block, space->n_trace_block))
        return bfail(b, C2G_ERR_INVALID, "candidate list without values");
    struct Cfg { int wave, streams, trav, block; };
    Cfg cur{b->wave_paths, b->n_streams, b->traversal, b->trace_block};
    auto apply = [&](const Cfg& c) {
        int rc = c2g_batch_tune(b, c.wave, c.streams);
        return rc ? rc : c2g_batch_set_trace(b, c.trav, c.block);
    };
    double best = -1.0;
    // a candidate whose wave buffers do not fit next to the other jobs' is infeasible: its trial
    // ends with C2G_ERR_OOM, every job's wave buffers are released and the search goes on
    auto trial = [&](const Cfg& c, double* rate) {
        int rc = apply(c);
        if (rc) return rc;
        c2g_batch_stats st{};
        rc = batch_pass(b, trial_spp, &st);
        if (rc == C2G_ERR_OOM) {
            for (BatchJob& j : b->jobs) {
                drop_graphs(j);
                j.ctx->gpu->release_wave_buffers(*j.ctx->arena);
                j.ctx->gpu->guide().release(*j.ctx->arena);  // its per-slot buffers follow the wave size
            }
            b->captured_wave_paths = -1;
            *rate = -1.0;
            return C2G_OK;
        }
        if (rc) return rc;
        *rate = st.mpaths_per_s;
        return C2G_OK;
    };
    int rc = trial(cur, &best);
    if (rc) return rc;
    const int* lists[4] = {space->wave_paths, space->streams, space->traversal, space->trace_block};
    const int counts[4] = {space->n_wave_paths, space->n_streams, space->n_traversal, space->n_trace_block};
    for (int dim = 0; dim < 4; dim++) {
        for (int i = 0; i < counts[dim]; i++) {
            Cfg c = cur;
            int* field = dim == 0 ? &c.wave : dim == 1 ? &c.streams : dim == 2 ? &c.trav : &c.block;
            if (*field == lists[dim][i]) continue;
            *field = lists[dim][i];
            double r = 0.0;
            rc = trial(c, &r);
            if (rc) return rc;
            if (r > best) { best = r; cur = c; }
        }
    }
    // trials leave samples in the films and train the networks: start the real run clean
    for (BatchJob& j : b->jobs) {
        drop_graphs(j);
        j.ctx->gpu->guide().release(*j.ctx->arena);
        j.ctx->gpu->film_clear(nullptr);
    }
    b->captured_wave_paths = -1;
    rc = apply(cur);
    if (rc) return rc;
    if (best_mpaths_per_s) *best_mpaths_per_s = best;
    return cudaDeviceSynchronize() == cudaSuccess ? C2G_OK : bfail(b, C2G_ERR_CUDA, "search");
}

int c2g_batch_run(c2g_batch* b, c2g_batch_stats* stats) {
    if (!b) return C2G_ERR_INVALID;
    if (b->jobs.empty()) return bfail(b, C2G_ERR_STATE, "empty batch");
    return batch_pass(b, 0, stats);
}

int c2g_batch_job_latency(c2g_batch* b, int i, double* ms) {
    if (!b || !ms || i < 0 || i >= (int)b->jobs.size()) return bfail(b, C2G_ERR_INVALID, "bad job index");
    *ms = b->jobs[i].latency_ms;
    return C2G_OK;
}

}  // extern "C"
