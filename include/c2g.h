/*
 * c2g.h - C ABI of the GB300 path-tracing hot path for Crystal2.
 *
 * The library replaces the subtree under crystal::Integrator::Render(Scene*, Camera*, FrameBuffer*)
 * (src/Integrators/Integrator.h:8-18) of the reference renderer: the per-sample loop of
 * SamplerIntegrator::Render (src/Integrators/SamplerIntegrator.cpp:17-72), the MIS path tracer
 * PathTracingIntegrator::Evaluate (src/Integrators/PathTracingIntegrator.cpp:28-278), BVH traversal
 * (src/Accelerators/BVH.cpp:56-154), shape intersection (src/Shapes/*.cpp), BSDF sampling and
 * evaluation (src/BSDFs/**), light sampling (src/Lights/*.cpp) and film accumulation
 * (src/Core/FrameBuffer.cpp:20-32).
 *
 * Conventions
 *  - Every entry point returns an int status (C2G_OK == 0); no C++ exception crosses the ABI.
 *    c2g_last_error() gives the message of the last failure on that context.
 *  - The context owns all device memory. Caller buffers are borrowed for the duration of a call.
 *  - Arrays are plain host pointers unless a name says `_dev` (device pointers, e.g. from
 *    cudaMalloc or torch). Streams are `cudaStream_t` passed as void* (NULL = the context stream).
 *  - One context per host thread; different contexts may be used concurrently.
 */
#ifndef C2G_H
#define C2G_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------------- */
#define C2G_OK 0
#define C2G_ERR_INVALID 1   /* bad argument (std::invalid_argument in the reference factories) */
#define C2G_ERR_IO 2        /* file missing or unreadable (JsonLoader.cpp:6-58, ObjLoader.cpp:96-116) */
#define C2G_ERR_PARSE 3     /* malformed JSON / OBJ (SJson ParseError family) */
#define C2G_ERR_CUDA 4      /* a CUDA runtime call failed */
#define C2G_ERR_OOM 5       /* device allocation failed or exceeded the context's memory cap */
#define C2G_ERR_DEVICE 6    /* a kernel reported an error word (stack/queue overflow, bounded-wait timeout) */
#define C2G_ERR_STATE 7     /* call out of order (e.g. render before a scene is loaded) */
#define C2G_ERR_UNSUPPORTED 8 /* feature the reference has but this library leaves out (textures, skybox) */

/* ---- enumerations ------------------------------------------------------------------------ */
/* Accelerator semantics (the reference's "Acceleration" key, Accelerator.cpp:6-25). */
#define C2G_ACCEL_BVH 0     /* BVH semantics: per-object box test; shadow test clipped to the object box (BVH.cpp:110-154) */
#define C2G_ACCEL_BRUTE 1   /* Brute semantics: no box tests; shadow test over [tMin, tMax] (Brute.cpp:19-55) */

/* Tree actually traversed on the GPU (either gives BVH semantics). */
#define C2G_TREE_REF_EQUAL_COUNT 0  /* bit-exact replica of BVH::_build with equal-count splits (BVH.cpp:156-188,269-279) */
#define C2G_TREE_SAH 1              /* binned-SAH tree, compact node layout (performance) */

/* Integrators (the reference's Integrator.Type, Integrator.cpp:14-47). */
#define C2G_INTEGRATOR_PATH 0    /* "PathTracer" */
#define C2G_INTEGRATOR_DIRECT 1  /* "DirectLight" */
#define C2G_INTEGRATOR_GUIDED 2  /* "GuidedPathTracer": path tracer plus the learned directional proposal */

/* Shape kinds of c2g_trace_rays outputs / scene objects. */
#define C2G_SHAPE_TRIANGLE 0
#define C2G_SHAPE_SPHERE 1
#define C2G_SHAPE_DISK 2

/* ---- plain structs ----------------------------------------------------------------------- */
typedef struct c2g_ctx c2g_ctx;

typedef struct {
    int device;                 /* CUDA device ordinal; -1 = host-only context (scene parsing and tree
                                   builds only; every device call returns C2G_ERR_STATE) */
    size_t mem_limit_bytes;     /* 0 = no cap; else allocations beyond this fail with C2G_ERR_OOM */
    int verbose;                /* print timings to stderr */
} c2g_device_opts;

typedef struct {
    int width, height;          /* film size (ConfigInfo.Width/Height) */
    int spp;                    /* samples per pixel (ConfigInfo.SamplesPerPixel) */
    int max_depth;              /* Integrator.Depth */
    int integrator;             /* C2G_INTEGRATOR_* */
    int accel;                  /* C2G_ACCEL_* */
    int sample_begin;           /* first sample index rendered by this call (progressive rendering) */
    int sample_count;           /* number of samples rendered by this call (<= spp - sample_begin) */
    int wave_paths;             /* paths in flight per wave (0 = automatic) */
    uint64_t seed;              /* seed of the hash RNG used for Halton dims >= 100 */
} c2g_render_params;

/* Kernel kinds of c2g_stats arrays. */
#define C2G_K_RAYGEN 0
#define C2G_K_EXTEND 1
#define C2G_K_SHADE 2
#define C2G_K_SHADOW 3
#define C2G_K_MIS 4
#define C2G_K_ACCUM 5
#define C2G_K_FILM 6
#define C2G_K_GUIDE 7   /* guide network inference */
#define C2G_K_TRAIN 8   /* guide training: batch build, fused forward/backward, Adam */
#define C2G_K_KINDS 10  /* size of the per-kind arrays */

/* Counting / timing switches of c2g_set_counting. */
#define C2G_COUNT_TRAVERSAL 1  /* rays, nodes visited and prims tested per traversal kernel */
#define C2G_COUNT_TIMING 2     /* CUDA events around every launch; per-kind device time */
#define C2G_COUNT_SERIAL 4     /* one stream: no side or look-ahead stream, so per-kind times are exclusive */

#define C2G_LEVELS 64  /* size of the per-bounce-level arrays (deeper levels add to the last entry) */

typedef struct {
    double seconds;             /* device time of the last c2g_render (CUDA events on its stream) */
    double paths;               /* camera paths traced by the last c2g_render */
    double rays[C2G_K_KINDS];             /* rays processed per kernel kind (C2G_COUNT_TRAVERSAL) */
    double nodes[C2G_K_KINDS];            /* BVH nodes visited per kernel kind (C2G_COUNT_TRAVERSAL) */
    double prims[C2G_K_KINDS];            /* primitives tested per kernel kind (C2G_COUNT_TRAVERSAL) */
    double kernel_ms[C2G_K_KINDS];        /* device time per kernel kind (C2G_COUNT_TIMING) */
    int kernel_count[C2G_K_KINDS];        /* launches per kernel kind */
    int kernel_launches;        /* kernels launched by the last c2g_render */
    int waves;                  /* waves of the last c2g_render */
    double level_ms[C2G_LEVELS];    /* device time per bounce level, summed over waves (C2G_COUNT_TIMING) */
    double level_paths[C2G_LEVELS]; /* paths entering each bounce level, summed over waves (C2G_COUNT_TRAVERSAL) */
    int levels;                 /* bounce levels run by the deepest wave */
} c2g_stats;

/* ---- lifecycle ------------------------------------------------------------------------------ */
int c2g_create(c2g_ctx** out, const c2g_device_opts* opts);
void c2g_destroy(c2g_ctx* ctx);
const char* c2g_last_error(const c2g_ctx* ctx);
const char* c2g_version(void);

/* ---- scene ---------------------------------------------------------------------------------- */
/* Load the reference's two JSON files (config + scene) exactly as RayTracer's constructor does
 * (src/Core/RayTracer.cpp:11-22): ConfigLoader keys, Scene::CreateScene (Scene.cpp:23-45),
 * Camera::CreateCamera (Camera.cpp:7-22), Integrator/Sampler factories. The tree is built with
 * `tree` (C2G_TREE_*). Relative OBJ paths resolve against the current directory, as fopen does
 * in ObjLoader::load (ObjLoader.cpp:96-116). */
int c2g_load_json(c2g_ctx* ctx, const char* config_path, const char* scene_path, int tree);
/* Same, from in-memory JSON text. */
int c2g_load_json_text(c2g_ctx* ctx, const char* config_json, const char* scene_json, int tree);
/* Register a decoded 8-bit RGB image (width x height x 3 bytes, row 0 = the file's first row) under
 * a path: scene textures ("Textures": {name: {"Path": ...}}) and skybox faces (<Path>/posx.jpg ...)
 * with that path use it instead of reading the file.  Stands in for the reference's stb_image
 * decode (Texel.cpp:4-13); the library itself reads binary PPM files.  Register before loading. */
int c2g_register_image(c2g_ctx* ctx, const char* path, int width, int height, const unsigned char* rgb8);
/* Rebuild the acceleration structure of the loaded scene (BVH::Build, BVH.cpp:45-54). */
int c2g_bvh_build(c2g_ctx* ctx, int tree);
/* Render parameters implied by the loaded config (Width, Height, SamplesPerPixel, Depth ...). */
int c2g_get_render_params(c2g_ctx* ctx, c2g_render_params* out);
int c2g_num_objects(c2g_ctx* ctx);
int c2g_num_lights(c2g_ctx* ctx);
/* Object order after the reference equal-count build (BVH::_objects), as scene indices. */
int c2g_bvh_order(c2g_ctx* ctx, int* order, int n);
/* Reference-tree nodes 1..n (n returned): bounds (6 floats), ch0/ch1 or start/count, axis (-1 leaf). */
int c2g_bvh_nodes(c2g_ctx* ctx, float* bounds, int* a, int* axis, int cap);

/* ---- rendering ------------------------------------------------------------------------------ */
/* Integrator::Render: trace samples [sample_begin, sample_begin + sample_count) of every pixel
 * and add them to the device film (FrameBuffer::AddSample semantics: NaN/Inf -> 0, weight 1). */
int c2g_render(c2g_ctx* ctx, const c2g_render_params* params, void* stream);
int c2g_film_clear(c2g_ctx* ctx, void* stream);
/* Per-pixel sums and weights, row y = sample-loop pixel y (not flipped). Either may be NULL. */
int c2g_film_download(c2g_ctx* ctx, float* rgb_sum, float* weight);
/* FrameBuffer::GetImageDataRGB32F (FrameBuffer.cpp:58-75): sum/weight, rows flipped. */
int c2g_film_image(c2g_ctx* ctx, float* rgb);
/* GetImageDataRGB8(gamma) (FrameBuffer.cpp:42-56): rows flipped like c2g_film_image, each channel
 * pow(mean, gamma) clamped to [0, 0.999] and scaled by 256; 3 bytes per pixel. */
int c2g_film_rgb8(c2g_ctx* ctx, float gamma, unsigned char* rgb8);
/* Radiance RGBE file of the film image (GetImageDataRGB32F order), the output RayTracer.cpp:40
 * writes with stbi_write_hdr: "-Y H +X W" header, run-length-encoded scanlines for widths
 * 8..32767, flat RGBE otherwise. */
int c2g_film_write_hdr(c2g_ctx* ctx, const char* path);
/* The same writer on caller data: rgb = height x width x 3 floats, row 0 written first.  Needs no
 * context or device; negative components are written as 0. */
int c2g_write_hdr(const char* path, int width, int height, const float* rgb);
/* Per-pixel sum of squares of the samples (variance estimates for parity tests). */
int c2g_film_download_m2(c2g_ctx* ctx, float* rgb_sumsq);
int c2g_get_stats(c2g_ctx* ctx, c2g_stats* out);
/* Allocation-free variant of c2g_render, for callers that cannot call cudaMalloc while they render
 * (an application that hands plug-ins no allocation rights and owns device memory through its own
 * pool, or a frame loop that must avoid cudaMalloc's implicit synchronisation).  No counterpart in
 * the reference.  It renders the same samples with the same kernels as c2g_render, but its working
 * memory is a static device array inside the library (about 14 MB, held by every GPU that loads the
 * library until the process exits) and the result is added to `film_dev`: caller-owned device
 * memory of width x height float4 (rgb sum, weight), in c2g_film_download's layout, which the
 * caller clears.  Limits: at most 16384 pixel slots (width and height rounded up to multiples of 8;
 * e.g. 128 x 128) and at most 8 lights; larger requests fail with C2G_ERR_INVALID.  The first call
 * on a device sets up the array's address and should come before any stream capture.  Calls share
 * the array: calls that overlap on the GPU race.  The call synchronises `stream` before returning. */
int c2g_render_noalloc(c2g_ctx* ctx, const c2g_render_params* params, float* film_dev, void* stream);
/* C2G_COUNT_* flags (0 = off): traversal counters (slower kernels) and per-launch timing. */
int c2g_set_counting(c2g_ctx* ctx, int flags);
/* SAH-tree traversal variant: 2 (binary nodes) or 4 (four-wide nodes, the default).  Both visit the
 * same leaves; no counterpart in the reference (its BVH is binary). */
int c2g_set_traversal(c2g_ctx* ctx, int width);
/* Threads per block of the traversal kernels (64, 128 or 256; default 128); no counterpart in the
 * reference. */
int c2g_set_trace_block(c2g_ctx* ctx, int threads);

/* L2 read bandwidth of `device` in GB/s: a `bytes` buffer (keep it well below the L2 size) read
 * `reps` times by every SM with L2-only loads, timed with CUDA events.  No counterpart in the
 * reference; it is the measured L2 roof beside which the traversal kernels' bandwidth is reported. */
int c2g_probe_l2_read(int device, size_t bytes, int reps, double* gbs);

/* ---- batched multi-job rendering ---------------------------------------------------------------
 * No counterpart in the reference (one scene per RayTracer).  A batch renders many jobs - each a
 * context with its own loaded scene and its own render parameters (path tracer or guided) - on one
 * GPU, and the films land in each job's context (c2g_film_download).  Two modes:
 *  - streams = 0 (default): the whole batch is one CUDA graph launched once; per job a chain of a
 *    sample-counter reset, device-side while loops (conditional graph nodes) that run the job's
 *    waves one after another, and a completion event; the jobs are spread over `lanes` chains
 *    (longest-first onto the least-loaded lane, shortest-first within a lane; default 8,
 *    c2g_batch_set_lanes) that the GPU runs side by side;
 *  - streams = S > 0: every job's wave is captured as its own graph that replays wave after wave,
 *    jobs spread over S concurrent streams (longest-first onto the least-loaded stream,
 *    shortest-first within a stream).
 * The wave size, the mode, the traversal variant and the traversal kernels' block size come from
 * c2g_batch_tune / c2g_batch_set_trace or the autotuners.  Jobs' contexts must live as long as the
 * batch; a context belongs to at most one batch. */
typedef struct c2g_batch c2g_batch;
typedef struct c2g_batch_stats {
    int jobs;
    double paths;               /* camera paths rendered by the run */
    double seconds;             /* device time from the first launch to the last job's end */
    double mpaths_per_s;
    double latency_p50_ms;      /* job completion times from the batch start (nearest rank) */
    double latency_p99_ms;
    double latency_max_ms;
    int wave_paths;             /* configuration the run used */
    int streams;
    int graph_launches;
    double latency_p90_ms;
    double latency_mean_ms;
    int traversal;              /* SAH node width of the run */
    int trace_block;            /* threads per block of the traversal kernels */
} c2g_batch_stats;
int c2g_batch_create(c2g_batch** out, int device);
void c2g_batch_destroy(c2g_batch* b);
const char* c2g_batch_last_error(c2g_batch* b);
/* Add a job: params->sample_count samples from params->sample_begin; *index = its job index. */
int c2g_batch_add(c2g_batch* b, c2g_ctx* job, const c2g_render_params* params, int* index);
/* Fix the configuration: paths per wave (rounded per job so that a wave holds whole samples that
 * divide the job's sample count) and the mode: 0 = one graph launch, 1..32 concurrent streams. */
int c2g_batch_tune(c2g_batch* b, int wave_paths, int streams);
/* Traversal variant of every job (SAH node width 2 or 4) and threads per block of the traversal
 * kernels (64, 128 or 256). */
int c2g_batch_set_trace(c2g_batch* b, int traversal, int trace_block);
/* One-launch mode: job chains that run side by side (1..256; 0 = every job on its own). */
int c2g_batch_set_lanes(c2g_batch* b, int lanes);
/* Candidate values per dimension of the batch configuration (n_x = 0: keep the current value). */
typedef struct {
    const int* wave_paths;
    int n_wave_paths;
    const int* streams;         /* 0 = one graph launch */
    int n_streams;
    const int* traversal;       /* 2 or 4 */
    int n_traversal;
    const int* trace_block;     /* 64, 128, 256 */
    int n_trace_block;
} c2g_batch_space;
/* Coordinate search: starting from the current configuration, each dimension in turn (wave size,
 * mode, traversal variant, block size) takes its candidate with the best aggregate rate on a trial
 * pass of every job (trial_spp samples each); films and networks are reset afterwards.  A candidate
 * whose trial runs out of device memory is skipped.  A trial's waves hold at most trial_spp samples
 * per pixel, so with trial_spp below a job's sample count the full run may need more memory than
 * its trial did. */
int c2g_batch_search(c2g_batch* b, const c2g_batch_space* space, int trial_spp, double* best_mpaths_per_s);
/* Time each (wave_paths, streams) pair of the candidate lists on a short trial of every job
 * (trial_spp samples each, films and networks reset afterwards), keep the fastest (an exhaustive
 * search over two dimensions; c2g_batch_search covers all four). */
int c2g_batch_autotune(c2g_batch* b, const int* wave_paths, int n_wave_paths, const int* streams, int n_streams,
                       int trial_spp, double* best_mpaths_per_s);
/* Render every job once (films accumulate; clear them with c2g_film_clear between runs). */
int c2g_batch_run(c2g_batch* b, c2g_batch_stats* stats);
/* Completion time of job i in the last run (ms from the batch start). */
int c2g_batch_job_latency(c2g_batch* b, int i, double* ms);

/* ---- learned guiding proposal (C2G_INTEGRATOR_GUIDED) -------------------------------------------
 * No counterpart in the reference, which has no guided integrator; these calls configure and
 * inspect the network the guided path tracer trains online.  The network maps (position in the
 * scene box, shading normal, outgoing direction) to an 8-lobe von Mises-Fisher mixture over
 * directions and the probability c = 0.05 + 0.75 sigmoid(s) of drawing from it rather than from the
 * BSDF; its weights are one flat FP32 vector of C2G_GUIDE_PARAMS values, layer by layer W (inputs x
 * outputs, row-major) then b, for layers 80->64->64->64->48 (outputs 41..47 are padding, kept
 * zero).  Loading a scene discards the network; a guided render creates one. */
#define C2G_GUIDE_PARAMS 16624
#define C2G_GUIDE_OUTPUTS 41
/* Draw a fresh seeded network for the box [lo, hi] (normalises positions) and clear Adam. */
int c2g_guide_reset(c2g_ctx* ctx, const float box_lo[3], const float box_hi[3], unsigned long long seed);
int c2g_guide_set_params(c2g_ctx* ctx, const float* params);
int c2g_guide_get_params(c2g_ctx* ctx, float* params);
/* Raw outputs (per lobe: mean direction xyz unnormalised, concentration pre-softplus, weight logit;
 * then the selection logit s) for n inputs of 9 floats (x, n, wo) -> out[n * C2G_GUIDE_OUTPUTS]. */
int c2g_guide_eval(c2g_ctx* ctx, int n, const float* xnw, float* out);
/* Summed gradient over n samples of 14 floats (x, n, wo, wi, w, p_bsdf) of
 * sum_j w_j * -log q_mix(wi_j), q_mix = (1 - c) p_bsdf + c q_guide, as the training kernel computes
 * it (BF16 operands, FP32 accumulation), written to grad[C2G_GUIDE_PARAMS];
 * loss = sum w (-log q_mix) / sum w.  No optimiser step. */
int c2g_guide_gradient(c2g_ctx* ctx, int n, const float* samples, float* grad, double* loss);
/* Training state of the last guided render: weighted NLL of the last batch, its size, Adam steps. */
int c2g_guide_stats(c2g_ctx* ctx, double* loss, int* records, int* steps);
/* learning_rate (Adam), bsdf_fraction (initial one-sample MIS probability of the BSDF technique,
 * (0, 1]; the network then learns it per vertex, within [0.2, 0.95]), warmup_waves (guided waves
 * that only train), train_steps (Adam steps per wave). */
int c2g_guide_config(c2g_ctx* ctx, float learning_rate, float bsdf_fraction, int warmup_waves, int train_steps);
/* Training batch of a guided wave: about records_per_wave recorded path vertices (every k-th path
 * records its bounces; default 262144, at least 1024) split into `windows` minibatch windows that
 * the wave's Adam steps take in turn (default 4, 1..64).  Takes effect at the next guided render. */
int c2g_guide_batch(c2g_ctx* ctx, int records_per_wave, int windows);
/* Regularisation of the learned mixture: the vMF concentration cap (1..500; default 500, about 2.5
 * degrees of spread), the clamp of the training weights at a multiple of their mean (>= 1;
 * default 20) and the learning-rate decay: Adam step t uses lr / (1 + t / decay_steps) (>= 0;
 * default 0 = constant).  Applies to the next inference and training launches. */
int c2g_guide_regularize(c2g_ctx* ctx, float kappa_max, float weight_clamp, float decay_steps);
/* Bounce levels, from the camera hit, whose vertices sample (and train) the guide; deeper vertices
 * use the plain tracer's estimator.  0 = every level; default 2. */
int c2g_guide_levels(c2g_ctx* ctx, int levels);

/* ---- ray queries (Scene::Intersect / Scene::IntersectTest, Scene.cpp:50-59) ---------------- */
/* Closest hit (any_hit = 0): obj = scene index of the hit object or -1, t = distance.
 * Any hit (any_hit = 1): obj = 1 if occluded else 0 over [tmin, tmax], ignoring object ignore[i]
 * (scene index or -1; the reference's ignoreShape). tmin/tmax/ignore may be NULL (0, inf, -1).
 * Host pointers; the copies are part of the call. */
int c2g_trace_rays(c2g_ctx* ctx, int n, const float* o, const float* d, const float* tmin,
                   const float* tmax, const int* ignore, int any_hit, int* obj, float* t);
/* Same over device pointers, on `stream`, without host synchronisation. */
int c2g_trace_rays_dev(c2g_ctx* ctx, int n, const float* o_dev, const float* d_dev,
                       const float* tmin_dev, const float* tmax_dev, const int* ignore_dev,
                       int any_hit, int* obj_dev, float* t_dev, void* stream);

/* ---- sampler / camera (HaltonSampler.cpp:118-291, PerspCamera.cpp:23-29) -------------------- */
/* SampleValue(GetVectorIndexForSample(sample), dim) for n (pixel, sample) pairs and dims
 * [0, ndim); film size width x height. Dims >= 100 come from the hash RNG. out: n * ndim. */
int c2g_halton(c2g_ctx* ctx, int width, int height, int n, const int* px, const int* py,
               const int* sample, int ndim, float* out);
/* Draws of the loaded scene's sampler (Config Integrator.Sampler: Halton, Default or Stratified;
 * Sampler::Get1D / Get2D, Sampler.cpp:10-53) at flat dimension `dim` for n (pixel, sample)
 * pairs: one float each (two_d = 0) or the pair (dim, dim + 1) (two_d = 1).  Dimension 0 is the
 * camera's pixel jitter.  out: n * (1 + two_d). */
int c2g_sampler_values(c2g_ctx* ctx, int n, const int* px, const int* py, const int* sample, int dim, int two_d,
                       float* out);
/* PerspCamera::GenerateRay for NDC points pos2 (n x 2) of the loaded camera. */
int c2g_camera_rays(c2g_ctx* ctx, int n, const float* pos2, float* o, float* d);

#ifdef __cplusplus
}
#endif
#endif /* C2G_H */
