// Host interface of the CUDA side: device scene upload, the wavefront renderer and the ray-query
// kernels.  Implemented in render.cu; called by the C ABI (capi.cpp).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>
#include <string>
#include <vector>

#include "../c2g_types.h"
#include "dev_scene.h"
#include "guide.h"
#include "../../../include/c2g.h"

namespace c2g {

struct HostScene;
struct RefTree;
struct SahTree;

// Device allocations owned by a context, with an optional cap.
class DeviceArena {
public:
    explicit DeviceArena(size_t cap = 0) : cap_(cap) {}
    ~DeviceArena();
    // Returns nullptr (and sets err) when the cap would be exceeded or cudaMalloc fails.
    void* alloc(size_t bytes, std::string& err);
    void free(void* p);
    void free_all();
    size_t used() const { return used_; }
    size_t cap() const { return cap_; }
    void set_cap(size_t c) { cap_ = c; }

private:
    struct Block { void* p; size_t n; };
    std::vector<Block> blocks_;
    size_t cap_ = 0, used_ = 0;
};

struct DeviceSceneBuffers;
struct WaveBuffers;

// Launch-independent arguments of the wave kernels (render.cu).
struct WaveArgs {
    int W, H;
    int tiles_x;
    int nslots;          // pixel slots (8x8 tiles)
    int wave_samples;    // samples of this wave
    int sample0;         // first sample index of the wave
    const int* sample0_dev;  // when set: the first sample index is read here (replayed graphs)
    int max_depth;
    int K;               // NEE slots per path
    int integrator;
};

// One render call's per-wave setup: scene view, wave arguments, samples per wave, bounce levels.
struct WavePlan {
    DevScene S;
    WaveArgs a;
    int spw = 1;
    int levels = 0;
    bool guided = false;
};

// Everything the kernels need for one loaded scene + its film.
class GpuScene {
public:
    GpuScene();
    ~GpuScene();
    // Upload scene, tree and sampler tables.  Returns a C2G status; err holds the message.
    int upload(const HostScene& s, int tree, const RefTree* ref, const SahTree* sah, DeviceArena& arena, std::string& err);
    int render(const HostScene& s, const c2g_render_params& p, cudaStream_t st, DeviceArena& arena, std::string& err);
    int film_clear(cudaStream_t st);
    int film_download(float* rgb_sum, float* weight, float* rgb_sumsq, std::string& err);
    int trace_rays_dev(int n, const float* o, const float* d, const float* tmin, const float* tmax, const int* ignore,
                       int any_hit, int* obj, float* t, cudaStream_t st, std::string& err);
    int sampler_values(int width, int n, const int* px, const int* py, const int* sample, int dim, int two_d, float* out,
                       DeviceArena& arena, std::string& err);
    int halton(int width, int height, int n, const int* px, const int* py, const int* sample, int ndim, float* out,
               DeviceArena& arena, std::string& err);
    int camera_rays(int n, const float* pos2, float* o, float* d, DeviceArena& arena, std::string& err);
    // Same render as render() into a caller-owned film, with no device allocation (render.cu).
    int render_noalloc(const c2g_render_params& p, float4* film_dev, cudaStream_t st, std::string& err);
    void set_counting(int flags) { counting_ = flags; }
    GuideStats guide_stats() { return guide_.stats(); }
    GuideTrainer& guide() { return guide_; }
    // Guided integrator schedule: waves of plain BSDF sampling before the mixture is used, and
    // Adam steps per wave.
    // Bounce levels (from the camera hit) that sample the guide and train it; 0 = every level.
    void set_guide_levels(int levels) { guide_levels_ = levels < 0 ? 0 : levels; }
    void set_guide_schedule(int warmup_waves, int train_steps) {
        guide_warmup_ = warmup_waves < 0 ? 0 : warmup_waves;
        guide_train_steps_ = train_steps < 0 ? 0 : train_steps;
    }
    const c2g_stats& stats() const { return stats_; }
    int check_device_error(std::string& err);
    // SAH traversal variant for the next upload and the loaded scene: 2 (binary nodes) or 4.
    void set_sah_width(int w);
    int sah_width() const { return sah_width_; }

    // ---- batched rendering (capi batch calls) ----
    // Capture one wave of p (samples per wave chosen by prepare) as a CUDA graph whose sample index
    // lives in device memory and is advanced by the graph itself, so the graph replays wave after
    // wave.  guide_sample: the guided integrator draws from the mixture in this graph.  Returns
    // the samples one launch renders in *wave_samples.
    int capture_wave(const c2g_render_params& p, bool guide_sample, cudaStream_t st, DeviceArena& arena,
                     cudaGraphExec_t* exec, int* wave_samples, std::string& err);
    // Record one wave of p into `body`, the body graph of a conditional while node of a larger
    // graph: the wave's kernels (as capture_wave), then one kernel that advances the device sample
    // counter by the wave's samples and sets the loop's condition `h` to (counter < end_sample), so
    // the loop renders wave after wave on the device.  Returns the samples per wave.
    int capture_wave_loop(const c2g_render_params& p, bool guide_sample, cudaGraph_t body, cudaGraphConditionalHandle h,
                          int end_sample, cudaStream_t st, DeviceArena& arena, int* wave_samples, std::string& err);
    // Append this scene's job (render parameters p, waves of up to wave_paths paths) to graph G as
    // one chain: a kernel that resets the device sample counter to p.sample_begin, a device-side
    // loop over the guided integrator's training-only waves, a loop over the remaining waves, and an
    // event record node on `done`.  The chain depends on deps[0..ndeps); *last = its final node.
    // *spw / *waves: samples per wave and the job's wave count.
    int append_job(cudaGraph_t G, const cudaGraphNode_t* deps, int ndeps, const c2g_render_params& p, int wave_paths,
                   cudaEvent_t done, cudaStream_t st, DeviceArena& arena, cudaGraphNode_t* last, int* spw, int* waves,
                   std::string& err);
    // Device counter the captured graphs read their first sample index from.
    int set_wave_counter(int sample, cudaStream_t st, DeviceArena& arena, std::string& err);
    // Free the wave's working buffers (the next render or capture sizes them anew).
    void release_wave_buffers(DeviceArena& arena);
    int* wave_counter() const { return wave_counter_; }
    // Threads per block of the traversal kernels (64, 128 or 256); taken by the next render or capture.
    void set_trace_block(int threads);
    int trace_block() const { return trace_block_; }
    int guide_warmup() const { return guide_warmup_; }

private:
    int prepare(const c2g_render_params& p, DeviceArena& arena, WavePlan& plan, std::string& err);
    size_t default_wave_paths(int K, const DeviceArena& arena) const;
    int enqueue_wave(const WavePlan& plan, const WaveArgs& a, const GuideView& gv, bool count, cudaStream_t st,
                     const std::function<void(int, cudaStream_t)>& begin, const std::function<void(cudaStream_t)>& end,
                     int& launches, std::string& err, bool advance = true);
    int capture_plan(const c2g_render_params& p, bool guide_sample, cudaStream_t st, DeviceArena& arena, WavePlan& plan,
                     GuideView& gv, std::string& err);
    DeviceSceneBuffers* sb_;
    int* wave_counter_ = nullptr;  // device sample index of captured wave graphs
    int sah_width_ = 4;            // SAH traversal variant (2 or 4 children per node)
    int trace_block_ = 128;        // threads per block of the traversal kernels
    WaveBuffers* wb_;
    int counting_ = 0;
    int present_buckets_ = 0;  // material buckets the loaded scene can produce
    GuideTrainer guide_;       // learned proposal of the guided integrator
    int guide_steps_ = 0;      // guided waves rendered on the loaded scene
    int guide_warmup_ = 2;     // guided waves that only record (BSDF sampling) before the mixture is used
    int guide_train_steps_ = 1;  // Adam steps per guided wave
    int guide_levels_ = 2;       // bounce levels served by the guide (0: all)
    // Second stream of a wave: independent kernels of a bounce level (shading buckets, the MIS
    // rays beside the shadow rays) run on it between fork and join events.  Eager renders only:
    // off while per-kernel timing events are recorded and in the graphs batched jobs replay.
    bool overlap_ = true;
    cudaStream_t side_ = nullptr;
    // Third stream of a wave: the next bounce level's extension starts on it as soon as this level's
    // shading has filled the next queue, beside this level's shadow and MIS rays and accumulation.
    cudaStream_t ahead_ = nullptr;
    cudaEvent_t fork_ev_[4] = {nullptr, nullptr, nullptr, nullptr}, join_ev_[4] = {nullptr, nullptr, nullptr, nullptr};
    int side_stream(std::string& err);
    float box_lo_[3] = {0, 0, 0}, box_hi_[3] = {1, 1, 1};  // scene bounds (network input range)
    c2g_stats stats_{};
    int film_w_ = 0, film_h_ = 0;
};

// L2 read bandwidth of the current device in GB/s: a buffer of `bytes` (small enough to stay in L2)
// read `reps` times by every SM with loads cached in L2 only.  The denominator of the traversal
// kernels' L2 roofline.
int probe_l2_read(size_t bytes, int reps, double* gbs, std::string& err);

}  // namespace c2g
