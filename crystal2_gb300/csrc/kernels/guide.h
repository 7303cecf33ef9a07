// Host interface of the learned guiding proposal (guide.cu): network state, inference over the
// shading buckets, training on recorded path vertices.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <string>

namespace c2g {

constexpr int kGuideIn = 80;
constexpr int kGuideHidden = 64;
constexpr int kGuideOut = 41;       // 8 lobes x 5, then the technique-selection logit
constexpr int kGuideOutPad = 48;    // output layer padded to a multiple of 16 (backward K)
constexpr int kGuideLobes = 8;
constexpr int kGuideFreqs = 12;
constexpr int kGuideLayers = 4;
constexpr float kGuideKappaMax = 500.f;   // vMF concentration cap (about 2.5 degrees of spread)
constexpr float kGuideSelMin = 0.05f;     // selection probability c in [0.05, 0.8]
constexpr float kGuideSelSpan = 0.75f;
// Layer shapes (inputs, outputs).
__host__ __device__ constexpr int guide_k(int l) { return l == 0 ? kGuideIn : kGuideHidden; }
__host__ __device__ constexpr int guide_n(int l) { return l == 3 ? kGuideOutPad : kGuideHidden; }
// Parameter offsets inside the flat FP32 master vector: W_l (K x N, row-major) then b_l (N).
__host__ __device__ constexpr int guide_w_off(int l) {
    return l == 0 ? 0 : guide_w_off(l - 1) + guide_k(l - 1) * guide_n(l - 1) + guide_n(l - 1);
}
__host__ __device__ constexpr int guide_b_off(int l) { return guide_w_off(l) + guide_k(l) * guide_n(l); }
constexpr int kGuideParams = guide_w_off(4);
// BF16 copies: wt_l (N x K) then wn_l (K x N) per layer.
__host__ __device__ constexpr int guide_bf_off(int l) { return l == 0 ? 0 : guide_bf_off(l - 1) + 2 * guide_k(l - 1) * guide_n(l - 1); }
constexpr int kGuideBf16 = guide_bf_off(4);

struct GuideNet {
    const __nv_bfloat16* bf;   // kGuideBf16 values
    const float* params;       // kGuideParams (biases read from here)
    float box_lo[3], box_inv[3];
    float alpha;               // probability of drawing the continuation from the BSDF
    int enabled;
    float kappa_max;           // vMF concentration cap (at most kGuideKappaMax)
    float weight_clamp;        // training weights clamped at this multiple of their mean
};

class DeviceArena;

// Per-wave view handed to the shading kernels.
struct GuideView {
    GuideNet net;
    const float* out;      // per guided work item: the packed mixture (kGuidePacked floats, field-major, guide.cuh)
    int out_stride;        // its field stride in float4 (the wave's path capacity)
    float4* rec;           // training records, 4 float4 per (recorded path, bounce)
    int rec_stride;        // every rec_stride-th path id records its vertices
    int rec_depth;         // records per recorded path (= max depth)
    int record;            // 1: write records this wave
    int sample;            // 1: draw continuations from the guide mixture
};

struct GuideStats {
    double loss;           // mean weighted negative log-likelihood of the last training batch
    int records;           // records used by the last training step
    int steps;             // Adam steps taken so far
};

class GuideTrainer {
public:
    GuideTrainer() = default;
    ~GuideTrainer();
    // Allocate the network (seeded init), Adam state and record buffers for waves of `paths`.
    int init(DeviceArena& arena, size_t paths, int max_depth, const float box_lo[3], const float box_hi[3],
             unsigned long long seed, std::string& err);
    bool ready() const { return params_ != nullptr; }
    // Free every device buffer; the next init() draws a fresh network.
    void release(DeviceArena& arena);
    // Network outputs for every slot in the given material buckets (encoding kernel, then the
    // tensor-core MLP kernel).
    // Returns the kernels launched (0 when no bucket of the mask is guided).
    int infer(cudaStream_t st, const void* S, const float4* ray_o, const float4* ray_d, const float4* hits,
              const int* bucket_cnt, const int* bucket_list, int cap, int bucket_mask);
    // Turn this wave's records into weighted samples and take `steps` Adam steps (a tensor-memory
    // wait that times out sets DEVERR_WAIT in *err).
    void train(cudaStream_t st, const float4* out_L, int wave_paths, int steps, int* err);
    GuideView view(bool record, bool sample) const;
    // Launch configuration (occupancy queries), done once before any stream capture.
    static void prepare_launch();
    // Partial gradients the training kernel writes per launch (one per warpgroup of its grid).
    static int train_parts();
    GuideStats stats();
    void set_learning_rate(float lr) { lr_ = lr; }
    void set_alpha(float a) { alpha_ = a; }
    // Regularisation of the mixture: concentration cap, training-weight clamp, learning-rate decay
    // (lr / (1 + step / decay_steps); 0 = constant).
    void set_regularisation(float kappa_max, float weight_clamp, float decay_steps) {
        kappa_max_ = kappa_max;
        weight_clamp_ = weight_clamp;
        lr_decay_ = decay_steps;
    }
    // Recorded vertices per wave and minibatch windows (the record buffers are re-sized by the next
    // init()).
    void set_batch(int records, int windows) {
        if (records != rec_target_) cap_ = 0;
        rec_target_ = records;
        windows_ = windows;
    }
    // Network weights as the flat FP32 vector (kGuideParams); setting them clears the Adam state.
    int set_params(const float* host, std::string& err);
    int get_params(float* host, std::string& err);
    // Raw outputs for n explicit inputs (x, n, wo: 9 floats each) -> n x kGuideOut floats.
    int eval(DeviceArena& arena, const float* host_xnw, int n, float* host_out, std::string& err);
    // Summed weight gradient of sum_j w_j * -log q_mix(wi_j | x_j, n_j, wo_j) over n samples (14
    // floats each: x, n, wo, wi, w, p_bsdf) with the fused training kernel; no Adam step.
    // loss = sum w (-log q_mix) / sum w.
    int gradient(DeviceArena& arena, const float* host_samples, int n, float* host_grad, double* loss, std::string& err);

private:
    float* params_ = nullptr;        // FP32 master weights
    float* grad_ = nullptr;          // summed gradient (explicit-batch entry point)
    float* part_ = nullptr;          // per-warpgroup partial gradients of the last training launch
    int nparts_ = 0;
    float* adam_m_ = nullptr;
    float* adam_v_ = nullptr;
    __nv_bfloat16* bf_ = nullptr;    // BF16 copies (both layouts)
    float* out_ = nullptr;           // per-slot outputs
    unsigned char* stage_ = nullptr; // network input records of the guided vertices (x, n, wo: 36 B per vertex)
    float4* rec_ = nullptr;
    float4* batch_ = nullptr;        // compacted training samples (x|w, n, wo, wi)
    int* batch_count_ = nullptr;
    float* loss_acc_ = nullptr;      // [0] weighted NLL sum, [1] weight sum, [2] raw weight sum,
                                     // [4..5] the last Adam step's [0..1]
    int* step_dev_ = nullptr;        // Adam steps taken (device copy: captured graphs advance it)
    size_t cap_ = 0;
    int rec_stride_ = 16, rec_depth_ = 1;
    int rec_target_ = 1 << 18;       // recorded vertices per wave (about)
    int windows_ = 4;                // minibatch windows per wave
    size_t rec_cap_ = 0;
    float box_lo_[3] = {0, 0, 0}, box_inv_[3] = {1, 1, 1};
    float lr_ = 2e-3f;
    float alpha_ = 0.5f;
    float kappa_max_ = kGuideKappaMax;
    float weight_clamp_ = 20.f;
    float lr_decay_ = 0.f;
    int steps_ = 0;
    int last_records_ = 0;
    GuideStats last_{};
};

}  // namespace c2g
