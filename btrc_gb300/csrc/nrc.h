// Neural radiance cache: a multiresolution hash-grid + spherical-harmonics encoding
// feeding a 5x64 ReLU MLP (BF16 weights and activations, FP32 accumulation) that predicts
// the outgoing radiance of a path vertex; trained online with FP32 Adam on radiance
// estimates the tracer produces (no counterpart in the reference).
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "bmath.h"

namespace bt {

// encoding
constexpr int NRC_LEVELS = 16;
constexpr int NRC_FEATURES = 2;                 // per level
constexpr int NRC_LOG2_TABLE = 19;              // 2^19 entries per level
constexpr uint32_t NRC_TABLE = 1u << NRC_LOG2_TABLE;
constexpr float NRC_MIN_RES = 16.0f;
constexpr float NRC_MAX_RES = 4096.0f;

// network: 80 inputs -> 5 hidden layers of 64 -> 3 outputs (padded to 16)
constexpr int NRC_IN = 80;                      // 32 hash + 16 SH(dir) + 16 SH(normal) + roughness + albedo(3) + 1 + pad
constexpr int NRC_WIDTH = 64;
constexpr int NRC_HIDDEN = 5;                   // hidden layers (outputs of width 64)
constexpr int NRC_OUT = 16;                     // 3 used
constexpr int NRC_LAYERS = NRC_HIDDEN + 1;      // weight matrices
// weight matrix l is K_l x N_l: K = {80, 64, 64, 64, 64, 64}, N = {64, 64, 64, 64, 64, 16}
constexpr int NRC_WEIGHTS = NRC_IN * NRC_WIDTH + (NRC_HIDDEN - 1) * NRC_WIDTH * NRC_WIDTH + NRC_WIDTH * NRC_OUT;

// a cache query: position, direction towards the viewer, shading normal, roughness,
// diffuse albedo
constexpr int NRC_QUERY_FLOATS = 13;
// a training sample: a query followed by the target radiance
constexpr int NRC_SAMPLE_FLOATS = 16;

struct NrcHyper
{
    float lr = 1e-2f;
    float beta1 = 0.9f, beta2 = 0.99f;
    float eps = 1e-8f;
    float rel_eps = 1e-2f;     // relative L2 loss: (y - t)^2 / (sg(y)^2 + rel_eps)
};

struct NrcDev
{
    float bbox_min[3], bbox_inv_extent[3];
    const __half2 *hash;        // [LEVELS][TABLE] features used by the encoding
    const uint2 *w_fwd;         // weights packed as mma B fragments for y = x W
    const uint2 *w_bwd;         // weights packed as mma B fragments for dx = dy W^T
    float2 *hash_grad;          // [LEVELS][TABLE]
    __nv_bfloat16 *act;         // training: layer inputs X_l, row-major per layer (see nrc.cu)
    __nv_bfloat16 *dact;        // training: pre-activation gradients dY_l
    float *loss;                // training: summed loss
    const __nv_bfloat16 *w_tc;  // weights as tcgen05 B operands (W_l^T, K-major core matrices)
    uint32_t *err;              // set when a tensor-core wait timed out
};

class Nrc
{
public:
    Nrc(const float bbox_min[3], const float bbox_max[3], uint64_t seed);
    ~Nrc();
    Nrc(const Nrc &) = delete;
    Nrc &operator=(const Nrc &) = delete;

    // predictions (3 floats per query, 4-float stride) for n queries
    cudaError_t infer(const float *d_queries, uint32_t n, float *d_out, cudaStream_t st);
    // one optimisation step over n training samples; its mean loss is added to a device
    // accumulator (reset_loss / read_loss). apply_adam = false computes gradients only.
    cudaError_t train(const float *d_samples, uint32_t n, bool apply_adam, cudaStream_t st);
    cudaError_t reset_loss(cudaStream_t st);
    // synchronises st and returns the accumulated loss
    cudaError_t read_loss(float *out, cudaStream_t st);
    // the loss accumulator copied to host memory on st without waiting (pinned `out`)
    cudaError_t copy_loss_async(float *out, cudaStream_t st);
    // synchronises st; cudaErrorLaunchTimeout when a tensor-core kernel gave up waiting
    cudaError_t check_error(cudaStream_t st);

    // parameters / gradients as FP32 host copies (test hooks). which: 0 MLP weights
    // (NRC_WEIGHTS, layer-major, row-major K x N), 1 hash features (LEVELS * TABLE * 2),
    // 2 MLP gradients, 3 hash gradients
    cudaError_t copy_params(int which, float *host, uint64_t count, bool set, cudaStream_t st);

    const NrcDev &dev() const { return d_; }
    uint64_t steps() const { return step_; }

private:
    cudaError_t ensure_batch(uint32_t n);
    cudaError_t repack(cudaStream_t st);

    NrcDev d_{};
    NrcHyper hyper_;
    float *w_master_ = nullptr, *w_grad_ = nullptr, *w_m_ = nullptr, *w_v_ = nullptr;
    float2 *h_master_ = nullptr, *h_m_ = nullptr, *h_v_ = nullptr;
    __half2 *h_f16_ = nullptr;
    uint2 *w_fwd_ = nullptr, *w_bwd_ = nullptr;
    __nv_bfloat16 *w_tc_ = nullptr;
    uint32_t *err_ = nullptr;
    bool use_tc_ = true;        // inference on tcgen05 (false: the mma.sync kernel)
    __nv_bfloat16 *act_ = nullptr, *dact_ = nullptr;
    float *loss_ = nullptr;
    uint32_t batch_cap_ = 0;
    uint64_t step_ = 0;
};

} // namespace bt
