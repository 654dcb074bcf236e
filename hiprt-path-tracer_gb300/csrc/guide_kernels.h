// Launch interface and parameter layout of the guiding network kernels (internal to libgbpt).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gbpt_guide.h"

namespace gbpt {
namespace guide {

// Packed BF16 weights in the tcgen05 K-major layout, as the kernels copy them into shared memory.
// Forward operands hold W^T (row = output unit, K = input unit): W1f, W2f, W3f (64 x 64), W4f
// (48 x 64). Backward operands hold W (row = input unit, K = output unit): W1b, W2b, W3b
// (64 x 64), W4b (64 x 48). Inference copies only the forward block.
constexpr int kW1f = 0, kW2f = kW1f + 64 * 64, kW3f = kW2f + 64 * 64, kW4f = kW3f + 64 * 64;
constexpr int kFwdWeights = kW4f + 48 * 64;
constexpr int kW1b = kFwdWeights, kW2b = kW1b + 64 * 64, kW3b = kW2b + 64 * 64, kW4b = kW3b + 64 * 64;
constexpr int kPackedWeights = kW4b + 64 * 48;  // bf16 elements
// offsets of W1..W4 in the FP32 parameter vector (W[in][out] row-major; the grid follows)
constexpr int kOffW1 = 0, kOffW2 = kOffW1 + 64 * 64, kOffW3 = kOffW2 + 64 * 64, kOffW4 = kOffW3 + 64 * 64;
constexpr int kNumWeights = kOffW4 + 64 * 48;
constexpr int64_t kNumParams = (int64_t)kNumWeights + GBPT_GUIDE_GRID_PARAMS;
static_assert(kNumWeights == GBPT_GUIDE_WEIGHTS, "weight count");

struct Net
{
    const float* params;        // [weights | grid], FP32 master
    const uint16_t* packed;     // BF16 kernel copies of the weights (kPackedWeights)
    const uint32_t* grid_bf16;  // BF16 copy of the grid, both features of an entry in one word
    float lo[3], inv_ext[3];    // hash-grid domain
    int wait_limit;             // polls of each tensor-core wait before it gives up (<= 0: none)
};

// A batch of rows: SoA position / normal / view / direction (3 floats per row), weight and BSDF
// pdf; the kernels process min(*count, n_max) rows when count is given (a device-side queue
// counter), else n_max rows. view points from the shading point towards the viewer.
struct Batch
{
    const float* pos;
    const float* nrm;
    const float* view;
    const float* dir;       // training only
    const float* weight;    // training only
    const float* bsdf_pdf;  // training only; null: the selection probability is not trained
    const int32_t* count;
    int64_t n_max;
};

cudaError_t launch_guide_init(float* params, uint32_t seed, cudaStream_t st);
// BF16 copies of the weights (tcgen05 layouts) and of the grid
cudaError_t launch_guide_pack(const float* params, uint16_t* packed, uint32_t* grid_bf16, cudaStream_t st);
cudaError_t launch_guide_weight_sum(const Batch& b, float* out_sum, cudaStream_t st);
// Forward + loss + backward over the batch; accumulates into grads (FP32, zeroed by the caller)
// and *loss; *err set to 1 if a tensor-core wait gave up.
cudaError_t launch_guide_train(const Net& net, const Batch& b, const float* weight_sum, float* grads, float* loss, int* err,
                               int n_sm, cudaStream_t st);
// Mixture per row: lobes[GBPT_GUIDE_ROW * row ..] = 8 x (mu xyz, kappa, weight), alpha
cudaError_t launch_guide_infer(const Net& net, const Batch& b, float* lobes, int* err, int n_sm, cudaStream_t st);
cudaError_t launch_guide_adam(float* params, const float* grads, float* m, float* v, float lr, float beta1, float beta2,
                              float eps, int step, cudaStream_t st);

// Entry points for the path tracer (guide_api.cpp): inference over a wavefront queue and one
// training step (gradients + Adam) on the frame's records, both reading device-side counts.
gbpt_status render_infer(gbpt_guide* g, const Batch& b, float* lobes, cudaStream_t cs);
gbpt_status render_train(gbpt_guide* g, const Batch& b, cudaStream_t cs);
int64_t max_batch(const gbpt_guide* g);

}  // namespace guide
}  // namespace gbpt
