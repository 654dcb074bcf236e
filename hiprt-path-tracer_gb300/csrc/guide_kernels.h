// Launch interface and shared-memory plan of the guiding network kernels (internal to libgbpt).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gbpt_guide.h"

namespace gbpt {
namespace guide {

// Packed BF16 weights in the tcgen05 K-major layout, as the kernels copy them into shared memory:
// forward operands W1f (64 x 32), W2f (64 x 64), W3f (48 x 64) hold W^T (row = output unit);
// backward operands W1b (32 x 64), W2b (64 x 64), W3b (64 x 48) hold W (row = input unit).
constexpr int kW1f = 0, kW2f = kW1f + 64 * 32, kW3f = kW2f + 64 * 64;
constexpr int kW1b = kW3f + 48 * 64, kW2b = kW1b + 32 * 64, kW3b = kW2b + 64 * 64;
constexpr int kPackedWeights = kW3b + 64 * 48;  // bf16 elements
// offsets of W1, W2, W3 in the FP32 parameter vector (grid follows the weights)
constexpr int kOffW1 = 0, kOffW2 = 32 * 64, kOffW3 = kOffW2 + 64 * 64;
constexpr int kNumWeights = kOffW3 + 64 * 48;
constexpr int kNumParams = kNumWeights + GBPT_GUIDE_GRID_PARAMS;

struct Net
{
    const float* params;            // [weights | grid], FP32 master
    const uint16_t* packed;         // BF16 kernel copies of the weights (kPackedWeights)
    float lo[3], inv_ext[3];        // hash-grid domain
};

// A batch of rows: SoA position / normal / view / direction (3 floats per row) and weight;
// the kernels process min(*count, n_max) rows when count is given (a device-side queue
// counter), else n_max rows. view points from the shading point towards the viewer.
struct Batch
{
    const float* pos;
    const float* nrm;
    const float* view;
    const float* dir;     // training only
    const float* weight;  // training only
    const int32_t* count;
    int64_t n_max;
};

cudaError_t launch_guide_init(float* params, uint32_t seed, cudaStream_t st);
cudaError_t launch_guide_pack(const float* params, uint16_t* packed, cudaStream_t st);
cudaError_t launch_guide_weight_sum(const Batch& b, float* out_sum, cudaStream_t st);
// Forward + loss + backward over the batch; accumulates into grads (FP32, zeroed by the caller)
// and *loss; *err set to 1 if a tensor-core wait gave up.
cudaError_t launch_guide_train(const Net& net, const Batch& b, const float* weight_sum, float* grads, float* loss, int* err,
                               int n_sm, cudaStream_t st);
// Mixture per row: lobes[40 row + 5 i ..] = lobe i (mu xyz, kappa, weight)
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
