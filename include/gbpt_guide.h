/*
 * gbpt — learned direction proposal for path guiding (no counterpart in the reference, which has
 * no path guiding; closest relatives are its NEE++ and ReGIR caches).
 *
 * A multiresolution hash-grid encoding of the shading position (8 levels x 2 features, 2^15
 * entries per level, resolutions 4..68 over the scene box) plus the shading normal and the
 * direction towards the viewer feeds a
 * 32 -> 64 -> 64 -> 48 ReLU MLP without biases (a constant input of 1 plays that role). Its
 * output is a mixture of 8 von Mises-Fisher lobes (direction, concentration kappa = softplus + 0.1,
 * clamped to 500, softmax weights). The MLP runs in BF16 on the tcgen05 tensor cores with FP32
 * accumulation; the hash grid, the head, the loss and Adam run in FP32.
 * Training minimises the KL divergence from the radiance-weighted target to the mixture: per
 * sample the loss is -w * log q(direction) with w = luminance(incident radiance * f * cos) / pdf,
 * normalised by the batch's sum of w. Forward, backward and Adam are hand-written kernels.
 * Sampling combines the mixture with BSDF sampling by one-sample MIS (gbpt_renderer_set_guide), so
 * the estimator stays unbiased. All pointers are device pointers unless stated.
 */
#ifndef GBPT_GUIDE_H
#define GBPT_GUIDE_H

#include "gbpt.h"

#ifdef __cplusplus
extern "C" {
#endif

#define GBPT_GUIDE_LEVELS 8
#define GBPT_GUIDE_TABLE 32768
#define GBPT_GUIDE_FEATURES 2
#define GBPT_GUIDE_GRID_PARAMS (GBPT_GUIDE_LEVELS * GBPT_GUIDE_TABLE * GBPT_GUIDE_FEATURES)
#define GBPT_GUIDE_IN 32
#define GBPT_GUIDE_HIDDEN 64
#define GBPT_GUIDE_OUT 48
#define GBPT_GUIDE_LOBES 8
/* W1 [32][64], W2 [64][64], W3 [64][48], row = input unit, column = output unit, concatenated */
#define GBPT_GUIDE_WEIGHTS (GBPT_GUIDE_IN * GBPT_GUIDE_HIDDEN + GBPT_GUIDE_HIDDEN * GBPT_GUIDE_HIDDEN + \
                            GBPT_GUIDE_HIDDEN * GBPT_GUIDE_OUT)

typedef struct gbpt_guide gbpt_guide;

typedef struct gbpt_guide_params {
    float scene_min[3], scene_max[3]; /* hash-grid domain (positions are clamped into it) */
    float learning_rate;              /* Adam, default 5e-3 */
    float beta1, beta2, epsilon;      /* default 0.9, 0.99, 1e-8 */
    uint32_t seed;                    /* initialisation */
    int32_t max_batch;                /* largest training batch, default 1 << 18 */
    int32_t reserved[6];
} gbpt_guide_params;

GBPT_API gbpt_status gbpt_guide_default_params(gbpt_guide_params* p);
GBPT_API gbpt_status gbpt_guide_create(const gbpt_guide_params* p, gbpt_guide** out);
GBPT_API gbpt_status gbpt_guide_destroy(gbpt_guide* g);

/* One Adam step on n training samples: position[3n], normal[3n], view[3n] (towards the viewer),
 * direction[3n] (the sampled incident direction; unit vectors), weight[n] (negative counts as 0).
 * *loss (host, may be NULL; synchronous when given) receives the normalised batch loss before the
 * step. */
GBPT_API gbpt_status gbpt_guide_train(gbpt_guide* g, const float* position, const float* normal, const float* view,
                                      const float* direction, const float* weight, int64_t n, float* loss, void* stream);
/* The gradients of the batch loss without an Adam step, copied to host arrays (either may be
 * NULL): grad_weights[GBPT_GUIDE_WEIGHTS], grad_grid[GBPT_GUIDE_GRID_PARAMS]. Synchronous. */
GBPT_API gbpt_status gbpt_guide_gradients(gbpt_guide* g, const float* position, const float* normal,
                                          const float* view, const float* direction, const float* weight, int64_t n,
                                          float* grad_weights, float* grad_grid, float* loss, void* stream);
/* Mixture per query: lobes[40 n] = 8 x (mu xyz, kappa, weight). */
GBPT_API gbpt_status gbpt_guide_infer(gbpt_guide* g, const float* position, const float* normal, const float* view,
                                      int64_t n, float* lobes, void* stream);
/* 1 if a bounded tensor-core wait of a guide kernel gave up since creation (the kernel then
 * stopped early and its outputs are incomplete), else 0. Synchronous. */
GBPT_API gbpt_status gbpt_guide_error_flag(gbpt_guide* g, int32_t* flag);
/* Parameters to / from host arrays (either may be NULL). Synchronous. */
GBPT_API gbpt_status gbpt_guide_get_params(gbpt_guide* g, float* weights, float* grid);
GBPT_API gbpt_status gbpt_guide_set_params(gbpt_guide* g, const float* weights, const float* grid);

#ifdef __cplusplus
}
#endif

#endif /* GBPT_GUIDE_H */
