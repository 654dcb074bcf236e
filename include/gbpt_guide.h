/*
 * gbpt — learned direction proposal for path guiding (no counterpart in the reference, which has
 * no path guiding; closest relatives are its NEE++ and ReGIR caches).
 *
 * Encoding: a multiresolution hash grid of the shading position, 16 levels x 2 features, 2^19
 * entries per level, resolutions floor(16 * 256^(l/15)) = 16 .. 4096 over the scene box (dense
 * indexing where (res+1)^3 fits, else the XOR-of-primes hash), features kept as FP32 master values
 * and read through a BF16 copy; plus the shading normal and the degree-4 real spherical-harmonic
 * encoding (16 coefficients) of the direction towards the viewer. 64 inputs (13 zero).
 * Network: 64 -> 64 -> 64 -> 64 -> 48, ReLU, no biases (the constant SH band plays that role),
 * BF16 weights and activations on the tcgen05 tensor cores with FP32 accumulation (forward,
 * backward and the weight gradients, accumulated in tensor memory).
 * Head: 8 von Mises-Fisher lobes (direction = normalised raw[5i..5i+2], concentration
 * kappa = softplus(raw[5i+3]) + 0.1 clamped to 500, weight = softmax(raw[5i+4])) and the
 * probability of sampling the mixture instead of the BSDF, alpha = 0.05 + 0.9 sigmoid(raw[40]).
 * Loss per sample, with w = weight / sum of the batch's weights:
 *   -w log q(direction)  (the KL divergence from the radiance-weighted target to the mixture),
 *   -w log(alpha q + (1 - alpha) p_bsdf)  with q held fixed (trains alpha; needs p_bsdf).
 * Adam with FP32 master weights, moments and gradients. All pointers are device pointers unless
 * stated.
 */
#ifndef GBPT_GUIDE_H
#define GBPT_GUIDE_H

#include "gbpt.h"

#ifdef __cplusplus
extern "C" {
#endif

#define GBPT_GUIDE_LEVELS 16
#define GBPT_GUIDE_TABLE 524288
#define GBPT_GUIDE_FEATURES 2
#define GBPT_GUIDE_GRID_PARAMS (GBPT_GUIDE_LEVELS * GBPT_GUIDE_TABLE * GBPT_GUIDE_FEATURES)
#define GBPT_GUIDE_IN 64
#define GBPT_GUIDE_HIDDEN 64
#define GBPT_GUIDE_OUT 48
#define GBPT_GUIDE_LOBES 8
/* floats per inferred row: 8 x (mu xyz, kappa, weight), alpha, 3 unused */
#define GBPT_GUIDE_ROW 44
/* W1 [64][64], W2 [64][64], W3 [64][64], W4 [64][48], row = input unit, column = output unit */
#define GBPT_GUIDE_WEIGHTS (3 * GBPT_GUIDE_HIDDEN * GBPT_GUIDE_HIDDEN + GBPT_GUIDE_HIDDEN * GBPT_GUIDE_OUT)

typedef struct gbpt_guide gbpt_guide;

typedef struct gbpt_guide_params {
    float scene_min[3], scene_max[3]; /* hash-grid domain (positions are clamped into it) */
    float learning_rate;              /* Adam, default 1e-2 */
    float beta1, beta2, epsilon;      /* default 0.9, 0.99, 1e-8 */
    uint32_t seed;                    /* initialisation */
    int32_t max_batch;                /* largest training batch, default 1 << 18 */
    /* Polls of each bounded tensor-core completion wait before it gives up: > 0 that many, 0 the
     * default (2^24), < 0 none at all. A wait that gives up lets the kernel's issued tensor-core
     * work finish (a second bounded wait), frees its TMEM, stops the kernel early and raises the
     * error flag (the call returns GBPT_ERROR_TIMEOUT); the device context stays usable. A
     * negative value makes every wait give up at once: the test of that path. */
    int32_t wait_limit;
    int32_t reserved[5];
} gbpt_guide_params;

GBPT_API gbpt_status gbpt_guide_default_params(gbpt_guide_params* p);
GBPT_API gbpt_status gbpt_guide_create(const gbpt_guide_params* p, gbpt_guide** out);
GBPT_API gbpt_status gbpt_guide_destroy(gbpt_guide* g);

/* One Adam step on n training samples: position[3n], normal[3n], view[3n] (towards the viewer),
 * direction[3n] (the sampled incident direction; unit vectors), weight[n] (negative counts as 0),
 * bsdf_pdf[n] (the BSDF's solid-angle pdf of direction; NULL: alpha is not trained).
 * *loss (host, may be NULL; synchronous when given) receives the batch loss before the step. */
GBPT_API gbpt_status gbpt_guide_train(gbpt_guide* g, const float* position, const float* normal, const float* view,
                                      const float* direction, const float* weight, const float* bsdf_pdf, int64_t n,
                                      float* loss, void* stream);
/* The gradients of the batch loss without an Adam step, copied to host arrays (either may be
 * NULL): grad_weights[GBPT_GUIDE_WEIGHTS], grad_grid[GBPT_GUIDE_GRID_PARAMS]. Synchronous. */
GBPT_API gbpt_status gbpt_guide_gradients(gbpt_guide* g, const float* position, const float* normal,
                                          const float* view, const float* direction, const float* weight,
                                          const float* bsdf_pdf, int64_t n, float* grad_weights, float* grad_grid,
                                          float* loss, void* stream);
/* Mixture per query: lobes[GBPT_GUIDE_ROW n] = 8 x (mu xyz, kappa, weight), alpha, 3 unused. */
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
