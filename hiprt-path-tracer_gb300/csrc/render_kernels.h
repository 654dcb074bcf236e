// Launch interface of the render-path kernels (internal to libgbpt).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gbpt {

struct SceneView;
struct Queue;
struct PathBuffers;

// Per-render constants, passed by value to every kernel.
struct RenderConst
{
    int32_t width, height, spp;
    int32_t nb_bounces;
    int32_t do_rr, rr_min_depth;
    float rr_clamp;
    int32_t light_sampling;
    int32_t bsdf;
    uint32_t seed;
    int32_t do_jittering;
    int32_t ggx_height_correlated;
    float inverse_view[16];
    float inverse_projection[16];
};

cudaError_t launch_light_table(const SceneView& s, float* power, double* partial, int n_partial, double* sum64,
                               double* q, float* prob, int32_t* alias, int32_t* smalls, int32_t* larges,
                               cudaStream_t st);
// The FP64 sum, normalisation and Vose partition of launch_light_table over a power list that
// the caller already holds on the device (power list -> prob/alias, sum into *sum64).
cudaError_t launch_alias_table(const float* power, int n, double* partial, int n_partial, double* sum64, double* q,
                               float* prob, int32_t* alias, int32_t* smalls, int32_t* larges, cudaStream_t st);
cudaError_t launch_camera(const RenderConst& rc, const PathBuffers& pb, const Queue& q, int32_t iteration_base,
                          unsigned long long* stats, int n_sm, cudaStream_t st);
cudaError_t launch_bounce(const SceneView& s, const RenderConst& rc, const PathBuffers& pb, const Queue& in,
                          const Queue& next, const Queue& shadow, const Queue& bsdfq, int bounce, int64_t capacity,
                          unsigned long long* stats, int n_sm, cudaStream_t st);
cudaError_t launch_accumulate(const RenderConst& rc, const PathBuffers& pb, float* acc32, double* acc64, int n_sm,
                              cudaStream_t st);

}  // namespace gbpt
