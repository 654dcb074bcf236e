// Launch interface of the render-path kernels (internal to libgbpt).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "render_common.h"
#include "restir.h"

namespace gbpt {

struct SceneView;
struct Queue;
struct PathBuffers;
struct GuideView;

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
    int32_t restir_final_visibility;  // ReSTIR DI final shading traces a shadow ray unless known unoccluded
    int32_t direct_ris;               // GBPT_DIRECT_RIS
    int32_t ris_light, ris_bsdf;      // RIS candidates
    int32_t rng_mode;                 // GBPT_RNG_*
    uint32_t random_number;           // GBPT_RNG_REFERENCE: HIPRTRenderData::random_number of the MegaKernel pass
    uint32_t random_number_camera;    // GBPT_RNG_REFERENCE: HIPRTRenderData::random_number of the G-buffer pass
    float inverse_view[16];
    float inverse_projection[16];
};

// One job of a batched render (device table): its scene and settings (rc.spp = samples per
// iteration), its first path slot and first accumulator pixel, and its total samples per pixel.
struct BatchJob
{
    SceneView s;
    RenderConst rc;
    int64_t slot_base;
    int64_t pixel_base;
    int32_t spp_total;
    int32_t iterations;  // ceil(spp_total / rc.spp)
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
// One bounce = extend (closest hit of the active queue) then shade (shade + shadow and BSDF-light
// traversal + resolve). 'restir' (null buffers when ReSTIR DI is off) holds the final reservoirs
// that replace next-event estimation at bounce 0.
// jobs / job_of_slot (batched rendering, else null): each ray traverses its slot's job's BVH.
// Closest-hit (any_hit = false: hits) or any-hit (occluded) traversal of a device-counted queue of
// at most 'capacity' rays.
cudaError_t launch_trace_queue(const SceneView& s, const Queue& q, bool any_hit, int64_t capacity, int n_sm,
                               cudaStream_t st);
cudaError_t launch_extend(const SceneView& s, const Queue& in, const Queue& next, const Queue& shadow,
                          const Queue& bsdfq, int64_t capacity, int n_sm, cudaStream_t st,
                          const BatchJob* jobs = nullptr, const int32_t* job_of_slot = nullptr);
// 'gv' (null lobes when guiding is off) holds the learned mixture per entry of 'in' and the
// training-record buffers. 'envq' (any-hit, 2 entries per path) takes the envmap direct-lighting
// rays when pb.env_entry is set (the scene's envmap is importance sampled).
cudaError_t launch_shade(const SceneView& s, const RenderConst& rc, const PathBuffers& pb, const Queue& in,
                         const Queue& next, const Queue& shadow, const Queue& bsdfq, const Queue& envq, int bounce,
                         int64_t capacity, unsigned long long* stats, const ReservoirBuf& restir, const GuideView& gv,
                         int n_sm, cudaStream_t st, const BatchJob* jobs = nullptr);
// Envmap tables: RGB9E5 texels and float luminance of n RGB float texels, the FP64 running sum
// over texels rounded to float (cdf) and the FP64 total (*sum64). tile_total / tile_offset hold
// envmap_scan_tiles(n) doubles each.
int envmap_scan_tiles(int64_t n);
cudaError_t launch_envmap_tables(const float* rgb, int64_t n, uint32_t* texels, float* lum, float* cdf,
                                 double* tile_total, double* tile_offset, double* sum64, cudaStream_t st);
// Guiding network inputs for each entry of 'in' (after its closest hits are known)
cudaError_t launch_guide_inputs(const SceneView& s, const Queue& in, const GuideView& gv, int64_t capacity, int n_sm,
                                cudaStream_t st);
// Training-record weights from the final path radiance (after the launch's last bounce)
cudaError_t launch_guide_weights(const PathBuffers& pb, const GuideView& gv, int n_sm, cudaStream_t st);
cudaError_t launch_restir_gbuffer(const SceneView& s, const Queue& q, const GBuffer& gb, int64_t n_pix, int packed_normals,
                                  int n_sm, cudaStream_t st);
// Light presampling of the frame into out (2 float4 per record, k.presample_subsets * size records)
cudaError_t launch_restir_presample(const SceneView& s, const RenderConst& rc, const RestirConst& k, float4* out,
                                    int n_sm, cudaStream_t st);
cudaError_t launch_restir_initial(const SceneView& s, const RenderConst& rc, const RestirConst& k, const GBuffer& gb,
                                  const ReservoirBuf& out, const InitialState& st, const Queue& qa, const Queue& qb,
                                  const Queue& vis, int64_t queue_capacity, int n_sm, cudaStream_t stream);
cudaError_t launch_restir_temporal(const SceneView& s, const RenderConst& rc, const RestirConst& k, const GBuffer& gb,
                                   const GBuffer& gb_prev, const ReservoirBuf& initial, const ReservoirBuf& prev,
                                   const ReservoirBuf& out, int2* ray_of, const Queue& rays, int n_sm, cudaStream_t st);
// Fused spatiotemporal reuse: initial + previous final reservoirs (and G-buffers) -> out
cudaError_t launch_restir_spatiotemporal(const SceneView& s, const RenderConst& rc, const RestirConst& k,
                                         const GBuffer& gb, const GBuffer& gb_prev, const ReservoirBuf& initial,
                                         const ReservoirBuf& prev, const ReservoirBuf& out, int32_t* ray_of,
                                         const Queue& rays, const InitialState& st, const Queue& vis, int n_sm,
                                         cudaStream_t stream);
cudaError_t launch_restir_spatial(const SceneView& s, const RenderConst& rc, const RestirConst& k, const GBuffer& gb,
                                  const ReservoirBuf& in, const ReservoirBuf& out, int pass, uint32_t neighbor_seed,
                                  int32_t* ray_of, const Queue& rays, const InitialState& st, const Queue& vis,
                                  int n_sm, cudaStream_t stream);
cudaError_t launch_accumulate(const RenderConst& rc, const PathBuffers& pb, float* acc32, double* acc64, int n_sm,
                              cudaStream_t st);
// Batched rendering (jobs: device table of n_jobs; iteration: device index of the iteration):
// camera rays of every job's samples of this iteration appended to q; per-job accumulation, then
// the completion stamps (global timer, ns) of the jobs that finish and the iteration advance.
cudaError_t launch_batch_camera(const BatchJob* jobs, int n_jobs, int64_t max_job_paths, const PathBuffers& pb,
                                const Queue& q, const int32_t* iteration, unsigned long long* stats, int n_sm,
                                cudaStream_t st);
cudaError_t launch_batch_accumulate(const BatchJob* jobs, int n_jobs, int64_t max_job_pixels, const PathBuffers& pb,
                                    const int32_t* iteration, float* acc32, double* acc64, int32_t* iteration_rw,
                                    unsigned long long* done_ns, int n_sm, cudaStream_t st);
// Writes the global timer (ns) to *out
cudaError_t launch_stamp(unsigned long long* out, cudaStream_t st);

}  // namespace gbpt
