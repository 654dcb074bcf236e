// ReSTIR DI state shared by the host glue and the kernels (internal to libgbpt).
//
// Reservoir record (32 B, two 16-byte words per pixel, SoA):
//   s = (point on the light xyz, target function p_hat at the owning pixel)
//   w = (emissive triangle index, (M << 9) | sample flags, weight_sum bits, UCW bits)
// Sample flags follow the reference's ReSTIRDISampleFlags (src/Device/includes/ReSTIR/DI/
// SampleFlags.h): bits 1-6 = the BSDF lobe a BSDF candidate was sampled from, bit 7 = unoccluded.
// G-buffer (per pixel, SoA): pos = (P, primitive bits, -1 = no hit), ns = (shading normal,
// material index bits), ng = (geometric normal, 1 if the camera ray is inside a transmissive
// object).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gbpt {

constexpr int kRestirFlagUnoccluded = 1 << 7;
constexpr int kRestirLobeMask = 0x7E;

struct GBuffer
{
    float4* pos;
    float4* ns;
    float4* ng;
};

struct ReservoirBuf
{
    float4* s;
    int4* w;
};

// Per-pixel state of the initial-candidates phases: the pending BSDF candidate (direction, pdf)
// and (PCG state low, high, lobe or a status below, queue index of the pixel's ray or -1).
struct InitialState
{
    float4* cand;
    int4* meta;
};
constexpr int kInitialDone = -1;        // no candidates (no surface or no emitter): reservoir final
constexpr int kInitialVisibility = -2;  // candidates done; meta.w = index in the visibility queue

struct RestirConst
{
    int32_t light_candidates, bsdf_candidates;
    int32_t visibility_reuse;
    int32_t do_temporal, temporal_search_count;
    float temporal_search_radius;
    int32_t do_spatial, spatial_passes, spatial_neighbors;
    float spatial_radius;
    int32_t m_cap, confidence_weights, bias_correction_visibility, final_visibility;
    float normal_similarity_cos, plane_distance;
    uint32_t frame, seed;
    int32_t has_prev;
    float camera_pos[3];
    float prev_camera_pos[3];
    float prev_view_projection[16];
    // light presampling (null: off): presample_subsets x presample_size records of two float4,
    // (point on the light, triangle bits) and (light normal, area pdf); the pixels of a
    // presample_tile^2 block share the subset that presample_seed picks for the frame
    const float4* presampled;
    int32_t presample_subsets, presample_size, presample_tile;
    uint32_t presample_seed;
    // GBPT_RNG_REFERENCE: each pass seeds a Xorshift32 per pixel from its own random number and the
    // sample number, as the reference's passes do (InitialCandidates.h:500-505,
    // TemporalReuse.h:69-74, SpatialReuse.h:62-69); the G-buffer holds the reference's packed
    // normals and the surfaces read the packed camera-hit materials
    int32_t rng_mode;
    uint32_t sample_number, rn_initial, rn_temporal, rn_spatial[4];
};

#ifdef __CUDACC__
}  // namespace gbpt
#include "render_common.h"
namespace gbpt {

struct Reservoir
{
    V3 point;
    float p_hat;
    int tri;
    int flags;
    int M;
    float w_sum;
    float ucw;
};

__device__ __forceinline__ Reservoir empty_reservoir()
{
    Reservoir r;
    r.point = v3(0.0f);
    r.p_hat = 0.0f;
    r.tri = -1;
    r.flags = 0;
    r.M = 0;
    r.w_sum = 0.0f;
    r.ucw = 0.0f;
    return r;
}

__device__ __forceinline__ Reservoir load_reservoir(const ReservoirBuf& b, int i)
{
    const float4 s = b.s[i];
    const int4 w = b.w[i];
    Reservoir r;
    r.point = xyz(s);
    r.p_hat = s.w;
    r.tri = w.x;
    r.flags = w.y & 0x1FF;
    r.M = (int)((unsigned)w.y >> 9);
    r.w_sum = __int_as_float(w.z);
    r.ucw = __int_as_float(w.w);
    return r;
}

__device__ __forceinline__ void store_reservoir(const ReservoirBuf& b, int i, const Reservoir& r)
{
    b.s[i] = f4(r.point, r.p_hat);
    b.w[i] = make_int4(r.tri, (r.M << 9) | (r.flags & 0x1FF), __float_as_int(r.w_sum), __float_as_int(r.ucw));
}

#endif  // __CUDACC__

}  // namespace gbpt
