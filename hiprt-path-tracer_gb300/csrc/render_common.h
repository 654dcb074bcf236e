// Device-side data layout and math shared by the wavefront path-tracing kernels.
//
// Restates, for sm_103a, the reference's per-vertex estimator of the megakernel path
// (src/Device/kernels/Megakernel.h:23-144) with direct lighting by 'sample_one_light_MIS'
// (src/Device/includes/LightSampling/Lights.h:123-226): one light sample with a shadow ray and one
// separate BSDF sample with its own ray, combined by the balance heuristic
// (src/Device/includes/Sampling.h:103-116); emission added at the camera hit only
// (Lights.h:384-389); continuation by a second BSDF sample with Russian roulette
// (src/Device/includes/PathTracing.h:44-101, src/Device/includes/RussianRoulette.h:20-55).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gbpt_bsdf.h"
#include "../../include/gbpt_render.h"
#include "hd_math.h"

namespace gbpt {

using namespace hd;

// ---------------------------------------------------------------------------------------------
// scene view and per-path buffers (all device pointers)
// ---------------------------------------------------------------------------------------------
struct DeviceMaterial
{
    float4 base_color;  // rgb, w unused
    float4 emission;    // rgb = emission colour * strength, w unused
};

// The world around the scene (WorldSettings, src/HostDeviceCommon/WorldSettings.h:14-53): nothing,
// a uniform colour, or an equirectangular Y-up environment map. Texel (x, y) covers u in
// [x/W, (x+1)/W), v in [y/H, (y+1)/H); v = 0 is the -y pole. Device pointers.
struct EnvView
{
    const uint32_t* texels;  // RGB9E5 shared-exponent texels (RGBE9995Packed), W*H
    const float* cdf;        // running luminance sum over texels in row-major order (binary search)
    const uint2* alias;      // per texel: (probability as float bits, alias index) (alias table)
    int32_t width, height;
    float intensity;         // envmap_intensity
    float total_sum;         // luminance sum of the unscaled texels (envmap_total_sum)
    float to_world[9];       // row-major rotation, world direction = to_world * envmap direction
    float to_env[9];         // its inverse
    float uniform[3];        // uniform_light_color
    int32_t ambient;         // GBPT_AMBIENT_*
    int32_t sampling;        // GBPT_ENVMAP_* (EnvmapSamplingStrategy)
    int32_t bsdf_mis;        // EnvmapSamplingDoBSDFMIS
    int32_t bilinear;        // EnvmapSamplingDoBilinearFiltering
    int32_t scale_background;  // envmap_scale_background_intensity
};

struct SceneView
{
    const float4* vertices;       // xyz per vertex
    const int32_t* indices;       // 3 per triangle
    const int32_t* material_of;   // per triangle
    const DeviceMaterial* materials;
    const int32_t* emissive;      // emissive triangle indices
    const float* alias_prob;      // power alias table (per emissive triangle)
    const int32_t* alias_index;
    float power_sum;              // sum of luminance(emission) * area over emissive triangles
    int32_t n_emissive;
    const uint4* bvh_nodes;
    const float4* bvh_tris;
    const gbpt_principled_material* pmats;  // effective principled materials (NULL: Lambertian scene)
    // packed materials (GBPT_MATERIALS_PACKED): the effective materials packed again, as the
    // reference's G-buffer stores the camera hit's material (NULL otherwise)
    const gbpt_principled_material* pmats_camera;
    EnvView env;
    const float4* normals;        // per vertex: smooth-shading normal, w = 1 when present (NULL: none)
};

struct Queue
{
    float4* origin_tmin;
    float4* dir_tmax;
    int32_t* last_prim;
    int32_t* slot;
    float4* hits;       // closest-hit output (extension and BSDF-light rays)
    uint8_t* occluded;  // any-hit output (shadow rays)
    int32_t* count;     // device counter
};

struct PathBuffers
{
    float4* throughput;     // rgb
    float4* radiance;       // rgb accumulated over the path
    uint64_t* rng;          // PCG state
    float4* pending_light;  // light-sample contribution waiting on its shadow ray
    float4* pending_bsdf;   // rgb = throughput * f * cos / pdf, w = BSDF pdf
    int32_t* shadow_entry;  // queue index of the slot's shadow ray this bounce, -1 if none
    int32_t* bsdf_entry;    // queue index of the slot's BSDF-light ray this bounce, -1 if none
    uint4* vol_stack;       // principled paths: the nested-dielectric stack (volume.h), 4 entries
    int4* vol_state;        // its incident / outgoing materials, position | inside << 8, distance
    float* wavelength;      // principled paths: the wavelength (nm) drawn at the first dispersive
                            // hit, negative until its colour filter is applied; 0: none yet
    int32_t* job;           // batched rendering: the job of each slot (null for a single renderer)
    float4* ris;            // RIS vertex: throughput before the continuation (rgb) and the light
                            // candidates' weight sum (w); w = -0.5: RIS without light candidates,
                            // w = -1: not a RIS vertex
    float* ris_u;           // GBPT_RNG_REFERENCE (null otherwise): the BSDF candidate's reservoir
                            // draw, taken where the reference draws it (before the continuation)
    // guided rendering (null otherwise): the one-sample MIS pdf of each path's last continuation
    // when it was a guided continuation (which doubles as next-event estimation's BSDF technique),
    // else 0; emission found by the next extension ray is weighted against light sampling with it
    float* guide_pdf;
    // environment-map direct lighting (null when the scene's envmap is not importance sampled):
    // the envmap sample's and the separate BSDF sample's contributions, each waiting on its
    // any-hit ray in the envmap queue
    int32_t* env_entry;     // queue index of the envmap-sample ray this bounce, -1 if none
    int32_t* envb_entry;    // queue index of the BSDF-sample ray this bounce, -1 if none
    float4* pending_env;
    float4* pending_envb;
};

// Learned path guiding in the wavefront (all device pointers; lobes == nullptr: guiding off).
// The continuation of a guidable vertex is drawn from the network's vMF mixture with probability
// alpha (the network's selection output, or 'prob' when that is > 0), else from the BSDF, and
// weighted by the one-sample MIS pdf alpha q + (1 - alpha) p_bsdf.
// Training records hold (position, normal, view, direction) and a weight, the MIS-weighted estimate
// of f cos L_i / pdf of that direction, for the two techniques of a recorded vertex:
//   continuation: throughput before the continuation and the path radiance after the light sample;
//                 after the launch the weight is luminance((final radiance - snapshot) / throughput)
//   light sample: weight = luminance(f cos Le w_light / p_light), zeroed if the shadow ray is
//                 occluded (slot -1: no snapshot)
// Vertices are recorded when a hash of (slot, bounce, frame) is below a device-side threshold that
// the end of each launch adapts to the launch's number of candidate vertices.
struct GuideView
{
    const float* lobes;  // per entry of the shaded queue: 8 x (mu xyz, kappa, weight), alpha
    float* in_pos;       // per queue entry: network inputs (3 floats each)
    float* in_nrm;
    float* in_view;
    float prob;
    int32_t* train_entry;        // per path slot: continuation record made at this bounce, -1 (null: no training)
    int32_t* train_light_entry;  // per path slot: light-sample record made at this bounce, -1
    float* rec_pos;        // per record: 3 floats each
    float* rec_nrm;
    float* rec_view;
    float* rec_dir;
    float4* rec_tp;
    float4* rec_snap;
    float* rec_weight;
    float* rec_pbsdf;  // BSDF pdf of the recorded direction (trains the selection probability)
    int32_t* rec_slot;
    int32_t* rec_count;
    int32_t* rec_candidates;         // guided vertices seen this launch
    uint32_t* rec_threshold;         // a vertex is recorded when its hash is below this (device)
    int32_t rec_cap;
    uint32_t frame;
    float weight_clamp;      // 0: none
};

#ifdef __CUDACC__
// ---------------------------------------------------------------------------------------------
// small vector helpers (the float3 type and operators shared with the BSDF live in hd_math.h)
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ V3 xyz(float4 f) { return v3(f.x, f.y, f.z); }
__device__ __forceinline__ float4 f4(V3 a, float w) { return make_float4(a.x, a.y, a.z, w); }

// ---------------------------------------------------------------------------------------------
// Random numbers of a path: one 64-bit state per path slot, two generators behind one interface.
//  - inc != 0: PCG32 (O'Neill 2014), stream selected by the render seed (the default);
//  - inc == 0: the reference's Xorshift32Generator (src/HostDeviceCommon/Xorshift.h:18-66) on the
//    low 32 bits of 'state' (GBPT_RNG_REFERENCE): xorshift 13/17/5, floats x / 2^32 clamped to
//    1 - 1e-7, random_index(n) = floor(x / 2^32 * n) clamped to n - 1. (float)x rounds to nearest
//    as the reference's conversion does, and x * 2^-32 equals its division by float(0xffffffff).
// ---------------------------------------------------------------------------------------------
struct Pcg32
{
    uint64_t state;
    uint64_t inc;

    __device__ __forceinline__ uint32_t next_u32()
    {
        if (inc == 0)
        {
            uint32_t x = (uint32_t)state;
            x ^= x << 13;
            x ^= x >> 17;
            x ^= x << 5;
            state = x;
            return x;
        }
        const uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        const uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        const uint32_t rot = (uint32_t)(old >> 59u);
        return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
    }
    // uniform float in [0, 1)
    __device__ __forceinline__ float next()
    {
        if (inc == 0) return fminf((float)next_u32() * (1.0f / 4294967296.0f), 1.0f - 1.0e-7f);
        return (float)(next_u32() >> 8) * (1.0f / 16777216.0f);
    }
    __device__ __forceinline__ float operator()() { return next(); }
    __device__ __forceinline__ int index(int n)
    {
        if (inc == 0)
        {
            const int i = (int)(__fmul_rn((float)next_u32() * (1.0f / 4294967296.0f), (float)n));
            return i < n - 1 ? i : n - 1;
        }
        int i = (int)(next() * (float)n);
        return i < n - 1 ? i : n - 1;
    }
};

// wang_hash (src/Device/includes/Hash.h:11-19)
__device__ __forceinline__ uint32_t wang_hash(uint32_t s)
{
    s = (s ^ 61u) ^ (s >> 16);
    s *= 9u;
    s = s ^ (s >> 4);
    s *= 0x27d4eb2du;
    s = s ^ (s >> 15);
    return s;
}

// The reference's generator of one pixel sample: Xorshift32 seeded by
// wang_hash((pixel + 1) * (sample_number + 1) * random_number), 32-bit wrap-around products
// (CameraRays.h:155-160, Megakernel.h:52-57).
__device__ __forceinline__ Pcg32 reference_seed(uint32_t pixel, uint32_t sample_number, uint32_t random_number)
{
    Pcg32 r;
    r.state = wang_hash((pixel + 1u) * (sample_number + 1u) * random_number);
    r.inc = 0;
    return r;
}

__device__ __forceinline__ uint64_t pcg_inc(uint32_t seed) { return ((uint64_t)seed << 1u) | 1u; }

// splitmix64 finaliser: decorrelates (pixel, iteration) into an initial PCG state
__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

__device__ __forceinline__ Pcg32 pcg_seed(uint32_t pixel, uint32_t iteration, uint32_t seed)
{
    Pcg32 r;
    r.state = 0;
    r.inc = pcg_inc(seed);
    r.next_u32();
    r.state += mix64(((uint64_t)iteration << 32) | pixel);
    r.next_u32();
    return r;
}

// Row-major 4x4 times point (w = 1) with perspective divide, as the reference's matrix_X_point
// (src/HostDeviceCommon/Math.h:617-640).
__device__ __forceinline__ V3 mat_x_point(const float* m, V3 p)
{
    float x = m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3];
    float y = m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7];
    float z = m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11];
    float w = m[12] * p.x + m[13] * p.y + m[14] * p.z + m[15];
    float inv_w = 1.0f;
    if (!(w < 1.0e-10f && w > -1.0e-10f)) inv_w = 1.0f / w;
    return v3(x * inv_w, y * inv_w, z * inv_w);
}

// Octahedral24BitNormalPadded32b pack then unpack (src/HostDeviceCommon/Packing.h:237-367; the
// octahedral map of Cigolle et al. 2014): the reference's G-buffer stores its camera-hit normals
// as two 12-bit snorms in three bytes. Every step is exact or a single rounding (no contraction
// changes a result), so the round trip matches the reference's bit for bit up to the final
// normalisation.
__device__ __forceinline__ float sign_nz(float k) { return k >= 0.0f ? 1.0f : -1.0f; }
__device__ __forceinline__ V3 oct24_roundtrip(V3 n)
{
    const float l1 = __fdiv_rn(1.0f, __fadd_rn(__fadd_rn(fabsf(n.x), fabsf(n.y)), fabsf(n.z)));
    float ex = __fmul_rn(n.x, l1), ey = __fmul_rn(n.y, l1);
    if (n.z < 0.0f)
    {
        const float ax = fabsf(ey), ay = fabsf(ex);
        ex = (1.0f - ax) * sign_nz(ex);
        ey = (1.0f - ay) * sign_nz(ey);
    }
    const float sx = roundf(__fmul_rn(fminf(fmaxf(ex + 1.0f, 0.0f), 2.0f), 2047.0f));
    const float sy = roundf(__fmul_rn(fminf(fmaxf(ey + 1.0f, 0.0f), 2.0f), 2047.0f));
    // the two 12-bit values round-trip through the three bytes unchanged (integer arithmetic)
    const float px = sx, py = sy;
    const float dx = fminf(fmaxf(__fdiv_rn(px, 2047.0f) - 1.0f, -1.0f), 1.0f);
    const float dy = fminf(fmaxf(__fdiv_rn(py, 2047.0f) - 1.0f, -1.0f), 1.0f);
    V3 v = v3(dx, dy, 1.0f - fabsf(dx) - fabsf(dy));
    if (v.z < 0.0f)
    {
        const float tx = v.x, ty = v.y;
        v.x = (1.0f - fabsf(ty)) * sign_nz(tx);
        v.y = (1.0f - fabsf(tx)) * sign_nz(ty);
    }
    return normalize(v);
}

// GBPT_RNG_REFERENCE, camera hit: the vertex as the reference's MegaKernel rebuilds it from its
// packed G-buffer (Megakernel.h:59-70): octahedral-24 normals written after the backface fix
// (CameraRays.h:178-181) and renormalised on read, and the view direction from the camera
// position (the translation column of the inverse view, Camera::to_hiprt) to the stored hit
// point (GBufferDevice::get_view_direction), negated into a ray direction, normalised and negated.
__device__ __forceinline__ void reference_gbuffer_vertex(const float* inverse_view, V3 P, V3& ng, V3& ns, V3& view)
{
    ng = normalize(oct24_roundtrip(ng));
    ns = normalize(oct24_roundtrip(ns));
    const V3 cam = v3(inverse_view[3], inverse_view[7], inverse_view[11]);
    view = -normalize(-normalize(cam - P));
}

// ---------------------------------------------------------------------------------------------
// sampling helpers
// ---------------------------------------------------------------------------------------------

// Cosine-weighted direction around n: normalize(n + uniform point on the unit sphere)
// (the construction of src/Device/includes/Sampling.h:180-201).
__device__ __forceinline__ V3 cosine_sample(V3 n, float r1, float r2u)
{
    float r2 = 2.0f * r2u - 1.0f;
    if (r1 < 1.0e-8f && r2 < -0.999999f && n.z > 0.999999f)
    {
        r1 += 1.0e-7f;
        r2 += 1.0e-7f;
    }
    const float theta = kTwoPi * r1;
    const float s = sqrtf(fmaxf(0.0f, 1.0f - r2 * r2));
    float st, ct;
    sincosf(theta, &st, &ct);
    return normalize(n + v3(s * ct, s * st, r2));
}

// Heitz 2019 square-to-triangle map (src/Device/includes/LightSampling/LightUtils.h:150-164).
__device__ __forceinline__ void square_to_triangle(float& x, float& y)
{
    if (y > x)
    {
        x *= 0.5f;
        y -= x;
    }
    else
    {
        y *= 0.5f;
        x -= y;
    }
}

__device__ __forceinline__ float balance_heuristic(float pdf_a, float pdf_b)
{
    if (pdf_a == 0.0f) return 0.0f;
    return pdf_a / (pdf_a + pdf_b);
}

__device__ __forceinline__ float area_to_solid_angle_pdf(float area_pdf, float dist, float cos_light)
{
    if (cos_light < 1.0e-8f) return 0.0f;
    return area_pdf * dist * dist / cos_light;
}

__device__ __forceinline__ void load_triangle(const SceneView& s, int prim, V3& a, V3& b, V3& c)
{
    const int i0 = __ldg(s.indices + 3 * prim), i1 = __ldg(s.indices + 3 * prim + 1), i2 = __ldg(s.indices + 3 * prim + 2);
    a = xyz(__ldg(s.vertices + i0));
    b = xyz(__ldg(s.vertices + i1));
    c = xyz(__ldg(s.vertices + i2));
}

// get_shading_normal (src/Device/includes/Intersect.h:114-134) without normal maps: the vertex
// normals interpolated at the hit's barycentrics (uv_interpolate, src/Device/includes/Texture.h:248-251)
// when the triangle's first vertex has one, else the geometric normal. Called before the backface fix.
__device__ __forceinline__ V3 shading_normal(const SceneView& s, int prim, float u, float v, V3 ng)
{
    if (!s.normals) return ng;
    const int i0 = __ldg(s.indices + 3 * prim);
    const float4 n0 = __ldg(s.normals + i0);
    if (n0.w == 0.0f) return ng;
    const float4 n1 = __ldg(s.normals + __ldg(s.indices + 3 * prim + 1));
    const float4 n2 = __ldg(s.normals + __ldg(s.indices + 3 * prim + 2));
    return normalize(xyz(n1) * u + xyz(n2) * v + xyz(n0) * (1.0f - u - v));
}

#endif  // __CUDACC__

}  // namespace gbpt
