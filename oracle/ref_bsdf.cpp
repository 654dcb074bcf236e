/*
 * TEST INFRASTRUCTURE ONLY — C entry points into the reference's OWN principled BSDF, compiled
 * from the reference's sources where they lie (oracle/Makefile, target 'ref'), behind the
 * clean-room shim headers in oracle/shim/. Output goes to oracle/_ref/ (git-ignored). Used by
 * tests/golden/make_bsdf_golden.py to write the golden vectors that pin this project's BSDF.
 *
 * Calls, unmodified: principled_bsdf_eval / principled_bsdf_pdf / principled_bsdf_sample
 * (src/Device/includes/BSDFs/Principled.h:1620-1941).
 * Compile-time options, set below after the reference's option headers and before the BSDF code
 * is parsed (their #ifndef guards make these the values the BSDF sees):
 *   - PrincipledBSDFDoEnergyCompensation = false: the energy-compensation terms need the
 *     precomputed directional-albedo tables of data/BRDFsData, which this project does not ship;
 *   - PrincipledBSDFDoMicrofacetRegularization = false: regularization is biased, and the
 *     unbiasedness tests need it off (it is a path-space heuristic, not part of the BSDF);
 *   - everything else at the reference's defaults (Lambertian diffuse lobe, Heitz 2018 VNDF
 *     sampling, height-uncorrelated Smith masking-shadowing (BRDFsData default), delta-distribution optimisation on, no fresnel-based lobe sampling).
 * Material layout: gbpt_principled_material (include/gbpt_bsdf.h), 64 words per material.
 * Query layout (16 floats): view(3), shading normal(3), geometric normal(3), to_light(3),
 * eta_incident, eta_outgoing, inside (0/1), incident light info (integer value as float).
 */
#include "HostDeviceCommon/KernelOptions/KernelOptions.h"

#ifdef REF_DIFFUSE_LOBE
#undef PrincipledBSDFDiffuseLobe
#define PrincipledBSDFDiffuseLobe REF_DIFFUSE_LOBE
#endif
#undef PrincipledBSDFDoEnergyCompensation
#define PrincipledBSDFDoEnergyCompensation KERNEL_OPTION_FALSE
#undef PrincipledBSDFDoMicrofacetRegularization
#define PrincipledBSDFDoMicrofacetRegularization KERNEL_OPTION_FALSE

#include "Device/includes/BSDFs/Principled.h"

#include <cmath>
#include <cstdint>
#include <cstring>

namespace {

DeviceUnpackedEffectiveMaterial unpack(const float* w)
{
    DeviceUnpackedEffectiveMaterial m;
    m.base_color = ColorRGB32F(w[0], w[1], w[2]);
    m.roughness = w[3];
    m.emission = ColorRGB32F(w[4], w[5], w[6]);
    m.metallic = w[7];
    m.metallic_F82 = ColorRGB32F(w[8], w[9], w[10]);
    m.metallic_F90_falloff_exponent = w[11];
    m.metallic_F90 = ColorRGB32F(w[12], w[13], w[14]);
    m.anisotropy = w[15];
    m.anisotropy_rotation = w[16];
    m.second_roughness_weight = w[17];
    m.second_roughness = w[18];
    m.specular = w[19];
    m.specular_color = ColorRGB32F(w[20], w[21], w[22]);
    m.specular_tint = w[23];
    m.specular_darkening = w[24];
    m.coat = w[25];
    m.coat_roughness = w[26];
    m.coat_roughening = w[27];
    m.coat_medium_absorption = ColorRGB32F(w[28], w[29], w[30]);
    m.coat_medium_thickness = w[31];
    m.coat_darkening = w[32];
    m.coat_anisotropy = w[33];
    m.coat_anisotropy_rotation = w[34];
    m.coat_ior = w[35];
    m.sheen = w[36];
    m.ior = w[37];
    m.specular_transmission = w[38];
    m.diffuse_transmission = w[39];
    m.absorption_color = ColorRGB32F(w[40], w[41], w[42]);
    m.absorption_at_distance = w[43];
    int32_t thin;
    std::memcpy(&thin, w + 44, 4);
    m.thin_walled = thin != 0;
    m.oren_nayar_sigma = w[46];
    m.thin_film = w[47];
    m.thin_film_ior = w[48];
    m.thin_film_thickness = w[49];
    m.thin_film_kappa_3 = w[50];
    m.thin_film_hue_shift_degrees = w[51];  // the unpacked material holds turns (degrees / 360)
    m.thin_film_base_ior_override = w[52];
    int32_t tf_override;
    std::memcpy(&tf_override, w + 53, 4);
    m.thin_film_do_ior_override = tf_override != 0;
    m.dispersion_scale = w[54];
    m.dispersion_abbe_number = w[55];
    return m;
}

// Render data and volume state for one query: the incident medium is material slot 0 of a
// two-entry IOR table, the outgoing medium slot 1 (air = MAX_MATERIAL_INDEX when its IOR is 1).
struct Ctx
{
    HIPRTRenderData rd;
    float iors[2];
    ColorRGB24bFloat0_1Packed absorption[2];
    float absorption_distance[2] = {1.0f, 1.0f};
    RayVolumeState vs;
    // absorption: the colour of the material slot the ray travels in (Beer-Lambert when leaving
    // a volume, Principled.h:332-357); the golden materials use white (no absorption)
    Ctx(const float* q, const DeviceUnpackedEffectiveMaterial& m, float wavelength = 0.0f)
    {
        iors[0] = q[12];
        iors[1] = q[13];
        absorption[0].set_color(m.absorption_color);
        absorption[1].set_color(m.absorption_color);
        absorption_distance[0] = absorption_distance[1] = m.absorption_at_distance;
        rd.buffers.materials_buffer.ior = iors;
        rd.buffers.materials_buffer.absorption_color_packed = absorption;
        rd.buffers.materials_buffer.absorption_at_distance = absorption_distance;
        vs.incident_mat_index = q[12] == 1.0f ? NestedDielectricsInteriorStack::MAX_MATERIAL_INDEX : 0;
        vs.outgoing_mat_index = q[13] == 1.0f ? NestedDielectricsInteriorStack::MAX_MATERIAL_INDEX : 1;
        vs.inside_material = q[14] != 0.0f;
        vs.sampled_wavelength = wavelength;
        // a NaN caught by the BSDF's CPU sanity check is zeroed rather than written to the
        // (absent) frame buffer
        rd.render_settings.display_NaNs = false;
    }
};

float3 f3(const float* p) { return make_float3(p[0], p[1], p[2]); }

void eval_query(const float* mat, const float* q, float* out, float wavelength = 0.0f)
{
    DeviceUnpackedEffectiveMaterial m = unpack(mat);
    Ctx c(q, m, wavelength);
    BSDFIncidentLightInfo info = (BSDFIncidentLightInfo)(int)q[15];
    BSDFContext ctx(f3(q), f3(q + 3), f3(q + 6), f3(q + 9), info, c.vs, false, m, 0, 0.0f);
    float pdf = 0.0f;
    ColorRGB32F col = principled_bsdf_eval(c.rd, ctx, pdf);
    out[0] = col.r;
    out[1] = col.g;
    out[2] = col.b;
    out[3] = pdf;
}

void sample_query(const float* mat, const float* q, uint32_t seed, float* o, int32_t* lobe, uint32_t* rng_after,
                  float wavelength = 0.0f)
{
    DeviceUnpackedEffectiveMaterial m = unpack(mat);
    Ctx c(q, m, wavelength);
    BSDFIncidentLightInfo info = BSDFIncidentLightInfo::NO_INFO;
    BSDFContext ctx(f3(q), f3(q + 3), f3(q + 6), make_float3(0.0f, 0.0f, 0.0f), info, c.vs, false, m, 0, 0.0f);
    Xorshift32Generator rng(seed);
    float3 dir = make_float3(0.0f, 0.0f, 0.0f);
    float pdf = 0.0f;
    ColorRGB32F col = principled_bsdf_sample(c.rd, ctx, dir, pdf, rng);
    o[0] = dir.x;
    o[1] = dir.y;
    o[2] = dir.z;
    o[3] = col.r;
    o[4] = col.g;
    o[5] = col.b;
    o[6] = pdf;
    o[7] = 0.0f;
    *lobe = (int32_t)info;
    *rng_after = rng.m_state.seed;
}

}  // namespace

extern "C" {
// the entry points stay visible in a build with -fvisibility=hidden (the Oren-Nayar build, whose
// inline reference functions must not bind to the default build's)
#pragma GCC visibility push(default)

/* out: 4 floats per query (rgb, pdf). wavelengths (may be NULL): the path's sampled wavelength
 * per query (RayVolumeState::sampled_wavelength), for dispersive materials. */
void ref_principled_eval(const float* mats, const int32_t* mat_index, const float* queries, const float* wavelengths,
                         int64_t n, float* out)
{
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; i++)
        eval_query(mats + 64 * (int64_t)mat_index[i], queries + 16 * i, out + 4 * i, wavelengths ? wavelengths[i] : 0.0f);
}

void ref_principled_pdf(const float* mats, const int32_t* mat_index, const float* queries, const float* wavelengths,
                        int64_t n, float* out)
{
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; i++)
    {
        const float* q = queries + 16 * i;
        DeviceUnpackedEffectiveMaterial m = unpack(mats + 64 * (int64_t)mat_index[i]);
        Ctx c(q, m, wavelengths ? wavelengths[i] : 0.0f);
        BSDFIncidentLightInfo info = (BSDFIncidentLightInfo)(int)q[15];
        BSDFContext ctx(f3(q), f3(q + 3), f3(q + 6), f3(q + 9), info, c.vs, false, m, 0, 0.0f);
        out[i] = principled_bsdf_pdf(c.rd, ctx);
    }
}

/* Samples with a Xorshift32 generator seeded by seeds[i]. out: 8 floats per query
 * (direction xyz, rgb, pdf, 0); info_out = the lobe the direction was sampled from;
 * rng_out = generator state after sampling (counts the draws). */
void ref_principled_sample(const float* mats, const int32_t* mat_index, const float* queries, const float* wavelengths,
                           const uint32_t* seeds, int64_t n, float* out, int32_t* info_out, uint32_t* rng_out)
{
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; i++)
        sample_query(mats + 64 * (int64_t)mat_index[i], queries + 16 * i, seeds[i], out + 8 * i, info_out + i, rng_out + i,
                     wavelengths ? wavelengths[i] : 0.0f);
}

/* Single-query forms with the same layouts, handed to the path-tracing oracle (pt_oracle.cpp) as
 * function pointers so that it shades with the reference's own BSDF. The sample form returns in
 * out[7] the bits of the Xorshift32 state after sampling. */
void ref_principled_eval_one(const float* mat, const float* q, float* out) { eval_query(mat, q, out); }

void ref_principled_sample_one(const float* mat, const float* q, uint32_t seed, float* out, int32_t* lobe)
{
    uint32_t rng_after;
    sample_query(mat, q, seed, out, lobe, &rng_after);
    // With a thin film the glass lobe can pick refraction at a totally reflecting interface, where
    // the reference's refraction gives a NaN direction (and pdf). The path-tracing oracle needs a
    // defined outcome there: the sample is reported as no direction, f = 0, pdf = 0 (the path
    // ends), which is what the library's BSDF returns in that case.
    if (!std::isfinite(out[0]) || !std::isfinite(out[1]) || !std::isfinite(out[2]))
    {
        out[0] = q[3];
        out[1] = q[4];
        out[2] = q[5];
        out[3] = out[4] = out[5] = out[6] = 0.0f;
    }
    std::memcpy(out + 7, &rng_after, 4);  // the generator's state after sampling, bit for bit
}

#pragma GCC visibility pop
}  // extern "C"
