/*
 * gbpt — principled BSDF: material record and batched eval / pdf / sample entry points.
 *
 * The material mirrors the reference's DeviceUnpackedEffectiveMaterial
 * (src/HostDeviceCommon/Material/MaterialUnpacked.h) as a plain 256-byte record. The BSDF is the
 * reference's layered principled BSDF (src/Device/includes/BSDFs/Principled.h:1515-1941): coat,
 * sheen, two metal lobes, specular over diffuse, glass and diffuse transmission, blended by the
 * same lobe weights and sampled with the same lobe probabilities.
 * Built without: energy compensation (it needs the reference's precomputed directional-albedo
 * tables), microfacet regularization (biased) and the sheen
 * lobe: the entry points below treat 'sheen' as 0, and scene creation rejects materials with
 * sheen > 0 (GBPT_ERROR_UNSUPPORTED). A query whose material index is out of range returns zeros.
 * See gbpt.h for status codes; all pointers below are device pointers.
 */
#ifndef GBPT_BSDF_H
#define GBPT_BSDF_H

#include "gbpt.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Effective (post-texture, post-coat-roughening) material, 64 words. Defaults as the reference. */
typedef struct gbpt_principled_material {
    float base_color[3];
    float roughness;
    float emission[3];             /* colour * strength * global emissive factor */
    float metallic;
    float metallic_F82[3];
    float metallic_F90_falloff_exponent;
    float metallic_F90[3];
    float anisotropy;
    float anisotropy_rotation;     /* in half turns (times pi radians) */
    float second_roughness_weight;
    float second_roughness;
    float specular;
    float specular_color[3];
    float specular_tint;
    float specular_darkening;
    float coat;
    float coat_roughness;
    float coat_roughening;         /* applied on the host before upload (Material.h:122-146) */
    float coat_medium_absorption[3];
    float coat_medium_thickness;
    float coat_darkening;
    float coat_anisotropy;
    float coat_anisotropy_rotation;
    float coat_ior;
    float sheen;                   /* not built: treated as 0 */
    float ior;
    float specular_transmission;
    float diffuse_transmission;
    float absorption_color[3];
    float absorption_at_distance;
    int32_t thin_walled;
    int32_t diffuse_lobe;          /* GBPT_DIFFUSE_* [GBPT_DIFFUSE_LAMBERTIAN] */
    float oren_nayar_sigma;        /* GBPT_DIFFUSE_OREN_NAYAR: roughness, the standard deviation of
                                      the facet slope angle in radians (the reference's default is
                                      20 degrees, 0.349066) */
    /* thin-film interference over the metal, specular and glass interfaces (Belcour and Barla
     * 2017, the reference's thin_film_fresnel, src/Device/includes/BSDFs/ThinFilm.h:124-226):
     * each lobe's Fresnel term becomes lerp(its own, the film's RGB reflectance, thin_film) */
    float thin_film;               /* weight in [0, 1] [0] */
    float thin_film_ior;           /* the film's IOR [1.3] */
    float thin_film_thickness;     /* nanometres [500] */
    float thin_film_kappa_3;       /* extinction of the base under the film, with the override [0] */
    float thin_film_hue_shift;     /* in turns (degrees / 360, as the reference's unpacked material) [0] */
    float thin_film_base_ior_override; /* the base's IOR under the film, with the override [1] */
    int32_t thin_film_do_ior_override; /* 0: the base is the material's own IOR, kappa 0 */
    /* dispersion of the glass lobe (the reference's compute_dispersion_ior,
     * src/Device/includes/Dispersion.h:485-499, OpenPBR's Cauchy fit from the Abbe number): the
     * glass lobe's IORs become those at the path's sampled wavelength when dispersion_scale > 0 */
    float dispersion_scale;        /* [0] */
    float dispersion_abbe_number;  /* [20] */
    int32_t reserved[8];
} gbpt_principled_material;

/* The diffuse lobe of the principled BSDF's glossy base (gbpt_principled_material.diffuse_lobe):
 * the reference selects one for all materials at compile time (PrincipledBSDFDiffuseLobe,
 * src/HostDeviceCommon/KernelOptions/PrincipledBSDFKernelOptions.h:63-72), here per material:
 *   GBPT_DIFFUSE_LAMBERTIAN: base_color / pi (the reference's default);
 *   GBPT_DIFFUSE_OREN_NAYAR: the Oren-Nayar qualitative model (src/Device/includes/BSDFs/
 *     OrenNayar.h:14-63, MaterialUtils::get_oren_nayar_AB), sampled by the cosine distribution. */
enum { GBPT_DIFFUSE_LAMBERTIAN = 0, GBPT_DIFFUSE_OREN_NAYAR = 1 };

/* Which lobe a direction was sampled from: the reference's BSDFIncidentLightInfo values
 * (src/Device/includes/BSDFs/BSDFIncidentLightInfo.h). */
enum {
    GBPT_LOBE_NONE = 0,
    GBPT_LOBE_COAT = 1 << 1,
    GBPT_LOBE_METAL_1 = 1 << 2,
    GBPT_LOBE_METAL_2 = 1 << 3,
    GBPT_LOBE_SPECULAR = 1 << 4,
    GBPT_LOBE_GLASS_REFLECT = 1 << 5,
    GBPT_LOBE_GLASS_REFRACT = 1 << 6,
    GBPT_LOBE_DIFFUSE = 1 << 7,
    GBPT_LOBE_DIFFUSE_TRANSMISSION = 1 << 8
};

/* One BSDF query: world-space unit directions (view points away from the surface), the media
 * on both sides (IOR of the medium the ray travels in and of the one behind the surface; 1 =
 * air), whether the ray is inside the object and the path's wavelength. Mirrors BSDFContext
 * (src/Device/includes/BSDFs/BSDFContext.h:13-54) with RayVolumeState reduced to those IORs. */
typedef struct gbpt_bsdf_query {
    float view[3];
    float shading_normal[3];
    float geometric_normal[3];
    float to_light[3];          /* ignored by gbpt_bsdf_sample */
    float eta_incident;
    float eta_outgoing;
    int32_t inside;
    int32_t incident_lobe;      /* GBPT_LOBE_* the light direction came from (eval/pdf) */
    float wavelength;           /* the path's sampled wavelength in nm (its magnitude; 0: none),
                                   for materials with dispersion (RayVolumeState::sampled_wavelength) */
    int32_t reserved[3];
} gbpt_bsdf_query;

typedef struct gbpt_bsdf_options {
    int32_t ggx_height_correlated; /* 0 = height-uncorrelated Smith G2 (the reference's default) */
    int32_t reserved[7];
} gbpt_bsdf_options;

/* out_rgb_pdf: 4 floats per query (f without the cosine, pdf). Replaces principled_bsdf_eval
 * (src/Device/includes/BSDFs/Principled.h:1620-1715) behind bsdf_dispatcher_eval
 * (src/Device/includes/Dispatcher.h:21-45). options may be NULL. */
GBPT_API gbpt_status gbpt_bsdf_eval(const gbpt_principled_material* materials, int32_t n_materials,
                                    const int32_t* material_index, const gbpt_bsdf_query* queries, int64_t n,
                                    const gbpt_bsdf_options* options, float* out_rgb_pdf, void* stream);
/* Replaces principled_bsdf_pdf (Principled.h:1717-1795). */
GBPT_API gbpt_status gbpt_bsdf_pdf(const gbpt_principled_material* materials, int32_t n_materials,
                                   const int32_t* material_index, const gbpt_bsdf_query* queries, int64_t n,
                                   const gbpt_bsdf_options* options, float* out_pdf, void* stream);
/* Samples one direction per query with the reference's Xorshift32 generator
 * (src/HostDeviceCommon/Xorshift.h:18-66) seeded by seeds[i], drawing in the reference's order,
 * then evaluates the BSDF for it. out: 8 floats per query (direction xyz, f rgb, pdf, 0);
 * out_lobe: GBPT_LOBE_*; out_rng_state (may be NULL): generator state afterwards.
 * Replaces principled_bsdf_sample (Principled.h:1803-1941). */
GBPT_API gbpt_status gbpt_bsdf_sample(const gbpt_principled_material* materials, int32_t n_materials,
                                      const int32_t* material_index, const gbpt_bsdf_query* queries,
                                      const uint32_t* seeds, int64_t n, const gbpt_bsdf_options* options, float* out,
                                      int32_t* out_lobe, uint32_t* out_rng_state, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GBPT_BSDF_H */
