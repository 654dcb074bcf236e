/*
 * gbpt — render path C ABI: scene upload, emissive power alias table, wavefront path tracer.
 *
 * Mirrors the reference's render-data / render-settings surface for the parts this path uses
 * (HIPRTRenderData src/HostDeviceCommon/RenderData.h:93-129, HIPRTRenderSettings
 * src/HostDeviceCommon/RenderSettings.h:24-278, HIPRTCamera src/HostDeviceCommon/HIPRTCamera.h:16-53)
 * and its per-pass kernel entry points (CameraRays src/Device/kernels/CameraRays.h:83,
 * MegaKernel src/Device/kernels/Megakernel.h:23). Plain C types only; see gbpt.h for the status codes.
 */
#ifndef GBPT_RENDER_H
#define GBPT_RENDER_H

#include "gbpt.h"
#include "gbpt_bsdf.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gbpt_scene gbpt_scene;
typedef struct gbpt_renderer gbpt_renderer;

/* Material subset of the reference's CPUMaterial (src/HostDeviceCommon/Material/MaterialUnpacked.h):
 * base colour and emission (= emission colour * emission_strength * global_emissive_factor). */
typedef struct gbpt_material {
    float base_color[3];
    float emission[3];
} gbpt_material;

/* Mirrors the reference's Scene (src/Scene/SceneParser.h:109-170): flat triangle soup with a
 * material index per triangle. Host pointers.
 * principled_materials (optional, n_materials entries) are the reference's CPUMaterial parameters
 * (src/HostDeviceCommon/Material/MaterialCPU.h) in the gbpt_principled_material record; the
 * library applies the reference's coat roughening (src/Device/includes/Material.h:122-146) once
 * at upload, and takes base colour and emission from them when 'materials' is NULL. Materials
 * with sheen > 0 are rejected (GBPT_ERROR_UNSUPPORTED). */
typedef struct gbpt_scene_desc {
    const float* positions;          /* 3 per vertex */
    int64_t n_vertices;
    const int32_t* indices;          /* 3 per triangle */
    int64_t n_triangles;
    const int32_t* material_indices; /* 1 per triangle */
    const gbpt_material* materials;
    int32_t n_materials;
    const gbpt_principled_material* principled_materials;
    /* Optional smooth-shading normals, 3 per vertex (NULL: every triangle shades with its
     * geometric normal). A triangle whose first vertex has a zero normal shades flat, as the
     * reference's per-vertex has_vertex_normals flag (src/HostDeviceCommon/RenderBuffers.h:34-37)
     * selects it in get_shading_normal (src/Device/includes/Intersect.h:114-134): the shading
     * normal is normalize(n_b u + n_c v + n_a (1 - u - v)) at the hit's barycentrics, then the
     * backface fix. Normal maps are not built. */
    const float* vertex_normals;
    /* GBPT_MATERIALS_* [GBPT_MATERIALS_FLOAT]. GBPT_MATERIALS_PACKED stores every material as the
     * reference does (DevicePackedEffectiveMaterial / DevicePackedTexturedMaterialSoA,
     * src/HostDeviceCommon/Material/MaterialPacked.h:16-520): colours and the [0, 1] parameters
     * truncated to 8 bits (base colour and roughness, metallic, F82, F90, diffuse transmission,
     * anisotropy and its rotation, second roughness and its weight, specular, its colour, tint and
     * darkening, coat, its roughness, roughening, darkening, anisotropy, rotation and medium
     * absorption, sheen, specular transmission, absorption colour), every other field in float. */
    int32_t material_packing;
} gbpt_scene_desc;

enum {
    GBPT_MATERIALS_FLOAT = 0,  /* material parameters kept in float */
    GBPT_MATERIALS_PACKED = 1  /* the reference's 8-bit packed material records */
};

/* The reference's packed material record read back, on the host: n materials through
 * CPUMaterial::pack_to_GPU and DevicePackedEffectiveMaterial::unpack
 * (src/HostDeviceCommon/Material/MaterialCPU.h:31-118, MaterialPacked.h:16-520) — what
 * GBPT_MATERIALS_PACKED stores before the coat roughening. in and out may alias. */
GBPT_API gbpt_status gbpt_material_pack_8bit(const gbpt_principled_material* in, int32_t n, gbpt_principled_material* out);

/* Uploads the scene, builds its BVH (gbpt_bvh_build), the emissive-triangle list (triangles
 * whose material has non-black emission, in triangle order, as the reference's scene parser
 * collects them) and the power alias table on the device.
 * Replaces GPURenderer::set_scene (src/Renderer/GPURenderer.cpp:952-958) and
 * compute_emissives_power_alias_table (src/Renderer/GPURenderer.cpp:173,221-295 with
 * Utils::compute_alias_table src/Utils/Utils.cpp:63-131). Power = luminance(emission) * area in
 * float as the reference computes it; the sum and the normalisation run in FP64 on the device
 * (the reference sums in float), then the Vose partition with the reference's queue order. */
GBPT_API gbpt_status gbpt_scene_create(const gbpt_scene_desc* desc, const gbpt_bvh_params* bvh_params,
                                       gbpt_scene** out, void* stream);
GBPT_API gbpt_status gbpt_scene_destroy(gbpt_scene* scene);
/* Borrowed pointer to the scene's BVH (owned by the scene). */
GBPT_API gbpt_status gbpt_scene_get_bvh(const gbpt_scene* scene, const gbpt_bvh** out);
/* Copies the emissive list and power alias table to host arrays of n_emissive entries each
 * (DeviceAliasTable src/Device/includes/AliasTable.h:11-29). Any pointer may be NULL. */
GBPT_API gbpt_status gbpt_scene_get_light_table(const gbpt_scene* scene, int32_t* n_emissive, int32_t* emissive,
                                                float* probas, int32_t* alias, float* power_sum, double* power_sum64);

/* ---- scene ingestion from glTF 2.0 (the reference's sample scenes in data/GLTFs) ----
 * Replaces SceneParser::parse_scene_file (src/Scene/SceneParser.cpp:19-226, ASSIMP with
 * aiProcess_PreTransformVertices | aiProcess_Triangulate) and read_material_properties
 * (SceneParser.cpp:391-438) for this path: a .gltf file with external or base64 buffers; the
 * default scene's node tree flattened to world space (matrix or TRS); triangle primitives (mode 4),
 * indexed (u8/u16/u32) or not, float VEC3 positions with any byte stride. Materials follow the
 * reference's mapping: base colour, metallic and roughness factors (glTF defaults), emissive
 * factor times KHR_materials_emissive_strength, and, when their extension is present,
 * KHR_materials_ior, _transmission, _clearcoat (factor, roughness), _specular (factor; tint and
 * colour to 1) and _volume (attenuation colour and distance); every other field keeps
 * CPUMaterial's default; then CPUMaterial::make_safe's clamps. Primitives without a material get
 * the glTF default material, appended after the file's materials. Also a .glb container. Not read:
 * textures and texture coordinates, skins and morph targets (the base mesh is loaded); sparse accessors, non-float positions and
 * unknown required extensions are errors. Triangle order is node traversal order (ASSIMP's
 * pre-transform step groups meshes by material instead). A KHR_materials_sheen material loads
 * with sheen = 1, as the reference maps it, which gbpt_scene_create then rejects. */
typedef struct gbpt_gltf gbpt_gltf;
typedef struct gbpt_gltf_camera {
    int32_t present;                 /* 1 when a node of the scene carries a perspective camera */
    float position[3], forward[3], up[3]; /* world space, from the first camera node's transform */
    float yfov;                      /* radians (the glTF value; the reference's ASSIMP route adds 0.425) */
    float aspect_ratio;              /* 0 when the file gives none */
    float znear, zfar;
} gbpt_gltf_camera;

GBPT_API gbpt_status gbpt_gltf_load(const char* path, gbpt_gltf** out);
/* The loaded scene as a scene description (principled materials only; vertex normals from the
 * primitives' NORMAL attributes moved to world space by the inverse transpose of their node's
 * transform and normalised, zero for primitives without one, NULL when no primitive has one;
 * pointers owned by 'g', valid until gbpt_gltf_destroy) for gbpt_scene_create. */
GBPT_API gbpt_status gbpt_gltf_scene_desc(const gbpt_gltf* g, gbpt_scene_desc* out);
GBPT_API gbpt_status gbpt_gltf_get_camera(const gbpt_gltf* g, gbpt_gltf_camera* out);
GBPT_API gbpt_status gbpt_gltf_destroy(gbpt_gltf* g);

/* Largest emitter count gbpt_alias_table_build_noalloc accepts. */
#define GBPT_ALIAS_NOALLOC_MAX_EMITTERS 131072

/* No counterpart in the reference: an extra entry point of this library for callers that cannot
 * allocate device memory. An interactive render loop that rebuilds the light table after an
 * emission edit cannot afford cudaMalloc/cudaFree (they can synchronise the whole device and stall
 * the frame), and a host application that hands the library a fixed device-memory budget up front
 * cannot let it allocate later. This call allocates nothing: it takes a device power list
 * (luminance(emission) * area per emitter, n entries) and writes the same table as the light-table
 * build of gbpt_scene_create — FP64 sum into *power_sum64, then probas[n] and alias[n] — all three
 * device pointers owned by the caller.
 * Limits: n <= GBPT_ALIAS_NOALLOC_MAX_EMITTERS, else GBPT_ERROR_INVALID_ARG. Its scratch is one
 * fixed 2 MiB device array inside libgbpt that every device which loads the library holds until
 * exit. The first call in each CUDA context looks up that array's device address (with the device
 * current; again after cudaDeviceReset or in another context): make that first call before any
 * stream capture. All calls share the one array: two calls that
 * overlap on the GPU (different streams, or different host threads) race and must be serialised
 * by the caller. Asynchronous on 'stream'. */
GBPT_API gbpt_status gbpt_alias_table_build_noalloc(const float* power, int32_t n, float* probas, int32_t* alias,
                                                    double* power_sum64, void* stream);

/* ---- the world around the scene: ambient light and environment map ----
 * Mirrors WorldSettings (src/HostDeviceCommon/WorldSettings.h:14-53), RendererEnvmap
 * (src/Renderer/RendererEnvmap.cpp:40-209) and the envmap kernel options
 * (src/HostDeviceCommon/KernelOptions/KernelOptions.h:53-55,155-170). */
enum {
    GBPT_AMBIENT_NONE = 0,    /* AmbientLightType::NONE: misses are black */
    GBPT_AMBIENT_UNIFORM = 1, /* AmbientLightType::UNIFORM: misses see uniform_color at every bounce */
    GBPT_AMBIENT_ENVMAP = 2   /* AmbientLightType::ENVMAP */
};
enum {
    GBPT_ENVMAP_NO_SAMPLING = 0,   /* ESS_NO_SAMPLING: the envmap is only found by misses */
    GBPT_ENVMAP_BINARY_SEARCH = 1, /* ESS_BINARY_SEARCH: texel drawn by a search of the luminance CDF */
    GBPT_ENVMAP_ALIAS_TABLE = 2    /* ESS_ALIAS_TABLE (the reference's default) */
};

/* envmap_rgb: width*height RGB float texels (finite, >= 0), row-major, row 0 at v = 0 — the -y
 * pole (the reference's envmap after its vertical flip at load). Direction of (u, v):
 * phi = 2 pi u, theta = pi v, d = (-sin theta cos phi, -cos theta, -sin theta sin phi) in envmap
 * space, rotated to the world by envmap_to_world (row-major, d_world = M d). world_to_envmap is its
 * inverse (the reference keeps both matrices; the library checks that they are inverses). */
typedef struct gbpt_world_desc {
    int32_t ambient;                /* GBPT_AMBIENT_* */
    float uniform_color[3];         /* uniform_light_color */
    const float* envmap_rgb;        /* host pointer (GBPT_AMBIENT_ENVMAP) */
    int32_t envmap_width, envmap_height;
    float envmap_intensity;         /* scale on every texel (envmap_intensity) */
    int32_t envmap_scale_background;/* 0: camera misses see the unscaled texel [0] */
    float envmap_to_world[9];
    float world_to_envmap[9];
    int32_t envmap_sampling;        /* GBPT_ENVMAP_* [GBPT_ENVMAP_ALIAS_TABLE] */
    int32_t envmap_bsdf_mis;        /* EnvmapSamplingDoBSDFMIS: a BSDF sample MIS-combined with the envmap sample [1] */
    int32_t envmap_bilinear;        /* EnvmapSamplingDoBilinearFiltering [0] */
} gbpt_world_desc;

/* Fills *w with the reference's defaults: no ambient light, identity rotation, intensity 1, alias
 * table sampling with BSDF MIS, nearest-texel lookups. */
GBPT_API gbpt_status gbpt_world_default(gbpt_world_desc* w);
/* Sets the scene's world; renderers of the scene see it from their next launch. Fails with
 * GBPT_ERROR_INVALID_ARG while a batch renders the scene (destroy the batch first). For an envmap the library packs the texels to
 * RGB9E5 and, on the device, takes each texel's luminance from the float input, their FP64 sum,
 * the FP64 running sum over texels stored as float (the binary-search CDF) and the Vose alias
 * table of the luminances normalised by the FP64 sum (Image32Bit::compute_cdf and
 * compute_alias_table, src/Image/Image.cpp:625-672, which sum in float). Synchronous. */
GBPT_API gbpt_status gbpt_scene_set_world(gbpt_scene* scene, const gbpt_world_desc* w, void* stream);
/* Copies the envmap's device tables to host arrays of width*height entries (any may be NULL):
 * packed texels, CDF, alias probabilities and indices; total_sum = the float sum the sampler
 * uses, total_sum64 = the FP64 sum. GBPT_ERROR_INVALID_ARG when the world has no envmap. */
GBPT_API gbpt_status gbpt_scene_get_envmap_tables(const gbpt_scene* scene, uint32_t* texels, float* cdf,
                                                  float* probas, int32_t* alias, float* total_sum,
                                                  double* total_sum64);

enum {
    GBPT_LIGHT_UNIFORM = 0, /* LSS_BASE_UNIFORM */
    GBPT_LIGHT_POWER = 1    /* LSS_BASE_POWER */
};
enum {
    GBPT_BSDF_LAMBERTIAN = 1, /* BSDFOverride = BSDF_LAMBERTIAN (src/Device/includes/Dispatcher.h:21-82) */
    GBPT_BSDF_PRINCIPLED = 3  /* BSDF_PRINCIPLED: the layered BSDF of gbpt_bsdf.h (needs principled materials) */
};

/* Subset of HIPRTRenderSettings + HIPRTCamera used by the render path. */
/* Direct lighting at a path vertex (DirectLightSamplingBaseStrategy,
 * src/HostDeviceCommon/KernelOptions/DirectLightSamplingOptions.h):
 *   GBPT_DIRECT_MIS: one light sample and one BSDF sample combined by the balance heuristic
 *     (LSS_ONE_LIGHT_MIS, sample_one_light_MIS, src/Device/includes/LightSampling/Lights.h:123-226);
 *   GBPT_DIRECT_RIS: resampled importance sampling over ris_light_candidates light samples and
 *     ris_bsdf_candidates BSDF samples (LSS_RIS_BSDF_AND_LIGHT, the reference's default,
 *     src/Device/includes/RIS/RIS.h:83-255), one shadow ray for the selected light sample.
 * Vertices guided by the learned proposal and the ReSTIR DI bounce keep their own estimators. */
enum { GBPT_DIRECT_MIS = 0, GBPT_DIRECT_RIS = 1 };

/* Random numbers of the paths (gbpt_render_settings.rng_mode):
 *   GBPT_RNG_PCG: one PCG32 stream per pixel sample, keyed on (pixel, sample index, seed);
 *   GBPT_RNG_REFERENCE: the reference's generator and draw order, for sample-by-sample comparison
 *     with its own kernels: Xorshift32 (src/HostDeviceCommon/Xorshift.h:18-66) seeded by
 *     wang_hash((pixel + 1) * (sample index + 1) * random_number) (src/Device/kernels/CameraRays.h:155-160),
 *     the camera pass and the bounce loop each seeding their own generator from their own pass's
 *     random_number (Megakernel.h:52-57), BSDF samples drawing from the path's generator, and the
 *     camera hit shaded from the packed G-buffer (octahedral 24-bit normals, the view direction
 *     from the camera position, the material re-packed after its coat roughening;
 *     CameraRays.h:178-201, Megakernel.h:59-72). Each launch is one sample of the reference's GPU
 *     renderer: a host Xorshift32 generator seeded with gbpt_render_settings.random_number (42
 *     when 0, GPURenderer.cpp:750-751) gives one number to each pass in launch order, the G-buffer
 *     pass first and the MegaKernel pass last (FillGBufferRenderPass.cpp:91,
 *     MegaKernelRenderPass.cpp:53; with ReSTIR DI its passes draw theirs in between,
 *     ReSTIRDIRenderPass.cpp:449-578). The environment map's direct lighting keeps its own draw
 *     position (before the emissive light sample) in both modes. */
enum { GBPT_RNG_PCG = 0, GBPT_RNG_REFERENCE = 1 };

typedef struct gbpt_render_settings {
    int32_t width, height;
    int32_t samples_per_launch;      /* spp traced together in one wavefront (>= 1) */
    int32_t nb_bounces;              /* render_settings.nb_bounces */
    int32_t do_russian_roulette;     /* render_settings.do_russian_roulette */
    int32_t russian_roulette_min_depth;
    float russian_roulette_throughput_clamp; /* 0 = no clamp */
    int32_t light_sampling;          /* GBPT_LIGHT_* */
    int32_t bsdf;                    /* GBPT_BSDF_* */
    uint32_t seed;
    int32_t do_jittering;            /* HIPRTCamera::do_jittering */
    int32_t ggx_height_correlated;   /* BRDFsData::GGX_masking_shadowing: 0 = height-uncorrelated (default) */
    int32_t direct_lighting;         /* GBPT_DIRECT_* (DirectLightSamplingBaseStrategy) */
    int32_t ris_light_candidates;    /* RISSettings::number_of_light_candidates [4] */
    int32_t ris_bsdf_candidates;     /* RISSettings::number_of_bsdf_candidates, 0 or 1 [1] */
    int32_t rng_mode;                /* GBPT_RNG_* [GBPT_RNG_PCG] */
    float inverse_view[16];          /* row-major, points multiplied on the right */
    float inverse_projection[16];
    uint32_t random_number;          /* GBPT_RNG_REFERENCE: seed of the per-launch random numbers (0: 42) */
} gbpt_render_settings;

typedef struct gbpt_render_stats {
    int64_t samples;         /* path samples accumulated since the last reset */
    int64_t extension_rays;  /* closest-hit rays traced (camera + bounce) */
    int64_t shadow_rays;     /* any-hit rays traced */
    int64_t bsdf_light_rays; /* closest-hit rays traced for the MIS BSDF sample */
} gbpt_render_stats;

GBPT_API gbpt_status gbpt_renderer_create(const gbpt_scene* scene, const gbpt_render_settings* settings,
                                          gbpt_renderer** out);
GBPT_API gbpt_status gbpt_renderer_destroy(gbpt_renderer* r);
GBPT_API gbpt_status gbpt_renderer_reset(gbpt_renderer* r, void* stream);
/* Sample index of the next launch's first sample (the PCG streams are seeded by pixel and sample
 * index): a rank rendering launches [a, a + n) of a sample-range-sharded image sets a * spp here
 * after gbpt_renderer_reset, and the ranks' FP64 sums add up to the single-GPU image. */
GBPT_API gbpt_status gbpt_renderer_set_sample_index(gbpt_renderer* r, int64_t first_sample);

/* Full frame: n_launches x (camera rays + nb_bounces+1 wavefront bounces + accumulate), each
 * launch adding samples_per_launch samples per pixel. Replaces the render loop of
 * GPURendererThread::render_path_tracing (src/Renderer/GPURendererThread.cpp:311-330) over the
 * FillGBuffer and MegaKernel passes. */
GBPT_API gbpt_status gbpt_render(gbpt_renderer* r, int32_t n_launches, void* stream);

/* The same passes one by one (for callers that schedule passes themselves):
 * camera rays   <- CameraRays (src/Device/kernels/CameraRays.h:83)
 * bounce k      <- one iteration of MegaKernel's bounce loop (src/Device/kernels/Megakernel.h:88-131)
 * accumulate    <- path_tracing_accumulate_color (src/Device/includes/PathTracing.h:176-217) */
GBPT_API gbpt_status gbpt_pass_camera_rays(gbpt_renderer* r, void* stream);
GBPT_API gbpt_status gbpt_pass_bounce(gbpt_renderer* r, int32_t bounce, void* stream);
GBPT_API gbpt_status gbpt_pass_accumulate(gbpt_renderer* r, void* stream);

/* Copies the accumulated sums (not divided by the sample count) to host memory:
 * rgb32 = FP32 sums (W*H*3), rgb64 = FP64 sums (W*H*3); either may be NULL. Pixel (x, y) is at
 * index x + y*W with y = 0 the bottom row (the reference's NDC convention). Synchronous. */
GBPT_API gbpt_status gbpt_renderer_get_image(gbpt_renderer* r, float* rgb32, double* rgb64, void* stream);
GBPT_API gbpt_status gbpt_renderer_get_stats(gbpt_renderer* r, gbpt_render_stats* out, void* stream);

/* ReSTIR DI at the camera hit (the reference's LSS_RESTIR_DI direct lighting,
 * src/HostDeviceCommon/ReSTIR/ReSTIRDISettings.h:11-161 and KernelOptions/ReSTIRDIOptions.h;
 * defaults in brackets). Requires GBPT_BSDF_PRINCIPLED and samples_per_launch = 1: one launch is
 * one frame, whose final reservoirs feed the next frame's temporal pass. Always on: visibility
 * reuse in the final reservoirs' shadow test, pairwise MIS bias correction, geometric-normal and
 * plane-distance neighbour heuristics; the envmap is not a ReSTIR candidate (vertices sample it
 * on their own). */
typedef struct gbpt_restir_di_settings {
    int32_t enabled;
    int32_t light_candidates;           /* number_of_initial_light_candidates [4] */
    int32_t bsdf_candidates;            /* number_of_initial_bsdf_candidates [1] */
    int32_t do_visibility_reuse;        /* ReSTIR_DI_DoVisibilityReuse [1] */
    int32_t do_temporal;                /* common_temporal_pass.do_temporal_reuse_pass [1] */
    int32_t temporal_search_count;      /* max_neighbor_search_count [8] */
    float temporal_search_radius;       /* neighbor_search_radius, pixels [4] */
    int32_t do_spatial;                 /* do_spatial_reuse_pass [1] */
    int32_t spatial_passes;             /* number_of_passes [1] */
    int32_t spatial_neighbors;          /* reuse_neighbor_count, 1..32 [5] */
    float spatial_radius;               /* reuse_radius, pixels [16] */
    int32_t m_cap;                      /* temporal M cap, 0 = none [3] */
    int32_t use_confidence_weights;     /* [1] */
    int32_t bias_correction_visibility; /* ReSTIR_DI_BiasCorrectionUseVisibility [1] */
    int32_t do_final_shading_visibility;/* [1] */
    float normal_similarity_cos;        /* normal_similarity_angle_precomp [0.906307787] */
    float plane_distance_threshold;     /* [0.1] */
    int32_t do_fused_spatiotemporal;    /* do_fused_spatiotemporal: one pass of temporal + spatial reuse [0] */
    int32_t do_light_presampling;       /* ReSTIR_DI_DoLightPresampling [0] */
    int32_t presampling_subsets;        /* light_presampling.number_of_subsets [128] */
    int32_t presampling_subset_size;    /* light_presampling.subset_size [1024] */
    int32_t presampling_tile_size;      /* light_presampling.tile_size, pixels [8] */
    int32_t reserved[10];
} gbpt_restir_di_settings;

/* Fills 's' with the reference's defaults (enabled = 1). */
GBPT_API gbpt_status gbpt_restir_di_default_settings(gbpt_restir_di_settings* s);
/* Allocates the G-buffers and reservoir buffers and turns ReSTIR DI on (or off with enabled = 0). */
GBPT_API gbpt_status gbpt_renderer_set_restir_di(gbpt_renderer* r, const gbpt_restir_di_settings* s);
/* Moves the camera for the next launch (row-major inverse view / projection as in
 * gbpt_render_settings); the previous frame's camera is kept for temporal backprojection
 * (HIPRTRenderData::prev_camera, src/HostDeviceCommon/RenderData.h:93-129). */
GBPT_API gbpt_status gbpt_renderer_set_camera(gbpt_renderer* r, const float* inverse_view, const float* inverse_projection);

/* Pass-level scheduling with ReSTIR DI (what gbpt_render does per launch):
 *   gbpt_pass_camera_rays, gbpt_pass_extend(0), gbpt_pass_restir_di_initial,
 *   gbpt_pass_restir_di_temporal, gbpt_pass_restir_di_spatial(0..passes-1), gbpt_pass_shade(0),
 *   gbpt_pass_bounce(1..nb_bounces), gbpt_pass_accumulate (which also ends the frame);
 *   with do_fused_spatiotemporal, gbpt_pass_restir_di_spatiotemporal then
 *   gbpt_pass_restir_di_spatial(1..passes-1) replace the temporal and spatial passes.
 * extend = closest hit of the bounce's queue; shade = shading, shadow and BSDF-light rays and
 * their resolve (gbpt_pass_bounce = extend + shade). */
GBPT_API gbpt_status gbpt_pass_extend(gbpt_renderer* r, int32_t bounce, void* stream);
GBPT_API gbpt_status gbpt_pass_shade(gbpt_renderer* r, int32_t bounce, void* stream);
/* Fills the G-buffer from the camera hits and runs ReSTIR_DI_InitialCandidates
 * (src/Device/kernels/ReSTIR/DI/InitialCandidates.h:478). */
GBPT_API gbpt_status gbpt_pass_restir_di_initial(gbpt_renderer* r, void* stream);
/* ReSTIR_DI_TemporalReuse (src/Device/kernels/ReSTIR/DI/TemporalReuse.h:50). */
GBPT_API gbpt_status gbpt_pass_restir_di_temporal(gbpt_renderer* r, void* stream);
/* ReSTIR_DI_SpatialReuse (src/Device/kernels/ReSTIR/DI/SpatialReuse.h:43), pass 'pass_index'. */
GBPT_API gbpt_status gbpt_pass_restir_di_spatial(gbpt_renderer* r, int32_t pass_index, void* stream);
/* ReSTIR_DI_SpatiotemporalReuse (src/Device/kernels/ReSTIR/DI/FusedSpatiotemporalReuse.h:152): the
 * temporal neighbour and the spatial neighbours (taken from the previous frame's final reservoirs
 * around the backprojected position) and the initial candidates resampled in one pass; its output
 * is the final reservoirs (spatial pass 0). */
GBPT_API gbpt_status gbpt_pass_restir_di_spatiotemporal(gbpt_renderer* r, void* stream);

enum {
    GBPT_RESERVOIRS_INITIAL = 0,
    GBPT_RESERVOIRS_TEMPORAL = 1,
    GBPT_RESERVOIRS_FINAL = 2,    /* what the shading of the current frame reads */
    GBPT_RESERVOIRS_PREVIOUS = 3  /* the previous frame's final reservoirs (temporal input) */
};
/* Reservoir buffers as 8 words per pixel: light point xyz, target function, emissive triangle
 * (int32), (M << 9) | flags (int32), weight sum, UCW (ReSTIRDIReservoir, Reservoir.h:22-187).
 * Synchronous. 'set' lets a caller inject reservoirs, e.g. to test one pass on given candidates. */
GBPT_API gbpt_status gbpt_restir_di_get_reservoirs(gbpt_renderer* r, int32_t which, float* host_out, void* stream);
GBPT_API gbpt_status gbpt_restir_di_set_reservoirs(gbpt_renderer* r, int32_t which, const float* host_in, void* stream);

/* ---- learned path guiding (the network: include/gbpt_guide.h) ----
 * With a guide attached, each bounce runs the network on the shaded queue (after extend, inside
 * gbpt_pass_shade) and draws the continuation of every vertex whose material has neither delta
 * lobes nor transmission from the vMF mixture with probability alpha (the network's learned
 * selection probability, or guide_probability when that is > 0), else from the BSDF; the path
 * weight uses the one-sample MIS pdf alpha q + (1 - alpha) p_bsdf, so the image stays unbiased
 * whatever the network has learned. Direct lighting (NEE, ReSTIR DI) is unchanged.
 * With train = 1, guided vertices are recorded (a hash of pixel sample, bounce and frame picks
 * about max_records records per launch, the fraction adapting to the previous launch's vertex
 * count): one record for the continuation and one for the light sample, each weighted by its
 * MIS-weighted estimate of f cos L_i / pdf; gbpt_pass_accumulate ends the launch with one Adam
 * step on them.
 * gbpt_renderer_reset restarts the sample index, so the launches after it draw the random numbers
 * of the launches the network was trained on: for an estimate independent of the training
 * samples, keep rendering (differences of accumulated images) or change the seed. */
typedef struct gbpt_guide gbpt_guide;
typedef struct gbpt_guide_render_settings {
    int32_t enabled;          /* [1] */
    int32_t train;            /* [1] */
    float guide_probability;  /* fixed alpha in (0, 1), or 0 = the network's [0] */
    int32_t max_records;      /* per launch, <= the guide's max_batch [2^18] */
    float weight_clamp;       /* upper bound of a record's weight, 0 = none [50] */
    int32_t reserved[11];
} gbpt_guide_render_settings;

GBPT_API gbpt_status gbpt_guide_render_default_settings(gbpt_guide_render_settings* s);
/* Attaches 'g' (not owned; it must outlive its use) or detaches it (g NULL or enabled = 0). */
GBPT_API gbpt_status gbpt_renderer_set_guide(gbpt_renderer* r, gbpt_guide* g, const gbpt_guide_render_settings* s);
/* The last launch's training records, 15 floats each: position xyz, normal xyz, view xyz,
 * direction xyz, weight, BSDF pdf of the direction, pixel-sample slot (int32 bits; -1 for a
 * light-sample record). Copies min(count, capacity) records to
 * host_out (may be NULL) and the number made (before the max_records cap) to *count. Synchronous. */
GBPT_API gbpt_status gbpt_renderer_get_guide_records(gbpt_renderer* r, float* host_out, int32_t capacity, int32_t* count,
                                                     void* stream);

/* ---- batched rendering: many independent jobs in one wavefront ----
 * Every job has its own scene (BVH, materials, lights) and settings (resolution, camera, bounces,
 * seed, ...; settings.samples_per_launch is the job's TOTAL samples per pixel). All jobs' paths
 * share every wavefront launch: one camera launch, then per bounce one extension, shading,
 * shadow, BSDF-light and resolve launch over the union of the jobs' queues, one accumulation
 * launch; a ray traverses its own job's BVH. An iteration renders samples_per_iteration samples
 * of every pixel of every unfinished job; jobs finish after ceil(spp / samples_per_iteration)
 * iterations. With use_graph one iteration is captured as a CUDA graph and replayed (the
 * iteration index lives in device memory). A job's image equals, bit for bit, the image of a
 * gbpt_renderer with samples_per_launch = samples_per_iteration run for the same samples (the
 * last launch truncated to the job's spp), because each path keeps its pixel and sample index
 * and its PCG stream. All jobs must use the same bsdf mode; ReSTIR DI and guiding are per
 * renderer and not available in a batch. */
typedef struct gbpt_batch gbpt_batch;
typedef struct gbpt_batch_job {
    const gbpt_scene* scene;
    gbpt_render_settings settings;
} gbpt_batch_job;
typedef struct gbpt_batch_params {
    int32_t samples_per_iteration; /* [4] */
    int32_t use_graph;             /* [1] */
    int32_t reserved[6];
} gbpt_batch_params;

GBPT_API gbpt_status gbpt_batch_default_params(gbpt_batch_params* p);
GBPT_API gbpt_status gbpt_batch_create(const gbpt_batch_job* jobs, int32_t n_jobs, const gbpt_batch_params* p,
                                       gbpt_batch** out);
GBPT_API gbpt_status gbpt_batch_destroy(gbpt_batch* b);
/* Renders every job from zero to completion; asynchronous on 'stream'. */
GBPT_API gbpt_status gbpt_batch_render(gbpt_batch* b, void* stream);
/* Per job: seconds from the start of the last gbpt_batch_render to the end of the job's last
 * iteration (device global timer). Synchronous. */
GBPT_API gbpt_status gbpt_batch_job_seconds(gbpt_batch* b, double* seconds);
/* A job's FP32 / FP64 radiance sums (width*height*3 each; either may be NULL). Synchronous. */
GBPT_API gbpt_status gbpt_batch_get_image(gbpt_batch* b, int32_t job, float* rgb32, double* rgb64, void* stream);
/* Rays traced by the last render, summed over the jobs (samples = sum of width*height*spp). */
GBPT_API gbpt_status gbpt_batch_get_stats(gbpt_batch* b, gbpt_render_stats* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GBPT_RENDER_H */
