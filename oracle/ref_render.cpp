/*
 * TEST INFRASTRUCTURE ONLY — C entry points into the reference's OWN render kernels, compiled
 * from the reference's sources where they lie (oracle/Makefile, target 'ref'), behind the
 * clean-room shim headers in oracle/shim/. Output goes to oracle/_ref/ (git-ignored). Used by
 * tests/golden/make_ref_render_golden.py to write golden images that pin this project's
 * wavefront path tracer sample by sample.
 *
 * Calls, unmodified, one frame per call over every pixel (OpenMP rows, as
 * CPURenderer::debug_render_pass, src/Renderer/CPURenderer.cpp:613-686, walks them):
 *   - CameraRays(render_data, x, y)  (src/Device/kernels/CameraRays.h:83-213): jittered camera
 *     ray, closest hit through the CPU BVH (BVH::intersect, src/Renderer/BVH.h:132-223), the
 *     packed G-buffer (8-bit material, octahedral-24 normals);
 *   - MegaKernel(render_data, x, y)  (src/Device/kernels/Megakernel.h:23-144): the bounce loop
 *     with next-event estimation, BSDF continuation, Russian roulette and accumulation.
 * Scene set-up follows CPURenderer::set_scene (src/Renderer/CPURenderer.cpp:297-420): materials
 * packed by CPUMaterial::pack_to_GPU (src/HostDeviceCommon/Material/MaterialCPU.h:31-118) into
 * the CPU material SoA, triangle areas as ThreadFunctions::load_scene_compute_triangle_areas
 * (src/Threads/ThreadFunctions.cpp:221-243), the emissive list in triangle order, and for power
 * sampling the float power list + float running sum + Utils::compute_alias_table
 * (CPURenderer::compute_emissives_power_alias_table, src/Renderer/CPURenderer.cpp:426-465;
 * the alias function is the reference's own, extracted from src/Utils/Utils.cpp by the Makefile).
 *
 * Compile-time options (-D on the command line, applied after the reference's option headers):
 *   REF_BSDF = BSDF_LAMBERTIAN (1) or BSDF_PRINCIPLED (3) -> BSDFOverride
 *   REF_LIGHT_BASE = LSS_BASE_UNIFORM (0) or LSS_BASE_POWER (1) -> DirectLightSamplingBaseStrategy
 *   REF_DIRECT = the DirectLightSamplingStrategy, LSS_MIS_LIGHT_BSDF (one light sample + one
 *     BSDF sample, balance heuristic; the default here) or LSS_RIS_BSDF_AND_LIGHT (RIS over
 *     light and BSDF candidates, src/Device/includes/RIS/RIS.h:83-255)
 * and always: energy compensation and microfacet regularization off (as the BSDF
 * harness builds them), alpha testing off (render_settings.do_alpha_testing = false: untextured
 * materials would otherwise draw a random number per candidate hit), adaptive sampling and the
 * pixel noise threshold off, no envmap (ambient light NONE).
 *
 * Material records: the 64-word gbpt_principled_material layout (include/gbpt_bsdf.h), emission
 * already multiplied by strength and global factor.
 */
#include "HostDeviceCommon/KernelOptions/KernelOptions.h"

#ifndef REF_DIRECT
#define REF_DIRECT LSS_MIS_LIGHT_BSDF
#endif
#undef DirectLightSamplingStrategy
#define DirectLightSamplingStrategy REF_DIRECT
#undef DirectLightSamplingBaseStrategy
#define DirectLightSamplingBaseStrategy REF_LIGHT_BASE
#undef BSDFOverride
#define BSDFOverride REF_BSDF
#undef PrincipledBSDFDoEnergyCompensation
#define PrincipledBSDFDoEnergyCompensation KERNEL_OPTION_FALSE
#undef PrincipledBSDFDoMicrofacetRegularization
#define PrincipledBSDFDoMicrofacetRegularization KERNEL_OPTION_FALSE

#include "Device/kernels/CameraRays.h"
#include "Device/kernels/Megakernel.h"
#if REF_RESTIR
#include "Device/kernels/ReSTIR/DI/InitialCandidates.h"
#include "Device/kernels/ReSTIR/DI/SpatialReuse.h"
#include "Device/kernels/ReSTIR/DI/TemporalReuse.h"
#endif
#include "HostDeviceCommon/Material/MaterialCPU.h"
#include "Renderer/BVH.h"
#include "Renderer/CPUDataStructures/MaterialPackedSoACPUData.h"
#include "Utils/Utils.h"

#include <atomic>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

CPUMaterial cpu_material(const float* w)
{
    CPUMaterial m;
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
    m.thin_film_hue_shift_degrees = w[51] * 360.0f;  // pack_to_GPU stores degrees / 360
    m.thin_film_base_ior_override = w[52];
    int32_t tf_override;
    std::memcpy(&tf_override, w + 53, 4);
    m.thin_film_do_ior_override = tf_override != 0;
    m.dispersion_scale = w[54];
    m.dispersion_abbe_number = w[55];
    // the reference's scene parser calls make_safe on every material
    // (src/Scene/SceneParser.cpp:391-438); its clamps only touch fields this layout does not
    // carry, the thin-film ranges (weight and hue in range, film IOR >= 1.0005) and the dielectric
    // priority of non-transmissive materials
    m.make_safe();
    return m;
}

struct RefRenderScene
{
    std::vector<int> indices;
    std::vector<float3> positions;
    std::vector<float3> normals;
    std::vector<float2> texcoords;  // zeros: the path reads them, nothing textured uses them
    std::vector<unsigned char> has_normals;
    std::vector<int> material_of;
    std::vector<float> areas;
    std::vector<int> emissive;
    std::vector<unsigned char> opaque;
    std::vector<float> alias_probas;
    std::vector<int> alias_alias;
    float power_sum = 0.0f;
    DevicePackedTexturedMaterialSoACPUData materials;
    std::vector<Triangle> tris, emissive_tris;
    BVH* bvh = nullptr;
    BVH* light_bvh = nullptr;
};

}  // namespace

#define REF_EXPORT extern "C" __attribute__((visibility("default")))

REF_EXPORT void* refr_scene_create(const float* positions, int64_t n_vertices, const int32_t* indices, int64_t n_triangles,
                        const int32_t* material_indices, const float* materials, int32_t n_materials,
                        const float* vertex_normals)
{
    RefRenderScene* s = new RefRenderScene();
    s->indices.assign(indices, indices + 3 * n_triangles);
    s->positions.resize(n_vertices);
    s->normals.resize(n_vertices);
    s->has_normals.resize(n_vertices);
    s->texcoords.assign(n_vertices, make_float2(0.0f, 0.0f));
    for (int64_t v = 0; v < n_vertices; v++)
    {
        s->positions[v] = make_float3(positions[3 * v], positions[3 * v + 1], positions[3 * v + 2]);
        float3 n = vertex_normals ? make_float3(vertex_normals[3 * v], vertex_normals[3 * v + 1], vertex_normals[3 * v + 2])
                                  : make_float3(0.0f, 0.0f, 0.0f);
        s->normals[v] = n;
        s->has_normals[v] = (n.x != 0.0f || n.y != 0.0f || n.z != 0.0f) ? 1 : 0;
    }
    s->material_of.assign(material_indices, material_indices + n_triangles);

    std::vector<CPUMaterial> cpu(n_materials);
    std::vector<DevicePackedTexturedMaterial> packed(n_materials);
    for (int m = 0; m < n_materials; m++)
    {
        cpu[m] = cpu_material(materials + 64 * (int64_t)m);
        packed[m] = cpu[m].pack_to_GPU();
    }
    s->materials.upload_data(packed);
    s->opaque.assign(n_materials, 0);

    s->areas.resize(n_triangles);
    for (int64_t t = 0; t < n_triangles; t++)
    {
        float3 A = s->positions[s->indices[3 * t]], B = s->positions[s->indices[3 * t + 1]], C = s->positions[s->indices[3 * t + 2]];
        float3 normal = hippt::cross(B - A, C - A);
        s->areas[t] = hippt::length(normal) * 0.5f;
        if (cpu[s->material_of[t]].is_emissive()) s->emissive.push_back((int)t);
    }

    // power list in float, float running sum (CPURenderer.cpp:437-456)
    std::vector<float> power(s->emissive.size());
    float sum = 0.0f;
    for (size_t i = 0; i < s->emissive.size(); i++)
    {
        int t = s->emissive[i];
        float3 A = s->positions[s->indices[3 * t]], B = s->positions[s->indices[3 * t + 1]], C = s->positions[s->indices[3 * t + 2]];
        float3 normal = hippt::cross(B - A, C - A);
        float area = 0.5f * hippt::length(normal);
        const CPUMaterial& m = cpu[s->material_of[t]];
        float lum = m.emission.luminance() * m.emission_strength * m.global_emissive_factor;
        power[i] = lum * area;
        sum += power[i];
    }
    s->power_sum = sum;
    if (!power.empty()) Utils::compute_alias_table(power, sum, s->alias_probas, s->alias_alias);

    s->tris.resize(n_triangles);
    for (int64_t t = 0; t < n_triangles; t++)
        s->tris[t] = Triangle(s->positions[s->indices[3 * t]], s->positions[s->indices[3 * t + 1]], s->positions[s->indices[3 * t + 2]]);
    for (int t : s->emissive) s->emissive_tris.push_back(s->tris[t]);
    s->bvh = new BVH(&s->tris);
    s->light_bvh = new BVH(&s->emissive_tris);
    return s;
}

REF_EXPORT void refr_scene_free(void* h)
{
    RefRenderScene* s = static_cast<RefRenderScene*>(h);
    delete s->bvh;
    delete s->light_bvh;
    delete s;
}

/* The emissive list and the power alias table the reference builds (float sum). Arrays of
 * n_emissive entries; any pointer may be NULL. */
REF_EXPORT void refr_scene_light_table(void* h, int32_t* n_emissive, int32_t* emissive, float* probas, int32_t* alias, float* power_sum)
{
    RefRenderScene* s = static_cast<RefRenderScene*>(h);
    if (n_emissive) *n_emissive = (int32_t)s->emissive.size();
    for (size_t i = 0; i < s->emissive.size(); i++)
    {
        if (emissive) emissive[i] = s->emissive[i];
        if (probas && !s->alias_probas.empty()) probas[i] = s->alias_probas[i];
        if (alias && !s->alias_alias.empty()) alias[i] = s->alias_alias[i];
    }
    if (power_sum) *power_sum = s->power_sum;
}

/* Utils::compute_alias_table(input, in_input_total_sum, ...) on a caller's power list and sum. */
REF_EXPORT void refr_alias_table(const float* power, int32_t n, float sum, float* probas, int32_t* alias)
{
    std::vector<float> in(power, power + n), p;
    std::vector<int> a;
    Utils::compute_alias_table(in, sum, p, a);
    for (int32_t i = 0; i < n; i++)
    {
        probas[i] = p[i];
        alias[i] = a[i];
    }
}

namespace {

// The buffers of one frame and the render data pointing at them (CPURenderer's per-frame state).
struct Frame
{
    int W, H;
    std::vector<ColorRGB32F> accum;
    std::vector<unsigned char> pixel_active;
    std::vector<float3> den_normals;
    std::vector<ColorRGB32F> den_albedo;
    std::vector<DevicePackedEffectiveMaterial> gb_mat;
    std::vector<Octahedral24BitNormalPadded32b> gb_gn, gb_sn;
    std::vector<float3> gb_pos;
    std::vector<int> gb_prim;
    unsigned char still_active = 0;
    AtomicType<unsigned int> converged{0};
    HIPRTRenderData rd;

    Frame(RefRenderScene* s, const int32_t* settings_i, const float* settings_f, const float* inverse_view,
          const float* inverse_projection, uint32_t sample_number, uint32_t random_number)
        : W(settings_i[0]), H(settings_i[1])
    {
        const int n_pix = W * H;
        accum.assign(n_pix, ColorRGB32F(0.0f));
        pixel_active.assign(n_pix, 0);
        den_normals.resize(n_pix);
        den_albedo.resize(n_pix);
        gb_mat.resize(n_pix);
        gb_gn.resize(n_pix);
        gb_sn.resize(n_pix);
        gb_pos.resize(n_pix);
        gb_prim.assign(n_pix, -1);

        rd.random_number = random_number;
        rd.buffers.accumulated_ray_colors = accum.data();
        rd.buffers.triangles_indices = s->indices.data();
        rd.buffers.vertices_positions = s->positions.data();
        rd.buffers.has_vertex_normals = s->has_normals.data();
        rd.buffers.vertex_normals = s->normals.data();
        rd.buffers.texcoords = s->texcoords.data();
        rd.buffers.triangles_areas = s->areas.data();
        rd.buffers.material_indices = s->material_of.data();
        rd.buffers.materials_buffer = s->materials.get_device_SoA_struct();
        rd.buffers.material_opaque = s->opaque.data();
        rd.buffers.emissive_triangles_count = (int)s->emissive.size();
        rd.buffers.emissive_triangles_primitive_indices = s->emissive.data();
        rd.buffers.emissive_triangles_primitive_indices_and_emissive_textures = s->emissive.data();
        rd.buffers.emissives_power_alias_table.alias_table_probas = s->alias_probas.data();
        rd.buffers.emissives_power_alias_table.alias_table_alias = s->alias_alias.data();
        rd.buffers.emissives_power_alias_table.sum_elements = s->power_sum;
        rd.buffers.emissives_power_alias_table.size = (int)s->emissive.size();

        rd.aux_buffers.pixel_active = pixel_active.data();
        rd.aux_buffers.denoiser_normals = den_normals.data();
        rd.aux_buffers.denoiser_albedo = den_albedo.data();
        rd.aux_buffers.still_one_ray_active = &still_active;
        rd.aux_buffers.pixel_count_converged_so_far = &converged;

        rd.g_buffer.materials = gb_mat.data();
        rd.g_buffer.geometric_normals = gb_gn.data();
        rd.g_buffer.shading_normals = gb_sn.data();
        rd.g_buffer.primary_hit_position = gb_pos.data();
        rd.g_buffer.first_hit_prim_index = gb_prim.data();

        HIPRTRenderSettings& rs = rd.render_settings;
        rs.render_resolution = make_int2(W, H);
        rs.need_to_reset = true;
        rs.sample_number = sample_number;
        rs.nb_bounces = settings_i[2];
        rs.do_russian_roulette = settings_i[3] != 0;
        rs.russian_roulette_min_depth = settings_i[4];
        rs.russian_roulette_throughput_clamp = settings_f[0];
        rs.do_alpha_testing = false;
        rs.enable_adaptive_sampling = false;
        rs.stop_pixel_noise_threshold = 0.0f;
        rs.do_update_status_buffers = false;
        rs.ris_settings.number_of_light_candidates = settings_i[6];
        rs.ris_settings.number_of_bsdf_candidates = settings_i[7];

        rd.world_settings.ambient_light_type = AmbientLightType::NONE;

        HIPRTCamera cam;
        std::memcpy(&cam.inverse_view, inverse_view, 16 * sizeof(float));
        std::memcpy(&cam.inverse_projection, inverse_projection, 16 * sizeof(float));
        cam.position = make_float3(inverse_view[3], inverse_view[7], inverse_view[11]);
        cam.do_jittering = settings_i[5] != 0;
        cam.sensor_width = W;
        cam.sensor_height = H;
        rd.current_camera = cam;
        rd.prev_camera = cam;

        rd.cpu_only.bvh = s->bvh;
        rd.cpu_only.light_bvh = s->light_bvh;
    }
};

}  // namespace

/* One frame: CameraRays then MegaKernel over every pixel. settings_i = {width, height,
 * nb_bounces, do_russian_roulette, russian_roulette_min_depth, do_jittering, RIS light
 * candidates, RIS BSDF candidates}, settings_f =
 * {russian_roulette_throughput_clamp}; inverse_view / inverse_projection row-major as
 * HIPRTCamera holds them; the camera position is the translation column of inverse_view
 * (what Camera::to_hiprt's row-vector product with it gives, src/Scene/Camera.cpp:24-25).
 * random_number_camera / random_number_megakernel: HIPRTRenderData::random_number of the two
 * launches. out_rgb (W*H*3): the frame's sample of every pixel. Also returns, when not NULL, the
 * packed G-buffer the camera pass wrote: gbuf_prim (W*H), gbuf_pos (W*H*3). */
REF_EXPORT void refr_render(void* h, const int32_t* settings_i, const float* settings_f, const float* inverse_view,
                            const float* inverse_projection, uint32_t sample_number, uint32_t random_number_camera,
                            uint32_t random_number_megakernel, float* out_rgb, int32_t* gbuf_prim, float* gbuf_pos)
{
    RefRenderScene* s = static_cast<RefRenderScene*>(h);
    Frame f(s, settings_i, settings_f, inverse_view, inverse_projection, sample_number, random_number_camera);
    const int W = f.W, H = f.H;
    HIPRTRenderData& rd = f.rd;

#pragma omp parallel for schedule(dynamic)
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) CameraRays(rd, x, y);
    // each render pass sets its own random number before its launch (FillGBufferRenderPass and
    // MegaKernelRenderPass::launch_async draw one each from the renderer's generator)
    rd.random_number = random_number_megakernel;
#pragma omp parallel for schedule(dynamic)
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) MegaKernel(rd, x, y);

    for (int i = 0; i < W * H; i++)
    {
        out_rgb[3 * i] = f.accum[i].r;
        out_rgb[3 * i + 1] = f.accum[i].g;
        out_rgb[3 * i + 2] = f.accum[i].b;
        if (gbuf_prim) gbuf_prim[i] = f.gb_prim[i];
        if (gbuf_pos)
        {
            gbuf_pos[3 * i] = f.gb_pos[i].x;
            gbuf_pos[3 * i + 1] = f.gb_pos[i].y;
            gbuf_pos[3 * i + 2] = f.gb_pos[i].z;
        }
    }
}

/* The material the reference's kernels see after packing (pack_to_GPU, the 8-bit fields of
 * DevicePackedEffectiveMaterial, src/HostDeviceCommon/Material/MaterialPacked.h) and unpacking,
 * written back in the 64-word layout (word 45, the diffuse-lobe selector, copied; 56..63 zero). */
REF_EXPORT void refr_pack_unpack_material(const float* in, float* out)
{
    CPUMaterial c = cpu_material(in);
    DevicePackedEffectiveMaterial p = c.pack_to_GPU();
    DeviceUnpackedEffectiveMaterial m = p.unpack();
    float w[64] = {};
    w[0] = m.base_color.r; w[1] = m.base_color.g; w[2] = m.base_color.b;
    w[3] = m.roughness;
    w[4] = m.emission.r; w[5] = m.emission.g; w[6] = m.emission.b;
    w[7] = m.metallic;
    w[8] = m.metallic_F82.r; w[9] = m.metallic_F82.g; w[10] = m.metallic_F82.b;
    w[11] = m.metallic_F90_falloff_exponent;
    w[12] = m.metallic_F90.r; w[13] = m.metallic_F90.g; w[14] = m.metallic_F90.b;
    w[15] = m.anisotropy;
    w[16] = m.anisotropy_rotation;
    w[17] = m.second_roughness_weight;
    w[18] = m.second_roughness;
    w[19] = m.specular;
    w[20] = m.specular_color.r; w[21] = m.specular_color.g; w[22] = m.specular_color.b;
    w[23] = m.specular_tint;
    w[24] = m.specular_darkening;
    w[25] = m.coat;
    w[26] = m.coat_roughness;
    w[27] = m.coat_roughening;
    w[28] = m.coat_medium_absorption.r; w[29] = m.coat_medium_absorption.g; w[30] = m.coat_medium_absorption.b;
    w[31] = m.coat_medium_thickness;
    w[32] = m.coat_darkening;
    w[33] = m.coat_anisotropy;
    w[34] = m.coat_anisotropy_rotation;
    w[35] = m.coat_ior;
    w[36] = m.sheen;
    w[37] = m.ior;
    w[38] = m.specular_transmission;
    w[39] = m.diffuse_transmission;
    w[40] = m.absorption_color.r; w[41] = m.absorption_color.g; w[42] = m.absorption_color.b;
    w[43] = m.absorption_at_distance;
    int32_t thin = m.thin_walled ? 1 : 0;
    std::memcpy(w + 44, &thin, 4);
    w[45] = in[45];  // the diffuse-lobe selector: a compile-time option of the reference, copied
    w[46] = m.oren_nayar_sigma;
    w[47] = m.thin_film;
    w[48] = m.thin_film_ior;
    w[49] = m.thin_film_thickness;
    w[50] = m.thin_film_kappa_3;
    w[51] = m.thin_film_hue_shift_degrees;
    w[52] = m.thin_film_base_ior_override;
    int32_t tf_override = m.thin_film_do_ior_override ? 1 : 0;
    std::memcpy(w + 53, &tf_override, 4);
    w[54] = m.dispersion_scale;
    w[55] = m.dispersion_abbe_number;
    std::memcpy(out, w, sizeof(w));
}

/* Octahedral24BitNormalPadded32b pack then unpack (src/HostDeviceCommon/Packing.h:237-367) of n
 * normals; packed (may be NULL) gets the three bytes x | y << 8 | z << 16. */
REF_EXPORT void refr_oct24(const float* in, int64_t n, float* out, uint32_t* packed)
{
    for (int64_t i = 0; i < n; i++)
    {
        Octahedral24BitNormalPadded32b p = Octahedral24BitNormalPadded32b::pack_static(make_float3(in[3 * i], in[3 * i + 1], in[3 * i + 2]));
        float3 u = p.unpack();
        out[3 * i] = u.x;
        out[3 * i + 1] = u.y;
        out[3 * i + 2] = u.z;
        if (packed)
        {
            unsigned char b[4];
            std::memcpy(b, &p, 4);
            packed[i] = (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16);
        }
    }
}


#if REF_RESTIR
/* ReSTIR DI frames (build with REF_DIRECT = LSS_RESTIR_DI): the reference's GPU renderer's pass
 * sequence per frame (FillGBufferRenderPass, ReSTIRDIRenderPass::launch_async and its configure_*
 * functions, src/Renderer/RenderPasses/ReSTIRDIRenderPass.cpp:440-600, MegaKernelRenderPass),
 * run on the CPU kernels pixel by pixel:
 *   CameraRays (G-buffer; the previous frame's kept in g_buffer_prev_frame),
 *   ReSTIR_DI_InitialCandidates -> initial reservoirs,
 *   ReSTIR_DI_TemporalReuse (input: last frame's output; output: the initial buffer when spatial
 *     reuse follows, else the spatial buffer of the frame's parity),
 *   ReSTIR_DI_SpatialReuse per pass (pass 0: temporal/initial output -> spatial 1, then ping-pong),
 *   MegaKernel (ReSTIR DI final shading at the camera hit; RIS at later bounces, the reference's
 *     ReSTIR_DI_LaterBouncesSamplingStrategy default).
 * The camera moves (render_settings.accumulate = false): the temporal pass backprojects through
 * prev_camera.view_projection. Reservoirs are exported as 8 words per pixel: point xyz, target
 * function, triangle, (M << 9) | flags, weight sum, UCW. */
namespace {

struct RefRestirState
{
    int W = 0, H = 0;
    bool first = true, odd_frame = false;
    std::vector<DevicePackedEffectiveMaterial> mat, pmat;
    std::vector<Octahedral24BitNormalPadded32b> gn, sn, pgn, psn;
    std::vector<float3> pos, ppos;
    std::vector<int> prim, pprim;
    std::vector<ReSTIRDIReservoir> initial, spatial1, spatial2;
    ReSTIRDIReservoir* last_output = nullptr;
};

void export_reservoirs(const std::vector<ReSTIRDIReservoir>& in, const ReSTIRDIReservoir* src, float* out)
{
    if (!out || !src) return;
    for (size_t i = 0; i < in.size(); i++)
    {
        const ReSTIRDIReservoir& r = src[i];
        float* o = out + 8 * i;
        o[0] = r.sample.point_on_light_source.x;
        o[1] = r.sample.point_on_light_source.y;
        o[2] = r.sample.point_on_light_source.z;
        o[3] = r.sample.target_function;
        int32_t t = r.sample.emissive_triangle_index, mf = (r.M << 9) | (int32_t)(r.sample.flags & 0x1FF);
        std::memcpy(o + 4, &t, 4);
        std::memcpy(o + 5, &mf, 4);
        o[6] = r.weight_sum;
        o[7] = r.UCW;
    }
}

}  // namespace

REF_EXPORT void* refr_restir_create(int32_t W, int32_t H)
{
    RefRestirState* st = new RefRestirState();
    const size_t n = (size_t)W * H;
    st->W = W;
    st->H = H;
    st->mat.resize(n);
    st->pmat.resize(n);
    st->gn.resize(n);
    st->sn.resize(n);
    st->pgn.resize(n);
    st->psn.resize(n);
    st->pos.assign(n, make_float3(0.0f, 0.0f, 0.0f));
    st->ppos.assign(n, make_float3(0.0f, 0.0f, 0.0f));
    st->prim.assign(n, -1);
    st->pprim.assign(n, -1);
    st->initial.resize(n);
    st->spatial1.resize(n);
    st->spatial2.resize(n);
    return st;
}

REF_EXPORT void refr_restir_free(void* h) { delete static_cast<RefRestirState*>(h); }

/* One frame. settings_i: refr_render's eight, then {light candidates, BSDF candidates, temporal
 * reuse on, temporal search count, temporal search radius, spatial reuse on, spatial passes,
 * spatial neighbours, spatial radius, M-cap, confidence weights}; settings_f: {RR throughput
 * clamp, normal similarity cosine, plane distance threshold}. prev_inverse_view / prev_vp: the
 * previous frame's camera (position from the translation column; view-projection row-major).
 * random_numbers: the passes' HIPRTRenderData::random_number in launch order: camera, initial,
 * [temporal, permutation bits], spatial pass 0..P-1, MegaKernel. Any output may be NULL:
 * out_rgb (W*H*3), reservoirs after the initial / temporal / last spatial pass (W*H*8), the final
 * (shaded) reservoirs, the G-buffer's primitives and positions. */
REF_EXPORT void refr_restir_frame(void* scene, void* state, const int32_t* settings_i, const float* settings_f,
                                  const float* inverse_view, const float* inverse_projection,
                                  const float* prev_inverse_view, const float* prev_vp, uint32_t sample_number,
                                  const uint32_t* random_numbers, float* out_rgb, float* res_initial, float* res_temporal,
                                  float* res_final, int32_t* gbuf_prim, float* gbuf_pos)
{
    RefRenderScene* s = static_cast<RefRenderScene*>(scene);
    RefRestirState* st = static_cast<RefRestirState*>(state);
    Frame f(s, settings_i, settings_f, inverse_view, inverse_projection, sample_number, random_numbers[0]);
    const int W = f.W, H = f.H;
    HIPRTRenderData& rd = f.rd;
    HIPRTRenderSettings& rs = rd.render_settings;
    rs.need_to_reset = st->first;
    rs.accumulate = false;

    rd.g_buffer.materials = st->mat.data();
    rd.g_buffer.geometric_normals = st->gn.data();
    rd.g_buffer.shading_normals = st->sn.data();
    rd.g_buffer.primary_hit_position = st->pos.data();
    rd.g_buffer.first_hit_prim_index = st->prim.data();
    rd.g_buffer_prev_frame.materials = st->pmat.data();
    rd.g_buffer_prev_frame.geometric_normals = st->pgn.data();
    rd.g_buffer_prev_frame.shading_normals = st->psn.data();
    rd.g_buffer_prev_frame.primary_hit_position = st->ppos.data();
    rd.g_buffer_prev_frame.first_hit_prim_index = st->pprim.data();

    HIPRTCamera prev = rd.current_camera;
    prev.position = make_float3(prev_inverse_view[3], prev_inverse_view[7], prev_inverse_view[11]);
    std::memcpy(&prev.inverse_view, prev_inverse_view, 16 * sizeof(float));
    std::memcpy(&prev.view_projection, prev_vp, 16 * sizeof(float));
    rd.prev_camera = prev;

    ReSTIRDISettings& rds = rs.restir_di_settings;
    rds.initial_candidates.number_of_initial_light_candidates = settings_i[8];
    rds.initial_candidates.number_of_initial_bsdf_candidates = settings_i[9];
    rds.common_temporal_pass.do_temporal_reuse_pass = settings_i[10] != 0;
    rds.common_temporal_pass.max_neighbor_search_count = settings_i[11];
    rds.common_temporal_pass.neighbor_search_radius = settings_i[12];
    rds.common_spatial_pass.do_spatial_reuse_pass = settings_i[13] != 0;
    rds.common_spatial_pass.number_of_passes = settings_i[14];
    rds.common_spatial_pass.reuse_neighbor_count = settings_i[15];
    rds.common_spatial_pass.neighbor_visibility_count = settings_i[15];
    rds.common_spatial_pass.reuse_radius = settings_i[16];
    rds.common_spatial_pass.auto_reuse_radius = false;
    rds.m_cap = settings_i[17];
    rds.use_confidence_weights = settings_i[18] != 0;
    rds.neighbor_similarity_settings.normal_similarity_angle_precomp = settings_f[1];
    rds.neighbor_similarity_settings.plane_distance_threshold = settings_f[2];
    rds.light_presampling.light_samples = nullptr;
    const int passes = rds.common_spatial_pass.do_spatial_reuse_pass ? rds.common_spatial_pass.number_of_passes : 0;
    const bool temporal = rds.common_temporal_pass.do_temporal_reuse_pass;
    if (!st->last_output) st->last_output = st->spatial2.data();

    auto each_pixel = [&](auto&& fn) {
#pragma omp parallel for schedule(dynamic)
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) fn(x, y);
    };
    int k = 0;
    rd.random_number = random_numbers[k++];
    each_pixel([&](int x, int y) { CameraRays(rd, x, y); });

    rd.random_number = random_numbers[k++];
    rds.initial_candidates.output_reservoirs = st->initial.data();
    each_pixel([&](int x, int y) { ReSTIR_DI_InitialCandidates(rd, x, y); });
    export_reservoirs(st->initial, st->initial.data(), res_initial);

    ReSTIRDIReservoir* out = st->initial.data();
    if (temporal)
    {
        rd.random_number = random_numbers[k++];
        rds.common_temporal_pass.permutation_sampling_random_bits = random_numbers[k++];
        rds.temporal_pass.input_reservoirs = st->last_output;
        rds.temporal_pass.output_reservoirs =
            passes > 0 ? st->initial.data() : (st->odd_frame ? st->spatial1.data() : st->spatial2.data());
        each_pixel([&](int x, int y) { ReSTIR_DI_TemporalReuse(rd, x, y); });
        out = rds.temporal_pass.output_reservoirs;
        export_reservoirs(st->initial, out, res_temporal);
    }
    for (int p = 0; p < passes; p++)
    {
        rd.random_number = random_numbers[k++];
        rds.common_spatial_pass.spatial_pass_index = p;
        if (p == 0)
        {
            rds.spatial_pass.input_reservoirs = out;
            rds.spatial_pass.output_reservoirs = st->spatial1.data();
        }
        else if ((p & 1) == 0)
        {
            rds.spatial_pass.input_reservoirs = st->spatial2.data();
            rds.spatial_pass.output_reservoirs = st->spatial1.data();
        }
        else
        {
            rds.spatial_pass.input_reservoirs = st->spatial1.data();
            rds.spatial_pass.output_reservoirs = st->spatial2.data();
        }
        each_pixel([&](int x, int y) { ReSTIR_DI_SpatialReuse(rd, x, y); });
        out = rds.spatial_pass.output_reservoirs;
    }
    rds.restir_output_reservoirs = out;
    st->last_output = out;
    st->odd_frame = !st->odd_frame;

    rd.random_number = random_numbers[k++];
    each_pixel([&](int x, int y) { MegaKernel(rd, x, y); });
    export_reservoirs(st->initial, out, res_final);
    st->first = false;

    for (int i = 0; i < W * H; i++)
    {
        if (out_rgb)
        {
            out_rgb[3 * i] = f.accum[i].r;
            out_rgb[3 * i + 1] = f.accum[i].g;
            out_rgb[3 * i + 2] = f.accum[i].b;
        }
        if (gbuf_prim) gbuf_prim[i] = st->prim[i];
        if (gbuf_pos)
        {
            gbuf_pos[3 * i] = st->pos[i].x;
            gbuf_pos[3 * i + 1] = st->pos[i].y;
            gbuf_pos[3 * i + 2] = st->pos[i].z;
        }
    }
}
#endif
