// C ABI of the render path: scene upload + light table, renderer buffers, pass scheduling
// (declared in include/gbpt_render.h).
//
// Replaces, for this path, the reference's GPURenderer scene upload and alias-table build
// (src/Renderer/GPURenderer.cpp:173-295,822-958), its RAII device buffers
// (src/HIPRT-Orochi/OrochiBuffer.h:21) and the render-thread pass loop
// (src/Renderer/GPURendererThread.cpp:311-330).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/gbpt_render.h"
#include "guide_kernels.h"
#include "handles.h"
#include "render_common.h"
#include "render_kernels.h"

namespace {

using gbpt::cuda_error;
using gbpt::set_error;

struct DevMem
{
    std::vector<void*> ptrs;
    cudaError_t err = cudaSuccess;
    template <typename T>
    T* alloc(size_t count)
    {
        if (err != cudaSuccess) return nullptr;
        void* p = nullptr;
        size_t bytes = count * sizeof(T);
        if (bytes == 0) bytes = 16;
        err = cudaMalloc(&p, bytes);
        if (err != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        return static_cast<T*>(p);
    }
    void release()
    {
        for (void* p : ptrs) cudaFree(p);
        ptrs.clear();
        err = cudaSuccess;
    }
};

int sm_count()
{
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

}  // namespace

struct gbpt_scene
{
    gbpt_bvh* bvh = nullptr;
    bool principled = false;
    DevMem mem;
    gbpt::SceneView view;
    int32_t n_emissive = 0;
    double power_sum64 = 0.0;
    // the world: ambient light and envmap tables (view.env points into env_mem)
    DevMem env_mem;
    float* env_cdf = nullptr;
    uint2* env_alias = nullptr;
    double env_sum64 = 0.0;
    mutable int batch_refs = 0;  // batches holding a copy of 'view' (the world cannot change under them)
};

struct gbpt_renderer
{
    const gbpt_scene* scene = nullptr;
    gbpt::RenderConst rc;
    // GBPT_RNG_REFERENCE: the host generator of the per-launch random numbers (CPURenderer::m_rng)
    uint32_t rng_seed = 42u, host_rng = 42u;
    // ... and the ReSTIR DI passes' numbers of the current sample: initial, temporal, spatial 0..3
    uint32_t rn_initial = 0u, rn_temporal = 0u, rn_spatial[4] = {0u, 0u, 0u, 0u};
    DevMem mem;
    gbpt::PathBuffers pb;
    gbpt::Queue q[2], shadow, bsdfq;
    int cur = 0;
    int64_t capacity = 0;
    float* acc32 = nullptr;
    double* acc64 = nullptr;
    unsigned long long* stats = nullptr;  // extension, shadow, bsdf-light rays
    int64_t iteration = 0;
    int64_t samples = 0;
    int n_sm = 1;
    // ReSTIR DI
    bool restir = false;
    gbpt_restir_di_settings restir_settings;
    DevMem restir_mem;
    gbpt::GBuffer gb[2];
    int gb_cur = 0;
    gbpt::ReservoirBuf res[5];  // initial, temporal, spatial ping, spatial pong, previous
    float4* presampled = nullptr;  // light presampling records (null: off)
    gbpt::InitialState initial_state{};  // per-pixel state between the initial-candidates phases
    int32_t* spatial_ray_of = nullptr;   // spatial reuse: bias-correction ray per pixel and neighbour
    gbpt::Queue spatial_rays{};          // their any-hit queue (pixels x spatial neighbours)
    int2* temporal_ray_of = nullptr;     // temporal reuse: its two bias-correction rays per pixel
    gbpt::Queue temporal_rays{};         // their any-hit queue (2 x pixels)
    int res_final = 0;
    bool has_prev = false;
    float prev_inverse_view[16];
    // learned path guiding
    gbpt_guide* guide = nullptr;
    gbpt_guide_render_settings guide_settings;
    DevMem guide_mem;
    gbpt::GuideView gv;  // gv.lobes == nullptr: off
    float* guide_lobes = nullptr;
    float* guide_pdf = nullptr;  // per path: MIS pdf of the last guided continuation
    // envmap direct lighting: per-path entries and the any-hit queue (allocated once the scene's
    // envmap is importance sampled)
    DevMem env_mem;
    gbpt::Queue envq;
    bool env_ready = false;
};

namespace {

gbpt::Queue make_queue(DevMem& m, int64_t cap, bool closest_out, bool any_out)
{
    gbpt::Queue q;
    std::memset(&q, 0, sizeof(q));
    q.origin_tmin = m.alloc<float4>(cap);
    q.dir_tmax = m.alloc<float4>(cap);
    q.last_prim = m.alloc<int32_t>(cap);
    q.slot = m.alloc<int32_t>(cap);
    q.hits = closest_out ? m.alloc<float4>(cap) : nullptr;
    q.occluded = any_out ? m.alloc<uint8_t>(cap) : nullptr;
    q.count = m.alloc<int32_t>(1);
    return q;
}

bool is_emissive(const gbpt_material& m) { return m.emission[0] > 0.0f || m.emission[1] > 0.0f || m.emission[2] > 0.0f; }

float lerpf(float a, float b, float t) { return (1.0f - t) * a + t * b; }

// inverse of a row-major 4x4 (Gauss-Jordan with partial pivoting, in double); false if singular
bool invert4(const double* m, double* out)
{
    double a[4][8];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 8; j++) a[i][j] = j < 4 ? m[4 * i + j] : (j - 4 == i ? 1.0 : 0.0);
    for (int c = 0; c < 4; c++)
    {
        int piv = c;
        for (int r = c + 1; r < 4; r++)
            if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
        if (std::fabs(a[piv][c]) < 1e-300) return false;
        if (piv != c)
            for (int j = 0; j < 8; j++) std::swap(a[c][j], a[piv][j]);
        const double d = a[c][c];
        for (int j = 0; j < 8; j++) a[c][j] /= d;
        for (int r = 0; r < 4; r++)
            if (r != c)
            {
                const double f = a[r][c];
                for (int j = 0; j < 8; j++) a[r][j] -= f * a[c][j];
            }
    }
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) out[4 * i + j] = a[i][j + 4];
    return true;
}

// view-projection (world -> NDC, points on the right) of a camera given by its inverse view and
// inverse projection: the inverse of inverse_view * inverse_projection
bool view_projection(const float* iv, const float* ip, float* vp)
{
    double prod[16], inv[16];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
        {
            double acc = 0.0;
            for (int k = 0; k < 4; k++) acc += (double)iv[4 * i + k] * (double)ip[4 * k + j];
            prod[4 * i + j] = acc;
        }
    if (!invert4(prod, inv)) return false;
    for (int i = 0; i < 16; i++) vp[i] = (float)inv[i];
    return true;
}

void camera_position(const float* iv, float* pos)
{
    const float w = iv[15] != 0.0f ? iv[15] : 1.0f;
    pos[0] = iv[3] / w;
    pos[1] = iv[7] / w;
    pos[2] = iv[11] / w;
}
float pow4f(float x)
{
    const float x2 = x * x;
    return x2 * x2;
}

// Coat roughening of the base and second metal roughness, as the reference's material fetch
// applies it (src/Device/includes/Material.h:122-146; OpenPBR coat roughening), done once here.
gbpt_principled_material effective_material(gbpt_principled_material m)
{
    const float coat = m.coat, roughening = m.coat_roughening;
    if (coat > 0.0f && roughening > 0.0f)
    {
        const float cr4 = pow4f(m.coat_roughness);
        const float base = m.roughness;
        const float target = sqrtf(sqrtf(std::min(1.0f, pow4f(base) + 2.0f * cr4)));
        m.roughness = lerpf(base, lerpf(base, target, coat), roughening);
        if (m.second_roughness_weight > 0.0f)
        {
            const float second = m.second_roughness;
            const float target2 = sqrtf(sqrtf(std::min(1.0f, pow4f(second) + 2.0f * cr4)));
            m.second_roughness = lerpf(second, lerpf(second, target2, coat), roughening);
        }
    }
    return m;
}

// The reference's 8-bit material fields (DevicePackedEffectiveMaterial,
// src/HostDeviceCommon/Material/MaterialPacked.h:16-520, with the accessors of
// src/HostDeviceCommon/Packing.h:16-200): a value in [0, 1] is stored as the byte (unsigned
// char)(x * 255) and read back as byte * (1 / 255); the green channel of a packed colour is read
// as (byte << 8) * (1 / 65280). Values outside [0, 1] are clamped to the byte range first.
uint32_t byte_of(float x)
{
    const float v = x * 255.0f;
    if (!(v > 0.0f)) return 0u;
    if (v >= 255.0f) return 255u;
    return (uint32_t)v;
}
float unpack_byte(float x) { return (float)byte_of(x) * (1.0f / 255.0f); }
void unpack_color(float* c)
{
    const uint32_t r = byte_of(c[0]), g = byte_of(c[1]), b = byte_of(c[2]);
    c[0] = (float)r * (1.0f / 255.0f);
    c[1] = (float)(g << 8) * (1.0f / 65280.0f);
    c[2] = (float)b * (1.0f / 255.0f);
}

// A material as the reference's kernels read it back from its packed record
// (CPUMaterial::pack_to_GPU then DevicePackedEffectiveMaterial::unpack)
gbpt_principled_material packed_material(gbpt_principled_material m)
{
    unpack_color(m.base_color);
    m.roughness = unpack_byte(m.roughness);
    m.metallic = unpack_byte(m.metallic);
    unpack_color(m.metallic_F82);
    unpack_color(m.metallic_F90);
    m.diffuse_transmission = unpack_byte(m.diffuse_transmission);
    m.anisotropy = unpack_byte(m.anisotropy);
    m.anisotropy_rotation = unpack_byte(m.anisotropy_rotation);
    m.second_roughness_weight = unpack_byte(m.second_roughness_weight);
    m.second_roughness = unpack_byte(m.second_roughness);
    unpack_color(m.specular_color);
    m.specular_tint = unpack_byte(m.specular_tint);
    m.specular = unpack_byte(m.specular);
    m.specular_darkening = unpack_byte(m.specular_darkening);
    m.coat_roughness = unpack_byte(m.coat_roughness);
    m.coat = unpack_byte(m.coat);
    unpack_color(m.coat_medium_absorption);
    m.coat_roughening = unpack_byte(m.coat_roughening);
    m.coat_darkening = unpack_byte(m.coat_darkening);
    m.coat_anisotropy = unpack_byte(m.coat_anisotropy);
    m.coat_anisotropy_rotation = unpack_byte(m.coat_anisotropy_rotation);
    m.sheen = unpack_byte(m.sheen);
    unpack_color(m.absorption_color);
    m.specular_transmission = unpack_byte(m.specular_transmission);
    m.thin_film = unpack_byte(m.thin_film);
    m.dispersion_scale = unpack_byte(m.dispersion_scale);
    m.thin_film_hue_shift = unpack_byte(m.thin_film_hue_shift);
    // the packed record's setter takes a bool (set_thin_film_base_ior_override,
    // MaterialPacked.h:347): any non-zero override IOR arrives as 1
    m.thin_film_base_ior_override = m.thin_film_base_ior_override != 0.0f ? 1.0f : 0.0f;
    return m;
}

uint32_t xorshift32_step(uint32_t& state)
{
    uint32_t x = state;
    x ^= x << 13;
    x ^= x >> 17;
    x ^= x << 5;
    state = x;
    return x;
}

}  // namespace

extern "C" {

gbpt_status gbpt_material_pack_8bit(const gbpt_principled_material* in, int32_t n, gbpt_principled_material* out)
{
    if (n < 0 || (n > 0 && (!in || !out))) return set_error(GBPT_ERROR_INVALID_ARG, "NULL material array or negative count");
    for (int32_t m = 0; m < n; m++) out[m] = packed_material(in[m]);
    return GBPT_OK;
}

gbpt_status gbpt_scene_create(const gbpt_scene_desc* d, const gbpt_bvh_params* bvh_params, gbpt_scene** out,
                              void* stream)
{
    if (!out) return set_error(GBPT_ERROR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (!d) return set_error(GBPT_ERROR_INVALID_ARG, "desc is NULL");
    if (d->n_triangles < 0 || d->n_vertices < 0 || d->n_materials < 0)
        return set_error(GBPT_ERROR_INVALID_ARG, "negative sizes");
    if (d->n_triangles > 0 && (!d->indices || !d->positions || !d->material_indices))
        return set_error(GBPT_ERROR_INVALID_ARG, "geometry buffers are NULL");
    if (d->n_materials > 0 && !d->materials && !d->principled_materials)
        return set_error(GBPT_ERROR_INVALID_ARG, "materials and principled_materials are both NULL");
    if (d->material_packing != GBPT_MATERIALS_FLOAT && d->material_packing != GBPT_MATERIALS_PACKED)
        return set_error(GBPT_ERROR_INVALID_ARG, "unknown material_packing");
    const bool packed = d->material_packing == GBPT_MATERIALS_PACKED;
    // the emission/base colour view used by light sampling: the plain materials, else the
    // principled ones
    std::vector<gbpt_material> plain;
    if (d->principled_materials)
    {
        for (int32_t m = 0; m < d->n_materials; m++)
        {
            const gbpt_principled_material& pm = d->principled_materials[m];
            if (pm.sheen != 0.0f)
                return set_error(GBPT_ERROR_UNSUPPORTED, "material " + std::to_string(m) + ": the sheen lobe is not built (sheen must be 0)");
            if (!(pm.ior > 0.0f) || !(pm.coat_ior > 0.0f))
                return set_error(GBPT_ERROR_INVALID_ARG, "material " + std::to_string(m) + " has a non-positive IOR");
            if (pm.diffuse_lobe != GBPT_DIFFUSE_LAMBERTIAN && pm.diffuse_lobe != GBPT_DIFFUSE_OREN_NAYAR)
                return set_error(GBPT_ERROR_INVALID_ARG, "material " + std::to_string(m) + ": unknown diffuse_lobe");
            if (pm.diffuse_lobe == GBPT_DIFFUSE_OREN_NAYAR && !(pm.oren_nayar_sigma >= 0.0f))
                return set_error(GBPT_ERROR_INVALID_ARG, "material " + std::to_string(m) + ": negative oren_nayar_sigma");
        }
        if (!d->materials)
        {
            plain.resize(d->n_materials);
            for (int32_t m = 0; m < d->n_materials; m++)
                for (int k = 0; k < 3; k++)
                {
                    plain[m].base_color[k] = d->principled_materials[m].base_color[k];
                    plain[m].emission[k] = d->principled_materials[m].emission[k];
                }
        }
    }
    const gbpt_material* materials = d->materials ? d->materials : plain.data();
    for (int64_t t = 0; t < d->n_triangles; t++)
        if (d->material_indices[t] < 0 || d->material_indices[t] >= d->n_materials)
            return set_error(GBPT_ERROR_INVALID_ARG, "triangle " + std::to_string(t) + " has an out-of-range material index");
    for (int32_t m = 0; m < d->n_materials; m++)
        for (int k = 0; k < 3; k++)
            if (!std::isfinite(materials[m].emission[k]) || materials[m].emission[k] < 0.0f)
                return set_error(GBPT_ERROR_INVALID_ARG, "material " + std::to_string(m) + " has an invalid emission");
    // smooth-shading normals: finite; a zero normal marks a vertex without one
    std::vector<float4> normals;
    if (d->vertex_normals)
    {
        normals.resize(d->n_vertices);
        for (int64_t v = 0; v < d->n_vertices; v++)
        {
            const float* n = d->vertex_normals + 3 * v;
            if (!std::isfinite(n[0]) || !std::isfinite(n[1]) || !std::isfinite(n[2]))
                return set_error(GBPT_ERROR_INVALID_ARG, "vertex " + std::to_string(v) + " has a non-finite normal");
            const bool has = n[0] != 0.0f || n[1] != 0.0f || n[2] != 0.0f;
            normals[v] = make_float4(n[0], n[1], n[2], has ? 1.0f : 0.0f);
        }
    }

    gbpt_scene* s = new (std::nothrow) gbpt_scene();
    if (!s) return set_error(GBPT_ERROR_OOM, "host allocation failed");
    gbpt_status st = gbpt_bvh_build(d->indices, d->positions, d->n_vertices, d->n_triangles, bvh_params, &s->bvh);
    if (st != GBPT_OK)
    {
        delete s;
        return st;
    }
    cudaStream_t cs = (cudaStream_t)stream;

    std::vector<float4> verts(d->n_vertices);
    for (int64_t v = 0; v < d->n_vertices; v++)
        verts[v] = make_float4(d->positions[3 * v], d->positions[3 * v + 1], d->positions[3 * v + 2], 0.0f);
    std::vector<gbpt::DeviceMaterial> mats(d->n_materials);
    for (int32_t m = 0; m < d->n_materials; m++)
    {
        const gbpt_material& src = materials[m];
        float base[3] = {src.base_color[0], src.base_color[1], src.base_color[2]};
        if (packed) unpack_color(base);
        mats[m].base_color = make_float4(base[0], base[1], base[2], 0.0f);
        mats[m].emission = make_float4(src.emission[0], src.emission[1], src.emission[2], 0.0f);
    }
    std::vector<int32_t> emissive;
    for (int64_t t = 0; t < d->n_triangles; t++)
        if (is_emissive(materials[d->material_indices[t]])) emissive.push_back((int32_t)t);
    const int32_t ne = (int32_t)emissive.size();

    DevMem& M = s->mem;
    float4* dv = M.alloc<float4>(verts.size());
    int32_t* di = M.alloc<int32_t>(3 * d->n_triangles);
    int32_t* dmo = M.alloc<int32_t>(d->n_triangles);
    gbpt::DeviceMaterial* dm = M.alloc<gbpt::DeviceMaterial>(mats.size());
    int32_t* de = M.alloc<int32_t>(ne);
    float* dprob = M.alloc<float>(ne);
    int32_t* dalias = M.alloc<int32_t>(ne);
    float* dpower = M.alloc<float>(ne);
    const int n_partial = 64;
    double* dpartial = M.alloc<double>(n_partial);
    double* dsum = M.alloc<double>(1);
    double* dq = M.alloc<double>(ne);
    int32_t* dsmall = M.alloc<int32_t>(ne);
    int32_t* dlarge = M.alloc<int32_t>(ne);
    float4* dn = normals.empty() ? nullptr : M.alloc<float4>(normals.size());
    gbpt_principled_material* dpm = nullptr;
    gbpt_principled_material* dpm_camera = nullptr;
    std::vector<gbpt_principled_material> pmats, pmats_camera;
    if (d->principled_materials)
    {
        // packed: quantised, then coat-roughened as the reference's material fetch does on the
        // unpacked record (Material.h:122-146); the camera-hit table packs that result again, as
        // the reference's G-buffer stores it (CameraRays.h:183)
        for (int32_t m = 0; m < d->n_materials; m++)
        {
            const gbpt_principled_material& raw = d->principled_materials[m];
            pmats.push_back(effective_material(packed ? packed_material(raw) : raw));
            if (packed) pmats_camera.push_back(packed_material(pmats.back()));
        }
        dpm = M.alloc<gbpt_principled_material>(pmats.size());
        if (packed) dpm_camera = M.alloc<gbpt_principled_material>(pmats_camera.size());
    }
    cudaError_t e = M.err;
    if (e == cudaSuccess && dpm)
        e = cudaMemcpyAsync(dpm, pmats.data(), pmats.size() * sizeof(gbpt_principled_material), cudaMemcpyHostToDevice, cs);
    if (e == cudaSuccess && dpm_camera)
        e = cudaMemcpyAsync(dpm_camera, pmats_camera.data(), pmats_camera.size() * sizeof(gbpt_principled_material),
                            cudaMemcpyHostToDevice, cs);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dv, verts.data(), verts.size() * sizeof(float4), cudaMemcpyHostToDevice, cs);
    if (e == cudaSuccess && dn)
        e = cudaMemcpyAsync(dn, normals.data(), normals.size() * sizeof(float4), cudaMemcpyHostToDevice, cs);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(di, d->indices, 3 * d->n_triangles * sizeof(int32_t), cudaMemcpyHostToDevice, cs);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dmo, d->material_indices, d->n_triangles * sizeof(int32_t), cudaMemcpyHostToDevice, cs);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dm, mats.data(), mats.size() * sizeof(gbpt::DeviceMaterial), cudaMemcpyHostToDevice, cs);
    if (e == cudaSuccess && ne > 0)
        e = cudaMemcpyAsync(de, emissive.data(), ne * sizeof(int32_t), cudaMemcpyHostToDevice, cs);

    gbpt::SceneView& v = s->view;
    std::memset(&v, 0, sizeof(v));
    v.vertices = dv;
    v.indices = di;
    v.material_of = dmo;
    v.materials = dm;
    v.emissive = de;
    v.alias_prob = dprob;
    v.alias_index = dalias;
    v.n_emissive = ne;
    v.bvh_nodes = static_cast<const uint4*>(s->bvh->dev.nodes);
    v.bvh_tris = static_cast<const float4*>(s->bvh->dev.tris);
    v.pmats = dpm;
    v.pmats_camera = dpm_camera;
    v.normals = dn;
    s->principled = dpm != nullptr;
    s->n_emissive = ne;
    if (e == cudaSuccess) e = gbpt::launch_light_table(v, dpower, dpartial, n_partial, dsum, dq, dprob, dalias, dsmall, dlarge, cs);
    if (e == cudaSuccess && ne > 0) e = cudaMemcpyAsync(&s->power_sum64, dsum, sizeof(double), cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
    if (e != cudaSuccess)
    {
        M.release();
        gbpt_bvh_destroy(s->bvh);
        delete s;
        return cuda_error(e, "scene upload");
    }
    v.power_sum = (float)s->power_sum64;
    *out = s;
    return GBPT_OK;
}

gbpt_status gbpt_scene_destroy(gbpt_scene* s)
{
    if (!s) return GBPT_OK;
    s->env_mem.release();
    s->mem.release();
    gbpt_status st = gbpt_bvh_destroy(s->bvh);
    delete s;
    return st;
}

gbpt_status gbpt_scene_get_bvh(const gbpt_scene* s, const gbpt_bvh** out)
{
    if (!s || !out) return set_error(GBPT_ERROR_INVALID_ARG, "NULL argument");
    *out = s->bvh;
    return GBPT_OK;
}

gbpt_status gbpt_scene_get_light_table(const gbpt_scene* s, int32_t* n_emissive, int32_t* emissive, float* probas,
                                       int32_t* alias, float* power_sum, double* power_sum64)
{
    if (!s) return set_error(GBPT_ERROR_INVALID_ARG, "scene is NULL");
    const int32_t n = s->n_emissive;
    if (n_emissive) *n_emissive = n;
    if (power_sum) *power_sum = s->view.power_sum;
    if (power_sum64) *power_sum64 = s->power_sum64;
    cudaError_t e = cudaSuccess;
    if (n > 0 && emissive) e = cudaMemcpy(emissive, s->view.emissive, n * sizeof(int32_t), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && n > 0 && probas) e = cudaMemcpy(probas, s->view.alias_prob, n * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && n > 0 && alias) e = cudaMemcpy(alias, s->view.alias_index, n * sizeof(int32_t), cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "light table read-back");
}

namespace {

bool scene_env_sampled(const gbpt_scene* s)
{
    const gbpt::EnvView& e = s->view.env;
    return e.ambient == GBPT_AMBIENT_ENVMAP && e.sampling != GBPT_ENVMAP_NO_SAMPLING && e.intensity > 0.0f;
}

bool finite_nonneg(float x) { return std::isfinite(x) && x >= 0.0f; }

// Vose's alias method over q (texel luminances scaled to mean 1) with FIFO small/large queues
// filled in index order: the partition of Utils::compute_alias_table (src/Utils/Utils.cpp:63-131);
// an entry never paired keeps probability 1 and alias 0, as in the reference's zero-filled vector.
// Runs on the host: it is one sequential O(n) pass, and on one GPU thread each of its steps would
// wait on a dependent memory access. Output: (probability as float bits, alias index) per texel.
void vose_host(std::vector<double>& q, std::vector<uint2>& out)
{
    const size_t n = q.size();
    std::vector<float> prob(n, 0.0f);
    std::vector<int32_t> alias(n, 0), smalls, larges;
    smalls.reserve(n);
    larges.reserve(n);
    for (size_t i = 0; i < n; i++)
    {
        (q[i] < 1.0 ? smalls : larges).push_back((int32_t)i);
    }
    size_t sh = 0, lh = 0;
    while (sh < smalls.size() && lh < larges.size())
    {
        const int32_t si = smalls[sh++], li = larges[lh++];
        prob[si] = (float)q[si];
        alias[si] = li;
        q[li] = (q[li] + q[si]) - 1.0;
        if (q[li] > 1.0)
            larges.push_back(li);
        else
            smalls.push_back(li);
    }
    while (lh < larges.size()) prob[larges[lh++]] = 1.0f;
    while (sh < smalls.size()) prob[smalls[sh++]] = 1.0f;
    out.resize(n);
    for (size_t i = 0; i < n; i++)
    {
        uint32_t bits;
        std::memcpy(&bits, &prob[i], sizeof(bits));
        out[i] = make_uint2(bits, (uint32_t)alias[i]);
    }
}

}  // namespace

gbpt_status gbpt_world_default(gbpt_world_desc* w)
{
    if (!w) return set_error(GBPT_ERROR_INVALID_ARG, "world is NULL");
    std::memset(w, 0, sizeof(*w));
    w->ambient = GBPT_AMBIENT_NONE;
    w->envmap_intensity = 1.0f;
    for (int k = 0; k < 3; k++) w->envmap_to_world[4 * k] = w->world_to_envmap[4 * k] = 1.0f;
    w->envmap_sampling = GBPT_ENVMAP_ALIAS_TABLE;
    w->envmap_bsdf_mis = 1;
    return GBPT_OK;
}

gbpt_status gbpt_scene_set_world(gbpt_scene* s, const gbpt_world_desc* w, void* stream)
{
    if (!s || !w) return set_error(GBPT_ERROR_INVALID_ARG, "NULL argument");
    if (s->batch_refs > 0) return set_error(GBPT_ERROR_INVALID_ARG, "a batch renders this scene: destroy it before changing the world");
    if (w->ambient < GBPT_AMBIENT_NONE || w->ambient > GBPT_AMBIENT_ENVMAP)
        return set_error(GBPT_ERROR_INVALID_ARG, "unknown ambient light type");
    for (int k = 0; k < 3; k++)
        if (!finite_nonneg(w->uniform_color[k])) return set_error(GBPT_ERROR_INVALID_ARG, "uniform_color must be finite and >= 0");
    gbpt::EnvView v;
    std::memset(&v, 0, sizeof(v));
    v.ambient = w->ambient;
    for (int k = 0; k < 3; k++) v.uniform[k] = w->uniform_color[k];
    DevMem fresh;
    double sum64 = 0.0;
    float* cdf = nullptr;
    uint2* alias = nullptr;
    if (w->ambient == GBPT_AMBIENT_ENVMAP)
    {
        const int64_t W = w->envmap_width, H = w->envmap_height, n = W * H;
        if (!w->envmap_rgb || W < 1 || H < 1 || W > 65536 || H > 65536 || n > ((int64_t)1 << 28))
            return set_error(GBPT_ERROR_INVALID_ARG, "envmap needs texels and 1 <= width, height <= 65536 with at most 2^28 texels");
        if (!finite_nonneg(w->envmap_intensity)) return set_error(GBPT_ERROR_INVALID_ARG, "envmap_intensity must be finite and >= 0");
        if (w->envmap_sampling < GBPT_ENVMAP_NO_SAMPLING || w->envmap_sampling > GBPT_ENVMAP_ALIAS_TABLE)
            return set_error(GBPT_ERROR_INVALID_ARG, "unknown envmap_sampling");
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
            {
                double acc = 0.0;
                for (int k = 0; k < 3; k++) acc += (double)w->envmap_to_world[3 * i + k] * w->world_to_envmap[3 * k + j];
                if (!std::isfinite(acc) || std::fabs(acc - (i == j ? 1.0 : 0.0)) > 1.0e-3)
                    return set_error(GBPT_ERROR_INVALID_ARG, "world_to_envmap is not the inverse of envmap_to_world");
            }
        for (int64_t i = 0; i < 3 * n; i++)
            if (!finite_nonneg(w->envmap_rgb[i]))
                return set_error(GBPT_ERROR_INVALID_ARG, "envmap texel " + std::to_string(i / 3) + " is not finite and >= 0");
        cudaStream_t cs = (cudaStream_t)stream;
        const int n_tiles = gbpt::envmap_scan_tiles(n);
        DevMem tmp;
        float* drgb = tmp.alloc<float>(3 * n);
        float* dlum = tmp.alloc<float>(n);
        double* dtile = tmp.alloc<double>(2 * (size_t)n_tiles + 1);
        uint32_t* texels = fresh.alloc<uint32_t>(n);
        cdf = fresh.alloc<float>(n);
        alias = fresh.alloc<uint2>(n);
        cudaError_t e = tmp.err != cudaSuccess ? tmp.err : fresh.err;
        if (e == cudaSuccess) e = cudaMemcpyAsync(drgb, w->envmap_rgb, 3 * n * sizeof(float), cudaMemcpyHostToDevice, cs);
        if (e == cudaSuccess)
            e = gbpt::launch_envmap_tables(drgb, n, texels, dlum, cdf, dtile, dtile + n_tiles, dtile + 2 * n_tiles, cs);
        std::vector<float> lum(n);
        if (e == cudaSuccess) e = cudaMemcpyAsync(lum.data(), dlum, n * sizeof(float), cudaMemcpyDeviceToHost, cs);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&sum64, dtile + 2 * n_tiles, sizeof(double), cudaMemcpyDeviceToHost, cs);
        if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
        std::vector<uint2> table;
        if (e == cudaSuccess)
        {
            if (sum64 > 0.0)
            {
                // alias table of the luminances normalised by the FP64 sum
                std::vector<double> q(n);
                for (int64_t i = 0; i < n; i++) q[i] = (double)lum[i] / sum64 * (double)n;
                vose_host(q, table);
            }
            else
                table.assign(n, make_uint2(0x3F800000u, 0u));  // black envmap: nothing to sample
            e = cudaMemcpyAsync(alias, table.data(), n * sizeof(uint2), cudaMemcpyHostToDevice, cs);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
        tmp.release();
        if (e != cudaSuccess)
        {
            fresh.release();
            return cuda_error(e, "envmap tables");
        }
        v.texels = texels;
        v.cdf = cdf;
        v.alias = alias;
        v.width = (int32_t)W;
        v.height = (int32_t)H;
        v.intensity = w->envmap_intensity;
        v.total_sum = (float)sum64;
        std::memcpy(v.to_world, w->envmap_to_world, sizeof(v.to_world));
        std::memcpy(v.to_env, w->world_to_envmap, sizeof(v.to_env));
        // a black envmap is never sampled (its pdfs would divide by a zero sum)
        v.sampling = sum64 > 0.0 ? w->envmap_sampling : GBPT_ENVMAP_NO_SAMPLING;
        v.bsdf_mis = w->envmap_bsdf_mis ? 1 : 0;
        v.bilinear = w->envmap_bilinear ? 1 : 0;
        v.scale_background = w->envmap_scale_background ? 1 : 0;
    }
    if (!s->env_mem.ptrs.empty())
    {
        // renderers on other streams may still read the old tables
        const cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess)
        {
            fresh.release();
            return cuda_error(e, "world change");
        }
    }
    s->env_mem.release();
    s->env_mem = fresh;
    s->env_cdf = cdf;
    s->env_alias = alias;
    s->env_sum64 = sum64;
    s->view.env = v;
    return GBPT_OK;
}

gbpt_status gbpt_scene_get_envmap_tables(const gbpt_scene* s, uint32_t* texels, float* cdf, float* probas,
                                         int32_t* alias, float* total_sum, double* total_sum64)
{
    if (!s) return set_error(GBPT_ERROR_INVALID_ARG, "scene is NULL");
    const gbpt::EnvView& v = s->view.env;
    if (v.ambient != GBPT_AMBIENT_ENVMAP) return set_error(GBPT_ERROR_INVALID_ARG, "the scene's world has no envmap");
    const int64_t n = (int64_t)v.width * v.height;
    if (total_sum) *total_sum = v.total_sum;
    if (total_sum64) *total_sum64 = s->env_sum64;
    cudaError_t e = cudaSuccess;
    if (texels) e = cudaMemcpy(texels, v.texels, n * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && cdf) e = cudaMemcpy(cdf, v.cdf, n * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && (probas || alias))
    {
        std::vector<uint2> t(n);
        e = cudaMemcpy(t.data(), v.alias, n * sizeof(uint2), cudaMemcpyDeviceToHost);
        for (int64_t i = 0; e == cudaSuccess && i < n; i++)
        {
            if (probas) std::memcpy(probas + i, &t[i].x, sizeof(float));
            if (alias) alias[i] = (int32_t)t[i].y;
        }
    }
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "envmap table read-back");
}

namespace {

gbpt_status check_settings(const gbpt_scene* scene, const gbpt_render_settings* st)
{
    if (!scene || !st) return set_error(GBPT_ERROR_INVALID_ARG, "NULL argument");
    if (st->width <= 0 || st->height <= 0 || st->samples_per_launch <= 0)
        return set_error(GBPT_ERROR_INVALID_ARG, "width, height and samples_per_launch must be positive");
    if (st->nb_bounces < 0 || st->nb_bounces > 64) return set_error(GBPT_ERROR_INVALID_ARG, "nb_bounces must be in 0..64");
    if (st->light_sampling != GBPT_LIGHT_UNIFORM && st->light_sampling != GBPT_LIGHT_POWER)
        return set_error(GBPT_ERROR_INVALID_ARG, "unknown light_sampling");
    if (st->bsdf != GBPT_BSDF_LAMBERTIAN && st->bsdf != GBPT_BSDF_PRINCIPLED)
        return set_error(GBPT_ERROR_UNSUPPORTED, "bsdf must be GBPT_BSDF_LAMBERTIAN or GBPT_BSDF_PRINCIPLED");
    if (st->bsdf == GBPT_BSDF_PRINCIPLED && !scene->principled)
        return set_error(GBPT_ERROR_INVALID_ARG, "GBPT_BSDF_PRINCIPLED needs a scene created with principled_materials");
    if (st->direct_lighting != GBPT_DIRECT_MIS && st->direct_lighting != GBPT_DIRECT_RIS)
        return set_error(GBPT_ERROR_INVALID_ARG, "unknown direct_lighting");
    if (st->rng_mode != GBPT_RNG_PCG && st->rng_mode != GBPT_RNG_REFERENCE)
        return set_error(GBPT_ERROR_INVALID_ARG, "unknown rng_mode");
    if (st->direct_lighting == GBPT_DIRECT_RIS &&
        (st->ris_light_candidates < 0 || st->ris_light_candidates > 64 || st->ris_bsdf_candidates < 0 ||
         st->ris_bsdf_candidates > 1 || st->ris_light_candidates + st->ris_bsdf_candidates == 0))
        return set_error(GBPT_ERROR_INVALID_ARG, "RIS needs 0..64 light and 0..1 BSDF candidates, at least one");
    return GBPT_OK;
}

gbpt::RenderConst render_const(const gbpt_render_settings* st, int32_t spp)
{
    gbpt::RenderConst rc;
    std::memset(&rc, 0, sizeof(rc));
    rc.width = st->width;
    rc.height = st->height;
    rc.spp = spp;
    rc.nb_bounces = st->nb_bounces;
    rc.do_rr = st->do_russian_roulette;
    rc.rr_min_depth = st->russian_roulette_min_depth;
    rc.rr_clamp = st->russian_roulette_throughput_clamp;
    rc.light_sampling = st->light_sampling;
    rc.bsdf = st->bsdf;
    rc.seed = st->seed;
    rc.do_jittering = st->do_jittering;
    rc.ggx_height_correlated = st->ggx_height_correlated;
    rc.direct_ris = st->direct_lighting == GBPT_DIRECT_RIS ? 1 : 0;
    rc.ris_light = st->ris_light_candidates;
    rc.ris_bsdf = st->ris_bsdf_candidates;
    rc.rng_mode = st->rng_mode;
    std::memcpy(rc.inverse_view, st->inverse_view, sizeof(rc.inverse_view));
    std::memcpy(rc.inverse_projection, st->inverse_projection, sizeof(rc.inverse_projection));
    return rc;
}

// Path state and the four queues of a wavefront of 'cap' paths
void alloc_paths(DevMem& M, int64_t cap, bool principled, bool batched, gbpt::PathBuffers& pb, gbpt::Queue* q,
                 gbpt::Queue& shadow, gbpt::Queue& bsdfq)
{
    std::memset(&pb, 0, sizeof(pb));
    pb.throughput = M.alloc<float4>(cap);
    pb.radiance = M.alloc<float4>(cap);
    pb.rng = M.alloc<uint64_t>(cap);
    pb.pending_light = M.alloc<float4>(cap);
    pb.pending_bsdf = M.alloc<float4>(cap);
    pb.shadow_entry = M.alloc<int32_t>(cap);
    pb.bsdf_entry = M.alloc<int32_t>(cap);
    pb.vol_stack = principled ? M.alloc<uint4>(cap) : nullptr;
    pb.vol_state = principled ? M.alloc<int4>(cap) : nullptr;
    pb.wavelength = principled ? M.alloc<float>(cap) : nullptr;
    pb.job = batched ? M.alloc<int32_t>(cap) : nullptr;
    pb.ris = M.alloc<float4>(cap);
    q[0] = make_queue(M, cap, true, false);
    q[1] = make_queue(M, cap, true, false);
    shadow = make_queue(M, cap, false, true);
    bsdfq = make_queue(M, cap, true, false);
}

// Envmap direct lighting of a wavefront of 'cap' paths: per-path entries and contributions, and
// the any-hit queue of the envmap-sample and BSDF-sample rays (two per path)
void alloc_env(DevMem& M, int64_t cap, gbpt::PathBuffers& pb, gbpt::Queue& envq)
{
    pb.env_entry = M.alloc<int32_t>(cap);
    pb.envb_entry = M.alloc<int32_t>(cap);
    pb.pending_env = M.alloc<float4>(cap);
    pb.pending_envb = M.alloc<float4>(cap);
    envq = make_queue(M, 2 * cap, false, true);
}

// Allocates a renderer's envmap buffers the first time its scene's envmap is importance sampled
gbpt_status ensure_env(gbpt_renderer* r, cudaStream_t cs)
{
    if (r->env_ready || !scene_env_sampled(r->scene)) return GBPT_OK;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(cs, &cap) == cudaSuccess && cap != cudaStreamCaptureStatusNone)
        return set_error(GBPT_ERROR_INVALID_ARG,
                         "the scene's envmap is sampled but this renderer has not shaded since: run one launch outside the stream capture first");
    alloc_env(r->env_mem, r->capacity, r->pb, r->envq);
    if (r->env_mem.err != cudaSuccess)
    {
        const cudaError_t e = r->env_mem.err;
        r->env_mem.release();
        r->pb.env_entry = r->pb.envb_entry = nullptr;
        r->pb.pending_env = r->pb.pending_envb = nullptr;
        return cuda_error(e, "envmap buffers");
    }
    r->env_ready = true;
    return GBPT_OK;
}

}  // namespace

gbpt_status gbpt_renderer_create(const gbpt_scene* scene, const gbpt_render_settings* st, gbpt_renderer** out)
{
    if (!out) return set_error(GBPT_ERROR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    gbpt_status chk = check_settings(scene, st);
    if (chk != GBPT_OK) return chk;
    const int64_t cap = (int64_t)st->width * st->height * st->samples_per_launch;
    if (cap > (int64_t)1 << 30) return set_error(GBPT_ERROR_INVALID_ARG, "width*height*samples_per_launch exceeds 2^30 paths");

    gbpt_renderer* r = new (std::nothrow) gbpt_renderer();
    if (!r) return set_error(GBPT_ERROR_OOM, "host allocation failed");
    r->scene = scene;
    r->capacity = cap;
    r->n_sm = sm_count();
    r->rc = render_const(st, st->samples_per_launch);
    r->rng_seed = r->host_rng = st->random_number != 0u ? st->random_number : 42u;

    DevMem& M = r->mem;
    alloc_paths(M, cap, st->bsdf == GBPT_BSDF_PRINCIPLED, false, r->pb, r->q, r->shadow, r->bsdfq);
    if (st->rng_mode == GBPT_RNG_REFERENCE) r->pb.ris_u = M.alloc<float>(cap);
    const int64_t npix = (int64_t)st->width * st->height;
    r->acc32 = M.alloc<float>(3 * npix);
    r->acc64 = M.alloc<double>(3 * npix);
    r->stats = M.alloc<unsigned long long>(4);
    cudaError_t e = M.err;
    if (e == cudaSuccess) e = cudaMemset(r->acc32, 0, 3 * npix * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(r->acc64, 0, 3 * npix * sizeof(double));
    if (e == cudaSuccess) e = cudaMemset(r->stats, 0, 4 * sizeof(unsigned long long));
    if (e != cudaSuccess)
    {
        M.release();
        delete r;
        return cuda_error(e, "renderer allocation");
    }
    *out = r;
    return GBPT_OK;
}

gbpt_status gbpt_renderer_destroy(gbpt_renderer* r)
{
    if (!r) return GBPT_OK;
    r->restir_mem.release();
    r->guide_mem.release();
    r->env_mem.release();
    r->mem.release();
    delete r;
    return GBPT_OK;
}

gbpt_status gbpt_renderer_reset(gbpt_renderer* r, void* stream)
{
    if (!r) return set_error(GBPT_ERROR_INVALID_ARG, "renderer is NULL");
    cudaStream_t cs = (cudaStream_t)stream;
    const int64_t npix = (int64_t)r->rc.width * r->rc.height;
    cudaError_t e = cudaMemsetAsync(r->acc32, 0, 3 * npix * sizeof(float), cs);
    if (e == cudaSuccess) e = cudaMemsetAsync(r->acc64, 0, 3 * npix * sizeof(double), cs);
    if (e == cudaSuccess) e = cudaMemsetAsync(r->stats, 0, 4 * sizeof(unsigned long long), cs);
    r->iteration = 0;
    r->samples = 0;
    r->host_rng = r->rng_seed;
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "reset");
}

gbpt_status gbpt_renderer_set_sample_index(gbpt_renderer* r, int64_t first_sample)
{
    if (!r) return set_error(GBPT_ERROR_INVALID_ARG, "renderer is NULL");
    if (first_sample < 0 || first_sample > INT32_MAX) return set_error(GBPT_ERROR_INVALID_ARG, "sample index out of range");
    r->iteration = first_sample;
    return GBPT_OK;
}

gbpt_status gbpt_pass_camera_rays(gbpt_renderer* r, void* stream)
{
    if (!r) return set_error(GBPT_ERROR_INVALID_ARG, "renderer is NULL");
    r->cur = 0;
    // the reference's GPU renderer draws one random number per pass from its generator, in launch
    // order: the G-buffer pass (FillGBufferRenderPass.cpp:91), the ReSTIR DI passes (initial
    // candidates; temporal reuse and its permutation-sampling bits; each spatial pass;
    // ReSTIRDIRenderPass.cpp:449-578), then the MegaKernel pass (MegaKernelRenderPass.cpp:53)
    if (r->rc.rng_mode == GBPT_RNG_REFERENCE)
    {
        r->rc.random_number_camera = xorshift32_step(r->host_rng);
        if (r->restir)
        {
            const gbpt_restir_di_settings& k = r->restir_settings;
            r->rn_initial = xorshift32_step(r->host_rng);
            if (k.do_temporal)
            {
                r->rn_temporal = xorshift32_step(r->host_rng);
                xorshift32_step(r->host_rng);  // permutation-sampling bits (permutation sampling off)
            }
            for (int p = 0; k.do_spatial && p < k.spatial_passes; p++) r->rn_spatial[p] = xorshift32_step(r->host_rng);
        }
        r->rc.random_number = xorshift32_step(r->host_rng);
    }
    cudaError_t e = gbpt::launch_camera(r->rc, r->pb, r->q[0], (int32_t)r->iteration, r->stats, r->n_sm,
                                        (cudaStream_t)stream);
    if (e == cudaSuccess && r->gv.rec_count) e = cudaMemsetAsync(r->gv.rec_count, 0, sizeof(int32_t), (cudaStream_t)stream);
    r->gv.frame = (uint32_t)r->iteration;
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "camera rays");
}

gbpt_status gbpt_pass_extend(gbpt_renderer* r, int32_t bounce, void* stream)
{
    if (!r) return set_error(GBPT_ERROR_INVALID_ARG, "renderer is NULL");
    if (bounce < 0 || bounce > r->rc.nb_bounces) return set_error(GBPT_ERROR_INVALID_ARG, "bounce out of range");
    cudaError_t e = gbpt::launch_extend(r->scene->view, r->q[r->cur], r->q[r->cur ^ 1], r->shadow, r->bsdfq, r->capacity,
                                        r->n_sm, (cudaStream_t)stream);
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "extend");
}

gbpt_status gbpt_pass_shade(gbpt_renderer* r, int32_t bounce, void* stream)
{
    if (!r) return set_error(GBPT_ERROR_INVALID_ARG, "renderer is NULL");
    if (bounce < 0 || bounce > r->rc.nb_bounces) return set_error(GBPT_ERROR_INVALID_ARG, "bounce out of range");
    gbpt::ReservoirBuf none = {nullptr, nullptr};
    const gbpt::ReservoirBuf& restir = (r->restir && bounce == 0) ? r->res[r->res_final] : none;
    cudaStream_t cs = (cudaStream_t)stream;
    const gbpt::Queue& in = r->q[r->cur];
    gbpt::GuideView gv = r->gv;
    if (bounce >= r->rc.nb_bounces) gv.lobes = nullptr;  // no continuation at the last bounce
    if (gv.lobes)
    {
        // network inputs and mixture for every entry of the shaded queue (count read on the device)
        cudaError_t e = gbpt::launch_guide_inputs(r->scene->view, in, gv, r->capacity, r->n_sm, cs);
        if (e != cudaSuccess) return cuda_error(e, "guide inputs");
        gbpt::guide::Batch b;
        std::memset(&b, 0, sizeof(b));
        b.pos = gv.in_pos;
        b.nrm = gv.in_nrm;
        b.view = gv.in_view;
        b.count = in.count;
        b.n_max = r->capacity;
        gbpt_status st = gbpt::guide::render_infer(r->guide, b, r->guide_lobes, cs);
        if (st != GBPT_OK) return st;
    }
    gbpt_status env_st = ensure_env(r, cs);
    if (env_st != GBPT_OK) return env_st;
    gbpt::PathBuffers pb = r->pb;
    if (!scene_env_sampled(r->scene)) pb.env_entry = nullptr;  // envmap direct lighting off
    pb.guide_pdf = r->guide_pdf;  // null without a guide
    cudaError_t e = gbpt::launch_shade(r->scene->view, r->rc, pb, in, r->q[r->cur ^ 1], r->shadow, r->bsdfq, r->envq,
                                       bounce, r->capacity, r->stats, restir, gv, r->n_sm, cs);
    r->cur ^= 1;
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "shade");
}

gbpt_status gbpt_pass_bounce(gbpt_renderer* r, int32_t bounce, void* stream)
{
    gbpt_status st = gbpt_pass_extend(r, bounce, stream);
    return st == GBPT_OK ? gbpt_pass_shade(r, bounce, stream) : st;
}

namespace {

uint32_t spatial_seed(uint32_t frame, int pass, uint32_t seed);

gbpt::RestirConst restir_const(const gbpt_renderer* r)
{
    const gbpt_restir_di_settings& k = r->restir_settings;
    gbpt::RestirConst c;
    std::memset(&c, 0, sizeof(c));
    c.light_candidates = k.light_candidates;
    c.bsdf_candidates = k.bsdf_candidates;
    c.visibility_reuse = k.do_visibility_reuse;
    c.do_temporal = k.do_temporal;
    c.temporal_search_count = k.temporal_search_count;
    c.temporal_search_radius = k.temporal_search_radius;
    c.do_spatial = k.do_spatial;
    c.spatial_passes = k.spatial_passes;
    c.spatial_neighbors = k.spatial_neighbors;
    c.spatial_radius = k.spatial_radius;
    c.m_cap = k.m_cap;
    c.confidence_weights = k.use_confidence_weights;
    c.bias_correction_visibility = k.bias_correction_visibility;
    c.final_visibility = k.do_final_shading_visibility;
    c.normal_similarity_cos = k.normal_similarity_cos;
    c.plane_distance = k.plane_distance_threshold;
    c.frame = (uint32_t)r->iteration;
    c.seed = r->rc.seed;
    c.has_prev = r->has_prev ? 1 : 0;
    c.rng_mode = r->rc.rng_mode;
    c.sample_number = (uint32_t)r->iteration;
    c.rn_initial = r->rn_initial;
    c.rn_temporal = r->rn_temporal;
    for (int p = 0; p < 4; p++) c.rn_spatial[p] = r->rn_spatial[p];
    camera_position(r->rc.inverse_view, c.camera_pos);
    camera_position(r->prev_inverse_view, c.prev_camera_pos);
    if (r->presampled)
    {
        c.presampled = r->presampled;
        c.presample_subsets = k.presampling_subsets;
        c.presample_size = k.presampling_subset_size;
        c.presample_tile = k.presampling_tile_size;
        // the frame's subset seed: the spatial-seed hash at a pass index no spatial pass uses
        c.presample_seed = spatial_seed(c.frame, 31, c.seed);
    }
    return c;
}

// Spatial-neighbour seed of a frame and pass, shared by every pixel (coalesced spatial reuse)
uint32_t spatial_seed(uint32_t frame, int pass, uint32_t seed)
{
    uint64_t z = ((uint64_t)frame << 32) ^ ((uint64_t)(uint32_t)pass << 16) ^ (uint64_t)seed ^ 0x5851F42D4C957F2DULL;
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    const uint32_t s = (uint32_t)((z ^ (z >> 31)) >> 16);
    return s != 0u ? s : 0x9E3779B9u;
}

gbpt_status restir_ready(gbpt_renderer* r)
{
    if (!r) return set_error(GBPT_ERROR_INVALID_ARG, "renderer is NULL");
    if (!r->restir) return set_error(GBPT_ERROR_INVALID_ARG, "ReSTIR DI is not enabled on this renderer");
    return GBPT_OK;
}

}  // namespace

gbpt_status gbpt_restir_di_default_settings(gbpt_restir_di_settings* s)
{
    if (!s) return set_error(GBPT_ERROR_INVALID_ARG, "settings is NULL");
    std::memset(s, 0, sizeof(*s));
    s->enabled = 1;
    s->light_candidates = 4;
    s->bsdf_candidates = 1;
    s->do_visibility_reuse = 1;
    s->do_temporal = 1;
    s->temporal_search_count = 8;
    s->temporal_search_radius = 4.0f;
    s->do_spatial = 1;
    s->spatial_passes = 1;
    s->spatial_neighbors = 5;
    s->spatial_radius = 16.0f;
    s->m_cap = 3;
    s->use_confidence_weights = 1;
    s->bias_correction_visibility = 1;
    s->do_final_shading_visibility = 1;
    s->normal_similarity_cos = 0.906307787f;
    s->plane_distance_threshold = 0.1f;
    s->do_fused_spatiotemporal = 0;
    s->do_light_presampling = 0;
    s->presampling_subsets = 128;
    s->presampling_subset_size = 1024;
    s->presampling_tile_size = 8;
    return GBPT_OK;
}

gbpt_status gbpt_renderer_set_restir_di(gbpt_renderer* r, const gbpt_restir_di_settings* k)
{
    if (!r || !k) return set_error(GBPT_ERROR_INVALID_ARG, "NULL argument");
    r->restir_mem.release();
    r->restir = false;
    r->has_prev = false;
    r->presampled = nullptr;
    r->rc.restir_final_visibility = 0;
    if (!k->enabled) return GBPT_OK;
    if (r->rc.bsdf != GBPT_BSDF_PRINCIPLED) return set_error(GBPT_ERROR_INVALID_ARG, "ReSTIR DI needs GBPT_BSDF_PRINCIPLED");
    if (r->rc.spp != 1) return set_error(GBPT_ERROR_INVALID_ARG, "ReSTIR DI needs samples_per_launch = 1");
    if (k->light_candidates < 0 || k->bsdf_candidates < 0 || k->light_candidates + k->bsdf_candidates == 0 ||
        k->light_candidates > 4096 || k->bsdf_candidates > 64)
        return set_error(GBPT_ERROR_INVALID_ARG, "candidate counts out of range");
    if (k->do_spatial && (k->spatial_neighbors < 1 || k->spatial_neighbors > 32 || k->spatial_passes < 1 ||
                          k->spatial_passes > 16 || !(k->spatial_radius > 0.0f)))
        return set_error(GBPT_ERROR_INVALID_ARG, "spatial settings out of range (1..32 neighbours, 1..16 passes)");
    if ((k->do_temporal || k->do_fused_spatiotemporal) && (k->temporal_search_count < 0 || k->temporal_search_count > 64))
        return set_error(GBPT_ERROR_INVALID_ARG, "temporal_search_count out of range");
    if (k->do_fused_spatiotemporal && (k->spatial_neighbors < 1 || k->spatial_neighbors > 32 || k->spatial_passes < 1 ||
                                       k->spatial_passes > 16 || !(k->spatial_radius > 0.0f)))
        return set_error(GBPT_ERROR_INVALID_ARG, "spatial settings out of range (1..32 neighbours, 1..16 passes)");
    if (k->do_light_presampling &&
        (k->presampling_subsets < 1 || k->presampling_subset_size < 1 || k->presampling_tile_size < 1 ||
         (int64_t)k->presampling_subsets * k->presampling_subset_size > ((int64_t)1 << 24)))
        return set_error(GBPT_ERROR_INVALID_ARG, "light presampling sizes out of range (at most 2^24 records)");
    if (r->rc.rng_mode == GBPT_RNG_REFERENCE &&
        (k->do_fused_spatiotemporal || k->do_light_presampling || (k->do_spatial && k->spatial_passes > 4)))
        return set_error(GBPT_ERROR_INVALID_ARG,
                         "GBPT_RNG_REFERENCE covers the separate temporal and spatial passes (at most 4), "
                         "without light presampling");
    const int64_t npix = (int64_t)r->rc.width * r->rc.height;
    DevMem& M = r->restir_mem;
    for (int g = 0; g < 2; g++)
    {
        r->gb[g].pos = M.alloc<float4>(npix);
        r->gb[g].ns = M.alloc<float4>(npix);
        r->gb[g].ng = M.alloc<float4>(npix);
    }
    for (int b = 0; b < 5; b++)
    {
        r->res[b].s = M.alloc<float4>(npix);
        r->res[b].w = M.alloc<int4>(npix);
    }
    r->presampled = k->do_light_presampling
                        ? M.alloc<float4>(2 * (size_t)k->presampling_subsets * k->presampling_subset_size)
                        : nullptr;
    r->initial_state.cand = M.alloc<float4>(npix);
    r->initial_state.meta = M.alloc<int4>(npix);
    r->spatial_ray_of = nullptr;
    std::memset(&r->spatial_rays, 0, sizeof(r->spatial_rays));
    r->temporal_ray_of = nullptr;
    std::memset(&r->temporal_rays, 0, sizeof(r->temporal_rays));
    if (k->do_temporal)
    {
        r->temporal_ray_of = M.alloc<int2>(npix);
        r->temporal_rays = make_queue(M, 2 * npix, false, true);
    }
    if (k->do_spatial || k->do_fused_spatiotemporal)
    {
        const int64_t n_rays = npix * (int64_t)(k->spatial_neighbors + 2);  // fused: + 2 temporal rays
        r->spatial_ray_of = M.alloc<int32_t>(n_rays);
        r->spatial_rays = make_queue(M, n_rays, false, true);
    }
    cudaError_t e = M.err;
    for (int b = 0; b < 5 && e == cudaSuccess; b++)
    {
        e = cudaMemset(r->res[b].s, 0, npix * sizeof(float4));
        if (e == cudaSuccess) e = cudaMemset(r->res[b].w, 0, npix * sizeof(int4));
    }
    if (e != cudaSuccess)
    {
        M.release();
        r->presampled = nullptr;
        return cuda_error(e, "ReSTIR DI buffers");
    }
    r->restir_settings = *k;
    r->restir = true;
    r->gb_cur = 0;
    r->res_final = 0;
    r->rc.restir_final_visibility = k->do_final_shading_visibility;
    std::memcpy(r->prev_inverse_view, r->rc.inverse_view, sizeof(r->prev_inverse_view));
    return GBPT_OK;
}

gbpt_status gbpt_renderer_set_camera(gbpt_renderer* r, const float* inverse_view, const float* inverse_projection)
{
    if (!r || !inverse_view || !inverse_projection) return set_error(GBPT_ERROR_INVALID_ARG, "NULL argument");
    std::memcpy(r->rc.inverse_view, inverse_view, sizeof(r->rc.inverse_view));
    std::memcpy(r->rc.inverse_projection, inverse_projection, sizeof(r->rc.inverse_projection));
    return GBPT_OK;
}

gbpt_status gbpt_pass_restir_di_initial(gbpt_renderer* r, void* stream)
{
    gbpt_status st = restir_ready(r);
    if (st != GBPT_OK) return st;
    cudaStream_t cs = (cudaStream_t)stream;
    const int64_t npix = (int64_t)r->rc.width * r->rc.height;
    const gbpt::GBuffer& gb = r->gb[r->gb_cur];
    const gbpt::RestirConst k = restir_const(r);
    cudaError_t e = gbpt::launch_restir_gbuffer(r->scene->view, r->q[r->cur], gb, npix,
                                                r->rc.rng_mode == GBPT_RNG_REFERENCE ? 1 : 0, r->n_sm, cs);
    if (e == cudaSuccess && r->presampled)
        e = gbpt::launch_restir_presample(r->scene->view, r->rc, k, r->presampled, r->n_sm, cs);
    // its BSDF-candidate and visibility rays go through the bounce's free queues (left empty after)
    if (e == cudaSuccess)
        e = gbpt::launch_restir_initial(r->scene->view, r->rc, k, gb, r->res[0], r->initial_state, r->bsdfq,
                                        r->q[r->cur ^ 1], r->shadow, r->capacity, r->n_sm, cs);
    r->res_final = 0;
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "ReSTIR DI initial candidates");
}

gbpt_status gbpt_pass_restir_di_temporal(gbpt_renderer* r, void* stream)
{
    gbpt_status st = restir_ready(r);
    if (st != GBPT_OK) return st;
    gbpt::RestirConst k = restir_const(r);
    if (!view_projection(r->prev_inverse_view, r->rc.inverse_projection, k.prev_view_projection))
        return set_error(GBPT_ERROR_INVALID_ARG, "the previous camera matrices are singular");
    if (!r->temporal_ray_of) return set_error(GBPT_ERROR_INVALID_ARG, "temporal reuse is not enabled on this renderer");
    cudaError_t e = gbpt::launch_restir_temporal(r->scene->view, r->rc, k, r->gb[r->gb_cur], r->gb[r->gb_cur ^ 1],
                                                 r->res[0], r->res[4], r->res[1], r->temporal_ray_of, r->temporal_rays,
                                                 r->n_sm, (cudaStream_t)stream);
    r->res_final = 1;
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "ReSTIR DI temporal reuse");
}

gbpt_status gbpt_pass_restir_di_spatiotemporal(gbpt_renderer* r, void* stream)
{
    gbpt_status st = restir_ready(r);
    if (st != GBPT_OK) return st;
    gbpt::RestirConst k = restir_const(r);
    if (!view_projection(r->prev_inverse_view, r->rc.inverse_projection, k.prev_view_projection))
        return set_error(GBPT_ERROR_INVALID_ARG, "the previous camera matrices are singular");
    if (!r->spatial_ray_of) return set_error(GBPT_ERROR_INVALID_ARG, "spatial reuse is not enabled on this renderer");
    cudaError_t e = gbpt::launch_restir_spatiotemporal(r->scene->view, r->rc, k, r->gb[r->gb_cur], r->gb[r->gb_cur ^ 1],
                                                       r->res[0], r->res[4], r->res[2], r->spatial_ray_of,
                                                       r->spatial_rays, r->initial_state, r->shadow, r->n_sm,
                                                       (cudaStream_t)stream);
    r->res_final = 2;
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "ReSTIR DI spatiotemporal reuse");
}

gbpt_status gbpt_pass_restir_di_spatial(gbpt_renderer* r, int32_t pass_index, void* stream)
{
    gbpt_status st = restir_ready(r);
    if (st != GBPT_OK) return st;
    if (pass_index < 0 || pass_index >= r->restir_settings.spatial_passes)
        return set_error(GBPT_ERROR_INVALID_ARG, "pass_index out of range");
    const int in = r->res_final;
    const int out = in == 2 ? 3 : 2;
    if (!r->spatial_ray_of) return set_error(GBPT_ERROR_INVALID_ARG, "spatial reuse is not enabled on this renderer");
    // its final visibility rays go through the bounce's shadow queue (left empty after)
    cudaError_t e = gbpt::launch_restir_spatial(r->scene->view, r->rc, restir_const(r), r->gb[r->gb_cur], r->res[in],
                                                r->res[out], pass_index,
                                                spatial_seed((uint32_t)r->iteration, pass_index, r->rc.seed),
                                                r->spatial_ray_of, r->spatial_rays, r->initial_state, r->shadow,
                                                r->n_sm, (cudaStream_t)stream);
    r->res_final = out;
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "ReSTIR DI spatial reuse");
}

namespace {

// end of a ReSTIR frame: the final reservoirs become the previous frame's, the G-buffers swap
cudaError_t restir_end_frame(gbpt_renderer* r, cudaStream_t cs)
{
    const int64_t npix = (int64_t)r->rc.width * r->rc.height;
    const gbpt::ReservoirBuf& f = r->res[r->res_final];
    cudaError_t e = cudaMemcpyAsync(r->res[4].s, f.s, npix * sizeof(float4), cudaMemcpyDeviceToDevice, cs);
    if (e == cudaSuccess) e = cudaMemcpyAsync(r->res[4].w, f.w, npix * sizeof(int4), cudaMemcpyDeviceToDevice, cs);
    r->gb_cur ^= 1;
    r->has_prev = true;
    std::memcpy(r->prev_inverse_view, r->rc.inverse_view, sizeof(r->prev_inverse_view));
    return e;
}

}  // namespace

gbpt_status gbpt_pass_accumulate(gbpt_renderer* r, void* stream)
{
    if (!r) return set_error(GBPT_ERROR_INVALID_ARG, "renderer is NULL");
    cudaError_t e = gbpt::launch_accumulate(r->rc, r->pb, r->acc32, r->acc64, r->n_sm, (cudaStream_t)stream);
    if (e == cudaSuccess && r->restir) e = restir_end_frame(r, (cudaStream_t)stream);
    if (e == cudaSuccess && r->gv.train_entry)
    {
        // one training step on this launch's guiding records
        e = gbpt::launch_guide_weights(r->pb, r->gv, r->n_sm, (cudaStream_t)stream);
        if (e == cudaSuccess)
        {
            gbpt::guide::Batch b;
            b.pos = r->gv.rec_pos;
            b.nrm = r->gv.rec_nrm;
            b.view = r->gv.rec_view;
            b.dir = r->gv.rec_dir;
            b.weight = r->gv.rec_weight;
            b.bsdf_pdf = r->gv.rec_pbsdf;
            b.count = r->gv.rec_count;
            b.n_max = r->gv.rec_cap;
            gbpt_status st = gbpt::guide::render_train(r->guide, b, (cudaStream_t)stream);
            if (st != GBPT_OK) return st;
        }
    }
    r->iteration += r->rc.spp;
    r->samples += r->rc.spp;
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "accumulate");
}

gbpt_status gbpt_render(gbpt_renderer* r, int32_t n_launches, void* stream)
{
    if (!r) return set_error(GBPT_ERROR_INVALID_ARG, "renderer is NULL");
    if (n_launches < 0) return set_error(GBPT_ERROR_INVALID_ARG, "n_launches is negative");
    for (int32_t k = 0; k < n_launches; k++)
    {
        gbpt_status st = gbpt_pass_camera_rays(r, stream);
        if (st == GBPT_OK && r->restir)
        {
            st = gbpt_pass_extend(r, 0, stream);
            if (st == GBPT_OK) st = gbpt_pass_restir_di_initial(r, stream);
            if (r->restir_settings.do_fused_spatiotemporal)
            {
                if (st == GBPT_OK) st = gbpt_pass_restir_di_spatiotemporal(r, stream);
                for (int p = 1; st == GBPT_OK && p < r->restir_settings.spatial_passes; p++)
                    st = gbpt_pass_restir_di_spatial(r, p, stream);
            }
            else
            {
                if (st == GBPT_OK && r->restir_settings.do_temporal) st = gbpt_pass_restir_di_temporal(r, stream);
                for (int p = 0; st == GBPT_OK && r->restir_settings.do_spatial && p < r->restir_settings.spatial_passes; p++)
                    st = gbpt_pass_restir_di_spatial(r, p, stream);
            }
            if (st == GBPT_OK) st = gbpt_pass_shade(r, 0, stream);
        }
        for (int b = r->restir ? 1 : 0; st == GBPT_OK && b <= r->rc.nb_bounces; b++) st = gbpt_pass_bounce(r, b, stream);
        if (st == GBPT_OK) st = gbpt_pass_accumulate(r, stream);
        if (st != GBPT_OK) return st;
    }
    return GBPT_OK;
}

gbpt_status gbpt_renderer_get_image(gbpt_renderer* r, float* rgb32, double* rgb64, void* stream)
{
    if (!r) return set_error(GBPT_ERROR_INVALID_ARG, "renderer is NULL");
    cudaStream_t cs = (cudaStream_t)stream;
    const int64_t npix = (int64_t)r->rc.width * r->rc.height;
    cudaError_t e = cudaSuccess;
    if (rgb32) e = cudaMemcpyAsync(rgb32, r->acc32, 3 * npix * sizeof(float), cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess && rgb64) e = cudaMemcpyAsync(rgb64, r->acc64, 3 * npix * sizeof(double), cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "image read-back");
}

namespace {

gbpt_status reservoir_buffer(gbpt_renderer* r, int32_t which, gbpt::ReservoirBuf& out)
{
    gbpt_status st = restir_ready(r);
    if (st != GBPT_OK) return st;
    switch (which)
    {
    case GBPT_RESERVOIRS_INITIAL: out = r->res[0]; break;
    case GBPT_RESERVOIRS_TEMPORAL: out = r->res[1]; break;
    case GBPT_RESERVOIRS_FINAL: out = r->res[r->res_final]; break;
    case GBPT_RESERVOIRS_PREVIOUS: out = r->res[4]; break;
    default: return set_error(GBPT_ERROR_INVALID_ARG, "unknown reservoir buffer");
    }
    return GBPT_OK;
}

}  // namespace

gbpt_status gbpt_restir_di_get_reservoirs(gbpt_renderer* r, int32_t which, float* host_out, void* stream)
{
    gbpt::ReservoirBuf b;
    gbpt_status st = reservoir_buffer(r, which, b);
    if (st != GBPT_OK) return st;
    if (!host_out) return set_error(GBPT_ERROR_INVALID_ARG, "host_out is NULL");
    const int64_t npix = (int64_t)r->rc.width * r->rc.height;
    std::vector<float4> s(npix);
    std::vector<int4> w(npix);
    cudaStream_t cs = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(s.data(), b.s, npix * sizeof(float4), cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess) e = cudaMemcpyAsync(w.data(), b.w, npix * sizeof(int4), cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
    if (e != cudaSuccess) return cuda_error(e, "reservoir read-back");
    for (int64_t i = 0; i < npix; i++)
    {
        std::memcpy(host_out + 8 * i, &s[i], 16);
        std::memcpy(host_out + 8 * i + 4, &w[i], 16);
    }
    return GBPT_OK;
}

gbpt_status gbpt_restir_di_set_reservoirs(gbpt_renderer* r, int32_t which, const float* host_in, void* stream)
{
    gbpt::ReservoirBuf b;
    gbpt_status st = reservoir_buffer(r, which, b);
    if (st != GBPT_OK) return st;
    if (!host_in) return set_error(GBPT_ERROR_INVALID_ARG, "host_in is NULL");
    const int64_t npix = (int64_t)r->rc.width * r->rc.height;
    std::vector<float4> s(npix);
    std::vector<int4> w(npix);
    for (int64_t i = 0; i < npix; i++)
    {
        std::memcpy(&s[i], host_in + 8 * i, 16);
        std::memcpy(&w[i], host_in + 8 * i + 4, 16);
    }
    cudaStream_t cs = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(b.s, s.data(), npix * sizeof(float4), cudaMemcpyHostToDevice, cs);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b.w, w.data(), npix * sizeof(int4), cudaMemcpyHostToDevice, cs);
    if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "reservoir upload");
}

gbpt_status gbpt_renderer_get_stats(gbpt_renderer* r, gbpt_render_stats* out, void* stream)
{
    if (!r || !out) return set_error(GBPT_ERROR_INVALID_ARG, "NULL argument");
    unsigned long long h[4];
    cudaStream_t cs = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(h, r->stats, sizeof(h), cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
    if (e != cudaSuccess) return cuda_error(e, "stats read-back");
    out->samples = r->samples * (int64_t)r->rc.width * r->rc.height;
    out->extension_rays = (int64_t)h[0];
    out->shadow_rays = (int64_t)h[1];
    out->bsdf_light_rays = (int64_t)h[2];
    return GBPT_OK;
}

gbpt_status gbpt_guide_render_default_settings(gbpt_guide_render_settings* s)
{
    if (!s) return set_error(GBPT_ERROR_INVALID_ARG, "settings is NULL");
    std::memset(s, 0, sizeof(*s));
    s->enabled = 1;
    s->train = 1;
    s->guide_probability = 0.0f;
    s->max_records = 1 << 18;
    s->weight_clamp = 50.0f;
    return GBPT_OK;
}

gbpt_status gbpt_renderer_set_guide(gbpt_renderer* r, gbpt_guide* g, const gbpt_guide_render_settings* s)
{
    if (!r) return set_error(GBPT_ERROR_INVALID_ARG, "renderer is NULL");
    r->guide_mem.release();
    std::memset(&r->gv, 0, sizeof(r->gv));
    r->guide = nullptr;
    r->guide_lobes = nullptr;
    r->guide_pdf = nullptr;
    if (!g || !s || !s->enabled) return GBPT_OK;
    if (!(s->guide_probability >= 0.0f && s->guide_probability < 1.0f))
        return set_error(GBPT_ERROR_INVALID_ARG, "guide_probability must be in [0, 1)");
    if (s->train && (s->max_records < 1 || s->max_records > gbpt::guide::max_batch(g)))
        return set_error(GBPT_ERROR_INVALID_ARG, "max_records must be in 1..the guide's max_batch");
    if (s->weight_clamp < 0.0f) return set_error(GBPT_ERROR_INVALID_ARG, "weight_clamp is negative");
    const int64_t cap = r->capacity;
    DevMem& M = r->guide_mem;
    gbpt::GuideView& gv = r->gv;
    gv.in_pos = M.alloc<float>(3 * cap);
    gv.in_nrm = M.alloc<float>(3 * cap);
    gv.in_view = M.alloc<float>(3 * cap);
    r->guide_lobes = M.alloc<float>((int64_t)GBPT_GUIDE_ROW * cap);
    r->guide_pdf = M.alloc<float>(cap);
    gv.prob = s->guide_probability;
    if (s->train)
    {
        const int64_t nr = s->max_records;
        gv.train_entry = M.alloc<int32_t>(cap);
        gv.train_light_entry = M.alloc<int32_t>(cap);
        gv.rec_candidates = M.alloc<int32_t>(1);
        gv.rec_threshold = M.alloc<uint32_t>(1);
        gv.rec_pos = M.alloc<float>(3 * nr);
        gv.rec_nrm = M.alloc<float>(3 * nr);
        gv.rec_view = M.alloc<float>(3 * nr);
        gv.rec_dir = M.alloc<float>(3 * nr);
        gv.rec_tp = M.alloc<float4>(nr);
        gv.rec_snap = M.alloc<float4>(nr);
        gv.rec_weight = M.alloc<float>(nr);
        gv.rec_pbsdf = M.alloc<float>(nr);
        gv.rec_slot = M.alloc<int32_t>(nr);
        gv.rec_count = M.alloc<int32_t>(1);
        gv.rec_cap = s->max_records;
        gv.weight_clamp = s->weight_clamp;
    }
    cudaError_t e = M.err;
    if (e == cudaSuccess && gv.rec_count)
    {
        // first launch: assume every path sample reaches every bounce (two records per vertex);
        // later launches adapt to the counted candidates
        const double expected = 2.0 * (double)cap * (r->rc.nb_bounces > 0 ? r->rc.nb_bounces : 1);
        const double frac = std::min(1.0, (double)s->max_records / expected);
        const uint32_t thr = frac >= 1.0 ? 0xFFFFFFFFu : (uint32_t)(frac * 4294967296.0);
        e = cudaMemset(gv.rec_count, 0, sizeof(int32_t));
        if (e == cudaSuccess) e = cudaMemset(gv.rec_candidates, 0, sizeof(int32_t));
        if (e == cudaSuccess) e = cudaMemcpy(gv.rec_threshold, &thr, sizeof(uint32_t), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess)
    {
        M.release();
        std::memset(&r->gv, 0, sizeof(r->gv));
        r->guide_lobes = nullptr;
        r->guide_pdf = nullptr;
        return e == cudaErrorMemoryAllocation ? set_error(GBPT_ERROR_OOM, "guiding buffers") : cuda_error(e, "guiding buffers");
    }
    gv.lobes = r->guide_lobes;
    r->guide = g;
    r->guide_settings = *s;
    return GBPT_OK;
}

gbpt_status gbpt_renderer_get_guide_records(gbpt_renderer* r, float* host_out, int32_t capacity, int32_t* count,
                                            void* stream)
{
    if (!r || !count) return set_error(GBPT_ERROR_INVALID_ARG, "NULL argument");
    if (!r->gv.rec_count) return set_error(GBPT_ERROR_INVALID_ARG, "no guide with training attached");
    cudaStream_t cs = (cudaStream_t)stream;
    int32_t n = 0;
    cudaError_t e = cudaMemcpyAsync(&n, r->gv.rec_count, sizeof(int32_t), cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
    if (e != cudaSuccess) return cuda_error(e, "record count read-back");
    *count = n;
    const int64_t k = std::min<int64_t>(std::min<int64_t>(n, r->gv.rec_cap), capacity > 0 ? capacity : 0);
    if (!host_out || k == 0) return GBPT_OK;
    std::vector<float> p(3 * k), nr(3 * k), v(3 * k), d(3 * k), w(k), pb(k);
    std::vector<int32_t> sl(k);
    e = cudaMemcpy(p.data(), r->gv.rec_pos, 3 * k * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(nr.data(), r->gv.rec_nrm, 3 * k * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(v.data(), r->gv.rec_view, 3 * k * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(d.data(), r->gv.rec_dir, 3 * k * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(w.data(), r->gv.rec_weight, k * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(pb.data(), r->gv.rec_pbsdf, k * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(sl.data(), r->gv.rec_slot, k * sizeof(int32_t), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_error(e, "record read-back");
    for (int64_t i = 0; i < k; i++)
    {
        float* o = host_out + 15 * i;
        for (int a = 0; a < 3; a++)
        {
            o[a] = p[3 * i + a];
            o[3 + a] = nr[3 * i + a];
            o[6 + a] = v[3 * i + a];
            o[9 + a] = d[3 * i + a];
        }
        o[12] = w[i];
        o[13] = pb[i];
        std::memcpy(o + 14, &sl[i], sizeof(int32_t));
    }
    return GBPT_OK;
}

struct gbpt_batch
{
    std::vector<gbpt::BatchJob> host_jobs;
    std::vector<const gbpt_scene*> scenes;
    gbpt_batch_params params;
    DevMem mem;
    gbpt::BatchJob* jobs = nullptr;
    gbpt::PathBuffers pb;
    gbpt::Queue q[2], shadow, bsdfq, envq;
    int64_t capacity = 0, max_job_paths = 0, max_job_pixels = 0, total_pixels = 0;
    int max_bounces = 0, max_iterations = 0, n_sm = 1;
    float* acc32 = nullptr;
    double* acc64 = nullptr;
    int32_t* iteration = nullptr;
    unsigned long long* stamps = nullptr;  // [0] render start, [1 + j] job j done (global timer, ns)
    unsigned long long* stats = nullptr;
    cudaStream_t capture_stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {

// One iteration of the batch: camera rays, the bounce loop over all jobs, accumulation + step
cudaError_t batch_iteration(gbpt_batch* b, cudaStream_t st)
{
    const gbpt::BatchJob& j0 = b->host_jobs[0];
    cudaError_t e = gbpt::launch_batch_camera(b->jobs, (int)b->host_jobs.size(), b->max_job_paths, b->pb, b->q[0],
                                              b->iteration, b->stats, b->n_sm, st);
    gbpt::ReservoirBuf none = {nullptr, nullptr};
    gbpt::GuideView no_guide;
    std::memset(&no_guide, 0, sizeof(no_guide));
    for (int bounce = 0; e == cudaSuccess && bounce <= b->max_bounces; bounce++)
    {
        const gbpt::Queue& in = b->q[bounce & 1];
        const gbpt::Queue& next = b->q[(bounce & 1) ^ 1];
        e = gbpt::launch_extend(j0.s, in, next, b->shadow, b->bsdfq, b->capacity, b->n_sm, st, b->jobs, b->pb.job);
        if (e == cudaSuccess)
            e = gbpt::launch_shade(j0.s, j0.rc, b->pb, in, next, b->shadow, b->bsdfq, b->envq, bounce, b->capacity,
                                   b->stats + 1, none, no_guide, b->n_sm, st, b->jobs);
    }
    if (e == cudaSuccess)
        e = gbpt::launch_batch_accumulate(b->jobs, (int)b->host_jobs.size(), b->max_job_pixels, b->pb, b->iteration,
                                          b->acc32, b->acc64, b->iteration, b->stamps + 1, b->n_sm, st);
    return e;
}

void batch_release(gbpt_batch* b)
{
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->capture_stream) cudaStreamDestroy(b->capture_stream);
    b->mem.release();
}

}  // namespace

gbpt_status gbpt_batch_default_params(gbpt_batch_params* p)
{
    if (!p) return set_error(GBPT_ERROR_INVALID_ARG, "params is NULL");
    std::memset(p, 0, sizeof(*p));
    p->samples_per_iteration = 4;
    p->use_graph = 1;
    return GBPT_OK;
}

gbpt_status gbpt_batch_create(const gbpt_batch_job* jobs, int32_t n_jobs, const gbpt_batch_params* p, gbpt_batch** out)
{
    if (!out) return set_error(GBPT_ERROR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    if (!jobs || !p || n_jobs < 1) return set_error(GBPT_ERROR_INVALID_ARG, "need at least one job and params");
    if (p->samples_per_iteration < 1 || p->samples_per_iteration > 1024)
        return set_error(GBPT_ERROR_INVALID_ARG, "samples_per_iteration must be in 1..1024");
    gbpt_batch* b = new (std::nothrow) gbpt_batch();
    if (!b) return set_error(GBPT_ERROR_OOM, "host allocation failed");
    b->params = *p;
    b->n_sm = sm_count();
    const int k = p->samples_per_iteration;
    for (int j = 0; j < n_jobs; j++)
    {
        const gbpt_render_settings* st = &jobs[j].settings;
        gbpt_status chk = check_settings(jobs[j].scene, st);
        if (chk == GBPT_OK && st->bsdf != jobs[0].settings.bsdf)
            chk = set_error(GBPT_ERROR_INVALID_ARG, "all jobs of a batch must use the same bsdf mode");
        if (chk == GBPT_OK && st->rng_mode != GBPT_RNG_PCG)
            chk = set_error(GBPT_ERROR_INVALID_ARG, "batched jobs draw PCG streams (rng_mode must be GBPT_RNG_PCG)");
        if (chk != GBPT_OK)
        {
            delete b;
            return chk;
        }
        gbpt::BatchJob J;
        std::memset(&J, 0, sizeof(J));
        J.s = jobs[j].scene->view;
        J.rc = render_const(st, k);
        J.slot_base = b->capacity;
        J.pixel_base = b->total_pixels;
        J.spp_total = st->samples_per_launch;
        J.iterations = (st->samples_per_launch + k - 1) / k;
        const int64_t npix = (int64_t)st->width * st->height;
        b->capacity += npix * k;
        b->total_pixels += npix;
        b->max_job_paths = std::max(b->max_job_paths, npix * k);
        b->max_job_pixels = std::max(b->max_job_pixels, npix);
        b->max_bounces = std::max(b->max_bounces, st->nb_bounces);
        b->max_iterations = std::max(b->max_iterations, J.iterations);
        b->host_jobs.push_back(J);
        b->scenes.push_back(jobs[j].scene);
    }
    if (b->capacity > (int64_t)1 << 30)
    {
        delete b;
        return set_error(GBPT_ERROR_INVALID_ARG, "the jobs' paths per iteration exceed 2^30");
    }
    DevMem& M = b->mem;
    alloc_paths(M, b->capacity, jobs[0].settings.bsdf == GBPT_BSDF_PRINCIPLED, true, b->pb, b->q, b->shadow, b->bsdfq);
    bool any_env = false;
    for (const gbpt_scene* sc : b->scenes) any_env = any_env || scene_env_sampled(sc);
    if (any_env) alloc_env(M, b->capacity, b->pb, b->envq);
    b->jobs = M.alloc<gbpt::BatchJob>(n_jobs);
    b->acc32 = M.alloc<float>(3 * b->total_pixels);
    b->acc64 = M.alloc<double>(3 * b->total_pixels);
    b->iteration = M.alloc<int32_t>(1);
    b->stamps = M.alloc<unsigned long long>(1 + n_jobs);
    b->stats = M.alloc<unsigned long long>(4);
    cudaError_t e = M.err;
    if (e == cudaSuccess)
        e = cudaMemcpy(b->jobs, b->host_jobs.data(), sizeof(gbpt::BatchJob) * n_jobs, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && p->use_graph)
    {
        // capture one iteration; the graph reads the iteration index from device memory
        e = cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaStreamBeginCapture(b->capture_stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess)
        {
            cudaError_t ei = batch_iteration(b, b->capture_stream);
            e = cudaStreamEndCapture(b->capture_stream, &b->graph);
            if (e == cudaSuccess) e = ei;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, b->graph, 0);
    }
    if (e != cudaSuccess)
    {
        batch_release(b);
        delete b;
        return e == cudaErrorMemoryAllocation ? set_error(GBPT_ERROR_OOM, "batch buffers") : cuda_error(e, "batch create");
    }
    for (const gbpt_scene* sc : b->scenes) sc->batch_refs++;
    *out = b;
    return GBPT_OK;
}

gbpt_status gbpt_batch_destroy(gbpt_batch* b)
{
    if (!b) return GBPT_OK;
    batch_release(b);
    for (const gbpt_scene* sc : b->scenes) sc->batch_refs--;
    delete b;
    return GBPT_OK;
}

gbpt_status gbpt_batch_render(gbpt_batch* b, void* stream)
{
    if (!b) return set_error(GBPT_ERROR_INVALID_ARG, "batch is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(b->acc32, 0, 3 * b->total_pixels * sizeof(float), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->acc64, 0, 3 * b->total_pixels * sizeof(double), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->iteration, 0, sizeof(int32_t), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->stats, 0, 4 * sizeof(unsigned long long), st);
    if (e == cudaSuccess) e = gbpt::launch_stamp(b->stamps, st);
    for (int it = 0; e == cudaSuccess && it < b->max_iterations; it++)
        e = b->exec ? cudaGraphLaunch(b->exec, st) : batch_iteration(b, st);
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "batch render");
}

gbpt_status gbpt_batch_job_seconds(gbpt_batch* b, double* seconds)
{
    if (!b || !seconds) return set_error(GBPT_ERROR_INVALID_ARG, "NULL argument");
    std::vector<unsigned long long> t(1 + b->host_jobs.size());
    cudaError_t e = cudaMemcpy(t.data(), b->stamps, t.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_error(e, "stamp read-back");
    for (size_t j = 0; j < b->host_jobs.size(); j++) seconds[j] = (double)(t[1 + j] - t[0]) * 1e-9;
    return GBPT_OK;
}

gbpt_status gbpt_batch_get_image(gbpt_batch* b, int32_t job, float* rgb32, double* rgb64, void* stream)
{
    if (!b) return set_error(GBPT_ERROR_INVALID_ARG, "batch is NULL");
    if (job < 0 || job >= (int32_t)b->host_jobs.size()) return set_error(GBPT_ERROR_INVALID_ARG, "job out of range");
    const gbpt::BatchJob& J = b->host_jobs[job];
    const int64_t npix = (int64_t)J.rc.width * J.rc.height;
    cudaStream_t cs = (cudaStream_t)stream;
    cudaError_t e = cudaSuccess;
    if (rgb32) e = cudaMemcpyAsync(rgb32, b->acc32 + 3 * J.pixel_base, 3 * npix * sizeof(float), cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess && rgb64)
        e = cudaMemcpyAsync(rgb64, b->acc64 + 3 * J.pixel_base, 3 * npix * sizeof(double), cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "batch image read-back");
}

gbpt_status gbpt_batch_get_stats(gbpt_batch* b, gbpt_render_stats* out, void* stream)
{
    if (!b || !out) return set_error(GBPT_ERROR_INVALID_ARG, "NULL argument");
    unsigned long long h[4];
    cudaStream_t cs = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(h, b->stats, sizeof(h), cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
    if (e != cudaSuccess) return cuda_error(e, "stats read-back");
    int64_t samples = 0;
    for (const gbpt::BatchJob& J : b->host_jobs) samples += (int64_t)J.rc.width * J.rc.height * J.spp_total;
    out->samples = samples;
    out->extension_rays = (int64_t)(h[0] + h[1]);
    out->shadow_rays = (int64_t)h[2];
    out->bsdf_light_rays = (int64_t)h[3];
    return GBPT_OK;
}

}  // extern "C"
