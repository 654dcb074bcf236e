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
};

struct gbpt_renderer
{
    const gbpt_scene* scene = nullptr;
    gbpt::RenderConst rc;
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

}  // namespace

extern "C" {

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
        mats[m].base_color = make_float4(src.base_color[0], src.base_color[1], src.base_color[2], 0.0f);
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
    gbpt_principled_material* dpm = nullptr;
    std::vector<gbpt_principled_material> pmats;
    if (d->principled_materials)
    {
        for (int32_t m = 0; m < d->n_materials; m++) pmats.push_back(effective_material(d->principled_materials[m]));
        dpm = M.alloc<gbpt_principled_material>(pmats.size());
    }
    cudaError_t e = M.err;
    if (e == cudaSuccess && dpm)
        e = cudaMemcpyAsync(dpm, pmats.data(), pmats.size() * sizeof(gbpt_principled_material), cudaMemcpyHostToDevice, cs);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dv, verts.data(), verts.size() * sizeof(float4), cudaMemcpyHostToDevice, cs);
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

gbpt_status gbpt_renderer_create(const gbpt_scene* scene, const gbpt_render_settings* st, gbpt_renderer** out)
{
    if (!out) return set_error(GBPT_ERROR_INVALID_ARG, "out is NULL");
    *out = nullptr;
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
    const int64_t cap = (int64_t)st->width * st->height * st->samples_per_launch;
    if (cap > (int64_t)1 << 30) return set_error(GBPT_ERROR_INVALID_ARG, "width*height*samples_per_launch exceeds 2^30 paths");

    gbpt_renderer* r = new (std::nothrow) gbpt_renderer();
    if (!r) return set_error(GBPT_ERROR_OOM, "host allocation failed");
    r->scene = scene;
    r->capacity = cap;
    r->n_sm = sm_count();
    gbpt::RenderConst& rc = r->rc;
    std::memset(&rc, 0, sizeof(rc));
    rc.width = st->width;
    rc.height = st->height;
    rc.spp = st->samples_per_launch;
    rc.nb_bounces = st->nb_bounces;
    rc.do_rr = st->do_russian_roulette;
    rc.rr_min_depth = st->russian_roulette_min_depth;
    rc.rr_clamp = st->russian_roulette_throughput_clamp;
    rc.light_sampling = st->light_sampling;
    rc.bsdf = st->bsdf;
    rc.seed = st->seed;
    rc.do_jittering = st->do_jittering;
    rc.ggx_height_correlated = st->ggx_height_correlated;
    std::memcpy(rc.inverse_view, st->inverse_view, sizeof(rc.inverse_view));
    std::memcpy(rc.inverse_projection, st->inverse_projection, sizeof(rc.inverse_projection));

    DevMem& M = r->mem;
    r->pb.throughput = M.alloc<float4>(cap);
    r->pb.radiance = M.alloc<float4>(cap);
    r->pb.rng = M.alloc<uint64_t>(cap);
    r->pb.pending_light = M.alloc<float4>(cap);
    r->pb.pending_bsdf = M.alloc<float4>(cap);
    r->pb.shadow_entry = M.alloc<int32_t>(cap);
    r->pb.bsdf_entry = M.alloc<int32_t>(cap);
    r->pb.medium = st->bsdf == GBPT_BSDF_PRINCIPLED ? M.alloc<int32_t>(cap) : nullptr;
    r->q[0] = make_queue(M, cap, true, false);
    r->q[1] = make_queue(M, cap, true, false);
    r->shadow = make_queue(M, cap, false, true);
    r->bsdfq = make_queue(M, cap, true, false);
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
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "reset");
}

gbpt_status gbpt_pass_camera_rays(gbpt_renderer* r, void* stream)
{
    if (!r) return set_error(GBPT_ERROR_INVALID_ARG, "renderer is NULL");
    r->cur = 0;
    cudaError_t e = gbpt::launch_camera(r->rc, r->pb, r->q[0], (int32_t)r->iteration, r->stats, r->n_sm,
                                        (cudaStream_t)stream);
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "camera rays");
}

gbpt_status gbpt_pass_bounce(gbpt_renderer* r, int32_t bounce, void* stream)
{
    if (!r) return set_error(GBPT_ERROR_INVALID_ARG, "renderer is NULL");
    if (bounce < 0 || bounce > r->rc.nb_bounces) return set_error(GBPT_ERROR_INVALID_ARG, "bounce out of range");
    const gbpt::Queue& in = r->q[r->cur];
    const gbpt::Queue& next = r->q[r->cur ^ 1];
    cudaError_t e = gbpt::launch_bounce(r->scene->view, r->rc, r->pb, in, next, r->shadow, r->bsdfq, bounce, r->capacity,
                                        r->stats, r->n_sm, (cudaStream_t)stream);
    r->cur ^= 1;
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "bounce");
}

gbpt_status gbpt_pass_accumulate(gbpt_renderer* r, void* stream)
{
    if (!r) return set_error(GBPT_ERROR_INVALID_ARG, "renderer is NULL");
    cudaError_t e = gbpt::launch_accumulate(r->rc, r->pb, r->acc32, r->acc64, r->n_sm, (cudaStream_t)stream);
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
        for (int b = 0; st == GBPT_OK && b <= r->rc.nb_bounces; b++) st = gbpt_pass_bounce(r, b, stream);
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

}  // extern "C"
