/*
 * TEST INFRASTRUCTURE ONLY — C entry points into the reference's OWN CPU intersection code,
 * compiled from the reference's sources where they lie (oracle/Makefile, target 'ref'), behind
 * the clean-room shim headers in oracle/shim/. Output goes to oracle/_ref/ (git-ignored).
 *
 * Calls, unmodified:
 *   - BVH::BVH / BVH::intersect (src/Renderer/BVH.cpp:23-70, src/Renderer/BVH.h:132-223),
 *     through intersect_scene_cpu (src/Device/includes/Intersect.h:180-195);
 *   - evaluate_shadow_ray_occluded (src/Device/includes/Intersect.h:276-324, CPU branch).
 * Alpha testing is off (render_settings.do_alpha_testing = false) so that the filter function
 * only rejects self-hits (src/Device/functions/FilterFunction.h:37-51).
 */
#include "Device/includes/Intersect.h"
#include "Renderer/BVH.h"

#include <cstdint>
#include <cstring>
#include <vector>

namespace {
struct RefScene
{
    std::vector<Triangle> tris;
    BVH* bvh = nullptr;
    HIPRTRenderData rd;
};
}

extern "C" {

void* ref_bvh_build(const float* tri_verts, int64_t n_tris)
{
    RefScene* s = new RefScene();
    s->tris.resize(n_tris);
    for (int64_t i = 0; i < n_tris; i++)
    {
        const float* p = tri_verts + 9 * i;
        s->tris[i] = Triangle(make_float3(p[0], p[1], p[2]), make_float3(p[3], p[4], p[5]), make_float3(p[6], p[7], p[8]));
    }
    s->bvh = new BVH(&s->tris);
    s->rd.render_settings.do_alpha_testing = false;
    s->rd.cpu_only.bvh = s->bvh;
    return s;
}

void ref_bvh_free(void* h)
{
    RefScene* s = static_cast<RefScene*>(h);
    delete s->bvh;
    delete s;
}

/* Same ray/hit layout as orc_octree_closest. */
void ref_bvh_closest(void* h, const float* origin_tmin, const float* dir_tmax, const int32_t* last_prim, int64_t n, float* hits)
{
    RefScene* s = static_cast<RefScene*>(h);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < n; i++)
    {
        hiprtRay ray;
        ray.origin = make_float3(origin_tmin[4 * i], origin_tmin[4 * i + 1], origin_tmin[4 * i + 2]);
        ray.minT = origin_tmin[4 * i + 3];
        ray.direction = make_float3(dir_tmax[4 * i], dir_tmax[4 * i + 1], dir_tmax[4 * i + 2]);
        Xorshift32Generator rng(1);
        hiprtHit hit = intersect_scene_cpu(s->rd, s->bvh, ray, last_prim ? last_prim[i] : -1, rng);
        int32_t prim = hit.hasHit() ? (int32_t)hit.primID : -1;
        float* out = hits + 4 * i;
        out[0] = hit.hasHit() ? hit.t : -1.0f;
        out[1] = hit.uv.x;
        out[2] = hit.uv.y;
        std::memcpy(out + 3, &prim, 4);
    }
}

/* The reference's shadow-ray decision: light_dist[i] is the t_max the reference passes
 * (the function itself subtracts 1e-4). */
void ref_shadow_occluded(void* h, const float* origin_tmin, const float* dir_tmax, const int32_t* last_prim, const float* light_dist,
                         int64_t n, uint8_t* occluded)
{
    RefScene* s = static_cast<RefScene*>(h);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < n; i++)
    {
        hiprtRay ray;
        ray.origin = make_float3(origin_tmin[4 * i], origin_tmin[4 * i + 1], origin_tmin[4 * i + 2]);
        ray.minT = origin_tmin[4 * i + 3];
        ray.direction = make_float3(dir_tmax[4 * i], dir_tmax[4 * i + 1], dir_tmax[4 * i + 2]);
        Xorshift32Generator rng(1);
        occluded[i] = evaluate_shadow_ray_occluded(s->rd, ray, light_dist[i], last_prim ? last_prim[i] : -1, 0, rng) ? 1 : 0;
    }
}

} // extern "C"
