// ReSTIR DI at the camera hit (sm_103a): G-buffer fill, initial candidates with visibility reuse,
// temporal reuse and spatial reuse with pairwise MIS and confidence weights.
//
// Follows the reference's passes (src/Device/kernels/ReSTIR/DI/InitialCandidates.h:180-538,
// TemporalReuse.h:50-298, SpatialReuse.h:43-322; reservoir src/Device/includes/ReSTIR/DI/
// Reservoir.h:22-187; target function TargetFunction.h:49-96; pairwise MIS weights
// src/Device/includes/ReSTIR/TemporalMISWeight.h:164-250 and SpatialMISWeight.h:100-160;
// neighbour selection UtilsSpatial.h, UtilsTemporal.h:27-98, NeighborSimilarity.h) with their
// default options: light candidates from the emissive triangles only (no envmap, no light
// presampling), visibility reuse on, bias correction with visibility, no visibility in the
// spatial target function, geometric-normal and plane-distance neighbour heuristics.
// One thread per pixel. The initial candidates' rays (BSDF candidates, visibility of the kept
// sample) go through device queues traced by the traversal kernels between phases; the reuse
// passes' rays (bias correction, visibility) are traced inline with the shared traversal core. Each pass draws from its own PCG stream per
// pixel; spatial neighbour offsets come from one per-frame Xorshift32 stream shared by all pixels
// (the reference's coalesced spatial reuse), regenerated for the counting and the reuse loops.
#include <cuda_runtime.h>
#include <stdint.h>

#include "render_device.h"
#include "restir.h"
#include "trace_core.h"

namespace gbpt {
namespace {

// ReSTIRDIReservoir::add_one_candidate (Reservoir.h:54-61)
__device__ __forceinline__ void add_candidate(Reservoir& r, V3 point, int tri, int flags, float p_hat, float weight, float u)
{
    r.M++;
    r.w_sum += weight;
    if (u < weight / r.w_sum)
    {
        r.point = point;
        r.tri = tri;
        r.flags = flags;
        r.p_hat = p_hat;
    }
}

// ReSTIRDIReservoir::combine_with (Reservoir.h:77-101): draws a number only when the other
// reservoir has a positive UCW
template <typename Rng>
__device__ __forceinline__ bool combine_with(Reservoir& r, const Reservoir& o, float mis, float p_hat, float jacobian,
                                             Rng& rng)
{
    if (o.ucw <= 0.0f)
    {
        r.M += o.M;
        return false;
    }
    const float w = mis * p_hat * o.ucw * jacobian;
    r.M += o.M;
    r.w_sum += w;
    if (rng() < w / r.w_sum)
    {
        r.point = o.point;
        r.tri = o.tri;
        r.flags = o.flags;
        r.p_hat = p_hat;
        return true;
    }
    return false;
}

// end() / end_with_normalization() (Reservoir.h:103-121)
__device__ __forceinline__ void end_reservoir(Reservoir& r)
{
    r.ucw = r.w_sum == 0.0f ? 0.0f : 1.0f / r.p_hat * r.w_sum;
}

__device__ __forceinline__ void end_with_normalization(Reservoir& r, float num, float den)
{
    if (r.w_sum == 0.0f || r.w_sum < 1.0e-10f || r.w_sum > 1.0e10f || den == 0.0f || num == 0.0f)
        r.ucw = 0.0f;
    else
        r.ucw = 1.0f / r.p_hat * r.w_sum * num / den;
    r.M = min(r.M, 1000000);
}

struct Surface
{
    V3 P, ns, ng, view;
    int prim;
    int mat;
    bool inside;
};

__device__ __forceinline__ Surface load_surface(const GBuffer& gb, int pixel, const float* cam_pos)
{
    const float4 p = gb.pos[pixel], n = gb.ns[pixel], g = gb.ng[pixel];
    Surface su;
    su.P = xyz(p);
    su.prim = __float_as_int(p.w);
    su.ns = xyz(n);
    su.mat = __float_as_int(n.w);
    su.ng = xyz(g);
    su.inside = __float_as_int(g.w) != 0;
    su.view = normalize(v3(cam_pos[0], cam_pos[1], cam_pos[2]) - su.P);
    return su;
}

__device__ __forceinline__ bsdf::Medium medium_of(const Surface& su, const bsdf::Material& m)
{
    bsdf::Medium md;
    md.inside = su.inside;
    md.eta_incident = su.inside ? m.ior : 1.0f;
    md.eta_outgoing = su.inside ? 1.0f : m.ior;
    return md;
}

__device__ __forceinline__ bool occluded(const SceneView& s, V3 P, V3 dir, float dist, int skip)
{
    uint32_t cn = 0, ct = 0;
    const float4 h = core::trace_ray<true, false>(s.bvh_nodes, s.bvh_tris, f4(P, 0.0f), f4(dir, dist - 1.0e-4f), skip, cn, ct);
    return __float_as_int(h.w) >= 0;
}

__device__ __forceinline__ V3 triangle_unit_normal(const SceneView& s, int tri)
{
    V3 a, b, c;
    load_triangle(s, tri, a, b, c);
    return normalize(cross(b - a, c - a));
}

__device__ __forceinline__ V3 emission_of(const SceneView& s, int tri)
{
    return xyz(s.materials[__ldg(s.material_of + tri)].emission);
}

// ReSTIR_DI_evaluate_target_function (TargetFunction.h:49-96)
__device__ float target_function(const SceneView& s, bool hc, const Surface& su, const bsdf::Material& m, V3 point,
                                 int tri, int flags, bool visibility)
{
    if (tri < 0) return 0.0f;
    V3 dir = point - su.P;
    const float dist = length(dir);
    dir = dir / dist;
    const float cosine = dot(su.ns, dir);
    if (cosine <= 0.0f) return 0.0f;
    bsdf::Query q;
    q.view = su.view;
    q.ns = su.ns;
    q.ng = su.ng;
    q.light = dir;
    float pdf;
    const V3 f = bsdf::eval_outlined(m, medium_of(su, m), hc, q, flags & kRestirLobeMask, pdf);
    const float G = fmaxf(0.0f, dot(triangle_unit_normal(s, tri), -dir)) / (dist * dist);
    const float p = luminance(f * emission_of(s, tri) * cosine * G);
    if (p == 0.0f) return 0.0f;
    if (visibility && occluded(s, su.P, dir, dist, su.prim)) return 0.0f;
    return p;
}

// ReSTIR_DI_visibility_test_kill_reservoir (src/Device/includes/ReSTIR/Utils.h:25-64)
__device__ void visibility_kill(const SceneView& s, Reservoir& r, const Surface& su)
{
    if (r.ucw <= 0.0f && r.w_sum <= 0.0f) return;
    if (r.flags & kRestirFlagUnoccluded) return;
    V3 dir = r.point - su.P;
    const float dist = length(dir);
    dir = dir / dist;
    if (occluded(s, su.P, dir, dist, su.prim))
        r.ucw = -1.0f;
    else
        r.flags |= kRestirFlagUnoccluded;
}

__device__ __forceinline__ Pcg32 pass_stream(const RestirConst& k, int pixel, int pass)
{
    if (k.rng_mode == GBPT_RNG_REFERENCE)
    {
        const uint32_t rn = pass == 1 ? k.rn_initial : pass == 2 ? k.rn_temporal : k.rn_spatial[(pass - 3) & 3];
        return reference_seed((uint32_t)pixel, k.sample_number, rn);
    }
    return pcg_seed((uint32_t)pixel, k.frame * 16u + (uint32_t)pass, k.seed);
}

// The material a G-buffer surface is shaded with: with the reference's generator, the packed
// camera-hit material the reference's G-buffer stores (DevicePackedEffectiveMaterial,
// CameraRays.h:178-201); else the scene's
__device__ __forceinline__ const gbpt_principled_material& surface_material(const SceneView& s, const RestirConst& k,
                                                                           int mat)
{
    return (k.rng_mode == GBPT_RNG_REFERENCE && s.pmats_camera) ? s.pmats_camera[mat] : s.pmats[mat];
}

// The spatial neighbours' generator of a pixel: with the reference's generator, seeded by one draw
// of the pixel's own (setup_adaptive_directional_spatial_reuse, UtilsSpatial.h:17-22); else the
// pass's seed shared by all pixels
__device__ __forceinline__ uint32_t neighbor_seed_of(const RestirConst& k, Pcg32& rng, uint32_t shared_seed)
{
    return k.rng_mode == GBPT_RNG_REFERENCE ? rng.next_u32() : shared_seed;
}

// neighbour heuristics (NeighborSimilarity.h:34-84): plane distance and geometric-normal angle;
// positions/primitives from 'gb_pos' (the previous frame's G-buffer for the temporal pass), the
// neighbour's normal from the current G-buffer as the reference reads it
__device__ __forceinline__ bool similar(const GBuffer& gb_pos, const GBuffer& gb_cur, int n_idx, int c_idx, V3 P, V3 n_center,
                                        const RestirConst& k)
{
    if (n_idx == c_idx) return true;
    const float4 np = gb_pos.pos[n_idx];
    if (__float_as_int(np.w) < 0) return false;
    if (!(fabsf(dot(xyz(np) - P, n_center)) < k.plane_distance)) return false;
    return dot(n_center, xyz(gb_cur.ng[n_idx])) > k.normal_similarity_cos;
}

// get_spatial_neighbor_pixel_index (UtilsSpatial.h:77-143): uniform disk of the reuse radius,
// offsets rounded to whole pixels; the centre itself for index == count
__device__ __forceinline__ int spatial_neighbor(int idx, int count, int cx, int cy, int W, int H, float radius,
                                                bsdf::Xorshift32& nrng)
{
    if (idx == count) return cx + cy * W;
    const float u = nrng();
    const float v = nrng();
    const float r = radius * sqrtf(v);
    float sn, cs;
    sincosf(kTwoPi * u, &sn, &cs);
    const int nx = cx + (int)roundf(r * cs), ny = cy + (int)roundf(r * sn);
    if (nx < 0 || nx >= W || ny < 0 || ny >= H) return -1;
    return nx + ny * W;
}

// ---------------------------------------------------------------------------------------------
// light presampling (ReSTIR_DI_LightsPresampling, src/Device/kernels/ReSTIR/DI/LightsPresampling.h:
// 74-109; use_presampled_light_candidate, InitialCandidates.h:33-69): once per frame, subsets of
// light samples drawn from the scene's light distribution; a pixel's light candidates come from
// the subset its tile draws, so neighbouring pixels read the same few kilobytes of light data
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) presample_kernel(SceneView s, RenderConst rc, RestirConst k, float4* out)
{
    const int n = k.presample_subsets * k.presample_size;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        Pcg32 rng = pcg_seed((uint32_t)i, k.frame, k.seed ^ 0x5BD1E995u);
        const LightSample ls = sample_light(s, rc, rng);
        out[2 * i] = f4(ls.point, __int_as_float(ls.triangle));
        out[2 * i + 1] = f4(ls.normal, ls.pdf_area);
    }
}

// the frame's subset for the tile of pixel (x, y): Cantor pairing of the tile coordinates scales
// the frame's seed of a Xorshift32 draw
__device__ __forceinline__ int presampled_subset(const RestirConst& k, int x, int y)
{
    const uint32_t tx = (uint32_t)(x / k.presample_tile), ty = (uint32_t)(y / k.presample_tile);
    const uint32_t cantor = (tx + ty + 1u) * (tx + ty) / 2u + ty;
    uint32_t seed = k.presample_seed * (cantor + 1u);
    if (seed == 0u) seed = 0x9E3779B9u;
    bsdf::Xorshift32 xr{seed};
    const int i = (int)(xr() * (float)k.presample_subsets);
    return min(i, k.presample_subsets - 1);
}

// ---------------------------------------------------------------------------------------------
// G-buffer from the camera hits (CameraRays, src/Device/kernels/CameraRays.h:178-201)
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) gbuffer_kernel(SceneView s, Queue q, GBuffer gb, int packed_normals)
{
    const int n = *q.count;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const int pixel = q.slot[i];
        const float4 hit = q.hits[i];
        const int prim = __float_as_int(hit.w);
        if (prim < 0)
        {
            gb.pos[pixel] = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1));
            continue;
        }
        const V3 o = xyz(q.origin_tmin[i]), d = xyz(q.dir_tmax[i]);
        const V3 P = o + hit.x * d;
        V3 a, b, c;
        load_triangle(s, prim, a, b, c);
        const V3 ng_raw = normalize(cross(b - a, c - a));
        V3 ng = ng_raw, ns = shading_normal(s, prim, hit.y, hit.z, ng_raw);
        const V3 view = -d;
        fix_backfacing(view, ng, ns);
        if (packed_normals)
        {
            // the reference's G-buffer stores octahedral 24-bit normals, read back unpacked as
            // they are by its ReSTIR surfaces (get_pixel_surface, ReSTIR/Surface.h:26-40)
            ns = oct24_roundtrip(ns);
            ng = oct24_roundtrip(ng);
        }
        const int mat = __ldg(s.material_of + prim);
        // the camera hit's volume state as the reference rebuilds it from the G-buffer
        // (RayVolumeState::reconstruct_first_hit, ReSTIR/Surface.h:31): the material pushed on a
        // stack holding only the air, so the ray enters it (camera in the air)
        const bool inside = false;
        gb.pos[pixel] = f4(P, __int_as_float(prim));
        gb.ns[pixel] = f4(ns, __int_as_float(mat));
        gb.ng[pixel] = f4(ng, __int_as_float(inside ? 1 : 0));
    }
}

// ---------------------------------------------------------------------------------------------
// initial candidates (InitialCandidates.h:180-538) as wavefront phases: the light candidates and
// the first BSDF candidate's direction (its ray appended to a queue), the queue traced by the
// traversal kernels, the BSDF candidate resolved (and the next one's ray appended), and so on per
// BSDF candidate; then the visibility rays of the kept samples, traced as one any-hit queue, and
// the kill. Tracing inside this kernel ran at its occupancy (168 registers, three CTAs per SM):
// the two rays of a 1080p frame cost 11.7 of its 17.8 ms. Random numbers are drawn in the
// reference's order: the pixel's PCG state travels between the phases.
// ---------------------------------------------------------------------------------------------

// the shared start of a pixel's phase: surface, material and medium
struct InitialPixel
{
    Surface su;
    bsdf::Material m;
    bsdf::Medium md;
};

// draws BSDF candidate 'round' of a pixel: the direction and its ray (appended to 'rays'), or no
// ray when its pdf is zero; the PCG state after the draw goes to the pixel state
__device__ __forceinline__ void initial_bsdf_draw(const InitialPixel& px, bool hc, Pcg32& rng, const Queue& rays,
                                                  const InitialState& st, int pixel)
{
    bsdf::Xorshift32 xr = bsdf_rng(rng);
    V3 dir;
    int lobe;
    float pdf;
    // the inlined evaluation: this kernel's light loop inlines it already
    bsdf::sample<bsdf::Xorshift32, true>(px.m, px.md, hc, px.su.view, px.su.ns, px.su.ng, xr, dir, lobe, pdf);
    const bool want = pdf > 0.0f;
    const int slot = warp_append(rays.count, want);
    if (want)
    {
        rays.origin_tmin[slot] = f4(px.su.P, 0.0f);
        rays.dir_tmax[slot] = f4(dir, 1.0e35f - 1.0e-4f);
        rays.last_prim[slot] = px.su.prim;
        rays.slot[slot] = pixel;
    }
    st.cand[pixel] = f4(dir, pdf);
    st.meta[pixel] = make_int4((int)(uint32_t)rng.state, (int)(uint32_t)(rng.state >> 32), lobe, want ? slot : -1);
}

// the end of the candidates: normalisation, M = 1, and the visibility ray of the kept sample
// (ReSTIR_DI_visibility_test_kill_reservoir, src/Device/includes/ReSTIR/Utils.h:25-64) appended to
// 'vis' when visibility reuse is on and the sample needs one; else the reservoir is final
__device__ __forceinline__ void initial_finish(const RestirConst& k, const Surface& su, Reservoir& r,
                                               const ReservoirBuf& out, const InitialState& st, const Queue& vis,
                                               int pixel)
{
    end_reservoir(r);
    r.M = 1;
    const bool test = k.visibility_reuse && !(r.ucw <= 0.0f && r.w_sum <= 0.0f) && !(r.flags & kRestirFlagUnoccluded);
    const int slot = warp_append(vis.count, test);
    if (test)
    {
        V3 dir = r.point - su.P;
        const float dist = length(dir);
        dir = dir / dist;
        vis.origin_tmin[slot] = f4(su.P, 0.0f);
        vis.dir_tmax[slot] = f4(dir, dist - 1.0e-4f);
        vis.last_prim[slot] = su.prim;
        vis.slot[slot] = pixel;
    }
    store_reservoir(out, pixel, r);
    st.meta[pixel] = make_int4(0, 0, kInitialVisibility, test ? slot : -1);
}

__device__ __forceinline__ bool initial_load(const SceneView& s, const RestirConst& k, const GBuffer& gb, int pixel,
                                             InitialPixel& px)
{
    px.su = load_surface(gb, pixel, k.camera_pos);
    if (px.su.prim < 0 || s.n_emissive == 0) return false;
    px.m = bsdf::load_material(surface_material(s, k, px.su.mat));
    px.md = medium_of(px.su, px.m);
    return true;
}

// the light candidates of a pixel; EXT: its material has extension lobes (the evaluation goes out
// of line, in its own copy of the loop, so that the common materials' loop makes no call)
template <bool EXT>
__device__ __forceinline__ void initial_light_candidates(const SceneView& s, const RenderConst& rc, const RestirConst& k,
                                                         const InitialPixel& px, bool hc, Pcg32& rng, Reservoir& r,
                                                         int pixel)
{
    const Surface& su = px.su;
    const float nl = (float)k.light_candidates, nb = (float)k.bsdf_candidates;
    const int subset = k.presampled ? presampled_subset(k, pixel % rc.width, pixel / rc.width) : 0;
    for (int c = 0; c < k.light_candidates; c++)
    {
        LightSample ls;
        if (k.presampled)
        {
            // a light of the tile's presampled subset, with the pdf it was drawn with
            const int e = subset * k.presample_size + rng.index(k.presample_size);
            const float4 a = __ldg(k.presampled + 2 * e), b = __ldg(k.presampled + 2 * e + 1);
            ls.point = xyz(a);
            ls.triangle = __float_as_int(a.w);
            ls.normal = xyz(b);
            ls.pdf_area = b.w;
            ls.emission = emission_of(s, ls.triangle);
        }
        else
        {
            // the reference first draws the envmap-or-light choice (sample_fresh_light_candidate,
            // InitialCandidates.h:100; without an envmap always a light)
            if (k.rng_mode == GBPT_RNG_REFERENCE) rng.next();
            ls = sample_light(s, rc, rng);
        }
        V3 wi = ls.point - su.P;
        const float dist = length(wi);
        wi = wi / dist;
        const float cosine = fmaxf(0.0f, dot(su.ns, wi));
        float weight = 0.0f, p_hat = 0.0f;
        if (cosine > 0.0f && ls.pdf_area > 0.0f)
        {
            bsdf::Query q;
            q.view = su.view;
            q.ns = su.ns;
            q.ng = su.ng;
            q.light = wi;
            float bsdf_pdf;
            const V3 f = EXT ? bsdf::eval_outlined(px.m, px.md, hc, q, GBPT_LOBE_NONE, bsdf_pdf)
                             : bsdf::eval_layers<false>(px.m, px.md, hc, q, GBPT_LOBE_NONE, bsdf_pdf);
            if (bsdf_pdf > 0.0f)
            {
                const float cos_l = fmaxf(0.0f, dot(ls.normal, -wi));
                // the reference's candidate carries ReSTIR_DI_evaluate_target_function's value
                p_hat = k.rng_mode == GBPT_RNG_REFERENCE
                            ? target_function(s, hc, su, px.m, ls.point, ls.triangle, 0, false)
                            : luminance(f * ls.emission * dot(su.ns, wi) * (cos_l / (dist * dist)));
                const float light_pdf = area_to_solid_angle_pdf(ls.pdf_area, dist, cos_l);
                const float mis = light_pdf == 0.0f ? 0.0f : light_pdf / (nl * light_pdf + nb * bsdf_pdf);
                weight = mis * p_hat / ls.pdf_area;
            }
        }
        add_candidate(r, ls.point, ls.triangle, 0, p_hat, weight, rng.next());
    }
}

// phase 1: the light candidates, then BSDF candidate 0's direction (or the end when there is none)
__global__ void __launch_bounds__(128, 3) initial_lights_kernel(SceneView s, RenderConst rc, RestirConst k, GBuffer gb,
                                                                ReservoirBuf out, InitialState st, Queue rays,
                                                                Queue vis)
{
    const int n_pix = rc.width * rc.height;
    const bool hc = rc.ggx_height_correlated != 0;
    for (int pixel = blockIdx.x * blockDim.x + threadIdx.x; pixel < n_pix; pixel += gridDim.x * blockDim.x)
    {
        Reservoir r = empty_reservoir();
        InitialPixel px;
        const bool live = initial_load(s, k, gb, pixel, px);
        Pcg32 rng = pass_stream(k, pixel, 1);
        if (live)
        {
            if (px.m.ext)
                initial_light_candidates<true>(s, rc, k, px, hc, rng, r, pixel);
            else
                initial_light_candidates<false>(s, rc, k, px, hc, rng, r, pixel);
        }
        if (!live)
        {
            store_reservoir(out, pixel, r);
            st.meta[pixel] = make_int4(0, 0, kInitialDone, -1);
        }
        else if (k.bsdf_candidates > 0)
        {
            store_reservoir(out, pixel, r);
            initial_bsdf_draw(px, hc, rng, rays, st, pixel);
        }
        else
            initial_finish(k, px.su, r, out, st, vis, pixel);
    }
}

// phase 2 (one launch per BSDF candidate): the traced candidate joins the reservoir; then the next
// candidate's direction, or the end
__global__ void __launch_bounds__(128, 3) initial_bsdf_kernel(SceneView s, RenderConst rc, RestirConst k, GBuffer gb,
                                                              ReservoirBuf out, InitialState st, Queue traced,
                                                              Queue rays, Queue vis, int round)
{
    const int n_pix = rc.width * rc.height;
    const bool hc = rc.ggx_height_correlated != 0;
    for (int pixel = blockIdx.x * blockDim.x + threadIdx.x; pixel < n_pix; pixel += gridDim.x * blockDim.x)
    {
        const int4 meta = st.meta[pixel];
        const bool live = meta.z >= 0;  // a lobe: the pixel still draws BSDF candidates
        if (!live) continue;
        InitialPixel px;
        Reservoir r = empty_reservoir();
        Pcg32 rng = pass_stream(k, pixel, 1);
        {
            initial_load(s, k, gb, pixel, px);
            r = load_reservoir(out, pixel);
            rng.state = (uint64_t)(uint32_t)meta.x | ((uint64_t)(uint32_t)meta.y << 32);
            if (meta.w >= 0)
            {
                const Surface& su = px.su;
                const float nl = (float)k.light_candidates, nb = (float)k.bsdf_candidates;
                const float4 cd = st.cand[pixel];
                const V3 dir = xyz(cd);
                const float pdf = cd.w;
                const int lobe = meta.z;
                const float4 h = traced.hits[meta.w];
                const int lt = __float_as_int(h.w);
                const V3 Le = lt >= 0 ? emission_of(s, lt) : v3(0.0f);
                if (lt >= 0 && !is_black(Le))
                {
                    const V3 point = su.P + dir * h.x;
                    const int flags = kRestirFlagUnoccluded | (lobe & kRestirLobeMask);
                    const float p_hat = target_function(s, hc, su, px.m, point, lt, flags, false);
                    const V3 nlt = triangle_unit_normal(s, lt);
                    const float cos_l = fmaxf(0.0f, dot(nlt, -dir));
                    float light_pdf = 0.0f;
                    if (!(dot(dir, su.ns) < 0.0f))
                    {
                        V3 a, b, cc;
                        load_triangle(s, lt, a, b, cc);
                        const float area = 0.5f * length(cross(b - a, cc - a));
                        float pa = 1.0f / area;
                        if (rc.light_sampling == GBPT_LIGHT_POWER)
                            pa *= (luminance(Le) * area) / s.power_sum;
                        else
                            pa /= (float)s.n_emissive;
                        light_pdf = area_to_solid_angle_pdf(pa, h.x, cos_l);
                    }
                    const float mis = pdf / (nb * pdf + nl * light_pdf);
                    const float pdf_area = pdf / (h.x * h.x) * cos_l;
                    // the back of a one-sided emitter: zero area pdf (the reference's weight would be 0/0)
                    if (pdf_area > 0.0f) add_candidate(r, point, lt, flags, p_hat, mis * p_hat / pdf_area, rng.next());
                }
            }
        }
        if (round + 1 < k.bsdf_candidates)
        {
            store_reservoir(out, pixel, r);
            initial_bsdf_draw(px, hc, rng, rays, st, pixel);
        }
        else
            initial_finish(k, px.su, r, out, st, vis, pixel);
    }
}

// the visibility results of the kept samples (initial candidates, spatial reuse): killed when
// occluded, marked unoccluded otherwise
__global__ void __launch_bounds__(256) visibility_apply_kernel(RenderConst rc, ReservoirBuf out, InitialState st,
                                                                 Queue vis)
{
    const int n_pix = rc.width * rc.height;
    for (int pixel = blockIdx.x * blockDim.x + threadIdx.x; pixel < n_pix; pixel += gridDim.x * blockDim.x)
    {
        const int4 meta = st.meta[pixel];
        if (meta.z != kInitialVisibility || meta.w < 0) continue;
        Reservoir r = load_reservoir(out, pixel);
        if (vis.occluded[meta.w])
            r.ucw = -1.0f;
        else
            r.flags |= kRestirFlagUnoccluded;
        store_reservoir(out, pixel, r);
    }
}

// ---------------------------------------------------------------------------------------------
// temporal reuse (TemporalReuse.h:50-298, pairwise MIS TemporalMISWeight.h:164-250)
// ---------------------------------------------------------------------------------------------
// The temporal neighbour of a pixel (UtilsTemporal.h:27-98): backprojection into the previous
// frame, then up to 'temporal_search_count' jittered tries; -1 when none is similar. Draws from
// 'rng' in the reference's order.
__device__ __forceinline__ int temporal_neighbor(const RestirConst& k, const GBuffer& gb, const GBuffer& gb_prev, int W,
                                                 int H, int pixel, const Surface& su, Pcg32& rng)
{
    const V3 ndc = mat_x_point(k.prev_view_projection, su.P);
    const float px = (ndc.x + 1.0f) * 0.5f * (float)W - 0.5f;
    const float py = (ndc.y + 1.0f) * 0.5f * (float)H - 0.5f;
    for (int i = 0; i < k.temporal_search_count + 1; i++)
    {
        float ox = 0.0f, oy = 0.0f;
        if (i > 0)
        {
            ox = (rng.next() - 0.5f) * k.temporal_search_radius;
            oy = (rng.next() - 0.5f) * k.temporal_search_radius;
        }
        const int tx = (int)roundf(px + ox), ty = (int)roundf(py + oy);
        if (tx < 0 || tx >= W || ty < 0 || ty >= H) continue;
        const int t_idx = tx + ty * W;
        // the reference's temporal pass compares against the centre's shading normal
        // (TemporalReuse.h:81-82); the other heuristics use the geometric one
        if (similar(gb_prev, gb, t_idx, pixel, su.P, k.rng_mode == GBPT_RNG_REFERENCE ? su.ns : su.ng, k)) return t_idx;
    }
    return -1;
}

// A previous-frame G-buffer surface. With the reference's generator its view direction runs from
// the previous camera to the CURRENT frame's hit point of that pixel, as the reference builds it
// (get_pixel_surface_previous_frame, ReSTIR/Surface.h:52)
__device__ __forceinline__ Surface previous_surface(const GBuffer& gb, const GBuffer& gb_prev, int idx, const RestirConst& k)
{
    Surface su = load_surface(gb_prev, idx, k.prev_camera_pos);
    if (k.rng_mode == GBPT_RNG_REFERENCE)
        su.view = normalize(v3(k.prev_camera_pos[0], k.prev_camera_pos[1], k.prev_camera_pos[2]) - xyz(gb.pos[idx]));
    return su;
}

// appends the shadow ray of a target-function evaluation (from P to the sample) when 'want'
__device__ __forceinline__ int append_sample_ray(const Queue& q, bool want, V3 P, V3 point, int skip, int pixel)
{
    const int slot = warp_append(q.count, want);
    if (want)
    {
        V3 dir = point - P;
        const float dist = length(dir);
        dir = dir / dist;
        q.origin_tmin[slot] = f4(P, 0.0f);
        q.dir_tmax[slot] = f4(dir, dist - 1.0e-4f);
        q.last_prim[slot] = skip;
        q.slot[slot] = pixel;
    }
    return slot;
}

// temporal reuse, phase 1: the two bias-correction rays of a pixel (the temporal sample seen from
// the pixel, the pixel's initial sample seen from the temporal neighbour), appended where their
// target functions without visibility are positive; slots in 'ray_of' (-1: no ray)
__global__ void __launch_bounds__(128, 3) temporal_rays_kernel(SceneView s, RenderConst rc, RestirConst k, GBuffer gb,
                                                               GBuffer gb_prev, ReservoirBuf initial, ReservoirBuf prev,
                                                               int2* ray_of, Queue rays)
{
    const int W = rc.width, H = rc.height, n_pix = W * H;
    const bool hc = rc.ggx_height_correlated != 0;
    for (int pixel = blockIdx.x * blockDim.x + threadIdx.x; pixel < n_pix; pixel += gridDim.x * blockDim.x)
    {
        ray_of[pixel] = make_int2(-1, -1);
        const Reservoir init = load_reservoir(initial, pixel);
        const Surface su = load_surface(gb, pixel, k.camera_pos);
        if (su.prim < 0 || !k.has_prev) continue;
        Pcg32 rng = pass_stream(k, pixel, 2);
        const int t_idx = temporal_neighbor(k, gb, gb_prev, W, H, pixel, su, rng);
        if (t_idx < 0) continue;
        const Reservoir tn = load_reservoir(prev, t_idx);
        const Surface ts = previous_surface(gb, gb_prev, t_idx, k);
        if (tn.M == 0 || ts.prim < 0 || !is_black(xyz(s.materials[ts.mat].emission))) continue;
        const bsdf::Material m = bsdf::load_material(surface_material(s, k, su.mat));
        const bsdf::Material tm = bsdf::load_material(surface_material(s, k, ts.mat));
        const bool a = tn.ucw > 0.0f && target_function(s, hc, su, m, tn.point, tn.tri, tn.flags, false) > 0.0f;
        const bool b = target_function(s, hc, ts, tm, init.point, init.tri, init.flags, false) > 0.0f;
        const int sa = append_sample_ray(rays, a, su.P, tn.point, su.prim, pixel);
        const int sb = append_sample_ray(rays, b, ts.P, init.point, ts.prim, pixel);
        ray_of[pixel] = make_int2(a ? sa : -1, b ? sb : -1);
    }
}

// temporal reuse, phase 2 (TemporalReuse.h:50-298): the resampling with the traced visibility
__global__ void __launch_bounds__(128, 3) temporal_kernel(SceneView s, RenderConst rc, RestirConst k, GBuffer gb,
                                                       GBuffer gb_prev, ReservoirBuf initial, ReservoirBuf prev,
                                                       ReservoirBuf out, const int2* __restrict__ ray_of, Queue traced)
{
    const int W = rc.width, H = rc.height, n_pix = W * H;
    const bool hc = rc.ggx_height_correlated != 0;
    for (int pixel = blockIdx.x * blockDim.x + threadIdx.x; pixel < n_pix; pixel += gridDim.x * blockDim.x)
    {
        const Reservoir init = load_reservoir(initial, pixel);
        const Surface su = load_surface(gb, pixel, k.camera_pos);
        if (su.prim < 0 || !k.has_prev)
        {
            store_reservoir(out, pixel, init);
            continue;
        }
        Pcg32 rng = pass_stream(k, pixel, 2);
        const int t_idx = temporal_neighbor(k, gb, gb_prev, W, H, pixel, su, rng);
        if (t_idx < 0)
        {
            store_reservoir(out, pixel, init);
            continue;
        }
        const Reservoir tn = load_reservoir(prev, t_idx);
        const Surface ts = previous_surface(gb, gb_prev, t_idx, k);
        if (tn.M == 0 || ts.prim < 0 || !is_black(xyz(s.materials[ts.mat].emission)))
        {
            store_reservoir(out, pixel, init);
            continue;
        }
        const bsdf::Material m = bsdf::load_material(surface_material(s, k, su.mat));
        const bsdf::Material tm = bsdf::load_material(surface_material(s, k, ts.mat));
        const bool vis = k.bias_correction_visibility != 0;
        const int2 rays = vis ? ray_of[pixel] : make_int2(-1, -1);
        Reservoir o = empty_reservoir();

        // temporal neighbour, pairwise MIS weight against the canonical (initial) reservoir
        float t_at_center = tn.ucw > 0.0f ? target_function(s, hc, su, m, tn.point, tn.tri, tn.flags, false) : 0.0f;
        if (vis && t_at_center > 0.0f && rays.x >= 0 && traced.occluded[rays.x]) t_at_center = 0.0f;
        const float tM = k.confidence_weights ? (float)tn.M : 1.0f;
        const float cM = k.confidence_weights ? (float)init.M : 1.0f;
        const float nsum = k.confidence_weights ? (float)tn.M : 1.0f;
        const float denom = tn.p_hat * nsum + t_at_center * cM;
        const float mi = denom == 0.0f ? 0.0f : tn.p_hat * tM / denom;
        float c_at_neighbor = target_function(s, hc, ts, tm, init.point, init.tri, init.flags, false);
        if (vis && c_at_neighbor > 0.0f && rays.y >= 0 && traced.occluded[rays.y]) c_at_neighbor = 0.0f;
        const float denom_mc = c_at_neighbor * nsum + init.p_hat * cM;
        float mc = 0.0f;
        if (denom_mc != 0.0f) mc += init.p_hat * cM / denom_mc * (k.confidence_weights ? tM / nsum : 1.0f);
        if (combine_with(o, tn, mi, t_at_center, 1.0f, rng))
        {
            if (vis)
                o.flags |= kRestirFlagUnoccluded;
            else
                o.flags &= ~kRestirFlagUnoccluded;
        }
        // canonical sample
        if (combine_with(o, init, mc == 0.0f ? 1.0f : mc, init.p_hat, 1.0f, rng))
        {
            if (vis)
                o.flags |= kRestirFlagUnoccluded;
            else
                o.flags |= init.flags & kRestirFlagUnoccluded;
        }
        end_with_normalization(o, 1.0f, 1.0f);
        if (k.m_cap > 0) o.M = min(o.M, k.m_cap);
        store_reservoir(out, pixel, o);
    }
}

// ---------------------------------------------------------------------------------------------
// spatial reuse (SpatialReuse.h:43-322, pairwise MIS SpatialMISWeight.h:100-160)
// ---------------------------------------------------------------------------------------------
// spatial reuse, phase 1: the bias-correction rays. Each valid neighbour evaluates the centre's
// sample with visibility (the MIS weight's c_at_n); the rays, from the neighbour's surface to the
// sample, depend only on the input reservoirs and the G-buffer, so they are appended here (one
// slot per pixel and neighbour in 'ray_of', -1 without a ray) and traced as one any-hit queue.
__global__ void __launch_bounds__(128) spatial_rays_kernel(SceneView s, RenderConst rc, RestirConst k, GBuffer gb,
                                                           ReservoirBuf in, int pass, uint32_t neighbor_seed,
                                                           int32_t* ray_of, Queue rays)
{
    const int W = rc.width, H = rc.height, n_pix = W * H;
    const bool hc = rc.ggx_height_correlated != 0;
    const int K = k.spatial_neighbors;
    for (int pixel = blockIdx.x * blockDim.x + threadIdx.x; pixel < n_pix; pixel += gridDim.x * blockDim.x)
    {
        int32_t* slots = ray_of + (int64_t)pixel * K;
        for (int j = 0; j < K; j++) slots[j] = -1;
        const Surface su = load_surface(gb, pixel, k.camera_pos);
        const Reservoir center = load_reservoir(in, pixel);
        if (su.prim < 0 || !(center.M > 0 && center.ucw > 0.0f)) continue;
        const int cx = pixel % W, cy = pixel / W;
        Pcg32 rng = pass_stream(k, pixel, 3 + pass);
        bsdf::Xorshift32 nrng{neighbor_seed_of(k, rng, neighbor_seed)};
        for (int j = 0; j < K; j++)
        {
            const int idx = spatial_neighbor(j, K, cx, cy, W, H, k.spatial_radius, nrng);
            bool want = idx >= 0 && center.tri >= 0 && similar(gb, gb, idx, pixel, su.P, su.ng, k);
            Surface ns_;
            if (want)
            {
                ns_ = load_surface(gb, idx, k.camera_pos);
                const bsdf::Material nm = bsdf::load_material(surface_material(s, k, ns_.mat));
                // the target function without visibility; a ray only where it is positive
                want = target_function(s, hc, ns_, nm, center.point, center.tri, center.flags, false) > 0.0f;
            }
            const int slot = warp_append(rays.count, want);
            if (!want) continue;
            V3 dir = center.point - ns_.P;
            const float dist = length(dir);
            dir = dir / dist;
            rays.origin_tmin[slot] = f4(ns_.P, 0.0f);
            rays.dir_tmax[slot] = f4(dir, dist - 1.0e-4f);
            rays.last_prim[slot] = ns_.prim;
            rays.slot[slot] = pixel;
            slots[j] = slot;
        }
    }
}

// spatial reuse, phase 2 (SpatialReuse.h:43-322): the resampling with the traced bias-correction
// visibility; the final visibility ray of the result goes to 'vis' (applied by
// visibility_apply_kernel), the reservoir is stored here
__global__ void __launch_bounds__(128) spatial_kernel(SceneView s, RenderConst rc, RestirConst k, GBuffer gb,
                                                      ReservoirBuf in, ReservoirBuf out, int pass, int last_pass,
                                                      uint32_t neighbor_seed, const int32_t* __restrict__ ray_of,
                                                      Queue traced, InitialState st, Queue visq)
{
    const int W = rc.width, H = rc.height, n_pix = W * H;
    const bool hc = rc.ggx_height_correlated != 0;
    const int K = k.spatial_neighbors;
    for (int pixel = blockIdx.x * blockDim.x + threadIdx.x; pixel < n_pix; pixel += gridDim.x * blockDim.x)
    {
        const Surface su = load_surface(gb, pixel, k.camera_pos);
        const Reservoir center = load_reservoir(in, pixel);
        if (su.prim < 0)
        {
            store_reservoir(out, pixel, center);
            st.meta[pixel] = make_int4(0, 0, kInitialDone, -1);
            continue;
        }
        Pcg32 rng = pass_stream(k, pixel, 3 + pass);
        const int cx = pixel % W, cy = pixel / W;
        const uint32_t nseed = neighbor_seed_of(k, rng, neighbor_seed);
        // count the valid neighbours and their confidence (count_valid_spatial_neighbors)
        bsdf::Xorshift32 nrng{nseed};
        int valid = 0, m_sum = 0;
        uint32_t cache = 0;
        for (int j = 0; j < K; j++)
        {
            const int idx = spatial_neighbor(j, K, cx, cy, W, H, k.spatial_radius, nrng);
            if (idx < 0) continue;
            if (!similar(gb, gb, idx, pixel, su.P, su.ng, k)) continue;
            m_sum += load_reservoir(in, idx).M;
            valid++;
            cache |= 1u << j;
        }
        const bsdf::Material m = bsdf::load_material(surface_material(s, k, su.mat));
        const bool vis = k.bias_correction_visibility != 0;
        const bool update_mc = center.M > 0 && center.ucw > 0.0f;
        const float cM = k.confidence_weights ? (float)center.M : 1.0f;
        const float nsum = k.confidence_weights ? (float)m_sum : 1.0f;
        const float div = k.confidence_weights ? 1.0f : (float)valid;
        float mc = 0.0f;
        Reservoir o = empty_reservoir();
        nrng = bsdf::Xorshift32{nseed};
        for (int j = m_sum == 0 ? K : 0; j < K + 1; j++)
        {
            if (j < K && !(cache & (1u << j)))
            {
                nrng();
                nrng();
                continue;
            }
            const int idx = spatial_neighbor(j, K, cx, cy, W, H, k.spatial_radius, nrng);
            if (idx < 0) continue;
            const Reservoir nbr = load_reservoir(in, idx);
            float t_at_center = 0.0f;
            if (nbr.ucw > 0.0f)
                t_at_center = j == K ? nbr.p_hat : target_function(s, hc, su, m, nbr.point, nbr.tri, nbr.flags, false);
            float mis;
            if (j < K)
            {
                const float rM = k.confidence_weights ? (float)nbr.M : 1.0f;
                const float denom = nbr.p_hat * nsum + t_at_center / div * cM;
                const float mi = denom == 0.0f ? 0.0f : nbr.p_hat * rM / denom;
                if (update_mc)
                {
                    const Surface ns_ = load_surface(gb, idx, k.camera_pos);
                    const bsdf::Material nm = bsdf::load_material(surface_material(s, k, ns_.mat));
                    float c_at_n = target_function(s, hc, ns_, nm, center.point, center.tri, center.flags, false);
                    if (vis && c_at_n > 0.0f)
                    {
                        const int32_t ray = ray_of[(int64_t)pixel * K + j];
                        if (ray >= 0 && traced.occluded[ray]) c_at_n = 0.0f;
                    }
                    const float nume_mc = center.p_hat / div * cM;
                    const float denom_mc = c_at_n * nsum + center.p_hat / div * cM;
                    const float conf = k.confidence_weights ? (nsum == 0.0f ? 0.0f : rM / nsum) : 1.0f;
                    if (denom_mc != 0.0f) mc += nume_mc / denom_mc / div * conf;
                }
                mis = mi / div;
            }
            else
                mis = mc == 0.0f ? 1.0f : mc;
            if (combine_with(o, nbr, mis, t_at_center, 1.0f, rng))
            {
                if (j == K)
                    o.flags |= nbr.flags & kRestirFlagUnoccluded;
                else
                    o.flags &= ~kRestirFlagUnoccluded;
            }
        }
        end_with_normalization(o, 1.0f, 1.0f);
        if (k.m_cap > 0) o.M = min(o.M, k.m_cap);  // SpatialReuse.h:317-319
        // visibility reuse of the result (visibility_kill) through the any-hit queue
        const bool test = k.visibility_reuse && vis && (k.do_temporal || pass != last_pass) &&
                          !(o.ucw <= 0.0f && o.w_sum <= 0.0f) && !(o.flags & kRestirFlagUnoccluded);
        const int slot = warp_append(visq.count, test);
        if (test)
        {
            V3 dir = o.point - su.P;
            const float dist = length(dir);
            dir = dir / dist;
            visq.origin_tmin[slot] = f4(su.P, 0.0f);
            visq.dir_tmax[slot] = f4(dir, dist - 1.0e-4f);
            visq.last_prim[slot] = su.prim;
            visq.slot[slot] = pixel;
        }
        st.meta[pixel] = make_int4(0, 0, kInitialVisibility, slot);
        store_reservoir(out, pixel, o);
    }
}

// ---------------------------------------------------------------------------------------------
// fused spatiotemporal reuse (FusedSpatiotemporalReuse.h:152-566, pairwise MIS
// SpatiotemporalMISWeight.h:140-224): the temporal neighbour, then K spatial neighbours from the
// previous frame's final reservoirs around the backprojected position (heuristics and MIS surfaces
// from the previous G-buffer), then the canonical initial reservoir, in one pass. The temporal
// neighbour is one more member of the pairwise MIS set. Neighbour offsets: a Xorshift32 stream
// seeded per pixel by one draw of the pixel's stream. As in the reference's fused kernel, an
// emissive temporal neighbour is resampled.
// ---------------------------------------------------------------------------------------------
// fused spatiotemporal reuse, phase 1: the bias-correction rays, replaying the pixel's neighbour
// seed, temporal search and neighbour offsets from its PCG stream. Slots per pixel (K + 2): the
// temporal sample seen from the pixel, the pixel's initial sample seen from the temporal
// neighbour, then from each spatial neighbour; -1 without a ray.
__global__ void __launch_bounds__(128, 3) spatiotemporal_rays_kernel(SceneView s, RenderConst rc, RestirConst k,
                                                                     GBuffer gb, GBuffer gb_prev, ReservoirBuf initial,
                                                                     ReservoirBuf prev, int32_t* ray_of, Queue rays)
{
    const int W = rc.width, H = rc.height, n_pix = W * H;
    const bool hc = rc.ggx_height_correlated != 0;
    const int K = k.spatial_neighbors;
    for (int pixel = blockIdx.x * blockDim.x + threadIdx.x; pixel < n_pix; pixel += gridDim.x * blockDim.x)
    {
        int32_t* slots = ray_of + (int64_t)pixel * (K + 2);
        for (int j = 0; j < K + 2; j++) slots[j] = -1;
        const Reservoir init = load_reservoir(initial, pixel);
        const Surface su = load_surface(gb, pixel, k.camera_pos);
        if (su.prim < 0 || !k.has_prev) continue;
        Pcg32 rng = pass_stream(k, pixel, 2);
        uint32_t nseed = rng.next_u32();
        if (nseed == 0u) nseed = 0x9E3779B9u;
        const V3 ndc = mat_x_point(k.prev_view_projection, su.P);
        const float px = (ndc.x + 1.0f) * 0.5f * (float)W - 0.5f;
        const float py = (ndc.y + 1.0f) * 0.5f * (float)H - 0.5f;
        const int tx0 = (int)roundf(px), ty0 = (int)roundf(py);
        const int t_idx = temporal_neighbor(k, gb, gb_prev, W, H, pixel, su, rng);
        const Reservoir tn = t_idx >= 0 ? load_reservoir(prev, t_idx) : empty_reservoir();
        const bool t_ok = t_idx >= 0 && tn.M > 0;
        bsdf::Xorshift32 nrng{nseed};
        int m_sum = t_ok ? tn.M : 0;
        uint32_t cache = 0;
        for (int j = 0; j < K; j++)
        {
            const int idx = spatial_neighbor(j, K, tx0, ty0, W, H, k.spatial_radius, nrng);
            if (idx < 0 || !similar(gb_prev, gb, idx, pixel, su.P, su.ng, k)) continue;
            m_sum += load_reservoir(prev, idx).M;
            cache |= 1u << j;
        }
        const bsdf::Material m = bsdf::load_material(surface_material(s, k, su.mat));
        const bool update_mc = init.M > 0 && init.ucw > 0.0f;
        if (t_ok)
        {
            const bool a = tn.ucw > 0.0f && target_function(s, hc, su, m, tn.point, tn.tri, tn.flags, false) > 0.0f;
            slots[0] = append_sample_ray(rays, a, su.P, tn.point, su.prim, pixel);
            bool b = false;
            Surface nsu = su;  // replaced by the neighbour's surface when it is evaluated
            if (update_mc)
            {
                nsu = load_surface(gb_prev, t_idx, k.prev_camera_pos);
                const bsdf::Material nm = bsdf::load_material(surface_material(s, k, nsu.mat));
                b = target_function(s, hc, nsu, nm, init.point, init.tri, init.flags, false) > 0.0f;
            }
            slots[1] = append_sample_ray(rays, b, nsu.P, init.point, nsu.prim, pixel);
            if (!a) slots[0] = -1;
            if (!b) slots[1] = -1;
        }
        if (!update_mc || m_sum == 0) continue;  // the spatial neighbours are not visited
        nrng = bsdf::Xorshift32{nseed};
        for (int j = 0; j < K; j++)
        {
            bool want = false;
            Surface nsu = su;  // replaced by the neighbour's surface when it is evaluated
            if (!(cache & (1u << j)))
            {
                nrng();
                nrng();
            }
            else
            {
                const int idx = spatial_neighbor(j, K, tx0, ty0, W, H, k.spatial_radius, nrng);
                if (idx >= 0)
                {
                    nsu = load_surface(gb_prev, idx, k.prev_camera_pos);
                    const bsdf::Material nm = bsdf::load_material(surface_material(s, k, nsu.mat));
                    want = target_function(s, hc, nsu, nm, init.point, init.tri, init.flags, false) > 0.0f;
                }
            }
            const int slot = append_sample_ray(rays, want, nsu.P, init.point, nsu.prim, pixel);
            if (want) slots[2 + j] = slot;
        }
    }
}

__global__ void __launch_bounds__(128) spatiotemporal_kernel(SceneView s, RenderConst rc, RestirConst k, GBuffer gb,
                                                             GBuffer gb_prev, ReservoirBuf initial, ReservoirBuf prev,
                                                             ReservoirBuf out, const int32_t* __restrict__ ray_of,
                                                             Queue traced, InitialState st, Queue visq)
{
    const int W = rc.width, H = rc.height, n_pix = W * H;
    const bool hc = rc.ggx_height_correlated != 0;
    const int K = k.spatial_neighbors;
    for (int pixel = blockIdx.x * blockDim.x + threadIdx.x; pixel < n_pix; pixel += gridDim.x * blockDim.x)
    {
        const Reservoir init = load_reservoir(initial, pixel);
        const Surface su = load_surface(gb, pixel, k.camera_pos);
        if (su.prim < 0 || !k.has_prev)
        {
            store_reservoir(out, pixel, init);
            st.meta[pixel] = make_int4(0, 0, kInitialDone, -1);
            continue;
        }
        const int32_t* slots = ray_of + (int64_t)pixel * (K + 2);
        Pcg32 rng = pass_stream(k, pixel, 2);
        uint32_t nseed = rng.next_u32();
        if (nseed == 0u) nseed = 0x9E3779B9u;
        const V3 ndc = mat_x_point(k.prev_view_projection, su.P);
        const float px = (ndc.x + 1.0f) * 0.5f * (float)W - 0.5f;
        const float py = (ndc.y + 1.0f) * 0.5f * (float)H - 0.5f;
        const int tx0 = (int)roundf(px), ty0 = (int)roundf(py);
        const int t_idx = temporal_neighbor(k, gb, gb_prev, W, H, pixel, su, rng);
        const Reservoir tn = t_idx >= 0 ? load_reservoir(prev, t_idx) : empty_reservoir();
        const bool t_ok = t_idx >= 0 && tn.M > 0;
        // valid spatial neighbours and their confidence (count_valid_spatiotemporal_neighbors)
        bsdf::Xorshift32 nrng{nseed};
        int valid = 0, m_sum = 0;
        uint32_t cache = 0;
        for (int j = 0; j < K; j++)
        {
            const int idx = spatial_neighbor(j, K, tx0, ty0, W, H, k.spatial_radius, nrng);
            if (idx < 0) continue;
            if (!similar(gb_prev, gb, idx, pixel, su.P, su.ng, k)) continue;
            m_sum += load_reservoir(prev, idx).M;
            valid++;
            cache |= 1u << j;
        }
        if (t_ok)
        {
            valid++;
            m_sum += tn.M;
        }
        const bsdf::Material m = bsdf::load_material(surface_material(s, k, su.mat));
        const bool vis = k.bias_correction_visibility != 0;
        const bool update_mc = init.M > 0 && init.ucw > 0.0f;
        const float cM = k.confidence_weights ? (float)init.M : 1.0f;
        const float nsum = k.confidence_weights ? (float)m_sum : 1.0f;
        const float div = k.confidence_weights ? 1.0f : (float)valid;
        float mc = 0.0f;
        // One loop over the resampled reservoirs in the reference's order: the temporal neighbour
        // (j = -1), the spatial neighbours (0..K-1), the canonical initial reservoir (K); each
        // target-function evaluation has one call site, keeping the kernel's code small.
        Reservoir o = empty_reservoir();
        nrng = bsdf::Xorshift32{nseed};
        const int first = t_ok ? -1 : (m_sum == 0 ? K : 0);
        for (int j = first; j < K + 1; j++)
        {
            if (j == 0 && m_sum == 0) j = K;  // no spatial neighbour to resample: the canonical one
            if (j >= 0 && j < K && !(cache & (1u << j)))
            {
                nrng();
                nrng();
                continue;
            }
            int idx;
            if (j < 0)
                idx = t_idx;
            else if (j == K)
                idx = pixel;
            else
                idx = spatial_neighbor(j, K, tx0, ty0, W, H, k.spatial_radius, nrng);
            if (idx < 0) continue;
            const Reservoir nb = j < 0 ? tn : (j == K ? init : load_reservoir(prev, idx));
            float t_at_center = 0.0f;
            if (nb.ucw > 0.0f)
                t_at_center = j == K ? nb.p_hat : target_function(s, hc, su, m, nb.point, nb.tri, nb.flags, false);
            if (j < 0 && vis && t_at_center > 0.0f && slots[0] >= 0 && traced.occluded[slots[0]]) t_at_center = 0.0f;
            float mis;
            if (j < K)
            {
                // pairwise MIS weight of a neighbour, accumulating the canonical one (mc)
                const float rM = k.confidence_weights ? (float)nb.M : 1.0f;
                const float denom = nb.p_hat * nsum + t_at_center / div * cM;
                const float mi = denom == 0.0f ? 0.0f : nb.p_hat * rM / denom;
                if (update_mc)
                {
                    const Surface nsu = load_surface(gb_prev, idx, k.prev_camera_pos);
                    const bsdf::Material nm = bsdf::load_material(surface_material(s, k, nsu.mat));
                    float c_at_n = target_function(s, hc, nsu, nm, init.point, init.tri, init.flags, false);
                    const int32_t ray = slots[j < 0 ? 1 : 2 + j];
                    if (vis && c_at_n > 0.0f && ray >= 0 && traced.occluded[ray]) c_at_n = 0.0f;
                    const float nume_mc = init.p_hat / div * cM;
                    const float denom_mc = c_at_n * nsum + init.p_hat / div * cM;
                    const float conf = k.confidence_weights ? (nsum == 0.0f ? 0.0f : rM / nsum) : 1.0f;
                    if (denom_mc != 0.0f) mc += nume_mc / denom_mc / div * conf;
                }
                mis = mi / div;
            }
            else
                mis = mc == 0.0f ? 1.0f : mc;
            if (combine_with(o, nb, mis, t_at_center, 1.0f, rng))
            {
                if (j < 0)
                {
                    if (vis)
                        o.flags |= kRestirFlagUnoccluded;
                    else
                        o.flags &= ~kRestirFlagUnoccluded;
                }
                else if (j == K)
                    o.flags |= nb.flags & kRestirFlagUnoccluded;
                else
                    o.flags &= ~kRestirFlagUnoccluded;
            }
        }
        end_with_normalization(o, 1.0f, 1.0f);
        if (k.m_cap > 0) o.M = min(o.M, k.m_cap);
        // visibility reuse of the result (visibility_kill) through the any-hit queue
        const bool test = k.visibility_reuse && vis && !(o.ucw <= 0.0f && o.w_sum <= 0.0f) &&
                          !(o.flags & kRestirFlagUnoccluded);
        const int slot = append_sample_ray(visq, test, su.P, o.point, su.prim, pixel);
        st.meta[pixel] = make_int4(0, 0, kInitialVisibility, test ? slot : -1);
        store_reservoir(out, pixel, o);
    }
}

inline int grid_for(int64_t n, int threads, int max_blocks)
{
    int64_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > max_blocks) b = max_blocks;
    return (int)b;
}

}  // namespace

cudaError_t launch_restir_gbuffer(const SceneView& s, const Queue& q, const GBuffer& gb, int64_t n_pix, int packed_normals,
                                  int n_sm, cudaStream_t st)
{
    gbuffer_kernel<<<grid_for(n_pix, 256, n_sm * 8), 256, 0, st>>>(s, q, gb, packed_normals);
    return cudaGetLastError();
}

cudaError_t launch_restir_presample(const SceneView& s, const RenderConst& rc, const RestirConst& k, float4* out,
                                    int n_sm, cudaStream_t st)
{
    const int64_t n = (int64_t)k.presample_subsets * k.presample_size;
    if (n <= 0 || s.n_emissive <= 0) return cudaSuccess;
    presample_kernel<<<grid_for(n, 256, n_sm * 8), 256, 0, st>>>(s, rc, k, out);
    return cudaGetLastError();
}

cudaError_t launch_restir_initial(const SceneView& s, const RenderConst& rc, const RestirConst& k, const GBuffer& gb,
                                  const ReservoirBuf& out, const InitialState& st, const Queue& qa, const Queue& qb,
                                  const Queue& vis, int64_t queue_capacity, int n_sm, cudaStream_t stream)
{
    const int64_t n = (int64_t)rc.width * rc.height;
    if (n > queue_capacity) return cudaErrorInvalidValue;
    const int grid = grid_for(n, 128, n_sm * 16);
    cudaError_t e = cudaSuccess;
    for (const Queue* q : {&qa, &qb, &vis})
        if (e == cudaSuccess) e = cudaMemsetAsync(q->count, 0, sizeof(int32_t), stream);
    if (e != cudaSuccess) return e;
    initial_lights_kernel<<<grid, 128, 0, stream>>>(s, rc, k, gb, out, st, qa, vis);
    // BSDF candidate c traces queue c % 2 and appends candidate c + 1's rays to the other one
    for (int c = 0; c < k.bsdf_candidates && e == cudaSuccess; c++)
    {
        const Queue& traced = (c & 1) ? qb : qa;
        const Queue& next = (c & 1) ? qa : qb;
        e = launch_trace_queue(s, traced, false, n, n_sm, stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(next.count, 0, sizeof(int32_t), stream);
        if (e == cudaSuccess)
            initial_bsdf_kernel<<<grid, 128, 0, stream>>>(s, rc, k, gb, out, st, traced, next, vis, c);
    }
    if (e == cudaSuccess && k.visibility_reuse)
    {
        e = launch_trace_queue(s, vis, true, n, n_sm, stream);
        if (e == cudaSuccess)
            visibility_apply_kernel<<<grid_for(n, 256, n_sm * 8), 256, 0, stream>>>(rc, out, st, vis);
    }
    // the queues belong to the bounce's shading: leave them empty
    for (const Queue* q : {&qa, &qb, &vis})
        if (e == cudaSuccess) e = cudaMemsetAsync(q->count, 0, sizeof(int32_t), stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    return e;
}

cudaError_t launch_restir_temporal(const SceneView& s, const RenderConst& rc, const RestirConst& k, const GBuffer& gb,
                                   const GBuffer& gb_prev, const ReservoirBuf& initial, const ReservoirBuf& prev,
                                   const ReservoirBuf& out, int2* ray_of, const Queue& rays, int n_sm, cudaStream_t st)
{
    const int64_t n = (int64_t)rc.width * rc.height;
    const int grid = grid_for(n, 128, n_sm * 16);
    cudaError_t e = cudaSuccess;
    if (k.bias_correction_visibility && k.has_prev)
    {
        e = cudaMemsetAsync(rays.count, 0, sizeof(int32_t), st);
        if (e == cudaSuccess)
        {
            temporal_rays_kernel<<<grid, 128, 0, st>>>(s, rc, k, gb, gb_prev, initial, prev, ray_of, rays);
            e = launch_trace_queue(s, rays, true, 2 * n, n_sm, st);
        }
    }
    if (e == cudaSuccess) temporal_kernel<<<grid, 128, 0, st>>>(s, rc, k, gb, gb_prev, initial, prev, out, ray_of, rays);
    if (e == cudaSuccess) e = cudaGetLastError();
    return e;
}

cudaError_t launch_restir_spatiotemporal(const SceneView& s, const RenderConst& rc, const RestirConst& k,
                                         const GBuffer& gb, const GBuffer& gb_prev, const ReservoirBuf& initial,
                                         const ReservoirBuf& prev, const ReservoirBuf& out, int32_t* ray_of,
                                         const Queue& rays, const InitialState& st, const Queue& vis, int n_sm,
                                         cudaStream_t stream)
{
    const int64_t n = (int64_t)rc.width * rc.height;
    const int grid = grid_for(n, 128, n_sm * 16);
    cudaError_t e = cudaMemsetAsync(rays.count, 0, sizeof(int32_t), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(vis.count, 0, sizeof(int32_t), stream);
    if (e != cudaSuccess) return e;
    if (k.bias_correction_visibility && k.has_prev)
    {
        spatiotemporal_rays_kernel<<<grid, 128, 0, stream>>>(s, rc, k, gb, gb_prev, initial, prev, ray_of, rays);
        e = launch_trace_queue(s, rays, true, n * (k.spatial_neighbors + 2), n_sm, stream);
    }
    if (e == cudaSuccess)
        spatiotemporal_kernel<<<grid, 128, 0, stream>>>(s, rc, k, gb, gb_prev, initial, prev, out, ray_of, rays, st, vis);
    if (e == cudaSuccess) e = launch_trace_queue(s, vis, true, n, n_sm, stream);
    if (e == cudaSuccess) visibility_apply_kernel<<<grid_for(n, 256, n_sm * 8), 256, 0, stream>>>(rc, out, st, vis);
    if (e == cudaSuccess) e = cudaMemsetAsync(vis.count, 0, sizeof(int32_t), stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    return e;
}

cudaError_t launch_restir_spatial(const SceneView& s, const RenderConst& rc, const RestirConst& k, const GBuffer& gb,
                                  const ReservoirBuf& in, const ReservoirBuf& out, int pass, uint32_t neighbor_seed,
                                  int32_t* ray_of, const Queue& rays, const InitialState& st, const Queue& vis,
                                  int n_sm, cudaStream_t stream)
{
    const int64_t n = (int64_t)rc.width * rc.height;
    const int grid = grid_for(n, 128, n_sm * 16);
    cudaError_t e = cudaMemsetAsync(rays.count, 0, sizeof(int32_t), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(vis.count, 0, sizeof(int32_t), stream);
    if (e != cudaSuccess) return e;
    if (k.bias_correction_visibility)
    {
        spatial_rays_kernel<<<grid, 128, 0, stream>>>(s, rc, k, gb, in, pass, neighbor_seed, ray_of, rays);
        e = launch_trace_queue(s, rays, true, n * k.spatial_neighbors, n_sm, stream);
    }
    if (e == cudaSuccess)
        spatial_kernel<<<grid, 128, 0, stream>>>(s, rc, k, gb, in, out, pass, k.spatial_passes - 1, neighbor_seed,
                                                 ray_of, rays, st, vis);
    if (e == cudaSuccess) e = launch_trace_queue(s, vis, true, n, n_sm, stream);
    if (e == cudaSuccess) visibility_apply_kernel<<<grid_for(n, 256, n_sm * 8), 256, 0, stream>>>(rc, out, st, vis);
    if (e == cudaSuccess) e = cudaMemsetAsync(vis.count, 0, sizeof(int32_t), stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    return e;
}

}  // namespace gbpt
