// Wavefront path tracer kernels (sm_103a): camera rays, per-bounce shading with next-event
// estimation + BSDF MIS, resolve, accumulation, and the emissive power alias table build.
//
// One launch traces samples_per_launch samples of every pixel as one wavefront. Each bounce runs
//   extend (closest hit on the active queue) -> shade -> shadow (any hit) + BSDF-light (closest hit)
//   -> resolve,
// with the active paths compacted into the next queue by warp-aggregated appends. Path state is
// SoA indexed by a fixed slot (pixel + W*H*sample), so accumulation is deterministic.
#include <cuda_runtime.h>
#include <stdint.h>

#include "render_common.h"
#include "envmap.h"
#include "guide_device.h"
#include "principled.h"
#include "render_device.h"
#include "render_kernels.h"
#include "restir.h"
#include "trace_core.h"
#include "volume.h"

namespace gbpt {
namespace {

// ---------------------------------------------------------------------------------------------
// camera rays (CameraRays, src/Device/kernels/CameraRays.h:155-176; HIPRTCamera::get_camera_ray,
// src/HostDeviceCommon/HIPRTCamera.h:31-52)
// ---------------------------------------------------------------------------------------------
// Camera ray of a pixel sample and its path's PCG stream (seeded by pixel and sample index)
__device__ __forceinline__ void camera_ray(const RenderConst& rc, int pixel, int sample, V3& origin, V3& dir, Pcg32& rng)
{
    const int x = pixel % rc.width, y = pixel / rc.width;
    const bool ref_rng = rc.rng_mode == GBPT_RNG_REFERENCE;
    rng = ref_rng ? reference_seed((uint32_t)pixel, (uint32_t)sample, rc.random_number_camera)
                  : pcg_seed((uint32_t)pixel, (uint32_t)sample, rc.seed);
    float px = x + 0.5f, py = y + 0.5f;
    if (rc.do_jittering)
    {
        px += rng.next() - 0.5f;
        py += rng.next() - 0.5f;
    }
    // the reference's MegaKernel seeds a new generator from its own pass's random number
    // (Megakernel.h:52-57): the path continues with that one
    if (ref_rng) rng = reference_seed((uint32_t)pixel, (uint32_t)sample, rc.random_number);
    const float xn = px / rc.width * 2.0f - 1.0f;
    const float yn = py / rc.height * 2.0f - 1.0f;
    origin = mat_x_point(rc.inverse_view, v3(0.0f, 0.0f, 0.0f));
    const V3 p_vs = mat_x_point(rc.inverse_projection, v3(xn, yn, -1.0f));
    const V3 p_ws = mat_x_point(rc.inverse_view, p_vs);
    dir = normalize(p_ws - origin);
}

// Pixel of the l-th camera ray of a sample plane: the image is walked in bands of 8 rows and,
// inside a band, column by column (8 pixels of one column, then the next column), so that a warp
// of 32 consecutive rays covers a 4 x 8 pixel tile (coherent traversal). A bijection for any W, H.
__device__ __forceinline__ int64_t band_pixel(int64_t l, int W, int H)
{
    const int64_t band = 8LL * W;
    const int64_t full = H / 8;
    int64_t x, y;
    if (l < full * band)
    {
        const int64_t b = l / band, r = l - b * band;
        x = r >> 3;
        y = b * 8 + (r & 7);
    }
    else
    {
        const int64_t bh = H - full * 8, r = l - full * band;
        x = r / bh;
        y = full * 8 + r % bh;
    }
    return y * W + x;
}

__global__ void __launch_bounds__(256) camera_kernel(RenderConst rc, PathBuffers pb, Queue q, int32_t iteration_base,
                                                     unsigned long long* stats)
{
    const int64_t n_pix = (int64_t)rc.width * rc.height;
    const int64_t n = n_pix * rc.spp;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    {
        const int s = (int)(i / n_pix);
        const int pixel = (int)band_pixel(i - (int64_t)s * n_pix, rc.width, rc.height);
        const int64_t slot = pixel + (int64_t)s * n_pix;  // path slot: accumulation order is by slot
        V3 origin, dir;
        Pcg32 rng;
        camera_ray(rc, pixel, iteration_base + s, origin, dir, rng);
        q.origin_tmin[i] = f4(origin, 0.0f);
        q.dir_tmax[i] = f4(dir, INFINITY);
        q.last_prim[i] = -1;
        q.slot[i] = (int32_t)slot;
        pb.throughput[slot] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
        pb.radiance[slot] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (pb.vol_stack)
        {
            VolumeStack v;
            v.reset();
            v.store(pb.vol_stack, pb.vol_state, slot);
            pb.wavelength[slot] = 0.0f;
        }
        store_rng(pb.rng + slot, rng);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
    {
        *q.count = (int32_t)n;
        atomicAdd(stats + 0, (unsigned long long)n);
    }
}

// ---------------------------------------------------------------------------------------------
// traversal over a device-counted queue (grid-stride, count read from device memory)
// ---------------------------------------------------------------------------------------------
template <bool ANY_HIT>
__global__ void __launch_bounds__(128) trace_queue_kernel(const uint4* __restrict__ nodes,
                                                          const float4* __restrict__ tris, Queue q,
                                                          const BatchJob* __restrict__ jobs,
                                                          const int32_t* __restrict__ job_of_slot)
{
    const int n = *q.count;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const uint4* nd = nodes;
        const float4* tr = tris;
        if (jobs)
        {
            const BatchJob* J = jobs + job_of_slot[q.slot[i]];
            nd = J->s.bvh_nodes;
            tr = J->s.bvh_tris;
        }
        uint32_t cn = 0, ct = 0;
        const float4 h = core::trace_ray<ANY_HIT, false>(nd, tr, q.origin_tmin[i], q.dir_tmax[i], q.last_prim[i], cn, ct);
        if (ANY_HIT)
            q.occluded[i] = __float_as_int(h.w) >= 0 ? 1 : 0;
        else
            q.hits[i] = h;
    }
}

// ---------------------------------------------------------------------------------------------
// envmap direct lighting (sample_environment_map, src/Device/includes/LightSampling/Envmap.h:251-285)
// of every vertex of the shaded queue, run before shade so that its random numbers come first at a
// vertex: an envmap sample and a separate BSDF sample, each with an any-hit ray to 1e35 in envq,
// resolved with the vertex's other samples. Its own kernel keeps the shade kernels' registers as
// they are when no envmap is sampled. The ReSTIR DI bounce keeps it too: its reservoirs hold
// emissive triangles only.
// ---------------------------------------------------------------------------------------------
// The path's wavelength at a principled hit: drawn from the path's generator when the hit material
// is dispersive and the path has none yet (the reference draws it right after the hit,
// Intersect.h:259-267, and at the camera hit in reconstruct_first_hit, RayVolumeState.h:50-58,
// uniformly in [360, 830] nm, Dispersion.h:469-474), negative until its colour filter is applied.
__device__ __forceinline__ float path_wavelength(const PathBuffers& pb, int slot, const gbpt_principled_material& rec,
                                                 Pcg32& rng)
{
    float wl = pb.wavelength[slot];
    if (wl == 0.0f && bsdf::is_dispersive(rec))
    {
        wl = -(rng.next() * 470.0f + 360.0f);
        pb.wavelength[slot] = wl;
    }
    return wl;
}

template <bool PRINCIPLED>
__global__ void __launch_bounds__(128) env_kernel(SceneView s0, RenderConst rc0, PathBuffers pb, Queue in, Queue envq,
                                                  unsigned long long* stats, const BatchJob* __restrict__ jobs)
{
    const int n = *in.count;
    const int n_round = (n + 31) & ~31;  // whole warps for the warp-aggregated appends
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_round; i += gridDim.x * blockDim.x)
    {
        const bool valid = i < n;
        int slot = 0, prim = -1;
        float4 hit = make_float4(0, 0, 0, 0);
        if (valid)
        {
            slot = in.slot[i];
            hit = in.hits[i];
            prim = __float_as_int(hit.w);
            pb.env_entry[slot] = -1;
            pb.envb_entry[slot] = -1;
        }
        const BatchJob* J = (jobs && valid) ? jobs + pb.job[slot] : nullptr;
        const SceneView s = J ? J->s : s0;
        const RenderConst rc = J ? J->rc : rc0;
        EnvDirect ed;
        V3 P = v3(0.0f);
        if (valid && prim >= 0 && env_sampled(s.env))
        {
            Pcg32 rng = load_rng(rc, pb.rng[slot]);
            const V3 d = xyz(in.dir_tmax[i]);
            P = xyz(in.origin_tmin[i]) + hit.x * d;
            V3 a, b, c;
            load_triangle(s, prim, a, b, c);
            const V3 ng_raw = normalize(cross(b - a, c - a));
            V3 ng = ng_raw;
            V3 ns = shading_normal(s, prim, hit.y, hit.z, ng_raw);
            const V3 view = -d;
            fix_backfacing(view, ng, ns);
            const int mat = __ldg(s.material_of + prim);
            const V3 tp = xyz(pb.throughput[slot]);
            if constexpr (!PRINCIPLED)
            {
                const V3 albedo = xyz(s.materials[mat].base_color);
                ed = env_direct(
                    s.env, rng, ns, tp, true, [&](V3 wi, float& pdf) { return lambert_eval(albedo, dot(ns, wi), pdf); },
                    [&](V3& wi, float& pdf) {
                        const float r1 = rng.next(), r2 = rng.next();
                        wi = cosine_sample(ns, r1, r2);
                        return lambert_eval(albedo, dot(ns, wi), pdf);
                    });
            }
            else
            {
                const bsdf::Material m = bsdf::load_material(s.pmats[mat]);
                const bool hc = rc.ggx_height_correlated != 0;
                // the vertex's volume state, as shade derives it (the hit pushed on the path's stack)
                VolumeStack vol;
                vol.load(pb.vol_stack, pb.vol_state, slot);
                volume_hit(vol, s.pmats[mat], mat, hit.x);
                bsdf::Medium md = volume_medium(s, vol);
                md.wavelength = fabsf(path_wavelength(pb, slot, s.pmats[mat], rng));
                ed = env_direct(
                    s.env, rng, ns, tp, can_light_sample(m),
                    [&](V3 wi, float& pdf) {
                        bsdf::Query q;
                        q.view = view;
                        q.ns = ns;
                        q.ng = ng;
                        q.light = wi;
                        return bsdf::eval_outlined(m, md, hc, q, GBPT_LOBE_NONE, pdf);
                    },
                    [&](V3& wi, float& pdf) {
                        bsdf::Xorshift32 xr = bsdf_rng(rng);
                        int lobe;
                        const V3 f = bsdf::sample(m, md, hc, view, ns, ng, xr, wi, lobe, pdf);
                        bsdf_rng_done(rng, xr);
                        return f;
                    });
            }
            store_rng(pb.rng + slot, rng);
        }
        const int ei = warp_append(envq.count, ed.want_l);
        if (ed.want_l)
        {
            envq.origin_tmin[ei] = f4(P, 0.0f);
            envq.dir_tmax[ei] = f4(ed.dir_l, 1.0e35f);
            envq.last_prim[ei] = prim;
            envq.slot[ei] = slot;
            pb.env_entry[slot] = ei;
            pb.pending_env[slot] = f4(ed.c_l, 0.0f);
        }
        const int bi = warp_append(envq.count, ed.want_b);
        if (ed.want_b)
        {
            envq.origin_tmin[bi] = f4(P, 0.0f);
            envq.dir_tmax[bi] = f4(ed.dir_b, 1.0e35f);
            envq.last_prim[bi] = prim;
            envq.slot[bi] = slot;
            pb.envb_entry[slot] = bi;
            pb.pending_envb[slot] = f4(ed.c_b, 0.0f);
        }
        warp_count(stats + 1, ed.want_l);
        warp_count(stats + 1, ed.want_b);
    }
}

// ---------------------------------------------------------------------------------------------
// shade: one path vertex per active path. PRINCIPLED selects the layered principled BSDF with the
// reference's nested-dielectric volume tracking (volume.h: each hit pushes its material, the
// continuation pops what it leaves), else the Lambertian BSDF override.
// ---------------------------------------------------------------------------------------------
template <bool PRINCIPLED>
__global__ void __launch_bounds__(128) shade_kernel(SceneView s0, RenderConst rc0, PathBuffers pb, Queue in, Queue next,
                                                    Queue shadow, Queue bsdfq, int bounce, unsigned long long* stats,
                                                    ReservoirBuf restir, GuideView gv, const BatchJob* __restrict__ jobs)
{
    const int n = *in.count;
    // iterate in whole warps so that the warp-aggregated appends see converged lanes
    const int n_round = (n + 31) & ~31;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_round; i += gridDim.x * blockDim.x)
    {
        const bool valid = i < n;
        int slot = 0;
        int prim = -1;
        float4 hit = make_float4(0, 0, 0, 0);
        if (valid)
        {
            slot = in.slot[i];
            hit = in.hits[i];
            prim = __float_as_int(hit.w);
            pb.shadow_entry[slot] = -1;
            pb.bsdf_entry[slot] = -1;
            if (gv.train_entry)
            {
                gv.train_entry[slot] = -1;
                gv.train_light_entry[slot] = -1;
            }
            if (rc0.direct_ris) pb.ris[slot] = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
        }
        // batched rendering: the scene and settings of the slot's job
        const BatchJob* J = (jobs && valid) ? jobs + pb.job[slot] : nullptr;
        const SceneView s = J ? J->s : s0;
        const RenderConst rc = J ? J->rc : rc0;
        const bool alive = valid && prim >= 0;
        // a ray that left the scene: the world's radiance (path_tracing_miss_gather_envmap)
        if (valid && prim < 0 && s.env.ambient != GBPT_AMBIENT_NONE)
        {
            const V3 c = env_miss(s.env, xyz(in.dir_tmax[i]), bounce, xyz(pb.throughput[slot]));
            if (!is_black(c))
            {
                const float4 r = pb.radiance[slot];
                pb.radiance[slot] = make_float4(r.x + c.x, r.y + c.y, r.z + c.z, 0.0f);
            }
        }

        bool want_shadow = false, want_bsdf = false, want_next = false, want_record = false;
        bool guided_vertex = false, rec_vertex = false;
        V3 rec_tp = v3(0.0f), rec_dir = v3(0.0f), lrec_dir = v3(0.0f);
        float rec_pb = 0.0f, lrec_w = 0.0f, lrec_pb = 0.0f;
        const uint32_t rec_thr = gv.train_entry ? *gv.rec_threshold : 0u;
        float4 sh_o, sh_d, bs_d, nx_d;
        V3 P = v3(0, 0, 0), tp = v3(0, 0, 0);
        V3 light_contrib = v3(0, 0, 0);
        float light_target = 0.0f;  // RIS: target function of the kept light candidate
        float4 bsdf_pending = make_float4(0, 0, 0, 0);
        float guide_pdf_out = 0.0f;  // MIS pdf of this vertex's continuation when it is guided
        VolumeStack vol;  // principled paths: the volume state after this vertex
        Pcg32 rng = load_rng(rc, 0);
        if (alive)
        {
            rng.state = pb.rng[slot];
            const float4 o4 = in.origin_tmin[i], d4 = in.dir_tmax[i];
            const V3 o = xyz(o4), d = xyz(d4);
            P = o + hit.x * d;
            V3 a, b, c;
            load_triangle(s, prim, a, b, c);
            const V3 ng_raw = normalize(cross(b - a, c - a));
            V3 ng = ng_raw;
            V3 ns = shading_normal(s, prim, hit.y, hit.z, ng_raw);
            V3 view = -d;
            fix_backfacing(view, ng, ns);
            if (rc.rng_mode == GBPT_RNG_REFERENCE && bounce == 0) reference_gbuffer_vertex(rc.inverse_view, P, ng, ns, view);
            const int mat = __ldg(s.material_of + prim);
            tp = xyz(pb.throughput[slot]);
            V3 L = v3(0, 0, 0);
            if (bounce == 0)
                L = xyz(s.materials[mat].emission);
            else if (pb.guide_pdf)
            {
                // the previous vertex's guided continuation is next-event estimation's BSDF
                // technique there: the emission it found here, weighted against light sampling
                const float gprev = pb.guide_pdf[slot];
                const V3 Le = xyz(s.materials[mat].emission);
                if (gprev > 0.0f && !is_black(Le))
                {
                    const float lp = emitter_hit_pdf(s, rc, prim, Le, hit.x, d);
                    if (lp > 0.0f) L = tp * Le * balance_heuristic(gprev, lp);
                }
            }

            if constexpr (!PRINCIPLED)
            {
                const V3 albedo = xyz(s.materials[mat].base_color);
                // guided vertex: the continuation is drawn from the learned mixture / the BSDF and
                // doubles as the BSDF technique of next-event estimation (MIS pdf alpha q + (1-alpha) p)
                const float* GL = (gv.lobes && bounce < rc.nb_bounces) ? gv.lobes + guide::kRow * (int64_t)i : nullptr;
                const float alpha = GL ? (gv.prob > 0.0f ? gv.prob : guide::alpha_at(GL)) : 0.0f;
                guided_vertex = GL != nullptr;
                rec_vertex = GL && gv.train_entry && record_hash((uint32_t)slot, (uint32_t)bounce, gv.frame) < rec_thr;
                const bool ris = rc.direct_ris && !GL && s.n_emissive > 0;
                if (ris)
                {
                    // ---- RIS direct lighting (sample_lights_RIS, RIS.h:83-255): light candidates
                    // now; the BSDF candidate's ray is traced and the reservoir finished in resolve ----
                    const RisPick pk = ris_light_candidates(s, rc, rng, P, ns, rc.ris_light, rc.ris_bsdf,
                                                            [&](V3 wi, float& pdf) { return lambert_eval(albedo, dot(ns, wi), pdf); });
                    if (pk.kept)
                    {
                        light_contrib = tp * pk.contrib;
                        light_target = pk.target;
                        want_shadow = true;
                        sh_o = f4(P, 0.0f);
                        sh_d = f4(pk.dir, pk.dist - 1.0e-4f);
                    }
                    pb.ris[slot] = f4(tp, pk.wsum);
                    if (rc.ris_bsdf > 0)
                    {
                        const float r1 = rng.next(), r2 = rng.next();
                        const V3 wi = cosine_sample(ns, r1, r2);
                        float pdf;
                        const V3 f = lambert_eval(albedo, dot(ns, wi), pdf);
                        if (pdf > 0.0f)
                        {
                            want_bsdf = true;
                            bs_d = f4(wi, 1.0e35f - 1.0e-4f);
                            bsdf_pending = f4(f * fabsf(dot(ns, wi)), pdf);
                        }
                        // the reference adds the BSDF candidate to the reservoir here, one draw
                        // (RISReservoir::add_one_candidate, RIS_Reservoir.h:35-42)
                        if (pb.ris_u) pb.ris_u[slot] = rng.next();
                    }
                }
                // ---- next-event estimation: light sample (sample_one_light_MIS, Lights.h:123-185) ----
                else if (s.n_emissive > 0)
                {
                    const LightSample ls = sample_light(s, rc, rng);
                    if (ls.pdf_area > 0.0f)
                    {
                        const V3 to_l = ls.point - P;
                        const float dist = length(to_l);
                        const V3 wi = to_l / dist;
                        float bsdf_pdf;
                        const V3 f = lambert_eval(albedo, dot(ns, wi), bsdf_pdf);
                        if (bsdf_pdf > 0.0f)
                        {
                            const float cos_l = fmaxf(0.0f, dot(ls.normal, -wi));
                            if (cos_l > 1.0e-5f)
                            {
                                const float light_pdf = area_to_solid_angle_pdf(ls.pdf_area, dist, cos_l);
                                const float other =
                                    GL ? alpha * guide::mixture_pdf_at(GL, wi) + (1.0f - alpha) * bsdf_pdf : bsdf_pdf;
                                const float mis = balance_heuristic(light_pdf, other);
                                const float cosine = fabsf(dot(ns, wi));
                                const V3 est = f * cosine * ls.emission * mis / light_pdf;
                                light_contrib = tp * est;
                                lrec_dir = wi;
                                lrec_w = luminance(est);
                                lrec_pb = bsdf_pdf;
                                if (!is_black(light_contrib))
                                {
                                    want_shadow = true;
                                    sh_o = f4(P, 0.0f);
                                    sh_d = f4(wi, dist - 1.0e-4f);
                                }
                            }
                        }
                    }
                }

                // ---- next-event estimation: BSDF sample (Lights.h:187-226) ----
                if (!GL && !ris)
                {
                    const float r1 = rng.next(), r2 = rng.next();
                    const V3 wi = cosine_sample(ns, r1, r2);
                    float pdf;
                    const V3 f = lambert_eval(albedo, dot(ns, wi), pdf);
                    if (pdf > 0.0f && s.n_emissive > 0)
                    {
                        const float cosine = fabsf(dot(ns, wi));
                        const V3 w = tp * (f * cosine / pdf);
                        want_bsdf = true;
                        bs_d = f4(wi, 1.0e35f - 1.0e-4f);
                        bsdf_pending = f4(w, pdf);
                    }
                }

                // ---- continuation (PathTracing.h:81-101, RussianRoulette.h:20-55); with guiding,
                // one-sample MIS of the learned mixture and cosine sampling ----
                if (bounce < rc.nb_bounces)
                {
                    V3 wi, f;
                    float pdf;
                    if (GL)
                    {
                        if (rng.next() < alpha)
                        {
                            const float u0 = rng.next(), u1 = rng.next(), u2 = rng.next();
                            wi = guide::sample_mixture_at(GL, u0, u1, u2);
                        }
                        else
                        {
                            const float r1 = rng.next(), r2 = rng.next();
                            wi = cosine_sample(ns, r1, r2);
                        }
                        float p_bsdf;
                        f = lambert_eval(albedo, dot(ns, wi), p_bsdf);
                        pdf = is_black(f) ? 0.0f : alpha * guide::mixture_pdf_at(GL, wi) + (1.0f - alpha) * p_bsdf;
                        rec_pb = p_bsdf;
                        // next-event estimation's BSDF technique is the continuation itself: the
                        // emission its extension ray finds is weighted at the next vertex
                        if (pdf > 0.0f && s.n_emissive > 0) guide_pdf_out = pdf;
                    }
                    else
                    {
                        const float r1 = rng.next(), r2 = rng.next();
                        wi = cosine_sample(ns, r1, r2);
                        f = lambert_eval(albedo, dot(ns, wi), pdf);
                    }
                    if (pdf > 0.0f)
                    {
                        const V3 atten = f * fabsf(dot(wi, ns)) / pdf;
                        bool survive = true;
                        V3 t2 = tp;
                        if (rc.do_rr && bounce >= rc.rr_min_depth)
                        {
                            const float p = fminf(max_comp(t2), 1.0f);
                            if (rng.next() > p)
                                survive = false;
                            else
                            {
                                float scale = 1.0f / p;
                                if (rc.rr_clamp > 0.0f) scale = fminf(scale, rc.rr_clamp);
                                t2 = t2 * scale;
                            }
                        }
                        if (survive)
                        {
                            want_record = rec_vertex;
                            rec_tp = tp;
                            rec_dir = wi;
                            t2 = t2 * atten;
                            t2 = v3(fmaxf(t2.x, 1.0e-5f), fmaxf(t2.y, 1.0e-5f), fmaxf(t2.z, 1.0e-5f));
                            tp = t2;
                            want_next = true;
                            nx_d = f4(wi, INFINITY);
                        }
                    }
                }
            }
            else
            {
                // under GBPT_RNG_REFERENCE the camera hit shades with the material as the
                // reference's G-buffer re-packed it (CameraRays.h:183, Megakernel.h:72)
                const gbpt_principled_material& rec =
                    (rc.rng_mode == GBPT_RNG_REFERENCE && bounce == 0 && s.pmats_camera) ? s.pmats_camera[mat] : s.pmats[mat];
                const bsdf::Material m = bsdf::load_material(rec);
                const bool hc = rc.ggx_height_correlated != 0;
                // volume state: the hit pushes its material on the path's nested-dielectric stack
                // (at the camera hit the stack holds only the air, as reconstruct_first_hit rebuilds it)
                vol.load(pb.vol_stack, pb.vol_state, slot);
                volume_hit(vol, s.pmats[mat], mat, hit.x);
                bsdf::Medium md = volume_medium(s, vol);
                // the path's wavelength: drawn at its first dispersive hit, before the vertex's other
                // draws (as the reference draws it right after the hit)
                float wavelength = path_wavelength(pb, slot, rec, rng);
                md.wavelength = fabsf(wavelength);
                // guided vertex (materials without delta lobes or transmission): the continuation is
                // drawn from the learned mixture / the BSDF and, outside ReSTIR's bounce 0, doubles as
                // the BSDF technique of next-event estimation (MIS pdf alpha q + (1 - alpha) p)
                const float* GL = (gv.lobes && bounce < rc.nb_bounces && guidable(m))
                                      ? gv.lobes + guide::kRow * (int64_t)i : nullptr;
                const float alpha = GL ? (gv.prob > 0.0f ? gv.prob : guide::alpha_at(GL)) : 0.0f;
                const bool restir_vertex = bounce == 0 && restir.s;
                guided_vertex = GL != nullptr;
                rec_vertex = GL && gv.train_entry && record_hash((uint32_t)slot, (uint32_t)bounce, gv.frame) < rec_thr;

                if (restir_vertex)
                {
                    // ---- direct lighting from the ReSTIR DI reservoir of the pixel
                    // (evaluate_ReSTIR_DI_reservoir, src/Device/includes/ReSTIR/DI/FinalShading.h:13-85) ----
                    const Reservoir R = load_reservoir(restir, slot);
                    if (R.ucw > 0.0f)
                    {
                        V3 wi = R.point - P;
                        const float dist = length(wi);
                        wi = wi / dist;
                        bsdf::Query q;
                        q.view = view;
                        q.ns = ns;
                        q.ng = ng;
                        q.light = wi;
                        float bsdf_pdf;
                        const V3 f = bsdf::eval_outlined(m, md, hc, q, R.flags & kRestirLobeMask, bsdf_pdf);
                        float cosine = dot(ns, wi);
                        if (R.flags & GBPT_LOBE_GLASS_REFRACT) cosine = fabsf(cosine);
                        if (cosine > 0.0f)
                        {
                            V3 la, lb, lc;
                            load_triangle(s, R.tri, la, lb, lc);
                            const V3 nl = normalize(cross(lb - la, lc - la));
                            const float conv = fmaxf(0.0f, dot(nl, -wi)) / (dist * dist);
                            const V3 Le = xyz(s.materials[__ldg(s.material_of + R.tri)].emission);
                            const V3 c = tp * (f * R.ucw * Le * cosine * conv);
                            if ((R.flags & kRestirFlagUnoccluded) || !rc.restir_final_visibility)
                                L = L + c;
                            else if (!is_black(c))
                            {
                                light_contrib = c;
                                want_shadow = true;
                                sh_o = f4(P, 0.0f);
                                sh_d = f4(wi, dist - 1.0e-4f);
                            }
                        }
                    }
                }
                else
                {
                    const bool ris = rc.direct_ris && !GL && s.n_emissive > 0;
                    if (ris)
                    {
                        // ---- RIS direct lighting (sample_lights_RIS, RIS.h:83-255; no light
                        // candidates when the material cannot be light-sampled, RIS.h:91-92) ----
                        const int M = can_light_sample(m) ? rc.ris_light : 0;
                        const RisPick pk = ris_light_candidates(s, rc, rng, P, ns, M, rc.ris_bsdf, [&](V3 wi, float& pdf) {
                            bsdf::Query q;
                            q.view = view;
                            q.ns = ns;
                            q.ng = ng;
                            q.light = wi;
                            return bsdf::eval_outlined(m, md, hc, q, GBPT_LOBE_NONE, pdf);
                        });
                        if (pk.kept)
                        {
                            light_contrib = tp * pk.contrib;
                            light_target = pk.target;
                            want_shadow = true;
                            sh_o = f4(P, 0.0f);
                            sh_d = f4(pk.dir, pk.dist - 1.0e-4f);
                        }
                        pb.ris[slot] = f4(tp, M > 0 ? pk.wsum : -0.5f);
                        if (rc.ris_bsdf > 0)
                        {
                            bsdf::Xorshift32 xr = bsdf_rng(rng);
                            V3 wi;
                            int lobe;
                            float pdf;
                            const V3 f = bsdf::sample(m, md, hc, view, ns, ng, xr, wi, lobe, pdf);
                            bsdf_rng_done(rng, xr);
                            if (pdf > 0.0f)
                            {
                                want_bsdf = true;
                                bs_d = f4(wi, 1.0e35f - 1.0e-4f);
                                bsdf_pending = f4(f * fabsf(dot(ns, wi)), pdf);
                            }
                            if (pb.ris_u) pb.ris_u[slot] = rng.next();
                        }
                    }
                    // ---- next-event estimation: light sample ----
                    if (!ris && s.n_emissive > 0 && can_light_sample(m))
                    {
                        const LightSample ls = sample_light(s, rc, rng);
                        if (ls.pdf_area > 0.0f)
                        {
                            const V3 to_l = ls.point - P;
                            const float dist = length(to_l);
                            const V3 wi = to_l / dist;
                            bsdf::Query q;
                            q.view = view;
                            q.ns = ns;
                            q.ng = ng;
                            q.light = wi;
                            float bsdf_pdf;
                            const V3 f = bsdf::eval_outlined(m, md, hc, q, GBPT_LOBE_NONE, bsdf_pdf);
                            if (bsdf_pdf > 0.0f)
                            {
                                const float cos_l = fmaxf(0.0f, dot(ls.normal, -wi));
                                if (cos_l > 1.0e-5f)
                                {
                                    const float light_pdf = area_to_solid_angle_pdf(ls.pdf_area, dist, cos_l);
                                    const float other =
                                        GL ? alpha * guide::mixture_pdf_at(GL, wi) + (1.0f - alpha) * bsdf_pdf : bsdf_pdf;
                                    const float mis = balance_heuristic(light_pdf, other);
                                    const float cosine = fabsf(dot(ns, wi));
                                    const V3 est = f * cosine * ls.emission * mis / light_pdf;
                                    light_contrib = tp * est;
                                    lrec_dir = wi;
                                    lrec_w = luminance(est);
                                    lrec_pb = bsdf_pdf;
                                    if (!is_black(light_contrib))
                                    {
                                        want_shadow = true;
                                        sh_o = f4(P, 0.0f);
                                        sh_d = f4(wi, dist - 1.0e-4f);
                                    }
                                }
                            }
                        }
                    }

                    // ---- next-event estimation: BSDF sample ----
                    if (!GL && !ris)
                    {
                        bsdf::Xorshift32 xr = bsdf_rng(rng);
                        V3 wi;
                        int lobe;
                        float pdf;
                        const V3 f = bsdf::sample(m, md, hc, view, ns, ng, xr, wi, lobe, pdf);
                        bsdf_rng_done(rng, xr);
                        if (pdf > 0.0f && s.n_emissive > 0)
                        {
                            const V3 w = tp * (f * fabsf(dot(ns, wi)) / pdf);
                            want_bsdf = true;
                            bs_d = f4(wi, 1.0e35f - 1.0e-4f);
                            bsdf_pending = f4(w, pdf);
                        }
                    }
                }

                // ---- continuation; with guiding (materials without delta lobes or transmission),
                // one-sample MIS of the learned mixture and BSDF sampling ----
                if (bounce < rc.nb_bounces)
                {
                    V3 wi, f;
                    int lobe = GBPT_LOBE_NONE;
                    float pdf;
                    if (GL)
                    {
                        float p_bsdf;
                        if (rng.next() < alpha)
                        {
                            const float u0 = rng.next(), u1 = rng.next(), u2 = rng.next();
                            wi = guide::sample_mixture_at(GL, u0, u1, u2);
                            bsdf::Query q;
                            q.view = view;
                            q.ns = ns;
                            q.ng = ng;
                            q.light = wi;
                            // directions below the geometric surface carry no BSDF value, as in BSDF sampling
                            f = dot(wi, ng) < 0.0f ? v3(0.0f) : bsdf::eval_outlined(m, md, hc, q, GBPT_LOBE_NONE, p_bsdf);
                            if (dot(wi, ng) < 0.0f) p_bsdf = 0.0f;
                        }
                        else
                        {
                            bsdf::Xorshift32 xr = bsdf_rng(rng);
                            f = bsdf::sample(m, md, hc, view, ns, ng, xr, wi, lobe, p_bsdf);
                            bsdf_rng_done(rng, xr);
                        }
                        pdf = is_black(f) ? 0.0f : alpha * guide::mixture_pdf_at(GL, wi) + (1.0f - alpha) * p_bsdf;
                        rec_pb = p_bsdf;
                        // next-event estimation's BSDF technique is the continuation itself (not on
                        // the ReSTIR DI bounce, whose reservoirs replace it)
                        if (pdf > 0.0f && s.n_emissive > 0 && !restir_vertex) guide_pdf_out = pdf;
                    }
                    else
                    {
                        bsdf::Xorshift32 xr = bsdf_rng(rng);
                        f = bsdf::sample(m, md, hc, view, ns, ng, xr, wi, lobe, pdf);
                        bsdf_rng_done(rng, xr);
                    }
                    // the continuation leaves the vertex's volume entries behind (a guided direction
                    // reflects off an opaque material: lobe NONE pops like a reflection lobe)
                    volume_after_sample(s, vol, m, view, ns, ng, wi, lobe);
                    if (pdf > 0.0f)
                    {
                        const V3 atten = f * fabsf(dot(wi, ns)) / pdf;
                        bool survive = true;
                        V3 t2 = tp;
                        if (rc.do_rr && bounce >= rc.rr_min_depth)
                        {
                            const float p = fminf(max_comp(t2), 1.0f);
                            if (rng.next() > p)
                                survive = false;
                            else
                            {
                                float scale = 1.0f / p;
                                if (rc.rr_clamp > 0.0f) scale = fminf(scale, rc.rr_clamp);
                                t2 = t2 * scale;
                            }
                        }
                        if (survive)
                        {
                            want_record = rec_vertex;
                            rec_tp = tp;
                            rec_dir = wi;
                            // a dispersive vertex filters the path by its wavelength's colour, once
                            // (get_dispersion_ray_color, Dispersion.h:512-525; PathTracing.h:51-52)
                            if (wavelength < 0.0f && rec.dispersion_scale > 0.0f)
                            {
                                t2 = t2 * bsdf::wavelength_rgb(-wavelength);
                                wavelength = -wavelength;
                                pb.wavelength[slot] = wavelength;
                            }
                            t2 = t2 * atten;
                            t2 = v3(fmaxf(t2.x, 1.0e-5f), fmaxf(t2.y, 1.0e-5f), fmaxf(t2.z, 1.0e-5f));
                            tp = t2;
                            want_next = true;
                            nx_d = f4(wi, INFINITY);
                        }
                    }
                }
            }
            if (!is_black(L))
            {
                float4 r = pb.radiance[slot];
                pb.radiance[slot] = make_float4(r.x + L.x, r.y + L.y, r.z + L.z, 0.0f);
            }
            store_rng(pb.rng + slot, rng);
        }

        const int si = warp_append(shadow.count, want_shadow);
        if (want_shadow)
        {
            shadow.origin_tmin[si] = sh_o;
            shadow.dir_tmax[si] = sh_d;
            shadow.last_prim[si] = prim;
            shadow.slot[si] = slot;
            pb.shadow_entry[slot] = si;
            pb.pending_light[slot] = f4(light_contrib, light_target);
        }
        const int bi = warp_append(bsdfq.count, want_bsdf);
        if (want_bsdf)
        {
            bsdfq.origin_tmin[bi] = f4(P, 0.0f);
            bsdfq.dir_tmax[bi] = bs_d;
            bsdfq.last_prim[bi] = prim;
            bsdfq.slot[bi] = slot;
            pb.bsdf_entry[slot] = bi;
            pb.pending_bsdf[slot] = bsdf_pending;
        }
        const int ni = warp_append(next.count, want_next);
        if (want_next)
        {
            next.origin_tmin[ni] = f4(P, 0.0f);
            next.dir_tmax[ni] = nx_d;
            next.last_prim[ni] = prim;
            next.slot[ni] = slot;
            pb.throughput[slot] = f4(tp, 0.0f);
            if (PRINCIPLED) vol.store(pb.vol_stack, pb.vol_state, slot);
            if (pb.guide_pdf) pb.guide_pdf[slot] = guide_pdf_out;
        }
        if (gv.train_entry)  // uniform: every lane of the warp takes the branch
        {
            const int ri = warp_append(gv.rec_count, want_record);
            if (want_record && ri < gv.rec_cap)
            {
                for (int a = 0; a < 3; a++)
                {
                    gv.rec_pos[3 * ri + a] = gv.in_pos[3 * (int64_t)i + a];
                    gv.rec_nrm[3 * ri + a] = gv.in_nrm[3 * (int64_t)i + a];
                    gv.rec_view[3 * ri + a] = gv.in_view[3 * (int64_t)i + a];
                }
                gv.rec_dir[3 * ri] = rec_dir.x;
                gv.rec_dir[3 * ri + 1] = rec_dir.y;
                gv.rec_dir[3 * ri + 2] = rec_dir.z;
                gv.rec_tp[ri] = f4(rec_tp, 0.0f);
                gv.rec_pbsdf[ri] = rec_pb;
                gv.rec_slot[ri] = slot;
                gv.train_entry[slot] = ri;
            }
            const bool want_lrec = rec_vertex && want_shadow && lrec_w > 0.0f;
            const int li = warp_append(gv.rec_count, want_lrec);
            if (want_lrec && li < gv.rec_cap)
            {
                for (int a = 0; a < 3; a++)
                {
                    gv.rec_pos[3 * li + a] = gv.in_pos[3 * (int64_t)i + a];
                    gv.rec_nrm[3 * li + a] = gv.in_nrm[3 * (int64_t)i + a];
                    gv.rec_view[3 * li + a] = gv.in_view[3 * (int64_t)i + a];
                }
                gv.rec_dir[3 * li] = lrec_dir.x;
                gv.rec_dir[3 * li + 1] = lrec_dir.y;
                gv.rec_dir[3 * li + 2] = lrec_dir.z;
                gv.rec_weight[li] = gv.weight_clamp > 0.0f ? fminf(lrec_w, gv.weight_clamp) : lrec_w;
                gv.rec_pbsdf[li] = lrec_pb;
                gv.rec_slot[li] = -1;
                gv.train_light_entry[slot] = li;
            }
            const unsigned m = __ballot_sync(0xffffffffu, guided_vertex);
            if ((threadIdx.x & 31) == 0 && m) atomicAdd(gv.rec_candidates, __popc(m));
        }
        warp_count(stats + 1, want_shadow);
        warp_count(stats + 2, want_bsdf);
        warp_count(stats + 0, want_next);
    }
}

// ---------------------------------------------------------------------------------------------
// resolve: add the light-sample and BSDF-sample contributions of this bounce, in a fixed order
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) resolve_kernel(SceneView s0, RenderConst rc0, PathBuffers pb, Queue in, Queue shadow,
                                                      Queue bsdfq, Queue envq, GuideView gv,
                                                      const BatchJob* __restrict__ jobs)
{
    const int n = *in.count;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const int slot = in.slot[i];
        const BatchJob* J = jobs ? jobs + pb.job[slot] : nullptr;
        const SceneView s = J ? J->s : s0;
        const RenderConst rc = J ? J->rc : rc0;
        const int se = pb.shadow_entry[slot];
        const int be = pb.bsdf_entry[slot];
        // envmap direct lighting of this vertex: the envmap sample, then the BSDF sample
        const int ee = pb.env_entry ? pb.env_entry[slot] : -1;
        const int eb = pb.env_entry ? pb.envb_entry[slot] : -1;
        const bool env_l = ee >= 0 && !envq.occluded[ee];
        const bool env_b = eb >= 0 && !envq.occluded[eb];
        // a guiding record of this vertex snapshots the radiance after its direct lighting; its
        // light-sample record loses its weight when the shadow ray is occluded
        const int te = gv.train_entry ? gv.train_entry[slot] : -1;
        const int tle = gv.train_entry ? gv.train_light_entry[slot] : -1;
        if (tle >= 0 && (se < 0 || shadow.occluded[se])) gv.rec_weight[tle] = 0.0f;
        if (rc.direct_ris)
        {
            const float4 ra = pb.ris[slot];
            if (ra.w > -0.75f)
            {
                // ---- RIS direct lighting, continued: the BSDF candidate (RIS.h:200-249) is added
                // to the light candidates' reservoir, then the kept sample is shaded
                // (evaluate_reservoir_sample, RIS.h:19-80; UCW = w_sum / p^) ----
                const int M = ra.w >= 0.0f ? rc.ris_light : 0, N = rc.ris_bsdf;
                float w_b = 0.0f, t_b = 0.0f;
                V3 c_b = v3(0.0f);
                if (be >= 0)
                {
                    const float4 h = bsdfq.hits[be];
                    const int lprim = __float_as_int(h.w);
                    if (lprim >= 0)
                    {
                        const V3 Le = xyz(s.materials[__ldg(s.material_of + lprim)].emission);
                        V3 a, b, c;
                        load_triangle(s, lprim, a, b, c);
                        const V3 nrm = cross(b - a, c - a);
                        const float len = length(nrm);
                        const V3 wi = xyz(bsdfq.dir_tmax[be]);
                        const float cos_l = fmaxf(0.0f, dot(nrm / len, -wi));
                        if (!is_black(Le) && cos_l > 0.0f)
                        {
                            const float area = 0.5f * len;
                            float pdf_area = 1.0f / area;
                            if (rc.light_sampling == GBPT_LIGHT_POWER)
                                pdf_area *= (luminance(Le) * area) / s.power_sum;
                            else
                                pdf_area /= (float)s.n_emissive;
                            const float light_pdf = area_to_solid_angle_pdf(pdf_area, h.x, cos_l);
                            const float4 pend = pb.pending_bsdf[slot];  // f |cos|, BSDF pdf
                            c_b = xyz(pend) * Le;
                            t_b = luminance(c_b);
                            w_b = balance_counts(pend.w, (float)N, light_pdf, (float)M) * t_b / pend.w;
                        }
                    }
                }
                const float4 pl = pb.pending_light[slot];  // T f Le cos of the kept light, its p^
                const bool light_ok = se >= 0 && !shadow.occluded[se];
                float wsum = fmaxf(ra.w, 0.0f);
                bool take_bsdf = false;
                if (N > 0)
                {
                    wsum += w_b;
                    if (pb.ris_u)
                        take_bsdf = pb.ris_u[slot] < w_b / wsum;
                    else
                    {
                        Pcg32 prng = load_rng(rc, pb.rng[slot]);
                        take_bsdf = prng.next() < w_b / wsum;
                        store_rng(pb.rng + slot, prng);
                    }
                }
                V3 add = v3(0.0f);
                if (take_bsdf)
                    add = xyz(ra) * c_b * (wsum / t_b);
                else if (light_ok && pl.w > 0.0f)
                    add = xyz(pl) * (wsum / pl.w);
                V3 rad = xyz(pb.radiance[slot]);
                if (env_l) rad = rad + xyz(pb.pending_env[slot]);
                if (env_b) rad = rad + xyz(pb.pending_envb[slot]);
                rad = rad + add;
                pb.radiance[slot] = f4(rad, 0.0f);
                continue;
            }
        }
        if (se < 0 && be < 0 && !env_l && !env_b)
        {
            if (te >= 0) gv.rec_snap[te] = pb.radiance[slot];
            continue;
        }
        // added one by one: the light sample, the envmap's two samples, the BSDF sample
        V3 rad = xyz(pb.radiance[slot]);
        if (se >= 0 && !shadow.occluded[se]) rad = rad + xyz(pb.pending_light[slot]);
        if (env_l) rad = rad + xyz(pb.pending_env[slot]);
        if (env_b) rad = rad + xyz(pb.pending_envb[slot]);
        // a guiding record's snapshot: after the vertex's light and envmap samples, before the
        // BSDF-technique emission (which arrives along the recorded direction and belongs to its
        // training target)
        if (te >= 0) gv.rec_snap[te] = f4(rad, 0.0f);
        if (be >= 0)
        {
            const float4 h = bsdfq.hits[be];
            const int lprim = __float_as_int(h.w);
            if (lprim >= 0)
            {
                const V3 Le = xyz(s.materials[__ldg(s.material_of + lprim)].emission);
                if (!is_black(Le))
                {
                    V3 a, b, c;
                    load_triangle(s, lprim, a, b, c);
                    const V3 nrm = cross(b - a, c - a);
                    const float len = length(nrm);
                    const V3 ln = nrm / len;
                    const V3 wi = xyz(bsdfq.dir_tmax[be]);
                    const float cos_l = fmaxf(0.0f, dot(ln, -wi));
                    if (cos_l > 0.0f)
                    {
                        const float area = 0.5f * len;
                        float pdf_area = 1.0f / area;
                        if (rc.light_sampling == GBPT_LIGHT_POWER)
                            pdf_area *= (luminance(Le) * area) / s.power_sum;
                        else
                            pdf_area /= (float)s.n_emissive;
                        const float light_pdf = area_to_solid_angle_pdf(pdf_area, h.x, cos_l);
                        const float4 pend = pb.pending_bsdf[slot];
                        const float mis = balance_heuristic(pend.w, light_pdf);
                        rad = rad + xyz(pend) * Le * mis;
                    }
                }
            }
        }
        pb.radiance[slot] = f4(rad, 0.0f);
    }
}

// ---------------------------------------------------------------------------------------------
// guiding: network inputs per queue entry (shading position, normal facing the viewer, view
// direction) and, after the launch, the weights of the training records
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(128) guide_inputs_kernel(SceneView s, Queue in, GuideView gv)
{
    const int n = *in.count;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const float4 hit = in.hits[i];
        const int prim = __float_as_int(hit.w);
        V3 P = v3(0.0f), ng = v3(0.0f), view = v3(0.0f);
        if (prim >= 0)
        {
            const V3 d = xyz(in.dir_tmax[i]);
            P = xyz(in.origin_tmin[i]) + hit.x * d;
            V3 a, b, c;
            load_triangle(s, prim, a, b, c);
            ng = normalize(cross(b - a, c - a));
            view = -d;
            if (dot(view, ng) < 0.0f) ng = -ng;
        }
        const int64_t o = 3 * (int64_t)i;
        gv.in_pos[o] = P.x;
        gv.in_pos[o + 1] = P.y;
        gv.in_pos[o + 2] = P.z;
        gv.in_nrm[o] = ng.x;
        gv.in_nrm[o + 1] = ng.y;
        gv.in_nrm[o + 2] = ng.z;
        gv.in_view[o] = view.x;
        gv.in_view[o + 1] = view.y;
        gv.in_view[o + 2] = view.z;
    }
}

// Recording fraction for the next launch: up to two records per candidate vertex, so that about
// rec_cap records are made; the candidate counter restarts
__global__ void guide_threshold_kernel(GuideView gv)
{
    const double cand = (double)max(*gv.rec_candidates, 1);
    const double frac = (double)gv.rec_cap / (2.0 * cand);
    *gv.rec_threshold = frac >= 1.0 ? 0xFFFFFFFFu : (uint32_t)(frac * 4294967296.0);
    *gv.rec_candidates = 0;
}

__global__ void guide_weights_kernel(PathBuffers pb, GuideView gv)
{
    const int n = min(*gv.rec_count, gv.rec_cap);
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
    {
        const int sl = gv.rec_slot[r];
        if (sl < 0) continue;  // light-sample record: weight already final
        const V3 R = xyz(pb.radiance[sl]);
        const V3 S = xyz(gv.rec_snap[r]);
        const V3 T = xyz(gv.rec_tp[r]);
        const V3 ratio = v3(T.x > 0.0f ? fmaxf(R.x - S.x, 0.0f) / T.x : 0.0f, T.y > 0.0f ? fmaxf(R.y - S.y, 0.0f) / T.y : 0.0f,
                            T.z > 0.0f ? fmaxf(R.z - S.z, 0.0f) / T.z : 0.0f);
        float w = luminance(ratio);
        if (!(w >= 0.0f)) w = 0.0f;  // NaN
        if (gv.weight_clamp > 0.0f) w = fminf(w, gv.weight_clamp);
        gv.rec_weight[r] = w;
    }
}

// ---------------------------------------------------------------------------------------------
// accumulate: per pixel, samples of this launch in sample order (FP32 and FP64 sums)
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) accumulate_kernel(RenderConst rc, PathBuffers pb, float* __restrict__ acc32,
                                                         double* __restrict__ acc64)
{
    const int n_pix = rc.width * rc.height;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n_pix; p += gridDim.x * blockDim.x)
    {
        float r = acc32[3 * p], g = acc32[3 * p + 1], b = acc32[3 * p + 2];
        double R = acc64[3 * p], G = acc64[3 * p + 1], B = acc64[3 * p + 2];
        for (int k = 0; k < rc.spp; k++)
        {
            const float4 v = pb.radiance[(int64_t)k * n_pix + p];
            r += v.x;
            g += v.y;
            b += v.z;
            R += v.x;
            G += v.y;
            B += v.z;
        }
        acc32[3 * p] = r;
        acc32[3 * p + 1] = g;
        acc32[3 * p + 2] = b;
        acc64[3 * p] = R;
        acc64[3 * p + 1] = G;
        acc64[3 * p + 2] = B;
    }
}

// ---------------------------------------------------------------------------------------------
// batched rendering: all jobs' paths share every wavefront launch; blockIdx.y selects the job in
// the per-job kernels. The iteration index lives in device memory so that a captured CUDA graph
// of one iteration replays unchanged.
// ---------------------------------------------------------------------------------------------
// samples per pixel job J renders in iteration it (0 once the job is done)
__device__ __forceinline__ int batch_samples(const BatchJob& J, int it)
{
    if (it >= J.iterations) return 0;
    const int left = J.spp_total - it * J.rc.spp;
    return left < J.rc.spp ? left : J.rc.spp;
}

__global__ void __launch_bounds__(256) camera_batch_kernel(const BatchJob* __restrict__ jobs, PathBuffers pb, Queue q,
                                                           const int32_t* __restrict__ iteration,
                                                           unsigned long long* stats)
{
    const int job = blockIdx.y;
    const BatchJob& J = jobs[job];
    const RenderConst rc = J.rc;
    const int it = *iteration;
    const int64_t n_pix = (int64_t)rc.width * rc.height;
    const int64_t n = n_pix * batch_samples(J, it);
    const int64_t n_round = (n + 31) & ~(int64_t)31;  // whole warps for the aggregated appends
    for (int64_t local = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; local < n_round;
         local += (int64_t)gridDim.x * blockDim.x)
    {
        const bool valid = local < n;
        V3 origin = v3(0.0f), dir = v3(0.0f);
        Pcg32 rng;
        rng.state = 0;
        rng.inc = 0;
        int64_t pslot = 0;
        if (valid)
        {
            const int s = (int)(local / n_pix);
            const int pixel = (int)band_pixel(local - (int64_t)s * n_pix, rc.width, rc.height);
            pslot = pixel + (int64_t)s * n_pix;
            camera_ray(rc, pixel, it * rc.spp + s, origin, dir, rng);
        }
        const int qi = warp_append(q.count, valid);
        if (valid)
        {
            const int64_t slot = J.slot_base + pslot;
            q.origin_tmin[qi] = f4(origin, 0.0f);
            q.dir_tmax[qi] = f4(dir, INFINITY);
            q.last_prim[qi] = -1;
            q.slot[qi] = (int32_t)slot;
            pb.throughput[slot] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
            pb.radiance[slot] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (pb.vol_stack)
        {
            VolumeStack v;
            v.reset();
            v.store(pb.vol_stack, pb.vol_state, slot);
            pb.wavelength[slot] = 0.0f;
        }
            pb.job[slot] = job;
            store_rng(pb.rng + slot, rng);
        }
        warp_count(stats + 0, valid);
    }
}

// per job: its pixels' samples of this iteration, in sample order, into its accumulators
__global__ void __launch_bounds__(256) accumulate_batch_kernel(const BatchJob* __restrict__ jobs, PathBuffers pb,
                                                               const int32_t* __restrict__ iteration,
                                                               float* __restrict__ acc32, double* __restrict__ acc64)
{
    const BatchJob& J = jobs[blockIdx.y];
    const int samples = batch_samples(J, *iteration);
    const int64_t n_pix = (int64_t)J.rc.width * J.rc.height;
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n_pix && samples > 0;
         p += (int64_t)gridDim.x * blockDim.x)
    {
        const int64_t a = 3 * (J.pixel_base + p);
        float r = acc32[a], g = acc32[a + 1], b = acc32[a + 2];
        double R = acc64[a], G = acc64[a + 1], B = acc64[a + 2];
        for (int k = 0; k < samples; k++)
        {
            const float4 v = pb.radiance[J.slot_base + (int64_t)k * n_pix + p];
            r += v.x;
            g += v.y;
            b += v.z;
            R += v.x;
            G += v.y;
            B += v.z;
        }
        acc32[a] = r;
        acc32[a + 1] = g;
        acc32[a + 2] = b;
        acc64[a] = R;
        acc64[a + 1] = G;
        acc64[a + 2] = B;
    }
}

// end of an iteration: stamps the global timer for the jobs that just finished, then advances
// the iteration index (one block)
__global__ void batch_step_kernel(const BatchJob* __restrict__ jobs, int n_jobs, int32_t* iteration,
                                  unsigned long long* done_ns)
{
    const int it = *iteration;
    for (int j = threadIdx.x; j < n_jobs; j += blockDim.x)
        if (it + 1 == jobs[j].iterations)
        {
            unsigned long long t;
            asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
            done_ns[j] = t;
        }
    __syncthreads();
    if (threadIdx.x == 0) *iteration = it + 1;
}

__global__ void stamp_kernel(unsigned long long* out)
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    *out = t;
}

__global__ void reset_counts_kernel(int32_t* a, int32_t* b, int32_t* c)
{
    if (a) *a = 0;
    if (b) *b = 0;
    if (c) *c = 0;
}

// ---------------------------------------------------------------------------------------------
// emissive power alias table
// ---------------------------------------------------------------------------------------------
// Power of one emissive triangle = luminance(emission) * area, with every float operation rounded
// separately in the reference's order (GPURenderer::compute_emissives_power_alias_table,
// src/Renderer/GPURenderer.cpp:256-275, computed on the host without FMA contraction), so the
// power list is bit-identical to the reference's.
__global__ void light_power_kernel(SceneView s, float* __restrict__ power)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < s.n_emissive; e += gridDim.x * blockDim.x)
    {
        const int t = s.emissive[e];
        V3 a, b, c;
        load_triangle(s, t, a, b, c);
        const V3 ab = v3(__fsub_rn(b.x, a.x), __fsub_rn(b.y, a.y), __fsub_rn(b.z, a.z));
        const V3 ac = v3(__fsub_rn(c.x, a.x), __fsub_rn(c.y, a.y), __fsub_rn(c.z, a.z));
        const V3 n = v3(__fsub_rn(__fmul_rn(ab.y, ac.z), __fmul_rn(ab.z, ac.y)),
                        __fsub_rn(__fmul_rn(ab.z, ac.x), __fmul_rn(ab.x, ac.z)),
                        __fsub_rn(__fmul_rn(ab.x, ac.y), __fmul_rn(ab.y, ac.x)));
        const float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(n.x, n.x), __fmul_rn(n.y, n.y)), __fmul_rn(n.z, n.z)));
        const float area = __fmul_rn(0.5f, len);
        const V3 Le = xyz(s.materials[s.material_of[t]].emission);
        const float lum = __fadd_rn(__fadd_rn(__fmul_rn(0.3086f, Le.x), __fmul_rn(0.6094f, Le.y)), __fmul_rn(0.0820f, Le.z));
        power[e] = __fmul_rn(lum, area);
    }
}

// Deterministic FP64 sum: fixed-shape tree per block, then one block over the partials.
constexpr int kSumThreads = 256;
__global__ void __launch_bounds__(kSumThreads) sum_f64_kernel(const float* __restrict__ x, int n,
                                                              double* __restrict__ partial)
{
    __shared__ double sh[kSumThreads];
    double acc = 0.0;
    const int chunk = (n + gridDim.x - 1) / gridDim.x;
    const int lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
    for (int i = lo + threadIdx.x; i < hi; i += kSumThreads) acc += (double)x[i];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = kSumThreads / 2; w > 0; w >>= 1)
    {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(kSumThreads) sum_partials_kernel(const double* __restrict__ partial, int n,
                                                                   double* __restrict__ out)
{
    __shared__ double sh[kSumThreads];
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += kSumThreads) acc += partial[i];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = kSumThreads / 2; w > 0; w >>= 1)
    {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

__global__ void normalize_f64_kernel(const float* __restrict__ power, int n, const double* __restrict__ sum,
                                     double* __restrict__ q)
{
    const double s = *sum;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        q[i] = (double)power[i] / s * (double)n;
}

// Vose's alias method with the reference's queue discipline (src/Utils/Utils.cpp:63-131):
// smalls/larges are FIFO queues filled in index order; a large that falls to <= 1 moves to the
// smalls; an entry never paired keeps probability 1 and alias 0 (the reference's value-initialised
// alias vector). Runs on one thread (O(n)); the queues are ring buffers of n entries each.
__global__ void alias_vose_kernel(double* __restrict__ q, int n, float* __restrict__ prob, int32_t* __restrict__ alias,
                                  int32_t* __restrict__ smalls, int32_t* __restrict__ larges)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    int s_head = 0, s_tail = 0, l_head = 0, l_tail = 0;  // tail - head = size; indices mod n
    for (int i = 0; i < n; i++)
    {
        alias[i] = 0;
        if (q[i] < 1.0)
            smalls[(s_tail++) % n] = i;
        else
            larges[(l_tail++) % n] = i;
    }
    while (s_tail > s_head && l_tail > l_head)
    {
        const int si = smalls[(s_head++) % n];
        const int li = larges[(l_head++) % n];
        prob[si] = (float)q[si];
        alias[si] = li;
        q[li] = (q[li] + q[si]) - 1.0;
        if (q[li] > 1.0)
            larges[(l_tail++) % n] = li;
        else
            smalls[(s_tail++) % n] = li;
    }
    while (l_tail > l_head) prob[larges[(l_head++) % n]] = 1.0f;
    while (s_tail > s_head) prob[smalls[(s_head++) % n]] = 1.0f;
}

inline int grid_for(int64_t n, int threads, int max_blocks)
{
    int64_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > max_blocks) b = max_blocks;
    return (int)b;
}

}  // namespace

cudaError_t launch_light_table(const SceneView& s, float* power, double* partial, int n_partial, double* sum64,
                               double* q, float* prob, int32_t* alias, int32_t* smalls, int32_t* larges,
                               cudaStream_t st)
{
    const int n = s.n_emissive;
    if (n <= 0) return cudaSuccess;
    light_power_kernel<<<grid_for(n, 256, 4096), 256, 0, st>>>(s, power);
    sum_f64_kernel<<<n_partial, kSumThreads, 0, st>>>(power, n, partial);
    sum_partials_kernel<<<1, kSumThreads, 0, st>>>(partial, n_partial, sum64);
    normalize_f64_kernel<<<grid_for(n, 256, 4096), 256, 0, st>>>(power, n, sum64, q);
    alias_vose_kernel<<<1, 1, 0, st>>>(q, n, prob, alias, smalls, larges);
    return cudaGetLastError();
}

cudaError_t launch_alias_table(const float* power, int n, double* partial, int n_partial, double* sum64, double* q,
                               float* prob, int32_t* alias, int32_t* smalls, int32_t* larges, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    sum_f64_kernel<<<n_partial, kSumThreads, 0, st>>>(power, n, partial);
    sum_partials_kernel<<<1, kSumThreads, 0, st>>>(partial, n_partial, sum64);
    normalize_f64_kernel<<<grid_for(n, 256, 4096), 256, 0, st>>>(power, n, sum64, q);
    alias_vose_kernel<<<1, 1, 0, st>>>(q, n, prob, alias, smalls, larges);
    return cudaGetLastError();
}

cudaError_t launch_camera(const RenderConst& rc, const PathBuffers& pb, const Queue& q, int32_t iteration_base,
                          unsigned long long* stats, int n_sm, cudaStream_t st)
{
    const int64_t n = (int64_t)rc.width * rc.height * rc.spp;
    camera_kernel<<<grid_for(n, 256, n_sm * 8), 256, 0, st>>>(rc, pb, q, iteration_base, stats);
    return cudaGetLastError();
}

cudaError_t launch_trace_queue(const SceneView& s, const Queue& q, bool any_hit, int64_t capacity, int n_sm,
                               cudaStream_t st)
{
    const int tgrid = grid_for(capacity, 128, n_sm * 16);
    if (any_hit)
        trace_queue_kernel<true><<<tgrid, 128, 0, st>>>(s.bvh_nodes, s.bvh_tris, q, nullptr, nullptr);
    else
        trace_queue_kernel<false><<<tgrid, 128, 0, st>>>(s.bvh_nodes, s.bvh_tris, q, nullptr, nullptr);
    return cudaGetLastError();
}

cudaError_t launch_extend(const SceneView& s, const Queue& in, const Queue& next, const Queue& shadow,
                          const Queue& bsdfq, int64_t capacity, int n_sm, cudaStream_t st, const BatchJob* jobs,
                          const int32_t* job_of_slot)
{
    const int tgrid = grid_for(capacity, 128, n_sm * 16);
    reset_counts_kernel<<<1, 1, 0, st>>>(next.count, shadow.count, bsdfq.count);
    trace_queue_kernel<false><<<tgrid, 128, 0, st>>>(s.bvh_nodes, s.bvh_tris, in, jobs, job_of_slot);
    return cudaGetLastError();
}

cudaError_t launch_shade(const SceneView& s, const RenderConst& rc, const PathBuffers& pb, const Queue& in,
                         const Queue& next, const Queue& shadow, const Queue& bsdfq, const Queue& envq, int bounce,
                         int64_t capacity, unsigned long long* stats, const ReservoirBuf& restir, const GuideView& gv,
                         int n_sm, cudaStream_t st, const BatchJob* jobs)
{
    const int tgrid = grid_for(capacity, 128, n_sm * 16);
    const bool principled = rc.bsdf == GBPT_BSDF_PRINCIPLED;
    if (pb.env_entry)
    {
        reset_counts_kernel<<<1, 1, 0, st>>>(envq.count, nullptr, nullptr);
        if (principled)
            env_kernel<true><<<tgrid, 128, 0, st>>>(s, rc, pb, in, envq, stats, jobs);
        else
            env_kernel<false><<<tgrid, 128, 0, st>>>(s, rc, pb, in, envq, stats, jobs);
    }
    if (principled)
        shade_kernel<true><<<tgrid, 128, 0, st>>>(s, rc, pb, in, next, shadow, bsdfq, bounce, stats, restir, gv, jobs);
    else
        shade_kernel<false><<<tgrid, 128, 0, st>>>(s, rc, pb, in, next, shadow, bsdfq, bounce, stats, restir, gv, jobs);
    trace_queue_kernel<true><<<tgrid, 128, 0, st>>>(s.bvh_nodes, s.bvh_tris, shadow, jobs, pb.job);
    trace_queue_kernel<false><<<tgrid, 128, 0, st>>>(s.bvh_nodes, s.bvh_tris, bsdfq, jobs, pb.job);
    if (pb.env_entry)
        trace_queue_kernel<true><<<grid_for(2 * capacity, 128, n_sm * 16), 128, 0, st>>>(s.bvh_nodes, s.bvh_tris, envq,
                                                                                         jobs, pb.job);
    resolve_kernel<<<tgrid, 128, 0, st>>>(s, rc, pb, in, shadow, bsdfq, envq, gv, jobs);
    return cudaGetLastError();
}

cudaError_t launch_guide_inputs(const SceneView& s, const Queue& in, const GuideView& gv, int64_t capacity, int n_sm,
                                cudaStream_t st)
{
    guide_inputs_kernel<<<grid_for(capacity, 128, n_sm * 16), 128, 0, st>>>(s, in, gv);
    return cudaGetLastError();
}

cudaError_t launch_guide_weights(const PathBuffers& pb, const GuideView& gv, int n_sm, cudaStream_t st)
{
    guide_weights_kernel<<<grid_for(gv.rec_cap, 256, n_sm * 8), 256, 0, st>>>(pb, gv);
    guide_threshold_kernel<<<1, 1, 0, st>>>(gv);
    return cudaGetLastError();
}

cudaError_t launch_accumulate(const RenderConst& rc, const PathBuffers& pb, float* acc32, double* acc64, int n_sm,
                              cudaStream_t st)
{
    accumulate_kernel<<<grid_for((int64_t)rc.width * rc.height, 256, n_sm * 8), 256, 0, st>>>(rc, pb, acc32, acc64);
    return cudaGetLastError();
}

cudaError_t launch_batch_camera(const BatchJob* jobs, int n_jobs, int64_t max_job_paths, const PathBuffers& pb,
                                const Queue& q, const int32_t* iteration, unsigned long long* stats, int n_sm,
                                cudaStream_t st)
{
    reset_counts_kernel<<<1, 1, 0, st>>>(q.count, nullptr, nullptr);
    const int gx = grid_for(max_job_paths, 256, (n_sm * 8 + n_jobs - 1) / n_jobs + 1);
    camera_batch_kernel<<<dim3(gx, n_jobs), 256, 0, st>>>(jobs, pb, q, iteration, stats);
    return cudaGetLastError();
}

cudaError_t launch_batch_accumulate(const BatchJob* jobs, int n_jobs, int64_t max_job_pixels, const PathBuffers& pb,
                                    const int32_t* iteration, float* acc32, double* acc64, int32_t* iteration_rw,
                                    unsigned long long* done_ns, int n_sm, cudaStream_t st)
{
    const int gx = grid_for(max_job_pixels, 256, (n_sm * 8 + n_jobs - 1) / n_jobs + 1);
    accumulate_batch_kernel<<<dim3(gx, n_jobs), 256, 0, st>>>(jobs, pb, iteration, acc32, acc64);
    batch_step_kernel<<<1, 256, 0, st>>>(jobs, n_jobs, iteration_rw, done_ns);
    return cudaGetLastError();
}

cudaError_t launch_stamp(unsigned long long* out, cudaStream_t st)
{
    stamp_kernel<<<1, 1, 0, st>>>(out);
    return cudaGetLastError();
}

}  // namespace gbpt
