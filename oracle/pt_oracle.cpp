/*
 * TEST INFRASTRUCTURE ONLY — CPU oracle of the path-tracing estimator and of the power alias table.
 *
 * Only tests/ and __graft_entry__.smoke() call this, as a checker. It restates, in plain C++ with
 * -ffp-contract=off, the reference's per-pixel estimator for a Lambertian scene:
 *   - camera ray with jitter: CameraRays (src/Device/kernels/CameraRays.h:162-172) and
 *     HIPRTCamera::get_camera_ray (src/HostDeviceCommon/HIPRTCamera.h:31-52, matrix_X_point
 *     src/HostDeviceCommon/Math.h:617-640);
 *   - bounce loop of MegaKernel (src/Device/kernels/Megakernel.h:88-131): emission at bounce 0
 *     (src/Device/includes/LightSampling/Lights.h:384-389), direct lighting by
 *     sample_one_light_MIS (Lights.h:123-226) = one light sample (uniform or power alias,
 *     LightUtils.h:248-309, Heitz square-to-triangle LightUtils.h:150-199, area->solid angle
 *     PDFConversion.h:32-38, one-sided lights PDFConversion.h:19-30) + one BSDF sample with its
 *     own closest-hit ray (Intersect.h:544-643), balance heuristic (Sampling.h:103-116);
 *   - continuation: Lambertian sample (Lambertian.h:14-58, Sampling.h:180-201), throughput update
 *     and Russian roulette (PathTracing.h:44-101, RussianRoulette.h:20-55), 1e-5 throughput floor;
 *   - fix_backfacing_normals (Intersect.h:142-176);
 *   - closest hit by exhaustive Moller-Trumbore (Triangle.h:20-63) with the self-hit filter.
 * Random numbers come from PCG32 in the same order as the GPU kernels draw them (camera jitter 2,
 * then per vertex: light index 1 [+1 for the alias test], light point 2, MIS BSDF sample 2,
 * continuation 2, Russian roulette 1), so GPU and oracle images agree sample by sample up to
 * floating-point contraction.
 *
 * orc_pt_render_principled runs the same estimator on principled materials with the BSDF
 * evaluated and sampled by callbacks — the reference's own principled BSDF
 * (src/Device/includes/BSDFs/Principled.h, compiled by oracle/Makefile 'ref') — with the light
 * sample skipped for all-delta materials (MaterialUtils::can_do_light_sampling,
 * src/HostDeviceCommon/Material/MaterialUtils.h:71-93) and one PCG draw seeding the Xorshift32
 * generator of each BSDF sample, as the GPU kernels draw them.
 *
 * orc_vose_alias restates Utils::compute_alias_table (src/Utils/Utils.cpp:63-131).
 */
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <deque>
#include <thread>
#include <vector>

#include "orc_common.h"

namespace {

// ---------------------------------------------------------------------------------------------
// RIS direct lighting (sample_bsdf_and_lights_RIS_reservoir + evaluate_reservoir_sample,
// src/Device/includes/RIS/RIS.h:19-255; RISReservoir, src/Device/includes/RIS/RIS_Reservoir.h):
// M light candidates with target p^ = luminance(f Le |cos|) and weight balance(p_l, M, p_b, N)
// p^ / p_l, then N (0 or 1) BSDF candidates whose ray is traced to find an emitter, weight
// balance(p_b, N, p_l, M) p^ / p_b; one reservoir draw per candidate (u < w / w_sum keeps it);
// UCW = w_sum / p^ of the kept sample; a kept light sample is shaded through a shadow ray, a
// kept BSDF sample without one. The balance heuristic leaves the count out of the numerator as
// the reference's does (src/Device/includes/Sampling.h:103-116).
// Random numbers (the GPU kernels' order): per light candidate the light sample's draws then the
// reservoir draw; the BSDF candidate's sample draws; then the vertex's continuation draws; then
// (in the GPU's resolve pass) the BSDF candidate's reservoir draw.
// ---------------------------------------------------------------------------------------------
float bal(float a, float na, float b, float nb) { return a == 0.0f ? 0.0f : a / (na * a + nb * b); }

struct LightDraw
{
    V lp, lnrm, Le;
    float pa;
};

LightDraw draw_light(const Scene& s, const Settings& st, Pcg& rng)
{
    int e;
    if (st.light == 1)
    {
        e = rng.index(s.ne);
        if (rng.next() > s.alias_prob[e]) e = s.alias_idx[e];
    }
    else
        e = rng.index(s.ne);
    int lt = s.emissive[e];
    float r1 = rng.next(), r2 = rng.next();
    if (r2 > r1) { r1 *= 0.5f; r2 -= r1; }
    else { r2 *= 0.5f; r1 -= r2; }
    V la = s.a(lt), ab = s.b(lt) - la, ac = s.c(lt) - la;
    V n = cross(ab, ac);
    float ln = len(n);
    LightDraw d;
    d.lp = la + ab * r1 + ac * r2;
    d.lnrm = n / ln;
    d.Le = s.emi(lt);
    d.pa = light_pdf_area(s, lt, 0.5f * ln, d.Le, st.light);
    return d;
}

struct Ris
{
    bool active = false, kept = false;
    V lp = mk(0, 0, 0), dir = mk(0, 0, 0), c_l = mk(0, 0, 0), c_b = mk(0, 0, 0);
    float dist = 0, t_l = 0, t_b = 0, w_l = 0, w_b = 0;
    int M = 0;
};

// light candidates; eval(wi, pdf) -> f
template <class Eval>
void ris_lights(const Scene& s, const Settings& st, Pcg& rng, V P, V ns, int M, int N, Eval eval, Ris& r)
{
    r.active = true;
    r.M = M;
    for (int i = 0; i < M; i++)
    {
        LightDraw ld = draw_light(s, st, rng);
        float w = 0.0f, target = 0.0f, dist = 0.0f;
        V c = mk(0, 0, 0), wi = mk(0, 0, 0);
        if (ld.pa > 0.0f)
        {
            V tl = ld.lp - P;
            dist = len(tl);
            wi = tl / dist;
            float cl = std::max(0.0f, dot(ld.lnrm, neg(wi)));
            float cp = std::fabs(dot(ns, wi));
            if (cp > 0.0f && cl > 1.0e-6f)
            {
                float pb;
                V f = eval(wi, pb);
                c = f * ld.Le * cp;
                target = lum(c);
                float pl = a2s(ld.pa, dist, cl);
                w = bal(pl, (float)M, pb, (float)N) * target / pl;
            }
        }
        r.w_l += w;
        if (rng.next() < w / r.w_l)
        {
            r.kept = true;
            r.lp = ld.lp;
            r.dir = wi;
            r.dist = dist;
            r.c_l = c;
            r.t_l = target;
        }
    }
}

// BSDF candidate given its sampled direction, BSDF value and pdf: traces the ray to an emitter
void ris_bsdf(const Scene& s, const Settings& st, V P, V ns, int prim, V wi, V f, float pdf, int N, Ris& r)
{
    if (pdf <= 0.0f) return;
    float th;
    int lp = closest(s, P, wi, prim, th);
    if (lp < 0 || !(th < 1.0e35f - 1.0e-4f)) return;
    V Le = s.emi(lp);
    V n = cross(s.b(lp) - s.a(lp), s.c(lp) - s.a(lp));
    float ln = len(n);
    float cl = std::max(0.0f, dot(n / ln, neg(wi)));
    if (black(Le) || !(cl > 0.0f)) return;
    float lpdf = a2s(light_pdf_area(s, lp, 0.5f * ln, Le, st.light), th, cl);
    r.c_b = f * std::fabs(dot(ns, wi)) * Le;
    r.t_b = lum(r.c_b);
    r.w_b = bal(pdf, (float)N, lpdf, (float)r.M) * r.t_b / pdf;
}

// the reservoir's last draw (BSDF candidate) and the shading of the kept sample
V ris_finish(const Scene& s, const Settings& st, Pcg& rng, V P, int prim, V tp, const Ris& r)
{
    float wsum = r.w_l;
    bool take_bsdf = false;
    if (st.ris_n > 0)
    {
        wsum += r.w_b;
        take_bsdf = rng.next() < r.w_b / wsum;
    }
    if (take_bsdf) return tp * r.c_b * (wsum / r.t_b);
    if (r.kept && r.t_l > 0.0f && !occluded(s, P, r.dir, prim, r.dist - 1.0e-4f)) return tp * r.c_l * (wsum / r.t_l);
    return mk(0, 0, 0);
}

V trace_path(const Scene& s, const Settings& st, int pixel, int iteration)
{
    const int x = pixel % st.width, y = pixel / st.width;
    Pcg rng = pcg_seed((uint32_t)pixel, (uint32_t)iteration, (uint32_t)st.seed);
    float px = x + 0.5f, py = y + 0.5f;
    if (st.jitter)
    {
        px += rng.next() - 0.5f;
        py += rng.next() - 0.5f;
    }
    float xn = px / st.width * 2.0f - 1.0f, yn = py / st.height * 2.0f - 1.0f;
    V o = mat_point(st.iv, mk(0, 0, 0));
    V pv = mat_point(st.ip, mk(xn, yn, -1.0f));
    V pw = mat_point(st.iv, pv);
    V d = nrm(pw - o);
    int skip = -1;
    V tp = mk(1, 1, 1), L = mk(0, 0, 0);
    for (int bounce = 0; bounce <= st.nb_bounces; bounce++)
    {
        float t;
        int prim = closest(s, o, d, skip, t);
        if (prim < 0) break;
        V P = o + d * t;
        V ng = nrm(cross(s.b(prim) - s.a(prim), s.c(prim) - s.a(prim)));
        V ns = ng;
        V view = neg(d);
        if (dot(view, ng) < 0.0f) { ng = neg(ng); ns = neg(ns); }
        if (dot(view, ns) < 0.0f) ns = neg(ns);
        V refl = ns * (2.0f * dot(view, ns)) - view;
        if (dot(refl, ng) <= 0.0f)
        {
            refl = refl - nrm(ng * (dot(refl, ng) - 0.01f));
            ns = nrm(view + refl);
        }
        V albedo = s.alb(prim);
        if (bounce == 0) L = L + s.emi(prim);
        Ris ris;
        const V tp0 = tp;
        if (st.direct == 1 && s.ne > 0)
        {
            ris_lights(s, st, rng, P, ns, st.ris_m, st.ris_n,
                       [&](V wi, float& pb) { return lambert(albedo, dot(ns, wi), pb); }, ris);
            if (st.ris_n > 0)
            {
                float r1 = rng.next(), r2 = rng.next();
                V wi = cosine_sample(ns, r1, r2);
                float pdf;
                V f = lambert(albedo, dot(ns, wi), pdf);
                ris_bsdf(s, st, P, ns, prim, wi, f, pdf, st.ris_n, ris);
            }
        }
        else if (s.ne > 0)
        {
            int e;
            if (st.light == 1)
            {
                e = rng.index(s.ne);
                if (rng.next() > s.alias_prob[e]) e = s.alias_idx[e];
            }
            else
                e = rng.index(s.ne);
            int lt = s.emissive[e];
            float r1 = rng.next(), r2 = rng.next();
            if (r2 > r1) { r1 *= 0.5f; r2 -= r1; }
            else { r2 *= 0.5f; r1 -= r2; }
            V la = s.a(lt), ab = s.b(lt) - la, ac = s.c(lt) - la;
            V n = cross(ab, ac);
            float ln = len(n);
            V lp = la + ab * r1 + ac * r2;
            V lnrm = n / ln;
            float area = 0.5f * ln;
            V Le = s.emi(lt);
            float pa = light_pdf_area(s, lt, area, Le, st.light);
            if (pa > 0.0f)
            {
                V tl = lp - P;
                float dist = len(tl);
                V wi = tl / dist;
                float bp;
                V f = lambert(albedo, dot(ns, wi), bp);
                if (bp > 0.0f)
                {
                    float cl = std::max(0.0f, dot(lnrm, neg(wi)));
                    if (cl > 1.0e-5f)
                    {
                        float lpdf = a2s(pa, dist, cl);
                        float mis = balance(lpdf, bp);
                        V c = tp * (f * std::fabs(dot(ns, wi)) * Le * mis / lpdf);
                        if (!black(c) && !occluded(s, P, wi, prim, dist - 1.0e-4f)) L = L + c;
                    }
                }
            }
        }
        if (!ris.active)
        {
            float r1 = rng.next(), r2 = rng.next();
            V wi = cosine_sample(ns, r1, r2);
            float pdf;
            V f = lambert(albedo, dot(ns, wi), pdf);
            if (pdf > 0.0f && s.ne > 0)
            {
                V w = tp * (f * std::fabs(dot(ns, wi)) / pdf);
                float th;
                int lp = closest(s, P, wi, prim, th);
                if (lp >= 0 && th < 1.0e35f - 1.0e-4f)
                {
                    V Le = s.emi(lp);
                    if (!black(Le))
                    {
                        V n = cross(s.b(lp) - s.a(lp), s.c(lp) - s.a(lp));
                        float ln = len(n);
                        float cl = std::max(0.0f, dot(n / ln, neg(wi)));
                        if (cl > 0.0f)
                        {
                            float lpdf = a2s(light_pdf_area(s, lp, 0.5f * ln, Le, st.light), th, cl);
                            L = L + w * Le * balance(pdf, lpdf);
                        }
                    }
                }
            }
        }
        // continuation (its draws precede the RIS reservoir's last draw, as on the GPU)
        auto cont = [&]() {
            float r1 = rng.next(), r2 = rng.next();
            V wi = cosine_sample(ns, r1, r2);
            float pdf;
            V f = lambert(albedo, dot(ns, wi), pdf);
            if (pdf <= 0.0f) return false;
            V att = f * std::fabs(dot(wi, ns)) / pdf;
            if (st.do_rr && bounce >= st.rr_min)
            {
                float p = std::min(std::max(tp.x, std::max(tp.y, tp.z)), 1.0f);
                if (rng.next() > p) return false;
                float sc = 1.0f / p;
                if (st.rr_clamp > 0.0f) sc = std::min(sc, st.rr_clamp);
                tp = tp * sc;
            }
            tp = tp * att;
            tp = mk(std::max(tp.x, 1.0e-5f), std::max(tp.y, 1.0e-5f), std::max(tp.z, 1.0e-5f));
            o = P;
            d = wi;
            skip = prim;
            return true;
        };
        const bool go = bounce < st.nb_bounces && cont();
        if (ris.active) L = L + ris_finish(s, st, rng, P, prim, tp0, ris);
        if (!go) break;
    }
    return L;
}

V trace_path_principled(const Scene& s, const PScene& ps, const Settings& st, int pixel, int iteration)
{
    const int x = pixel % st.width, y = pixel / st.width;
    Pcg rng = pcg_seed((uint32_t)pixel, (uint32_t)iteration, (uint32_t)st.seed);
    float px = x + 0.5f, py = y + 0.5f;
    if (st.jitter)
    {
        px += rng.next() - 0.5f;
        py += rng.next() - 0.5f;
    }
    float xn = px / st.width * 2.0f - 1.0f, yn = py / st.height * 2.0f - 1.0f;
    V o = mat_point(st.iv, mk(0, 0, 0));
    V pv = mat_point(st.ip, mk(xn, yn, -1.0f));
    V pw = mat_point(st.iv, pv);
    V d = nrm(pw - o);
    int skip = -1;
    int medium = -1;
    V tp = mk(1, 1, 1), L = mk(0, 0, 0);
    for (int bounce = 0; bounce <= st.nb_bounces; bounce++)
    {
        float t;
        int prim = closest(s, o, d, skip, t);
        if (prim < 0) break;
        V P = o + d * t;
        V ng_raw = nrm(cross(s.b(prim) - s.a(prim), s.c(prim) - s.a(prim)));
        V ng = ng_raw, ns = ng_raw;
        V view = neg(d);
        if (dot(view, ng) < 0.0f) { ng = neg(ng); ns = neg(ns); }
        if (dot(view, ns) < 0.0f) ns = neg(ns);
        V refl = ns * (2.0f * dot(view, ns)) - view;
        if (dot(refl, ng) <= 0.0f)
        {
            refl = refl - nrm(ng * (dot(refl, ng) - 0.01f));
            ns = nrm(view + refl);
        }
        const int mi = s.mat_of[prim];
        const float* m = ps.mat(mi);
        if (bounce == 0) L = L + s.emi(prim);
        int32_t thin;
        std::memcpy(&thin, m + 44, 4);
        const bool transmissive = (m[38] > 0.0f || m[39] > 0.0f) && thin == 0;
        const bool inside = transmissive && dot(view, ng_raw) < 0.0f;
        const float eta_i = inside ? m[37] : (medium >= 0 ? ps.mat(medium)[37] : 1.0f);
        const float eta_o = inside ? 1.0f : m[37];
        float q[16], out[8];
        Ris ris;
        const V tp0 = tp;
        if (st.direct == 1 && s.ne > 0)
        {
            const int M = can_light_sample(m) ? st.ris_m : 0;
            ris_lights(s, st, rng, P, ns, M, st.ris_n,
                       [&](V wi, float& pb) {
                           float qq[16], oo[8];
                           make_query(qq, view, ns, ng, wi, eta_i, eta_o, inside, 0);
                           ps.eval(m, qq, oo);
                           pb = oo[3];
                           return mk(oo[0], oo[1], oo[2]);
                       },
                       ris);
            if (st.ris_n > 0)
            {
                make_query(q, view, ns, ng, mk(0, 0, 0), eta_i, eta_o, inside, 0);
                int32_t lobe;
                ps.sample(m, q, bsdf_seed(rng), out, &lobe);
                ris_bsdf(s, st, P, ns, prim, mk(out[0], out[1], out[2]), mk(out[3], out[4], out[5]), out[6], st.ris_n, ris);
            }
        }
        else if (s.ne > 0 && can_light_sample(m))
        {
            int e;
            if (st.light == 1)
            {
                e = rng.index(s.ne);
                if (rng.next() > s.alias_prob[e]) e = s.alias_idx[e];
            }
            else
                e = rng.index(s.ne);
            int lt = s.emissive[e];
            float r1 = rng.next(), r2 = rng.next();
            if (r2 > r1) { r1 *= 0.5f; r2 -= r1; }
            else { r2 *= 0.5f; r1 -= r2; }
            V la = s.a(lt), ab = s.b(lt) - la, ac = s.c(lt) - la;
            V n = cross(ab, ac);
            float ln = len(n);
            V lp = la + ab * r1 + ac * r2;
            V lnrm = n / ln;
            float area = 0.5f * ln;
            V Le = s.emi(lt);
            float pa = light_pdf_area(s, lt, area, Le, st.light);
            if (pa > 0.0f)
            {
                V tl = lp - P;
                float dist = len(tl);
                V wi = tl / dist;
                make_query(q, view, ns, ng, wi, eta_i, eta_o, inside, 0);
                ps.eval(m, q, out);
                const float bp = out[3];
                if (bp > 0.0f)
                {
                    float cl = std::max(0.0f, dot(lnrm, neg(wi)));
                    if (cl > 1.0e-5f)
                    {
                        float lpdf = a2s(pa, dist, cl);
                        float mis = balance(lpdf, bp);
                        V f = mk(out[0], out[1], out[2]);
                        V c = tp * (f * std::fabs(dot(ns, wi)) * Le * mis / lpdf);
                        if (!black(c) && !occluded(s, P, wi, prim, dist - 1.0e-4f)) L = L + c;
                    }
                }
            }
        }
        if (!ris.active)
        {
            make_query(q, view, ns, ng, mk(0, 0, 0), eta_i, eta_o, inside, 0);
            int32_t lobe;
            ps.sample(m, q, bsdf_seed(rng), out, &lobe);
            const float pdf = out[6];
            V wi = mk(out[0], out[1], out[2]);
            if (pdf > 0.0f && s.ne > 0)
            {
                V f = mk(out[3], out[4], out[5]);
                V w = tp * (f * std::fabs(dot(ns, wi)) / pdf);
                float th;
                int lp = closest(s, P, wi, prim, th);
                if (lp >= 0 && th < 1.0e35f - 1.0e-4f)
                {
                    V Le = s.emi(lp);
                    if (!black(Le))
                    {
                        V n = cross(s.b(lp) - s.a(lp), s.c(lp) - s.a(lp));
                        float ln = len(n);
                        float cl = std::max(0.0f, dot(n / ln, neg(wi)));
                        if (cl > 0.0f)
                        {
                            float lpdf = a2s(light_pdf_area(s, lp, 0.5f * ln, Le, st.light), th, cl);
                            L = L + w * Le * balance(pdf, lpdf);
                        }
                    }
                }
            }
        }
        auto cont = [&]() {
            make_query(q, view, ns, ng, mk(0, 0, 0), eta_i, eta_o, inside, 0);
            int32_t lobe;
            ps.sample(m, q, bsdf_seed(rng), out, &lobe);
            const float pdf = out[6];
            if (pdf <= 0.0f) return false;
            V wi = mk(out[0], out[1], out[2]);
            V f = mk(out[3], out[4], out[5]);
            V att = f * std::fabs(dot(wi, ns)) / pdf;
            if (st.do_rr && bounce >= st.rr_min)
            {
                float p = std::min(std::max(tp.x, std::max(tp.y, tp.z)), 1.0f);
                if (rng.next() > p) return false;
                float sc = 1.0f / p;
                if (st.rr_clamp > 0.0f) sc = std::min(sc, st.rr_clamp);
                tp = tp * sc;
            }
            tp = tp * att;
            tp = mk(std::max(tp.x, 1.0e-5f), std::max(tp.y, 1.0e-5f), std::max(tp.z, 1.0e-5f));
            if (transmissive && (lobe == 64 || lobe == 256)) medium = inside ? -1 : mi;
            o = P;
            d = wi;
            skip = prim;
            return true;
        };
        const bool go = bounce < st.nb_bounces && cont();
        if (ris.active) L = L + ris_finish(s, st, rng, P, prim, tp0, ris);
        if (!go) break;
    }
    return L;
}

}  // namespace

extern "C" {

/* settings_i: width, height, nb_bounces, do_rr, rr_min_depth, light_sampling (0 uniform, 1 power),
 * seed, do_jittering, spp, iteration_base, direct lighting (0 MIS, 1 RIS), RIS light candidates,
 * RIS BSDF candidates. Adds the samples of iterations
 * [iteration_base, iteration_base + spp) to out_rgb (W*H*3 doubles). */
void orc_pt_render(const float* tri_verts, int n_tris, const int* mat_of, const float* albedo, const float* emission,
                   const int* emissive, int n_emissive, const float* alias_prob, const int* alias_idx, float power_sum,
                   const int* settings_i, float rr_clamp, const float* inv_view, const float* inv_proj, double* out_rgb,
                   int nthreads)
{
    Scene s{tri_verts, n_tris, mat_of, albedo, emission, emissive, n_emissive, alias_prob, alias_idx, power_sum};
    Settings st{settings_i[0], settings_i[1], settings_i[2], settings_i[3], settings_i[4], settings_i[5],
                settings_i[6], settings_i[7], settings_i[8], settings_i[9], rr_clamp, inv_view, inv_proj,
                settings_i[10], settings_i[11], settings_i[12]};
    const int npix = st.width * st.height;
    if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
    std::atomic<int> next{0};
    std::vector<std::thread> pool;
    for (int w = 0; w < nthreads; w++)
        pool.emplace_back([&]() {
            for (;;)
            {
                int p = next.fetch_add(1);
                if (p >= npix) break;
                double r = 0, g = 0, b = 0;
                for (int k = 0; k < st.spp; k++)
                {
                    V c = trace_path(s, st, p, st.iteration_base + k);
                    r += c.x;
                    g += c.y;
                    b += c.z;
                }
                out_rgb[3 * p] += r;
                out_rgb[3 * p + 1] += g;
                out_rgb[3 * p + 2] += b;
            }
        });
    for (auto& t : pool) t.join();
}

/* Emissive power list exactly as GPURenderer::compute_emissives_power_alias_table
 * (src/Renderer/GPURenderer.cpp:256-275): luminance(emission) * area in float, operations rounded
 * one by one (this file is compiled with -ffp-contract=off). tri_verts = 9 floats per triangle,
 * emission = 3 floats per material (colour * strength * global factor). */
void orc_emissive_power(const float* tri_verts, const int* mat_of, const float* emission, const int* emissive,
                        int n_emissive, float* out_power)
{
    for (int i = 0; i < n_emissive; i++)
    {
        const float* t = tri_verts + 9 * (size_t)emissive[i];
        V a = mk(t[0], t[1], t[2]), b = mk(t[3], t[4], t[5]), c = mk(t[6], t[7], t[8]);
        V n = cross(b - a, c - a);
        float area = 0.5f * len(n);
        const float* e = emission + 3 * mat_of[emissive[i]];
        out_power[i] = lum(mk(e[0], e[1], e[2])) * area;
    }
}

/* Principled scenes: as orc_pt_render, with 'pmats' (64-word effective materials) shaded through
 * the given BSDF callbacks (the reference's own BSDF from oracle/_ref/libref.so). */
void orc_pt_render_principled(const float* tri_verts, int n_tris, const int* mat_of, const float* albedo,
                              const float* emission, const float* pmats, void* eval_fn, void* sample_fn,
                              const int* emissive, int n_emissive, const float* alias_prob, const int* alias_idx,
                              float power_sum, const int* settings_i, float rr_clamp, const float* inv_view,
                              const float* inv_proj, double* out_rgb, int nthreads)
{
    Scene s{tri_verts, n_tris, mat_of, albedo, emission, emissive, n_emissive, alias_prob, alias_idx, power_sum};
    PScene ps{pmats, (bsdf_eval_fn)eval_fn, (bsdf_sample_fn)sample_fn};
    Settings st{settings_i[0], settings_i[1], settings_i[2], settings_i[3], settings_i[4], settings_i[5],
                settings_i[6], settings_i[7], settings_i[8], settings_i[9], rr_clamp, inv_view, inv_proj,
                settings_i[10], settings_i[11], settings_i[12]};
    const int npix = st.width * st.height;
    if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
    std::atomic<int> next{0};
    std::vector<std::thread> pool;
    for (int w = 0; w < nthreads; w++)
        pool.emplace_back([&]() {
            for (;;)
            {
                int p = next.fetch_add(1);
                if (p >= npix) break;
                double r = 0, g = 0, b = 0;
                for (int k = 0; k < st.spp; k++)
                {
                    V c = trace_path_principled(s, ps, st, p, st.iteration_base + k);
                    r += c.x;
                    g += c.y;
                    b += c.z;
                }
                out_rgb[3 * p] += r;
                out_rgb[3 * p + 1] += g;
                out_rgb[3 * p + 2] += b;
            }
        });
    for (auto& t : pool) t.join();
}

/* Vose alias table exactly as src/Utils/Utils.cpp:63-131: elements normalised in double by
 * 'total_sum' (as given) and scaled by n; FIFO small/large queues in index order. */
void orc_vose_alias(const float* input, int n, double total_sum, float* out_prob, int* out_alias)
{
    std::vector<double> q(n);
    for (int i = 0; i < n; i++) q[i] = (double)input[i] / total_sum * n;
    std::deque<int> smalls, larges;
    for (int i = 0; i < n; i++)
    {
        out_alias[i] = i;
        if (q[i] < 1.0f)
            smalls.push_back(i);
        else
            larges.push_back(i);
    }
    while (!smalls.empty() && !larges.empty())
    {
        int si = smalls.front(), li = larges.front();
        smalls.pop_front();
        larges.pop_front();
        out_prob[si] = (float)q[si];
        out_alias[si] = li;
        q[li] = (q[li] + q[si]) - 1.0f;
        if (q[li] > 1.0f)
            larges.push_back(li);
        else
            smalls.push_back(li);
    }
    while (!larges.empty())
    {
        out_prob[larges.front()] = 1.0f;
        larges.pop_front();
    }
    while (!smalls.empty())
    {
        out_prob[smalls.front()] = 1.0f;
        smalls.pop_front();
    }
}

} // extern "C"
