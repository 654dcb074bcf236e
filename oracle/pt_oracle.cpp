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
// Random numbers: per light candidate the light sample's draws then the reservoir draw; the BSDF
// candidate's sample draws; then, with the reference's generator (rng_mode 1), the BSDF
// candidate's reservoir draw as the reference makes it; then the vertex's continuation draws; with
// PCG streams the BSDF candidate's reservoir draw comes last (the GPU's resolve pass draws it).
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
    float u_b = -1.0f;  // the BSDF candidate's reservoir draw when drawn in the reference's place
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
        take_bsdf = (r.u_b >= 0.0f ? r.u_b : rng.next()) < r.w_b / wsum;
    }
    if (take_bsdf) return tp * r.c_b * (wsum / r.t_b);
    if (r.kept && r.t_l > 0.0f && !occluded(s, P, r.dir, prim, r.dist - 1.0e-4f)) return tp * r.c_l * (wsum / r.t_l);
    return mk(0, 0, 0);
}

// ---------------------------------------------------------------------------------------------
// The world and its environment map:
//   - RGB9E5 texels: RGBE9995Packed::pack / unpack (src/HostDeviceCommon/Packing.h:441-485);
//   - tables: luminance_of_pixel from the float texels (src/Image/Image.cpp:526-546), the running
//     sum of compute_cdf (Image.cpp:625-645) accumulated in double and stored as float, the Vose
//     table of compute_alias_table (Image.cpp:650-672) through orc_vose_alias below;
//   - lookups: eval_envmap_no_pdf (src/Device/includes/LightSampling/Envmap.h:27-37) through
//     sample_environment_map_texture (src/Device/includes/Texture.h:209-240), nearest or bilinear;
//   - sampling: envmap_cdf_search / envmap_sample / envmap_eval (Envmap.h:39-170): a texel by alias
//     table (index draw, alias-test draw) or CDF search (one draw), the direction of its (x/W, y/H)
//     corner, radiance and pdf read through the texture lookup at that corner;
//   - direct lighting: sample_environment_map_with_mis (Envmap.h:173-249), an envmap sample
//     (skipped when the material cannot be light-sampled) and a separate BSDF sample, balance
//     heuristic, any-hit visibility to 1e35; the ReSTIR DI bounce is not restated here;
//   - misses: path_tracing_miss_gather_envmap (src/Device/includes/PathTracing.h:122-169).
// Guards shared with the GPU kernels: asin's argument clamped to [-1, 1], texel indices clamped to
// the image, alias index split by integer division.
// Random numbers at a vertex: first the envmap texel draws (2 alias / 1 CDF) and the BSDF sample's
// draws (2 Lambertian / 1 Xorshift32 seed), then the emissive direct lighting's, then the
// continuation's (the GPU's envmap pass runs before its shade pass). Contributions are added in
// the order light sample, envmap sample, envmap BSDF sample, MIS BSDF sample.
// ---------------------------------------------------------------------------------------------
struct OrcEnv
{
    int32_t ambient;  // 0 none, 1 uniform, 2 envmap
    float uniform[3];
    const uint32_t* texels;
    const float* cdf;
    const float* probas;
    const int32_t* alias;
    int32_t width, height;
    float intensity, total_sum;
    float to_world[9], to_env[9];  // row-major, d' = M d
    int32_t sampling;              // 0 none, 1 binary search, 2 alias table
    int32_t bsdf_mis, bilinear, scale_background;
};

const float kInv2Pi = 0.15915494309189533577f, kInvPiF = 0.31830988618379067154f;
const float kTwoPiF = 6.28318530717958647693f, kPiF = 3.14159265358979323846f;
const float kTwoPiSq = 19.73920880217871723767f;

uint32_t fbits(float f)
{
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}
float bitsf(uint32_t u)
{
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

uint32_t rgb9e5_pack(float r, float g, float b)
{
    const float hi = bitsf(0x477F8000u), lo = bitsf(0x37800000u);
    r = std::min(std::max(r, 0.0f), hi);
    g = std::min(std::max(g, 0.0f), hi);
    b = std::min(std::max(b, 0.0f), hi);
    const float m = std::max(std::max(lo, r), std::max(g, b));
    const float bias = bitsf((fbits(m) + 0x07804000u) & 0x7F800000u);
    const uint32_t R = fbits(r + bias), G = fbits(g + bias), B = fbits(b + bias);
    const uint32_t E = (fbits(bias) << 4) + 0x10000000u;
    return E | (B << 18) | (G << 9) | (R & 0x1FFu);
}

V rgb9e5_unpack(uint32_t t)
{
    const float sc = std::ldexp(1.0f, (int)(t >> 27) - 24);
    return mk((float)(t & 0x1FFu) * sc, (float)((t >> 9) & 0x1FFu) * sc, (float)((t >> 18) & 0x1FFu) * sc);
}

V mat3(const float* m, V d)
{
    return mk(m[0] * d.x + m[1] * d.y + m[2] * d.z, m[3] * d.x + m[4] * d.y + m[5] * d.z,
              m[6] * d.x + m[7] * d.y + m[8] * d.z);
}

V env_texel(const OrcEnv& e, int x, int y)
{
    x = std::min(std::max(x, 0), e.width - 1);
    y = std::min(std::max(y, 0), e.height - 1);
    return rgb9e5_unpack(e.texels[(size_t)y * e.width + x]) * e.intensity;
}

V env_texture(const OrcEnv& e, float u, float v)
{
    const float fx = u * (float)(e.width - 1), fy = v * (float)(e.height - 1);
    if (!e.bilinear) return env_texel(e, (int)fx, (int)fy);
    const int x0 = (int)fx, y0 = (int)fy;
    const float tx = fx - std::floor(fx), ty = fy - std::floor(fy);
    const int x1 = std::min(x0 + 1, e.width - 1), y1 = std::min(y0 + 1, e.height - 1);
    const V a = env_texel(e, x0, y0) * (1.0f - tx) + env_texel(e, x1, y0) * tx;
    const V b = env_texel(e, x0, y1) * (1.0f - tx) + env_texel(e, x1, y1) * tx;
    return a * (1.0f - ty) + b * ty;
}

V env_lookup(const OrcEnv& e, V d)
{
    const V r = mat3(e.to_env, d);
    const float u = 0.5f + std::atan2(r.z, r.x) * kInv2Pi;
    const float v = 0.5f + std::asin(std::min(1.0f, std::max(-1.0f, r.y))) * kInvPiF;
    return env_texture(e, u, v);
}

float env_pdf(const OrcEnv& e, V L, float sin_theta)
{
    float pdf = lum(L) / (e.total_sum * e.intensity);
    pdf *= (float)(e.width * e.height);
    return pdf / (kTwoPiSq * sin_theta);
}

void env_cdf_search(const OrcEnv& e, float value, int& x, int& y)
{
    int lo = 0, hi = e.height - 1;
    while (lo < hi)
    {
        const int mid = (lo + hi) >> 1;
        if (value < e.cdf[(size_t)mid * e.width + (e.width - 1)])
            hi = mid;
        else
            lo = mid + 1;
    }
    y = std::min(lo, e.height - 1);
    lo = 0;
    hi = e.width - 1;
    while (lo < hi)
    {
        const int mid = (lo + hi) >> 1;
        if (value < e.cdf[(size_t)y * e.width + mid])
            hi = mid;
        else
            lo = mid + 1;
    }
    x = std::min(lo, e.width - 1);
}

struct EnvSampleO
{
    V dir, L;
    float pdf;
};

// direction, radiance and pdf of a sampled texel (envmap_sample after the texel choice)
EnvSampleO env_sample_texel(const OrcEnv& e, int x, int y)
{
    const float u = (float)x / (float)e.width, v = (float)y / (float)e.height;
    const float phi = u * kTwoPiF;
    const float theta = std::max(1.0e-5f, v * kPiF);
    const float ct = std::cos(theta), sn = std::sin(theta);
    EnvSampleO s;
    s.dir = mat3(e.to_world, mk(-sn * std::cos(phi), -ct, -sn * std::sin(phi)));
    s.L = env_texture(e, u, v);
    s.pdf = env_pdf(e, s.L, sn);
    return s;
}

EnvSampleO env_sample(const OrcEnv& e, Pcg& rng)
{
    int x, y;
    if (e.sampling == 1)
        env_cdf_search(e, rng.next() * e.total_sum, x, y);
    else
    {
        int i = rng.index(e.width * e.height);
        if (rng.next() > e.probas[i]) i = e.alias[i];
        y = i / e.width;
        x = i - y * e.width;
    }
    return env_sample_texel(e, x, y);
}

V env_eval(const OrcEnv& e, V d, float& pdf)
{
    const V L = env_lookup(e, d);
    pdf = env_pdf(e, L, std::sin(std::acos(-d.y)));
    return L;
}

bool env_sampled(const OrcEnv* e) { return e && e->ambient == 2 && e->sampling != 0 && e->intensity > 0.0f; }

V env_miss(const OrcEnv* e, V d, int bounce, V tp)
{
    if (!e) return mk(0, 0, 0);
    if (e->ambient == 1) return mk(e->uniform[0], e->uniform[1], e->uniform[2]) * tp;
    if (e->ambient != 2 || !(e->intensity > 0.0f)) return mk(0, 0, 0);
    const bool sampled = e->sampling != 0;
    if (sampled && bounce > 0) return mk(0, 0, 0);
    V c = env_lookup(*e, d);
    if (!e->scale_background && (sampled || bounce == 0)) c = c / e->intensity;
    return c * tp;
}

struct EnvDirectO
{
    V c_l = mk(0, 0, 0), c_b = mk(0, 0, 0);
};

// envmap sample + separate BSDF sample; eval(wi, pdf) -> f, sample(wi, pdf) -> f
template <class Eval, class Sample>
EnvDirectO env_direct(const OrcEnv& e, const Scene& s, Pcg& rng, V P, int prim, V ns, V tp, bool light_ok, Eval eval,
                      Sample sample)
{
    EnvDirectO r;
    const EnvSampleO es = env_sample(e, rng);
    if (light_ok)
    {
        const float cosine = dot(ns, es.dir);
        if (es.pdf > 0.0f && cosine > 0.0f)
        {
            float bp;
            const V f = eval(es.dir, bp);
            const float mis = e.bsdf_mis ? balance(es.pdf, bp) : 1.0f;
            const V c = tp * (f * cosine * mis * es.L / es.pdf);
            if (!black(c) && !occluded(s, P, es.dir, prim, 1.0e35f)) r.c_l = c;
        }
    }
    if (e.bsdf_mis)
    {
        V wi;
        float pdf;
        const V f = sample(wi, pdf);
        if (pdf > 0.0f)
        {
            const float cosine = std::fabs(dot(ns, wi));
            float pe;
            const V L = env_eval(e, wi, pe);
            if (pe > 0.0f)
            {
                const V c = tp * (L * balance(pdf, pe) * cosine * f / pdf);
                if (!black(c) && !occluded(s, P, wi, prim, 1.0e35f)) r.c_b = c;
            }
        }
    }
    return r;
}

// rng_mode 1, camera hit: the vertex as the reference's MegaKernel rebuilds it from the packed
// G-buffer (Megakernel.h:59-70): octahedral-24 normals written after the backface fix
// (CameraRays.h:178-181), renormalised on read, and the view direction from the camera position
// (the translation column of the inverse view, Camera::to_hiprt) to the stored hit point
// (GBufferDevice::get_view_direction), negated into a ray direction, normalised and negated back.
void gbuffer_vertex(const Settings& st, V P, V& ng, V& ns, V& view)
{
    ng = nrm(oct24(ng));
    ns = nrm(oct24(ns));
    const V cam = mk(st.iv[3], st.iv[7], st.iv[11]);
    view = neg(nrm(neg(nrm(cam - P))));
}

V trace_path(const Scene& s, const Settings& st, int pixel, int iteration)
{
    const int x = pixel % st.width, y = pixel / st.width;
    Pcg rng = st.rng_mode ? parity_seed((uint32_t)pixel, (uint32_t)iteration, st.random_number)
                          : pcg_seed((uint32_t)pixel, (uint32_t)iteration, (uint32_t)st.seed);
    float px = x + 0.5f, py = y + 0.5f;
    if (st.jitter)
    {
        px += rng.next() - 0.5f;
        py += rng.next() - 0.5f;
    }
    // the reference's MegaKernel seeds a new generator from its own pass's random number
    // (Megakernel.h:52-57; MegaKernelRenderPass::launch_async draws it after the camera pass's)
    if (st.rng_mode) rng = parity_seed((uint32_t)pixel, (uint32_t)iteration, st.random_number_shade);
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
        if (prim < 0)
        {
            L = L + env_miss(st.env, d, bounce, tp);
            break;
        }
        V P = o + d * t;
        V ng = nrm(cross(s.b(prim) - s.a(prim), s.c(prim) - s.a(prim)));
        V ns = shading_normal(s, prim, o, d, ng);
        V view = neg(d);
        if (dot(view, ng) < 0.0f) { ng = neg(ng); ns = neg(ns); }
        if (dot(view, ns) < 0.0f) ns = neg(ns);
        V refl = ns * (2.0f * dot(view, ns)) - view;
        if (dot(refl, ng) <= 0.0f)
        {
            refl = refl - nrm(ng * (dot(refl, ng) - 0.01f));
            ns = nrm(view + refl);
        }
        if (st.rng_mode && bounce == 0) gbuffer_vertex(st, P, ng, ns, view);
        V albedo = s.alb(prim);
        if (bounce == 0) L = L + s.emi(prim);
        // envmap direct lighting: its draws come first at a vertex (the GPU's envmap pass runs
        // before shade); its contributions are added after the light sample's
        EnvDirectO ed;
        if (env_sampled(st.env))
            ed = env_direct(
                *st.env, s, rng, P, prim, ns, tp, true, [&](V wi, float& pb) { return lambert(albedo, dot(ns, wi), pb); },
                [&](V& wi, float& pdf) {
                    float r1 = rng.next(), r2 = rng.next();
                    wi = cosine_sample(ns, r1, r2);
                    return lambert(albedo, dot(ns, wi), pdf);
                });
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
                if (st.rng_mode) ris.u_b = rng.next();
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
        V bsdf_c = mk(0, 0, 0);  // MIS BSDF sample, added after the envmap's samples as on the GPU
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
                            bsdf_c = w * Le * balance(pdf, lpdf);
                        }
                    }
                }
            }
        }
        L = L + ed.c_l;
        L = L + ed.c_b;
        L = L + bsdf_c;
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
    Pcg rng = st.rng_mode ? parity_seed((uint32_t)pixel, (uint32_t)iteration, st.random_number)
                          : pcg_seed((uint32_t)pixel, (uint32_t)iteration, (uint32_t)st.seed);
    float px = x + 0.5f, py = y + 0.5f;
    if (st.jitter)
    {
        px += rng.next() - 0.5f;
        py += rng.next() - 0.5f;
    }
    // the reference's MegaKernel seeds a new generator from its own pass's random number
    // (Megakernel.h:52-57; MegaKernelRenderPass::launch_async draws it after the camera pass's)
    if (st.rng_mode) rng = parity_seed((uint32_t)pixel, (uint32_t)iteration, st.random_number_shade);
    float xn = px / st.width * 2.0f - 1.0f, yn = py / st.height * 2.0f - 1.0f;
    V o = mat_point(st.iv, mk(0, 0, 0));
    V pv = mat_point(st.ip, mk(xn, yn, -1.0f));
    V pw = mat_point(st.iv, pv);
    V d = nrm(pw - o);
    int skip = -1;
    VolState vs;
    V tp = mk(1, 1, 1), L = mk(0, 0, 0);
    for (int bounce = 0; bounce <= st.nb_bounces; bounce++)
    {
        float t;
        int prim;
        // trace_main_path_ray (Intersect.h:200-270): every hit pushes its material on the volume
        // stack (distance travelled inside a volume accumulated), a skipped boundary (a lower
        // priority material inside a higher one) is passed through; at the camera hit the stack
        // restarts from the air (RayVolumeState::reconstruct_first_hit, Megakernel.h:78-82)
        for (;;)
        {
            prim = closest(s, o, d, skip, t);
            if (prim < 0) break;
            const int pm = s.mat_of[prim];
            if (bounce == 0)
            {
                vs = VolState();
                vs.push(pm, dielectric_priority(ps.mat(pm)));
                break;
            }
            const bool skipped = vs.push(pm, dielectric_priority(ps.mat(pm)));
            if (vs.inside) vs.distance += t;
            if (!skipped) break;
            o = o + d * t;
            vs.distance += t;
        }
        if (prim < 0)
        {
            L = L + env_miss(st.env, d, bounce, tp);
            break;
        }
        V P = o + d * t;
        V ng_raw = nrm(cross(s.b(prim) - s.a(prim), s.c(prim) - s.a(prim)));
        V ng = ng_raw, ns = shading_normal(s, prim, o, d, ng_raw);
        V view = neg(d);
        if (dot(view, ng) < 0.0f) { ng = neg(ng); ns = neg(ns); }
        if (dot(view, ns) < 0.0f) ns = neg(ns);
        V refl = ns * (2.0f * dot(view, ns)) - view;
        if (dot(refl, ng) <= 0.0f)
        {
            refl = refl - nrm(ng * (dot(refl, ng) - 0.01f));
            ns = nrm(view + refl);
        }
        if (st.rng_mode && bounce == 0) gbuffer_vertex(st, P, ng, ns, view);
        const int mi = s.mat_of[prim];
        // rng_mode 1: the camera hit shades with the material as the G-buffer re-packed it after
        // the fetch's coat roughening (CameraRays.h:183, Megakernel.h:72)
        const float* m = (st.rng_mode && bounce == 0 && st.gbuffer_materials) ? ps.mat(mi + st.gbuffer_materials) : ps.mat(mi);
        if (bounce == 0) L = L + s.emi(prim);
        const bool inside = vs.inside;
        const float eta_i = vol_ior(ps, vs.incident), eta_o = vol_ior(ps, vs.outgoing);
        // Beer-Lambert attenuation of a refraction out of a volume (principled_glass_eval and
        // principled_diffuse_transmission_eval apply it to refracted directions)
        const V beer = vol_beer(ps, vs);
        const float nov_b = dot(view, ns);
        auto refr = [&](V wi, V f) { return (nov_b * dot(wi, ns) <= 0.0f) ? f * beer : f; };
        float q[16], out[8];
        // envmap direct lighting first, as on the GPU
        EnvDirectO ed;
        if (env_sampled(st.env))
            ed = env_direct(
                *st.env, s, rng, P, prim, ns, tp, can_light_sample(m),
                [&](V wi, float& pb) {
                    float qq[16], oo[8];
                    make_query(qq, view, ns, ng, wi, eta_i, eta_o, inside, 0);
                    ps.eval(m, qq, oo);
                    pb = oo[3];
                    return refr(wi, mk(oo[0], oo[1], oo[2]));
                },
                [&](V& wi, float& pdf) {
                    float qq[16], oo[8];
                    make_query(qq, view, ns, ng, mk(0, 0, 0), eta_i, eta_o, inside, 0);
                    int32_t lobe;
                    ps.sample(m, qq, bsdf_seed(rng), oo, &lobe);
                    bsdf_seed_done(rng, oo);
                    wi = mk(oo[0], oo[1], oo[2]);
                    pdf = oo[6];
                    return refr(wi, mk(oo[3], oo[4], oo[5]));
                });
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
                           return refr(wi, mk(oo[0], oo[1], oo[2]));
                       },
                       ris);
            if (st.ris_n > 0)
            {
                make_query(q, view, ns, ng, mk(0, 0, 0), eta_i, eta_o, inside, 0);
                int32_t lobe;
                ps.sample(m, q, bsdf_seed(rng), out, &lobe);
            bsdf_seed_done(rng, out);
                ris_bsdf(s, st, P, ns, prim, mk(out[0], out[1], out[2]), refr(mk(out[0], out[1], out[2]), mk(out[3], out[4], out[5])), out[6], st.ris_n, ris);
                if (st.rng_mode) ris.u_b = rng.next();
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
                        V f = refr(wi, mk(out[0], out[1], out[2]));
                        V c = tp * (f * std::fabs(dot(ns, wi)) * Le * mis / lpdf);
                        if (!black(c) && !occluded(s, P, wi, prim, dist - 1.0e-4f)) L = L + c;
                    }
                }
            }
        }
        V bsdf_c = mk(0, 0, 0);  // MIS BSDF sample, added after the envmap's samples as on the GPU
        if (!ris.active)
        {
            make_query(q, view, ns, ng, mk(0, 0, 0), eta_i, eta_o, inside, 0);
            int32_t lobe;
            ps.sample(m, q, bsdf_seed(rng), out, &lobe);
            bsdf_seed_done(rng, out);
            const float pdf = out[6];
            V wi = mk(out[0], out[1], out[2]);
            if (pdf > 0.0f && s.ne > 0)
            {
                V f = refr(wi, mk(out[3], out[4], out[5]));
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
                            bsdf_c = w * Le * balance(pdf, lpdf);
                        }
                    }
                }
            }
        }
        L = L + ed.c_l;
        L = L + ed.c_b;
        L = L + bsdf_c;
        auto cont = [&]() {
            make_query(q, view, ns, ng, mk(0, 0, 0), eta_i, eta_o, inside, 0);
            int32_t lobe;
            ps.sample(m, q, bsdf_seed(rng), out, &lobe);
            bsdf_seed_done(rng, out);
            const float pdf = out[6];
            if (pdf <= 0.0f) return false;
            V wi = mk(out[0], out[1], out[2]);
            V f = refr(wi, mk(out[3], out[4], out[5]));
            if (!vol_after_sample(ps, vs, m, view, ns, ng, wi, lobe)) return false;
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

}  // namespace

extern "C" {

/* settings_i: width, height, nb_bounces, do_rr, rr_min_depth, light_sampling (0 uniform, 1 power),
 * seed, do_jittering, spp, iteration_base, direct lighting (0 MIS, 1 RIS), RIS light candidates,
 * RIS BSDF candidates, rng mode (0 PCG, 1 the reference's Xorshift32 + packed G-buffer), the
 * frame's random number (rng mode 1), the offset of the camera-hit material table in pmats (rng
 * mode 1, principled; 0: none). env: the world (NULL: none). tri_normals: corner normals, 9 floats per
 * triangle (NULL: flat shading). Adds the samples of iterations
 * [iteration_base, iteration_base + spp) to out_rgb (W*H*3 doubles). */
void orc_pt_render(const float* tri_verts, int n_tris, const int* mat_of, const float* albedo, const float* emission,
                   const int* emissive, int n_emissive, const float* alias_prob, const int* alias_idx, float power_sum,
                   const int* settings_i, float rr_clamp, const float* inv_view, const float* inv_proj, double* out_rgb,
                   int nthreads, const OrcEnv* env, const float* tri_normals)
{
    Scene s{tri_verts, n_tris, mat_of, albedo, emission, emissive, n_emissive, alias_prob, alias_idx, power_sum, tri_normals};
    Settings st{settings_i[0], settings_i[1], settings_i[2], settings_i[3], settings_i[4], settings_i[5],
                settings_i[6], settings_i[7], settings_i[8], settings_i[9], rr_clamp, inv_view, inv_proj,
                settings_i[10], settings_i[11], settings_i[12], env, settings_i[13], (uint32_t)settings_i[14], settings_i[15], (uint32_t)settings_i[16]};
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
                              const float* inv_proj, double* out_rgb, int nthreads, const OrcEnv* env,
                              const float* tri_normals)
{
    Scene s{tri_verts, n_tris, mat_of, albedo, emission, emissive, n_emissive, alias_prob, alias_idx, power_sum, tri_normals};
    PScene ps{pmats, (bsdf_eval_fn)eval_fn, (bsdf_sample_fn)sample_fn};
    Settings st{settings_i[0], settings_i[1], settings_i[2], settings_i[3], settings_i[4], settings_i[5],
                settings_i[6], settings_i[7], settings_i[8], settings_i[9], rr_clamp, inv_view, inv_proj,
                settings_i[10], settings_i[11], settings_i[12], env, settings_i[13], (uint32_t)settings_i[14], settings_i[15], (uint32_t)settings_i[16]};
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

/* The octahedral-24 normal round trip of the G-buffer restated (oct24 in orc_common.h). */
void orc_oct24(const float* in, int n, float* out)
{
    for (int i = 0; i < n; i++)
    {
        V u = oct24(mk(in[3 * i], in[3 * i + 1], in[3 * i + 2]));
        out[3 * i] = u.x;
        out[3 * i + 1] = u.y;
        out[3 * i + 2] = u.z;
    }
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
        out_alias[i] = 0;  // the reference's out_alias.resize(n) value-initialises
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

/* ---- envmap tables and functions (pinned against the reference's own code in tests) ---- */

/* RGB9E5 packing of n RGB float texels and the float luminance of each (luminance_of_pixel) */
void orc_env_pack(const float* rgb, int64_t n, uint32_t* texels, float* luminance)
{
    for (int64_t i = 0; i < n; i++)
    {
        const float r = rgb[3 * i], g = rgb[3 * i + 1], b = rgb[3 * i + 2];
        if (texels) texels[i] = rgb9e5_pack(r, g, b);
        if (luminance) luminance[i] = ((r * 0.3086f) + (g * 0.6094f)) + (b * 0.0820f);
    }
}

void orc_env_unpack(const uint32_t* texels, int64_t n, float* rgb)
{
    for (int64_t i = 0; i < n; i++)
    {
        const V c = rgb9e5_unpack(texels[i]);
        rgb[3 * i] = c.x;
        rgb[3 * i + 1] = c.y;
        rgb[3 * i + 2] = c.z;
    }
}

/* running sum of the luminances in double, each stored as float; *total = the double sum */
void orc_env_cdf(const float* luminance, int64_t n, float* cdf, double* total)
{
    double run = 0.0;
    for (int64_t i = 0; i < n; i++)
    {
        run += (double)luminance[i];
        cdf[i] = (float)run;
    }
    *total = run;
}

/* eval_envmap_no_pdf of n world directions */
void orc_env_lookup(const OrcEnv* e, const float* dirs, int n, float* rgb)
{
    for (int i = 0; i < n; i++)
    {
        const V c = env_lookup(*e, mk(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]));
        rgb[3 * i] = c.x;
        rgb[3 * i + 1] = c.y;
        rgb[3 * i + 2] = c.z;
    }
}

/* envmap_eval: radiance and pdf of n world directions */
void orc_env_eval(const OrcEnv* e, const float* dirs, int n, float* rgb, float* pdf)
{
    for (int i = 0; i < n; i++)
    {
        const V c = env_eval(*e, mk(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]), pdf[i]);
        rgb[3 * i] = c.x;
        rgb[3 * i + 1] = c.y;
        rgb[3 * i + 2] = c.z;
    }
}

/* envmap_sample from given draws: alias table (index[i], u[i]) when values is NULL, else the CDF
 * search of values[i]; out: direction, radiance, pdf and the texel (x, y) */
void orc_env_sample(const OrcEnv* e, const int32_t* index, const float* u, const float* values, int n, float* dir,
                    float* rgb, float* pdf, int32_t* xy)
{
    for (int i = 0; i < n; i++)
    {
        int x, y;
        if (values)
            env_cdf_search(*e, values[i], x, y);
        else
        {
            int k = index[i];
            if (u[i] > e->probas[k]) k = e->alias[k];
            y = k / e->width;
            x = k - y * e->width;
        }
        const EnvSampleO s = env_sample_texel(*e, x, y);
        dir[3 * i] = s.dir.x;
        dir[3 * i + 1] = s.dir.y;
        dir[3 * i + 2] = s.dir.z;
        rgb[3 * i] = s.L.x;
        rgb[3 * i + 1] = s.L.y;
        rgb[3 * i + 2] = s.L.z;
        pdf[i] = s.pdf;
        xy[2 * i] = x;
        xy[2 * i + 1] = y;
    }
}

} // extern "C"
