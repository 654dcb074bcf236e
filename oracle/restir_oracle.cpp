/*
 * TEST INFRASTRUCTURE ONLY — CPU oracle of ReSTIR DI at the camera hit. Only tests/ call this, as
 * a checker (golden reservoirs are generated here with the reference's own principled BSDF as the
 * shading callbacks, oracle/ref_bsdf.cpp).
 *
 * Restates, pass by pass, the reference's ReSTIR DI with its default options:
 *   - reservoir: ReSTIRDIReservoir add_one_candidate / combine_with / end / end_with_normalization
 *     (src/Device/includes/ReSTIR/DI/Reservoir.h:54-121);
 *   - target function: ReSTIR_DI_evaluate_target_function (src/Device/includes/ReSTIR/DI/
 *     TargetFunction.h:49-96), luminance(f * Le * cos * cos_light / d^2), optional shadow ray;
 *   - initial candidates: sample_light_candidates / sample_bsdf_candidates / end, M = 1, then the
 *     visibility-reuse kill (src/Device/kernels/ReSTIR/DI/InitialCandidates.h:180-538,
 *     src/Device/includes/ReSTIR/Utils.h:25-64);
 *   - temporal reuse with pairwise MIS and confidence weights (TemporalReuse.h:50-298,
 *     src/Device/includes/ReSTIR/TemporalMISWeight.h:164-250, UtilsTemporal.h:27-98);
 *   - spatial reuse with pairwise MIS and confidence weights (SpatialReuse.h:43-322,
 *     SpatialMISWeight.h:100-160, UtilsSpatial.h:77-220, NeighborSimilarity.h:34-84);
 *   - final shading of the reservoir (src/Device/includes/ReSTIR/DI/FinalShading.h:13-85).
 * Random numbers, rng_mode 0: one PCG32 stream per pixel and pass, pcg_seed(pixel, frame * 16 +
 * pass, seed) with pass 1 = initial, 2 = temporal, 3 + p = spatial pass p; each BSDF sample is
 * seeded with one 32-bit draw; spatial neighbour offsets from a Xorshift32 seeded per frame and
 * pass for all pixels. These are the GPU kernels' streams (hiprt-path-tracer_gb300/csrc/
 * restir.cu), so the oracle and the kernels select the same samples.
 * rng_mode 1 (the reference's generator and draw order): each pass seeds a Xorshift32 per pixel
 * with wang_hash((pixel + 1) (sample + 1) random_number) from its own random number
 * (InitialCandidates.h:500-505, TemporalReuse.h:69-74, SpatialReuse.h:62-69); a light candidate
 * first draws the envmap-or-light choice (sample_fresh_light_candidate, InitialCandidates.h:100);
 * BSDF samples draw from the pixel's generator; a spatial pass seeds each pixel's neighbour
 * generator with one draw of the pixel's (setup_adaptive_directional_spatial_reuse,
 * UtilsSpatial.h:17-22); the G-buffer holds octahedral 24-bit normals and the packed camera-hit
 * materials (offset 'gbuffer_materials' in the material table); the temporal heuristics compare
 * against the centre's shading normal (TemporalReuse.h:81-82) and a previous-frame surface's view
 * direction runs from the previous camera to the CURRENT frame's hit point of that pixel
 * (get_pixel_surface_previous_frame, src/Device/includes/ReSTIR/Surface.h:52).
 * Reservoir record: 8 words per pixel (point xyz, p_hat, triangle, (M << 9) | flags, w_sum, UCW).
 */
#include <atomic>
#include <thread>
#include <vector>

#include "orc_common.h"

namespace {

constexpr int kUnoccluded = 1 << 7;
constexpr int kLobeMask = 0x7E;

struct Res
{
    V point = mk(0, 0, 0);
    float p_hat = 0.0f;
    int tri = -1;
    int flags = 0;
    int M = 0;
    float w_sum = 0.0f;
    float ucw = 0.0f;
};

Res load_res(const float* b, int i)
{
    const float* p = b + 8 * (size_t)i;
    Res r;
    r.point = mk(p[0], p[1], p[2]);
    r.p_hat = p[3];
    int32_t t, mf;
    std::memcpy(&t, p + 4, 4);
    std::memcpy(&mf, p + 5, 4);
    r.tri = t;
    r.flags = mf & 0x1FF;
    r.M = (int)((uint32_t)mf >> 9);
    r.w_sum = p[6];
    r.ucw = p[7];
    return r;
}

void store_res(float* b, int i, const Res& r)
{
    float* p = b + 8 * (size_t)i;
    p[0] = r.point.x;
    p[1] = r.point.y;
    p[2] = r.point.z;
    p[3] = r.p_hat;
    int32_t t = r.tri, mf = (r.M << 9) | (r.flags & 0x1FF);
    std::memcpy(p + 4, &t, 4);
    std::memcpy(p + 5, &mf, 4);
    p[6] = r.w_sum;
    p[7] = r.ucw;
}

struct Xor32
{
    uint32_t s;
    uint32_t u32()
    {
        uint32_t x = s;
        x ^= x << 13;
        x ^= x >> 17;
        x ^= x << 5;
        return s = x;
    }
    float next() { return std::min((float)u32() * (1.0f / 4294967296.0f), 1.0f - 1.0e-7f); }
};

struct RSettings
{
    int width, height, seed, frame, has_prev, light_strategy;
    int n_light, n_bsdf, visibility_reuse, do_temporal, temporal_search, spatial_passes, spatial_neighbors, m_cap,
        confidence, bias_vis;
    float temporal_radius, spatial_radius, normal_cos, plane_dist;
    float cam[3], prev_cam[3];
    const float* prev_vp;
    // light presampling (presampled null: off): records of 8 floats (point, triangle bits,
    // normal, area pdf), 'subsets' x 'size' of them; tiles of 'tile' pixels share a subset
    const float* presampled = nullptr;
    int subsets = 0, size = 0, tile = 8;
    uint32_t presample_seed = 0;
    // rng_mode 1: the reference's per-pass random numbers (HIPRTRenderData::random_number)
    int rng_mode = 0;
    uint32_t sample_number = 0, rn_initial = 0, rn_temporal = 0, rn_spatial[4] = {0, 0, 0, 0};
    int gbuffer_materials = 0;  // offset of the packed camera-hit materials in the material table
};

struct Surf
{
    V P, ns, ng, view;
    int prim, mat;
    bool inside;
};

Surf load_surf(const float* gb, int i, const float* cam)
{
    const float* p = gb + 12 * (size_t)i;
    Surf s;
    s.P = mk(p[0], p[1], p[2]);
    std::memcpy(&s.prim, p + 3, 4);
    s.ns = mk(p[4], p[5], p[6]);
    std::memcpy(&s.mat, p + 7, 4);
    s.ng = mk(p[8], p[9], p[10]);
    int32_t ins;
    std::memcpy(&ins, p + 11, 4);
    s.inside = ins != 0;
    s.view = nrm(mk(cam[0], cam[1], cam[2]) - s.P);
    return s;
}

struct Ctx
{
    const Scene& s;
    const PScene& ps;
    const RSettings& st;
};

V tri_normal(const Scene& s, int t) { return nrm(cross(s.b(t) - s.a(t), s.c(t) - s.a(t))); }

float eta_in(const Surf& su, const float* m) { return su.inside ? m[37] : 1.0f; }
float eta_out(const Surf& su, const float* m) { return su.inside ? 1.0f : m[37]; }

const float* surf_mat(const Ctx& c, const Surf& su) { return c.ps.mat(su.mat + c.st.gbuffer_materials); }

V bsdf_eval(const Ctx& c, const Surf& su, V l, int lobe, float& pdf)
{
    const float* m = surf_mat(c, su);
    float q[16], out[4];
    make_query(q, su.view, su.ns, su.ng, l, eta_in(su, m), eta_out(su, m), su.inside, lobe);
    c.ps.eval(m, q, out);
    pdf = out[3];
    return mk(out[0], out[1], out[2]);
}

float target(const Ctx& c, const Surf& su, V point, int tri, int flags, bool vis)
{
    if (tri < 0) return 0.0f;
    V dir = point - su.P;
    float dist = len(dir);
    dir = dir / dist;
    float cosine = dot(su.ns, dir);
    if (cosine <= 0.0f) return 0.0f;
    float pdf;
    V f = bsdf_eval(c, su, dir, flags & kLobeMask, pdf);
    float G = std::max(0.0f, dot(tri_normal(c.s, tri), neg(dir))) / (dist * dist);
    float p = lum(f * c.s.emi(tri) * cosine * G);
    if (p == 0.0f) return 0.0f;
    if (vis && occluded(c.s, su.P, dir, su.prim, dist - 1.0e-4f)) return 0.0f;
    return p;
}

void add_candidate(Res& r, V point, int tri, int flags, float p_hat, float weight, float u)
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

bool combine(Res& r, const Res& o, float mis, float p_hat, Pcg& rng)
{
    if (o.ucw <= 0.0f)
    {
        r.M += o.M;
        return false;
    }
    float w = mis * p_hat * o.ucw * 1.0f;
    r.M += o.M;
    r.w_sum += w;
    if (rng.next() < w / r.w_sum)
    {
        r.point = o.point;
        r.tri = o.tri;
        r.flags = o.flags;
        r.p_hat = p_hat;
        return true;
    }
    return false;
}

void end_norm(Res& r)
{
    if (r.w_sum == 0.0f || r.w_sum < 1.0e-10f || r.w_sum > 1.0e10f)
        r.ucw = 0.0f;
    else
        r.ucw = 1.0f / r.p_hat * r.w_sum * 1.0f / 1.0f;
    r.M = std::min(r.M, 1000000);
}

void visibility_kill(const Ctx& c, Res& r, const Surf& su)
{
    if (r.ucw <= 0.0f && r.w_sum <= 0.0f) return;
    if (r.flags & kUnoccluded) return;
    V dir = r.point - su.P;
    float dist = len(dir);
    dir = dir / dist;
    if (occluded(c.s, su.P, dir, su.prim, dist - 1.0e-4f))
        r.ucw = -1.0f;
    else
        r.flags |= kUnoccluded;
}

Pcg stream(const RSettings& st, int pixel, int pass)
{
    if (st.rng_mode)
    {
        const uint32_t rn = pass == 1 ? st.rn_initial : pass == 2 ? st.rn_temporal : st.rn_spatial[(pass - 3) & 3];
        return parity_seed((uint32_t)pixel, st.sample_number, rn);
    }
    return pcg_seed((uint32_t)pixel, (uint32_t)st.frame * 16u + (uint32_t)pass, (uint32_t)st.seed);
}

// emissive-triangle light sample, as the path-tracing oracle draws it
struct LS
{
    V point, normal, emission;
    float pdf_area;
    int tri;
};

LS sample_light(const Scene& s, int strategy, Pcg& rng)
{
    int e;
    if (strategy == 1)
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
    LS ls;
    ls.tri = lt;
    ls.point = la + ab * r1 + ac * r2;
    ls.normal = n / ln;
    float area = 0.5f * ln;
    ls.emission = s.emi(lt);
    ls.pdf_area = light_pdf_area(s, lt, area, ls.emission, strategy);
    return ls;
}

// Light presampling (ReSTIR_DI_LightsPresampling, src/Device/kernels/ReSTIR/DI/
// LightsPresampling.h:74-109): record i is a light sample from its own PCG stream
// pcg_seed(i, frame, seed ^ 0x5BD1E995), as the GPU kernel draws it.
void presample(const Scene& s, int strategy, int n, uint32_t frame, uint32_t seed, float* out)
{
    for (int i = 0; i < n; i++)
    {
        Pcg rng = pcg_seed((uint32_t)i, frame, seed ^ 0x5BD1E995u);
        LS ls = sample_light(s, strategy, rng);
        float* o = out + 8 * (size_t)i;
        o[0] = ls.point.x; o[1] = ls.point.y; o[2] = ls.point.z;
        std::memcpy(o + 3, &ls.tri, 4);
        o[4] = ls.normal.x; o[5] = ls.normal.y; o[6] = ls.normal.z;
        o[7] = ls.pdf_area;
    }
}

// the frame's subset for the tile of pixel (x, y) (use_presampled_light_candidate,
// InitialCandidates.h:33-69): Cantor pairing of the tile coordinates scales the frame's seed
int presampled_subset(const RSettings& st, int x, int y)
{
    const uint32_t tx = (uint32_t)(x / st.tile), ty = (uint32_t)(y / st.tile);
    const uint32_t cantor = (tx + ty + 1u) * (tx + ty) / 2u + ty;
    uint32_t seed = st.presample_seed * (cantor + 1u);
    if (seed == 0u) seed = 0x9E3779B9u;
    Xor32 xr{seed};
    const int i = (int)(xr.next() * (float)st.subsets);
    return std::min(i, st.subsets - 1);
}

Res initial_pixel(const Ctx& c, const float* gb, int pixel)
{
    Res r;
    const Surf su = load_surf(gb, pixel, c.st.cam);
    if (su.prim < 0 || c.s.ne == 0) return r;
    Pcg rng = stream(c.st, pixel, 1);
    const float* m = surf_mat(c, su);
    const float nl = (float)c.st.n_light, nb = (float)c.st.n_bsdf;
    const int subset = c.st.presampled ? presampled_subset(c.st, pixel % c.st.width, pixel / c.st.width) : 0;
    for (int k = 0; k < c.st.n_light; k++)
    {
        LS ls;
        if (c.st.presampled)
        {
            const int e = subset * c.st.size + rng.index(c.st.size);
            const float* p = c.st.presampled + 8 * (size_t)e;
            ls.point = mk(p[0], p[1], p[2]);
            std::memcpy(&ls.tri, p + 3, 4);
            ls.normal = mk(p[4], p[5], p[6]);
            ls.pdf_area = p[7];
            ls.emission = c.s.emi(ls.tri);
        }
        else
        {
            if (c.st.rng_mode) rng.next();  // the envmap-or-light draw (no envmap: a light)
            ls = sample_light(c.s, c.st.light_strategy, rng);
        }
        V wi = ls.point - su.P;
        float dist = len(wi);
        wi = wi / dist;
        float cosine = std::max(0.0f, dot(su.ns, wi));
        float weight = 0.0f, p_hat = 0.0f;
        if (cosine > 0.0f && ls.pdf_area > 0.0f)
        {
            float bpdf;
            V f = bsdf_eval(c, su, wi, 0, bpdf);
            if (bpdf > 0.0f)
            {
                float cl = std::max(0.0f, dot(ls.normal, neg(wi)));
                // the reference's candidate carries ReSTIR_DI_evaluate_target_function's value
                p_hat = c.st.rng_mode ? target(c, su, ls.point, ls.tri, 0, false)
                                      : lum(f * ls.emission * dot(su.ns, wi) * (cl / (dist * dist)));
                float lpdf = a2s(ls.pdf_area, dist, cl);
                float mis = lpdf == 0.0f ? 0.0f : lpdf / (nl * lpdf + nb * bpdf);
                weight = mis * p_hat / ls.pdf_area;
            }
        }
        add_candidate(r, ls.point, ls.tri, 0, p_hat, weight, rng.next());
    }
    for (int k = 0; k < c.st.n_bsdf; k++)
    {
        float q[16], out[8];
        make_query(q, su.view, su.ns, su.ng, mk(0, 0, 0), eta_in(su, m), eta_out(su, m), su.inside, 0);
        int32_t lobe;
        c.ps.sample(m, q, bsdf_seed(rng), out, &lobe);
        bsdf_seed_done(rng, out);
        float pdf = out[6];
        if (!(pdf > 0.0f)) continue;
        V dir = mk(out[0], out[1], out[2]);
        float t;
        int lt = closest(c.s, su.P, dir, su.prim, t);
        if (lt < 0 || !(t < 1.0e35f - 1.0e-4f)) continue;
        V Le = c.s.emi(lt);
        if (black(Le)) continue;
        V point = su.P + dir * t;
        int flags = kUnoccluded | (lobe & kLobeMask);
        float p_hat = target(c, su, point, lt, flags, false);
        float cl = std::max(0.0f, dot(tri_normal(c.s, lt), neg(dir)));
        float lpdf = 0.0f;
        if (!(dot(dir, su.ns) < 0.0f))
        {
            float area = 0.5f * len(cross(c.s.b(lt) - c.s.a(lt), c.s.c(lt) - c.s.a(lt)));
            lpdf = a2s(light_pdf_area(c.s, lt, area, Le, c.st.light_strategy), t, cl);
        }
        float mis = pdf / (nb * pdf + nl * lpdf);
        float pdf_area = pdf / (t * t) * cl;
        if (!(pdf_area > 0.0f)) continue;
        add_candidate(r, point, lt, flags, p_hat, mis * p_hat / pdf_area, rng.next());
    }
    r.ucw = r.w_sum == 0.0f ? 0.0f : 1.0f / r.p_hat * r.w_sum;
    r.M = 1;
    if (c.st.visibility_reuse) visibility_kill(c, r, su);
    return r;
}

bool similar(const float* gb_pos, const float* gb_cur, int n_idx, int c_idx, V P, V nc, const RSettings& st)
{
    if (n_idx == c_idx) return true;
    const float* p = gb_pos + 12 * (size_t)n_idx;
    int32_t prim;
    std::memcpy(&prim, p + 3, 4);
    if (prim < 0) return false;
    if (!(std::fabs(dot(mk(p[0], p[1], p[2]) - P, nc)) < st.plane_dist)) return false;
    const float* g = gb_cur + 12 * (size_t)n_idx + 8;
    return dot(nc, mk(g[0], g[1], g[2])) > st.normal_cos;
}

Res temporal_pixel(const Ctx& c, const float* gb, const float* gb_prev, const float* initial, const float* prev, int pixel)
{
    const Res init = load_res(initial, pixel);
    const Surf su = load_surf(gb, pixel, c.st.cam);
    if (su.prim < 0 || !c.st.has_prev) return init;
    Pcg rng = stream(c.st, pixel, 2);
    const int W = c.st.width, H = c.st.height;
    V ndc = mat_point(c.st.prev_vp, su.P);
    float px = (ndc.x + 1.0f) * 0.5f * (float)W - 0.5f;
    float py = (ndc.y + 1.0f) * 0.5f * (float)H - 0.5f;
    int t_idx = -1;
    for (int i = 0; i < c.st.temporal_search + 1; i++)
    {
        float ox = 0.0f, oy = 0.0f;
        if (i > 0)
        {
            ox = (rng.next() - 0.5f) * c.st.temporal_radius;
            oy = (rng.next() - 0.5f) * c.st.temporal_radius;
        }
        int tx = (int)std::round(px + ox), ty = (int)std::round(py + oy);
        if (tx < 0 || tx >= W || ty < 0 || ty >= H) continue;
        t_idx = tx + ty * W;
        if (similar(gb_prev, gb, t_idx, pixel, su.P, c.st.rng_mode ? su.ns : su.ng, c.st)) break;
        t_idx = -1;
    }
    if (t_idx < 0) return init;
    const Res tn = load_res(prev, t_idx);
    Surf ts = load_surf(gb_prev, t_idx, c.st.prev_cam);
    if (c.st.rng_mode)
    {
        const float* pc = gb + 12 * (size_t)t_idx;
        ts.view = nrm(mk(c.st.prev_cam[0], c.st.prev_cam[1], c.st.prev_cam[2]) - mk(pc[0], pc[1], pc[2]));
    }
    if (tn.M == 0 || ts.prim < 0 || !black(mk(c.s.emission[3 * ts.mat], c.s.emission[3 * ts.mat + 1], c.s.emission[3 * ts.mat + 2])))
        return init;
    const bool vis = c.st.bias_vis != 0;
    Res o;
    float t_at_center = tn.ucw > 0.0f ? target(c, su, tn.point, tn.tri, tn.flags, vis) : 0.0f;
    float tM = c.st.confidence ? (float)tn.M : 1.0f;
    float cM = c.st.confidence ? (float)init.M : 1.0f;
    float nsum = c.st.confidence ? (float)tn.M : 1.0f;
    float denom = tn.p_hat * nsum + t_at_center * cM;
    float mi = denom == 0.0f ? 0.0f : tn.p_hat * tM / denom;
    float c_at_n = target(c, ts, init.point, init.tri, init.flags, vis);
    float denom_mc = c_at_n * nsum + init.p_hat * cM;
    float mc = 0.0f;
    if (denom_mc != 0.0f) mc += init.p_hat * cM / denom_mc * (c.st.confidence ? tM / nsum : 1.0f);
    if (combine(o, tn, mi, t_at_center, rng))
    {
        if (vis)
            o.flags |= kUnoccluded;
        else
            o.flags &= ~kUnoccluded;
    }
    if (combine(o, init, mc == 0.0f ? 1.0f : mc, init.p_hat, rng))
    {
        if (vis)
            o.flags |= kUnoccluded;
        else
            o.flags |= init.flags & kUnoccluded;
    }
    end_norm(o);
    if (c.st.m_cap > 0) o.M = std::min(o.M, c.st.m_cap);
    return o;
}

int spatial_neighbor(int j, int K, int cx, int cy, int W, int H, float radius, Xor32& nr)
{
    if (j == K) return cx + cy * W;
    float u = nr.next();
    float v = nr.next();
    float r = radius * std::sqrt(v);
    float ang = 6.28318530717958647693f * u;
    int nx = cx + (int)std::round(r * std::cos(ang)), ny = cy + (int)std::round(r * std::sin(ang));
    if (nx < 0 || nx >= W || ny < 0 || ny >= H) return -1;
    return nx + ny * W;
}

Res spatial_pixel(const Ctx& c, const float* gb, const float* in, int pixel, int pass, int last_pass, uint32_t seed)
{
    const Surf su = load_surf(gb, pixel, c.st.cam);
    const Res center = load_res(in, pixel);
    if (su.prim < 0) return center;
    Pcg rng = stream(c.st, pixel, 3 + pass);
    if (c.st.rng_mode) seed = rng.u32();  // the pixel's neighbour generator seed
    const int W = c.st.width, H = c.st.height, K = c.st.spatial_neighbors;
    const int cx = pixel % W, cy = pixel / W;
    Xor32 nr{seed};
    int valid = 0, m_sum = 0;
    uint32_t cache = 0;
    for (int j = 0; j < K; j++)
    {
        int idx = spatial_neighbor(j, K, cx, cy, W, H, c.st.spatial_radius, nr);
        if (idx < 0) continue;
        if (!similar(gb, gb, idx, pixel, su.P, su.ng, c.st)) continue;
        m_sum += load_res(in, idx).M;
        valid++;
        cache |= 1u << j;
    }
    const bool vis = c.st.bias_vis != 0;
    const bool update_mc = center.M > 0 && center.ucw > 0.0f;
    const float cM = c.st.confidence ? (float)center.M : 1.0f;
    const float nsum = c.st.confidence ? (float)m_sum : 1.0f;
    const float div = c.st.confidence ? 1.0f : (float)valid;
    float mc = 0.0f;
    Res o;
    nr = Xor32{seed};
    for (int j = m_sum == 0 ? K : 0; j < K + 1; j++)
    {
        if (j < K && !(cache & (1u << j)))
        {
            nr.next();
            nr.next();
            continue;
        }
        int idx = spatial_neighbor(j, K, cx, cy, W, H, c.st.spatial_radius, nr);
        if (idx < 0) continue;
        const Res nb = load_res(in, idx);
        float t_at_center = 0.0f;
        if (nb.ucw > 0.0f) t_at_center = j == K ? nb.p_hat : target(c, su, nb.point, nb.tri, nb.flags, false);
        float mis;
        if (j < K)
        {
            float rM = c.st.confidence ? (float)nb.M : 1.0f;
            float denom = nb.p_hat * nsum + t_at_center / div * cM;
            float mi = denom == 0.0f ? 0.0f : nb.p_hat * rM / denom;
            if (update_mc)
            {
                const Surf nsu = load_surf(gb, idx, c.st.cam);
                float c_at_n = target(c, nsu, center.point, center.tri, center.flags, vis);
                float nume_mc = center.p_hat / div * cM;
                float denom_mc = c_at_n * nsum + center.p_hat / div * cM;
                float conf = c.st.confidence ? (nsum == 0.0f ? 0.0f : rM / nsum) : 1.0f;
                if (denom_mc != 0.0f) mc += nume_mc / denom_mc / div * conf;
            }
            mis = mi / div;
        }
        else
            mis = mc == 0.0f ? 1.0f : mc;
        if (combine(o, nb, mis, t_at_center, rng))
        {
            if (j == K)
                o.flags |= nb.flags & kUnoccluded;
            else
                o.flags &= ~kUnoccluded;
        }
    }
    end_norm(o);
    if (c.st.visibility_reuse && vis && (c.st.do_temporal || pass != last_pass)) visibility_kill(c, o, su);
    if (c.st.m_cap > 0) o.M = std::min(o.M, c.st.m_cap);  // SpatialReuse.h:317-319
    return o;
}

// Fused spatiotemporal reuse (ReSTIR_DI_SpatiotemporalReuse, src/Device/kernels/ReSTIR/DI/
// FusedSpatiotemporalReuse.h:152-566; pairwise MIS SpatiotemporalMISWeight.h:140-224): one pass
// that resamples the temporal neighbour, then K spatial neighbours taken from the PREVIOUS frame's
// final reservoirs around the backprojected position (positions for the heuristics and surfaces
// for the MIS terms from the previous G-buffer), then the canonical initial reservoir. The
// temporal neighbour counts as one more neighbour of the pairwise MIS set (its M joins the
// confidence sum). Neighbour offsets come from a Xorshift32 stream seeded per pixel by one draw of
// the pixel's stream (the reference seeds it per pixel in this pass); visibility reuse on the
// output; M-cap. As in the reference's fused kernel, an emissive temporal neighbour is resampled.
Res spatiotemporal_pixel(const Ctx& c, const float* gb, const float* gb_prev, const float* initial, const float* prev,
                         int pixel)
{
    const Res init = load_res(initial, pixel);
    const Surf su = load_surf(gb, pixel, c.st.cam);
    if (su.prim < 0 || !c.st.has_prev) return init;
    Pcg rng = stream(c.st, pixel, 2);
    uint32_t nseed = rng.u32();
    if (nseed == 0u) nseed = 0x9E3779B9u;
    const int W = c.st.width, H = c.st.height, K = c.st.spatial_neighbors;
    V ndc = mat_point(c.st.prev_vp, su.P);
    float px = (ndc.x + 1.0f) * 0.5f * (float)W - 0.5f;
    float py = (ndc.y + 1.0f) * 0.5f * (float)H - 0.5f;
    const int tx0 = (int)std::round(px), ty0 = (int)std::round(py);
    int t_idx = -1;
    for (int i = 0; i < c.st.temporal_search + 1; i++)
    {
        float ox = 0.0f, oy = 0.0f;
        if (i > 0)
        {
            ox = (rng.next() - 0.5f) * c.st.temporal_radius;
            oy = (rng.next() - 0.5f) * c.st.temporal_radius;
        }
        int tx = (int)std::round(px + ox), ty = (int)std::round(py + oy);
        if (tx < 0 || tx >= W || ty < 0 || ty >= H) continue;
        t_idx = tx + ty * W;
        if (similar(gb_prev, gb, t_idx, pixel, su.P, su.ng, c.st)) break;
        t_idx = -1;
    }
    Res tn;
    if (t_idx >= 0) tn = load_res(prev, t_idx);
    const bool t_ok = t_idx >= 0 && tn.M > 0;
    // valid spatial neighbours and their confidence
    Xor32 nr{nseed};
    int valid = 0, m_sum = 0;
    uint32_t cache = 0;
    for (int j = 0; j < K; j++)
    {
        int idx = spatial_neighbor(j, K, tx0, ty0, W, H, c.st.spatial_radius, nr);
        if (idx < 0) continue;
        if (!similar(gb_prev, gb, idx, pixel, su.P, su.ng, c.st)) continue;
        m_sum += load_res(prev, idx).M;
        valid++;
        cache |= 1u << j;
    }
    if (t_ok)
    {
        valid++;
        m_sum += tn.M;
    }
    const bool vis = c.st.bias_vis != 0;
    const bool update_mc = init.M > 0 && init.ucw > 0.0f;
    const float cM = c.st.confidence ? (float)init.M : 1.0f;
    const float nsum = c.st.confidence ? (float)m_sum : 1.0f;
    const float div = c.st.confidence ? 1.0f : (float)valid;
    float mc = 0.0f;
    // pairwise MIS weight of a neighbour reservoir, accumulating the canonical weight
    auto pairwise = [&](const Res& nb, float t_at_center, const Surf& nsu) {
        float rM = c.st.confidence ? (float)nb.M : 1.0f;
        float denom = nb.p_hat * nsum + t_at_center / div * cM;
        float mi = denom == 0.0f ? 0.0f : nb.p_hat * rM / denom;
        if (update_mc)
        {
            float c_at_n = target(c, nsu, init.point, init.tri, init.flags, vis);
            float nume_mc = init.p_hat / div * cM;
            float denom_mc = c_at_n * nsum + init.p_hat / div * cM;
            float conf = c.st.confidence ? (nsum == 0.0f ? 0.0f : rM / nsum) : 1.0f;
            if (denom_mc != 0.0f) mc += nume_mc / denom_mc / div * conf;
        }
        return mi / div;
    };
    Res o;
    if (t_ok)
    {
        const float t_at_center = tn.ucw > 0.0f ? target(c, su, tn.point, tn.tri, tn.flags, vis) : 0.0f;
        const float mis = pairwise(tn, t_at_center, load_surf(gb_prev, t_idx, c.st.prev_cam));
        if (combine(o, tn, mis, t_at_center, rng))
        {
            if (vis)
                o.flags |= kUnoccluded;
            else
                o.flags &= ~kUnoccluded;
        }
    }
    nr = Xor32{nseed};
    for (int j = m_sum == 0 ? K : 0; j < K + 1; j++)
    {
        if (j < K && !(cache & (1u << j)))
        {
            nr.next();
            nr.next();
            continue;
        }
        const int idx = j == K ? pixel : spatial_neighbor(j, K, tx0, ty0, W, H, c.st.spatial_radius, nr);
        if (idx < 0) continue;
        const Res nb = j == K ? init : load_res(prev, idx);
        float t_at_center = 0.0f;
        if (nb.ucw > 0.0f) t_at_center = j == K ? nb.p_hat : target(c, su, nb.point, nb.tri, nb.flags, false);
        const float mis = j < K ? pairwise(nb, t_at_center, load_surf(gb_prev, idx, c.st.prev_cam)) : (mc == 0.0f ? 1.0f : mc);
        if (combine(o, nb, mis, t_at_center, rng))
        {
            if (j == K)
                o.flags |= nb.flags & kUnoccluded;
            else
                o.flags &= ~kUnoccluded;
        }
    }
    end_norm(o);
    if (c.st.visibility_reuse && vis) visibility_kill(c, o, su);
    if (c.st.m_cap > 0) o.M = std::min(o.M, c.st.m_cap);
    return o;
}

template <typename F>
void parallel_pixels(int n, int nthreads, F f)
{
    if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
    std::atomic<int> next{0};
    std::vector<std::thread> pool;
    for (int w = 0; w < nthreads; w++)
        pool.emplace_back([&]() {
            for (;;)
            {
                int p = next.fetch_add(1);
                if (p >= n) break;
                f(p);
            }
        });
    for (auto& t : pool) t.join();
}

RSettings settings_from(const int* si, const float* sf, const float* prev_vp)
{
    RSettings st;
    st.width = si[0];
    st.height = si[1];
    st.seed = si[2];
    st.frame = si[3];
    st.has_prev = si[4];
    st.light_strategy = si[5];
    st.n_light = si[6];
    st.n_bsdf = si[7];
    st.visibility_reuse = si[8];
    st.do_temporal = si[9];
    st.temporal_search = si[10];
    st.spatial_passes = si[11];
    st.spatial_neighbors = si[12];
    st.m_cap = si[13];
    st.confidence = si[14];
    st.bias_vis = si[15];
    st.temporal_radius = sf[0];
    st.spatial_radius = sf[1];
    st.normal_cos = sf[2];
    st.plane_dist = sf[3];
    for (int k = 0; k < 3; k++)
    {
        st.cam[k] = sf[4 + k];
        st.prev_cam[k] = sf[7 + k];
    }
    st.prev_vp = prev_vp;
    // settings_i[16..24]: rng mode, sample number, the initial / temporal / spatial passes' random
    // numbers (rng mode 1), the offset of the packed camera-hit materials
    st.rng_mode = si[16];
    st.sample_number = (uint32_t)si[17];
    st.rn_initial = (uint32_t)si[18];
    st.rn_temporal = (uint32_t)si[19];
    for (int k = 0; k < 4; k++) st.rn_spatial[k] = (uint32_t)si[20 + k];
    st.gbuffer_materials = si[24];
    return st;
}

}  // namespace

extern "C" {

/* G-buffer of the camera hits (12 floats per pixel: P, prim bits, ns, material bits, ng, inside
 * bits), with the GPU camera's jitter stream pcg_seed(pixel, frame, seed); with rng_mode 1, the
 * reference's camera pass instead (Xorshift32 seeded by wang_hash((pixel + 1) (frame + 1)
 * random_number), CameraRays.h:155-170) and its packed normals (octahedral 24 bits, written at
 * CameraRays.h:178-201). */
void orc_restir_gbuffer(const float* tri_verts, int n_tris, const int* mat_of, const float* pmats, int width, int height,
                        int seed, int frame, int jitter, const float* inv_view, const float* inv_proj, float* gb, int nthreads,
                        int rng_mode, uint32_t random_number)
{
    Scene s{tri_verts, n_tris, mat_of, nullptr, nullptr, nullptr, 0, nullptr, nullptr, 0.0f};
    parallel_pixels(width * height, nthreads, [&](int pixel) {
        const int x = pixel % width, y = pixel / width;
        Pcg rng = rng_mode ? parity_seed((uint32_t)pixel, (uint32_t)frame, random_number)
                           : pcg_seed((uint32_t)pixel, (uint32_t)frame, (uint32_t)seed);
        float px = x + 0.5f, py = y + 0.5f;
        if (jitter)
        {
            px += rng.next() - 0.5f;
            py += rng.next() - 0.5f;
        }
        float xn = px / width * 2.0f - 1.0f, yn = py / height * 2.0f - 1.0f;
        V o = mat_point(inv_view, mk(0, 0, 0));
        V pv = mat_point(inv_proj, mk(xn, yn, -1.0f));
        V pw = mat_point(inv_view, pv);
        V d = nrm(pw - o);
        float t;
        int prim = closest(s, o, d, -1, t);
        float* g = gb + 12 * (size_t)pixel;
        std::memset(g, 0, 48);
        int32_t pb = prim;
        std::memcpy(g + 3, &pb, 4);
        if (prim < 0) return;
        V P = o + d * t;
        V ng_raw = nrm(cross(s.b(prim) - s.a(prim), s.c(prim) - s.a(prim)));
        V ng = ng_raw, ns = ng_raw, view = neg(d);
        if (dot(view, ng) < 0.0f) { ng = neg(ng); ns = neg(ns); }
        if (dot(view, ns) < 0.0f) ns = neg(ns);
        V refl = ns * (2.0f * dot(view, ns)) - view;
        if (dot(refl, ng) <= 0.0f)
        {
            refl = refl - nrm(ng * (dot(refl, ng) - 0.01f));
            ns = nrm(view + refl);
        }
        if (rng_mode)
        {
            ns = oct24(ns);
            ng = oct24(ng);
        }
        const int mi = mat_of[prim];
        // the camera hit enters its material from the air: the reference rebuilds the surface's
        // volume state by pushing the hit material on a fresh stack (ReSTIR/Surface.h:31)
        int32_t inside = 0;
        g[0] = P.x; g[1] = P.y; g[2] = P.z;
        g[4] = ns.x; g[5] = ns.y; g[6] = ns.z;
        int32_t mb = mi;
        std::memcpy(g + 7, &mb, 4);
        g[8] = ng.x; g[9] = ng.y; g[10] = ng.z;
        std::memcpy(g + 11, &inside, 4);
    });
}

/* One ReSTIR DI pass over all pixels. pass: 0 = initial (out <- candidates), 1 = temporal
 * (in = initial, prev = previous final reservoirs, gb_prev = previous G-buffer), 2 = spatial pass
 * 'spatial_index' (in -> out) with the given neighbour seed, 3 = fused spatiotemporal (in =
 * initial, prev = previous final reservoirs, gb_prev = previous G-buffer).
 * presampled (NULL: off): light presampling records (orc_restir_presample) with presample_i =
 * subsets, subset size, tile size, the frame's subset seed (bits).
 * settings_i (25): width, height, seed, frame, has_prev, light strategy (0 uniform, 1 power), light
 *   candidates, bsdf candidates, visibility reuse, do temporal, temporal search count, spatial
 *   passes, spatial neighbours, m cap, confidence weights, bias-correction visibility, rng mode,
 *   sample number, random numbers of the initial / temporal / spatial passes 0..3, offset of the
 *   packed camera-hit materials.
 * settings_f: temporal radius, spatial radius, normal cos, plane distance, camera pos xyz,
 *   previous camera pos xyz. */
void orc_restir_pass(int pass, const float* tri_verts, int n_tris, const int* mat_of, const float* emission,
                     const int* emissive, int n_emissive, const float* alias_prob, const int* alias_idx, float power_sum,
                     const float* pmats, void* eval_fn, void* sample_fn, const int* settings_i, const float* settings_f,
                     const float* prev_vp, const float* gb, const float* gb_prev, const float* in, const float* prev,
                     float* out, int spatial_index, uint32_t spatial_seed, int nthreads, const float* presampled,
                     const int* presample_i)
{
    Scene s{tri_verts, n_tris, mat_of, nullptr, emission, emissive, n_emissive, alias_prob, alias_idx, power_sum};
    PScene ps{pmats, (bsdf_eval_fn)eval_fn, (bsdf_sample_fn)sample_fn};
    RSettings st = settings_from(settings_i, settings_f, prev_vp);
    if (presampled)
    {
        st.presampled = presampled;
        st.subsets = presample_i[0];
        st.size = presample_i[1];
        st.tile = presample_i[2];
        st.presample_seed = (uint32_t)presample_i[3];
    }
    Ctx c{s, ps, st};
    const int n = st.width * st.height;
    parallel_pixels(n, nthreads, [&](int pixel) {
        Res r;
        if (pass == 0)
            r = initial_pixel(c, gb, pixel);
        else if (pass == 1)
            r = temporal_pixel(c, gb, gb_prev, in, prev, pixel);
        else if (pass == 3)
            r = spatiotemporal_pixel(c, gb, gb_prev, in, prev, pixel);
        else
            r = spatial_pixel(c, gb, in, pixel, spatial_index, st.spatial_passes - 1, spatial_seed);
        store_res(out, pixel, r);
    });
}

/* Light presampling records of a frame: n = subsets * size records of 8 floats. */
void orc_restir_presample(const float* tri_verts, int n_tris, const int* mat_of, const float* emission,
                          const int* emissive, int n_emissive, const float* alias_prob, const int* alias_idx,
                          float power_sum, int strategy, int n, uint32_t frame, uint32_t seed, float* out)
{
    Scene s{tri_verts, n_tris, mat_of, nullptr, emission, emissive, n_emissive, alias_prob, alias_idx, power_sum};
    presample(s, strategy, n, frame, seed, out);
}

}  // extern "C"
