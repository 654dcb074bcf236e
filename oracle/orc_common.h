/*
 * TEST INFRASTRUCTURE ONLY — helpers shared by the CPU oracles (pt_oracle.cpp, restir_oracle.cpp):
 * float3 math, the PCG32 streams the GPU kernels use, the pinhole camera, brute-force
 * Moller-Trumbore intersection with the self-hit filter (src/Renderer/Triangle.h:20-63), light
 * pdfs, and the callback interface to the reference's principled BSDF. Compiled with
 * -ffp-contract=off.
 */
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

// The scene accelerator of the path-tracing and ReSTIR oracles, shared by their translation units
// (defined in trace_oracle.cpp)
extern "C" void* orc_scene_accel();
extern "C" int32_t orc_octree_closest_one(void* h, const float* o, const float* d, int32_t skip, float* t_out);

namespace {


struct V { float x, y, z; };
inline V mk(float x, float y, float z) { return V{x, y, z}; }
inline V operator+(V a, V b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V operator-(V a, V b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V operator*(V a, V b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
inline V operator*(V a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
inline V operator/(V a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
inline V neg(V a) { return mk(-a.x, -a.y, -a.z); }
inline float dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V cross(V a, V b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline float len(V a) { return std::sqrt(dot(a, a)); }
inline V nrm(V a) { return a / std::sqrt(dot(a, a)); }
inline bool black(V a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }
inline float lum(V c) { return 0.3086f * c.x + 0.6094f * c.y + 0.0820f * c.z; }

// Random numbers of a path. Two generators behind one interface:
//  - inc != 0: PCG32 (O'Neill 2014), the library's default streams;
//  - inc == 0: the reference's Xorshift32Generator (src/HostDeviceCommon/Xorshift.h:18-66), the
//    32-bit state in 'state': floats are x / 2^32 clamped to 1 - 1e-7, random_index(n) is
//    floor(x / 2^32 * n) clamped to n - 1.
struct Pcg
{
    uint64_t state, inc;
    uint32_t u32()
    {
        if (inc == 0)
        {
            uint32_t x = (uint32_t)state;
            x ^= x << 13;
            x ^= x >> 17;
            x ^= x << 5;
            state = x;
            return x;
        }
        uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xs >> rot) | (xs << ((32u - rot) & 31u));
    }
    float next()
    {
        if (inc == 0) return std::min((float)u32() / 4294967296.0f, 1.0f - 1.0e-7f);
        return (float)(u32() >> 8) * (1.0f / 16777216.0f);
    }
    int index(int n)
    {
        if (inc == 0)
        {
            int i = (int)((float)u32() / 4294967296.0f * (float)n);
            return std::min(i, n - 1);
        }
        int i = (int)(next() * (float)n);
        return i < n - 1 ? i : n - 1;
    }
};

// wang_hash (src/Device/includes/Hash.h:11-19)
uint32_t wang_hash(uint32_t s)
{
    s = (s ^ 61u) ^ (s >> 16);
    s *= 9u;
    s = s ^ (s >> 4);
    s *= 0x27d4eb2du;
    s = s ^ (s >> 15);
    return s;
}

// The reference's per-pixel generator of a frame: Xorshift32 seeded by
// wang_hash((pixel + 1) * (sample_number + 1) * random_number) (CameraRays.h:155-160,
// Megakernel.h:52-57), 32-bit wrap-around products.
Pcg parity_seed(uint32_t pixel, uint32_t sample_number, uint32_t random_number)
{
    Pcg r;
    r.state = wang_hash((pixel + 1u) * (sample_number + 1u) * random_number);
    r.inc = 0;
    return r;
}

uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

Pcg pcg_seed(uint32_t pixel, uint32_t iteration, uint32_t seed)
{
    Pcg r;
    r.state = 0;
    r.inc = ((uint64_t)seed << 1u) | 1u;
    r.u32();
    r.state += mix64(((uint64_t)iteration << 32) | pixel);
    r.u32();
    return r;
}

V mat_point(const float* m, V p)
{
    float x = m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3];
    float y = m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7];
    float z = m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11];
    float w = m[12] * p.x + m[13] * p.y + m[14] * p.z + m[15];
    float iw = 1.0f;
    if (!(w < 1.0e-10f && w > -1.0e-10f)) iw = 1.0f / w;
    return mk(x * iw, y * iw, z * iw);
}

struct Scene
{
    const float* tv;
    int nt;
    const int* mat_of;
    const float* albedo;
    const float* emission;
    const int* emissive;
    int ne;
    const float* alias_prob;
    const int* alias_idx;
    float power_sum;
    const float* tn = nullptr;  // corner normals, 9 per triangle (NULL: flat shading everywhere)
    V a(int t) const { return mk(tv[9 * t], tv[9 * t + 1], tv[9 * t + 2]); }
    V b(int t) const { return mk(tv[9 * t + 3], tv[9 * t + 4], tv[9 * t + 5]); }
    V c(int t) const { return mk(tv[9 * t + 6], tv[9 * t + 7], tv[9 * t + 8]); }
    V alb(int t) const { int m = mat_of[t]; return mk(albedo[3 * m], albedo[3 * m + 1], albedo[3 * m + 2]); }
    V emi(int t) const { int m = mat_of[t]; return mk(emission[3 * m], emission[3 * m + 1], emission[3 * m + 2]); }
};

bool mt(V A, V B, V C, V o, V d, float& t)
{
    const float EPS = 0.0000001f;
    V e1 = B - A, e2 = C - A;
    V h = cross(d, e2);
    float a = dot(e1, h);
    if (a > -EPS && a < EPS) return false;
    float f = 1.0f / a;
    V s = o - A;
    float u = f * dot(s, h);
    if (u < 0.0f || u > 1.0f) return false;
    V q = cross(s, e1);
    float v = f * dot(d, q);
    if (v < 0.0f || u + v > 1.0f) return false;
    t = f * dot(e2, q);
    return t > EPS;
}

// Barycentrics (u, v) of the ray's hit on triangle t (the Moller-Trumbore values of mt()).
void mt_uv(const Scene& s, int t, V o, V d, float& u, float& v)
{
    V A = s.a(t), B = s.b(t), C = s.c(t);
    V e1 = B - A, e2 = C - A;
    V h = cross(d, e2);
    float f = 1.0f / dot(e1, h);
    V sv = o - A;
    u = f * dot(sv, h);
    V q = cross(sv, e1);
    v = f * dot(d, q);
}

// get_shading_normal (src/Device/includes/Intersect.h:114-134) without normal maps: corner normals
// interpolated as uv_interpolate does (src/Device/includes/Texture.h:248-251) when the triangle's
// first corner has one, else the geometric normal.
V shading_normal(const Scene& s, int t, V o, V d, V ng)
{
    if (!s.tn) return ng;
    const float* n = s.tn + 9 * (size_t)t;
    if (n[0] == 0.0f && n[1] == 0.0f && n[2] == 0.0f) return ng;
    float u, v;
    mt_uv(s, t, o, d, u, v);
    V na = mk(n[0], n[1], n[2]), nb = mk(n[3], n[4], n[5]), nc = mk(n[6], n[7], n[8]);
    return nrm(nb * u + nc * v + na * (1.0f - u - v));
}

// closest hit with the self-hit filter; returns prim or -1 (lowest index on exact ties)
int closest(const Scene& s, V o, V d, int skip, float& t_out)
{
    // the scene accelerator (an orc_octree_build handle over the same triangles) when one is set
    // (orc_set_scene_accel, trace_oracle.cpp); else every triangle is tested
    if (void* accel = orc_scene_accel())
    {
        const float of[3] = {o.x, o.y, o.z}, df[3] = {d.x, d.y, d.z};
        return orc_octree_closest_one(accel, of, df, skip, &t_out);
    }
    int best = -1;
    float bt = 0.0f;
    for (int k = 0; k < s.nt; k++)
    {
        float t;
        if (k == skip || !mt(s.a(k), s.b(k), s.c(k), o, d, t)) continue;
        if (best < 0 || t < bt)
        {
            best = k;
            bt = t;
        }
    }
    t_out = bt;
    return best;
}

bool occluded(const Scene& s, V o, V d, int skip, float tmax)
{
    float t;
    int p = closest(s, o, d, skip, t);
    return p >= 0 && t < tmax;
}

V cosine_sample(V n, float r1, float r2u)
{
    float r2 = 2.0f * r2u - 1.0f;
    if (r1 < 1.0e-8f && r2 < -0.999999f && n.z > 0.999999f)
    {
        r1 += 1.0e-7f;
        r2 += 1.0e-7f;
    }
    float theta = 6.28318530717958647693f * r1;
    float sn = std::sqrt(std::max(0.0f, 1.0f - r2 * r2));
    return nrm(n + mk(sn * std::cos(theta), sn * std::sin(theta), r2));
}

V lambert(V albedo, float NoL, float& pdf)
{
    pdf = 0.0f;
    if (NoL <= 0.0f) return mk(0, 0, 0);
    pdf = NoL * 0.31830988618379067154f;
    return albedo * 0.31830988618379067154f;
}

float light_pdf_area(const Scene& s, int lt, float area, V Le, int strategy)
{
    float p = 1.0f / area;
    if (strategy == 1)
        p *= (lum(Le) * area) / s.power_sum;
    else
        p /= (float)s.ne;
    return p;
}

float balance(float a, float b) { return a == 0.0f ? 0.0f : a / (a + b); }

float a2s(float area_pdf, float dist, float cosl) { return cosl < 1.0e-8f ? 0.0f : area_pdf * dist * dist / cosl; }

struct OrcEnv;  // the world around the scene (pt_oracle.cpp)

struct Settings
{
    int width, height, nb_bounces, do_rr, rr_min, light, seed, jitter, spp, iteration_base;
    float rr_clamp;
    const float* iv;
    const float* ip;
    int direct = 0;             // 0: one light + one BSDF sample with MIS, 1: RIS
    int ris_m = 4, ris_n = 1;   // RIS light / BSDF candidates
    const OrcEnv* env = nullptr;  // ambient light / envmap (null: none)
    int rng_mode = 0;             // 0: PCG streams, 1: the reference's Xorshift32 + packed G-buffer
    uint32_t random_number = 0;   // rng_mode 1: HIPRTRenderData::random_number of the camera pass
    int gbuffer_materials = 0;    // rng_mode 1, principled: offset of the camera-hit material table in pmats
    uint32_t random_number_shade = 0;  // rng_mode 1: HIPRTRenderData::random_number of the MegaKernel pass
};

// ---------------------------------------------------------------------------------------------
// Principled scenes: the same estimator with the BSDF evaluated and sampled through callbacks
// (the reference's own principled BSDF, oracle/ref_bsdf.cpp) on 64-word material records and
// 16-float queries (view, shading normal, geometric normal, light, eta in, eta out, inside, lobe).
// Each BSDF sample is seeded with one 32-bit PCG draw (Xorshift32 seed, 0 -> 0x9E3779B9), as the
// GPU kernels do. Volume tracking: a path is inside a non-thin transmissive object after a glass
// refraction or diffuse transmission into it; its back face is then hit from inside.
// ---------------------------------------------------------------------------------------------
typedef void (*bsdf_eval_fn)(const float* mat, const float* q, float* out4);
typedef void (*bsdf_sample_fn)(const float* mat, const float* q, uint32_t seed, float* out8, int32_t* lobe);

struct PScene
{
    const float* pmats;  // effective materials, 64 words each
    bsdf_eval_fn eval;
    bsdf_sample_fn sample;
    const float* mat(int m) const { return pmats + 64 * (size_t)m; }
};

bool smooth(float r) { return r <= 1.0e-2f; }

bool can_light_sample(const float* m)
{
    const float rough = m[3], metallic = m[7], transmission = m[38], coat = m[25], coat_rough = m[26];
    const float second_w = m[17], second_r = m[18];
    bool smooth_base = smooth(rough) && (metallic == 1.0f || transmission == 1.0f);
    bool smooth_coat = coat == 0.0f || smooth(coat_rough);
    bool smooth_second = smooth(second_r) || second_w == 0.0f;
    return !(smooth_base && smooth_coat && smooth_second);
}

void make_query(float* q, V view, V ns, V ng, V l, float eta_i, float eta_o, bool inside, int lobe)
{
    q[0] = view.x; q[1] = view.y; q[2] = view.z;
    q[3] = ns.x; q[4] = ns.y; q[5] = ns.z;
    q[6] = ng.x; q[7] = ng.y; q[8] = ng.z;
    q[9] = l.x; q[10] = l.y; q[11] = l.z;
    q[12] = eta_i; q[13] = eta_o; q[14] = inside ? 1.0f : 0.0f; q[15] = (float)lobe;
}

uint32_t bsdf_seed(Pcg& rng)
{
    if (rng.inc == 0) return (uint32_t)rng.state;
    uint32_t s = rng.u32();
    return s != 0u ? s : 0x9E3779B9u;
}

// After a BSDF sample through the callback: with the reference's generator, the path continues
// from the sampler's final state (returned in out8[7]); a PCG path already advanced in bsdf_seed.
void bsdf_seed_done(Pcg& rng, const float* out8)
{
    if (rng.inc != 0) return;
    uint32_t st;
    std::memcpy(&st, out8 + 7, 4);
    rng.state = st;
}

// The reference's nested-dielectric volume state (RayVolumeState, src/Device/includes/RayVolumeState.h:20-80,
// with the NestedDielectricsInteriorStack of src/Device/includes/NestedDielectrics.h:119-258, Schmidt
// 2002): 4 stack entries packed as priority (4 bits) | topmost << 4 | odd parity << 5 | material << 6,
// entry 0 being the air (material 0x3FFFFFF, priority 0); a push per hit finds the last entered
// material and whether the hit enters or leaves its own material (parity), the BSDF pops it again.
struct VolState
{
    static constexpr int kSize = 4;
    static constexpr uint32_t kMaxMat = 0x3FFFFFFu;
    uint32_t e[kSize];
    int pos = 0;
    int incident = -1, outgoing = -1;
    bool inside = false;
    float distance = 0.0f;
    VolState()
    {
        for (int i = 0; i < kSize; i++) e[i] = (kMaxMat << 6) | (1u << 5) | (1u << 4);
    }
    static int mat(uint32_t x) { return (int)((x >> 6) & kMaxMat); }
    static bool topmost(uint32_t x) { return (x >> 4) & 1u; }
    static bool odd(uint32_t x) { return (x >> 5) & 1u; }
    static int prio(uint32_t x) { return (int)(x & 15u); }
    // returns true when the boundary is skipped (a lower-priority material inside a higher one)
    bool push(int m, int priority)
    {
        if (pos == kSize - 1) return false;
        int last;
        for (last = pos; last >= 0; last--)
            if (mat(e[last]) != m && topmost(e[last]) && odd(e[last])) break;
        bool par = true;
        for (int prev = pos; prev >= 0; prev--)
            if (mat(e[prev]) == m)
            {
                e[prev] &= ~(1u << 4);
                par = !odd(e[prev]);
                break;
            }
        inside = !par;
        if (pos < kSize - 1) pos++;
        e[pos] = ((uint32_t)(m & (int)kMaxMat) << 6) | ((par ? 1u : 0u) << 5) | (1u << 4) | ((uint32_t)priority & 15u);
        if (priority < prio(e[last])) return true;
        if (par)
        {
            incident = mat(e[last]);
            outgoing = m;
        }
        else
        {
            incident = m;
            outgoing = mat(e[last]);
        }
        return false;
    }
    void pop(bool in)
    {
        const int top = mat(e[pos]);
        if (pos > 0) pos--;
        if (in)
        {
            int prev;
            for (prev = pos; prev >= 0; prev--)
                if (mat(e[prev]) == top) break;
            if (prev >= 0)
                for (int i = prev + 1; i <= pos; i++) e[i - 1] = e[i];
            if (pos > 0) pos--;
        }
        for (int i = pos; i >= 0; i--)
            if (mat(e[i]) == top)
            {
                e[i] |= 1u << 4;
                break;
            }
    }
};

// The dielectric priority the reference's material packing gives (CPUMaterial::make_safe,
// MaterialCPU.h:200-212, then the unsigned-char field): 255 (stored as 15 in a stack entry) for a
// material without transmission, else the material's own priority (0 by default).
int dielectric_priority(const float* m) { return (m[38] == 0.0f && m[39] == 0.0f) ? 255 : 0; }

// IOR of a stack entry's material (1 for the air entry)
float vol_ior(const PScene& ps, int mat) { return (mat < 0 || mat == (int)VolState::kMaxMat) ? 1.0f : ps.mat(mat)[37]; }

// principled_beer_absorption (Principled.h:332-357): attenuation over the distance travelled in the
// volume being left (the incident entry), 1 when its absorption colour is white
V vol_beer(const PScene& ps, const VolState& vs)
{
    if (vs.incident < 0 || vs.incident == (int)VolState::kMaxMat) return mk(1, 1, 1);
    const float* m = ps.mat(vs.incident);
    if (m[40] == 1.0f && m[41] == 1.0f && m[42] == 1.0f) return mk(1, 1, 1);
    const float d = std::max(vs.distance, 1.0e-6f);
    return mk(std::exp(std::log(m[40]) / m[43] * d), std::exp(std::log(m[41]) / m[43] * d),
              std::exp(std::log(m[42]) / m[43] * d));
}

// MaterialUtils::get_thin_walled_roughness
float thin_rough(bool thin, float r, float eta)
{
    if (!thin) return r;
    const float x = r * std::sqrt(3.7f * (eta - 1.0f) * (eta - 0.5f) * (eta - 0.5f) / (eta * eta * eta));
    return std::min(std::max(x / 1.39f, 0.0f), 1.0f);
}

// The volume-stack updates of a continuation sample (the BSDF sample with update_ray_volume_state):
// a reflective lobe pops (principled_bsdf_sample, Principled.h:1851-1857), so does a glass
// reflection or a thin-walled refraction (principled_glass_sample, :793, :821); then the evaluation
// of the sampled direction pops when it refracts out of a volume through the glass lobe
// (principled_glass_eval, :536-556, past its early exits) or the diffuse transmission lobe
// (:844-860), and restarts the travelled distance. Returns false when the sample was rejected
// below the surface before its evaluation.
bool vol_after_sample(const PScene& ps, VolState& vs, const float* m, V view, V ns, V ng, V wi, int lobe)
{
    int32_t thin_i;
    std::memcpy(&thin_i, m + 44, 4);
    const bool thin = thin_i != 0;
    const bool through = lobe == 32 || lobe == 64 || lobe == 256;
    if (!through) vs.pop(false);
    if (lobe == 32 || (lobe == 64 && thin)) vs.pop(false);
    if (dot(wi, ng) < 0.0f && !through) return false;
    const bool outside = !vs.inside;
    const float metallic = m[7], trans = m[38], dt = m[39];
    const float w_glass = outside ? (1.0f - metallic) * (1.0f - dt) * trans : (1.0f - dt);
    const float w_dt = outside ? (1.0f - metallic) * dt : dt;
    const float nov = dot(view, ns), nol = dot(wi, ns);
    if (w_glass > 0.0f && std::fabs(nol) >= 1.0e-8f && !(nol * nov > 0.0f))
    {
        float eta = vol_ior(ps, vs.outgoing) / vol_ior(ps, vs.incident);
        if (std::fabs(eta - 1.0f) < 1.0e-5f) eta = 1.0f + 1.0e-5f;
        const float rough = thin_rough(thin, m[3], eta);
        V h;
        if (rough <= 1.0e-4f)
            h = ns;
        else if (thin)
            h = nrm((wi - ns * (2.0f * nol)) + view);
        else
            h = nrm(wi * eta + view);
        if (dot(h, ns) < 0.0f) h = neg(h);
        if (!(dot(wi, h) * nol < 0.0f || dot(view, h) * nov < 0.0f))
        {
            if (thin)
                vs.pop(vs.inside);
            else if (vs.incident != (int)VolState::kMaxMat)
            {
                vs.distance = 0.0f;
                if (vs.inside) vs.pop(vs.inside);
            }
        }
    }
    if (w_dt > 0.0f && nol < 0.0f && !(nov * nol > 0.0f) && vs.incident != (int)VolState::kMaxMat)
    {
        vs.distance = 0.0f;
        if (vs.inside) vs.pop(vs.inside);
    }
    return true;
}

// Octahedral24BitNormalPadded32b pack + unpack (src/HostDeviceCommon/Packing.h:237-367; Cigolle et
// al. 2014): octahedral projection, two 12-bit snorms in three bytes, decode and normalise.
float sign_nz(float k) { return k >= 0.0f ? 1.0f : -1.0f; }
V oct24(V n)
{
    const float l1 = 1.0f / (std::fabs(n.x) + std::fabs(n.y) + std::fabs(n.z));
    float ex = n.x * l1, ey = n.y * l1;
    if (n.z < 0.0f)
    {
        const float ax = std::fabs(ey), ay = std::fabs(ex);
        ex = (1.0f - ax) * sign_nz(ex);
        ey = (1.0f - ay) * sign_nz(ey);
    }
    const float sx = std::round(std::min(std::max(ex + 1.0f, 0.0f), 2.0f) * 2047.0f);
    const float sy = std::round(std::min(std::max(ey + 1.0f, 0.0f), 2.0f) * 2047.0f);
    const float ux = sx / 16.0f;
    const float t = std::floor(sy / 256.0f);
    const unsigned char bx = (unsigned char)ux;
    const unsigned char by = (unsigned char)((ux - std::floor(ux)) * 256.0f + t);
    const unsigned char bz = (unsigned char)(sy - t * 256.0f);
    const float tmp = by / 16.0f;
    const float px = bx * 16.0f + std::floor(tmp);
    const float py = (tmp - std::floor(tmp)) * 256.0f * 16.0f + bz;
    const float dx = std::min(std::max(px / 2047.0f - 1.0f, -1.0f), 1.0f);
    const float dy = std::min(std::max(py / 2047.0f - 1.0f, -1.0f), 1.0f);
    V v = mk(dx, dy, 1.0f - std::fabs(dx) - std::fabs(dy));
    if (v.z < 0.0f)
    {
        const float tx = v.x, ty = v.y;
        v.x = (1.0f - std::fabs(ty)) * sign_nz(tx);
        v.y = (1.0f - std::fabs(tx)) * sign_nz(ty);
    }
    return nrm(v);
}

}  // namespace
