// Layered principled BSDF: eval, pdf and sampling, for the CUDA kernels and for the host build
// that the CPU tests compile (tests/native/bsdf_emu.cpp).
//
// Behaviour follows the reference's principled BSDF with energy compensation, microfacet
// regularization, thin film, dispersion and sheen switched off
// (src/Device/includes/BSDFs/Principled.h:1515-1941 and the lobes it calls):
//   - lobe weights and sampling probabilities: Principled.h:1515-1618;
//   - layering (coat over sheen over metal / glass / glossy base / diffuse transmission, with the
//     fresnel transmission, coat absorption and darkening of each layer attenuating the ones
//     below): Principled.h:955-1060 (coat), 1129-1176 (metal), 1177-1218 (glass), 1219-1270
//     (diffuse transmission), 1272-1513 (specular over diffuse);
//   - GGX: anisotropic D, Smith G1/G2, Heitz 2018 visible-normal sampling, Torrance-Sparrow
//     reflection and Walter 2007 refraction: src/Device/includes/BSDFs/Microfacet.h:25-502;
//   - Fresnel: dielectric, Adobe F82-tint, d'Eon's hemispherical-albedo fit:
//     src/Device/includes/Fresnel.h:41-175;
//   - frames: Frisvad/Max ONB and the rotated ONB of anisotropy: src/Device/includes/ONB.h;
//   - delta-lobe handling (a perfectly smooth lobe contributes only when the direction was
//     sampled from a lobe with the same mirror peak): MaterialUtils.h:143-177, Microfacet.h:90-120.
// All directions are unit vectors; "view" points away from the surface. Lobe values exclude the
// cosine term, as in the reference.
#pragma once

#include "../../include/gbpt_bsdf.h"
#include "hd_math.h"

namespace gbpt {
namespace bsdf {

using namespace hd;

constexpr float kRoughnessClamp = 1.0e-4f;   // MaterialConstants::ROUGHNESS_CLAMP
constexpr float kSmoothRoughness = 1.0e-2f;  // MaterialConstants::PERFECTLY_SMOOTH_ROUGHNESS_THRESHOLD
constexpr float kDeltaValue = 1.0e9f;        // MaterialConstants::DELTA_DISTRIBUTION_HIGH_VALUE
constexpr float kDeltaAlign = 0.999999f;     // MaterialConstants::DELTA_DISTRIBUTION_ALIGNEMENT_THRESHOLD
constexpr float kGgxDotClamp = 1.0e-3f;      // GGX_DOT_PRODUCTS_CLAMP

// ---------------------------------------------------------------------------------------------
// random numbers: the reference's Xorshift32 (src/HostDeviceCommon/Xorshift.h:18-66)
// ---------------------------------------------------------------------------------------------
struct Xorshift32
{
    uint32_t state;
    GBPT_HD uint32_t next_u32()
    {
        uint32_t x = state;
        x ^= x << 13;
        x ^= x >> 17;
        x ^= x << 5;
        state = x;
        return x;
    }
    // uniform in [0, 1 - 1e-7]: the value / 2^32 (float(0xffffffff) == 2^32), clamped
    GBPT_HD float operator()() { return fminf((float)next_u32() * (1.0f / 4294967296.0f), 1.0f - 1.0e-7f); }
};

// ---------------------------------------------------------------------------------------------
// material, medium, sampled-lobe bookkeeping
// ---------------------------------------------------------------------------------------------
struct Material
{
    V3 base;
    float roughness, metallic;
    V3 f82, f90;
    float f90_exponent, anisotropy, anisotropy_rotation, second_weight, second_roughness;
    float specular, specular_tint, specular_darkening;
    V3 specular_color;
    float coat, coat_roughness, coat_thickness, coat_darkening, coat_anisotropy, coat_anisotropy_rotation, coat_ior;
    V3 coat_absorption;
    float sheen, ior, transmission, diffuse_transmission;
    bool thin_walled;
    bool oren_nayar;           // GBPT_DIFFUSE_OREN_NAYAR diffuse lobe
    float oren_a, oren_b;      // its A and B terms of the facet-slope deviation
};

GBPT_HD Material load_material(const gbpt_principled_material& s)
{
    Material m;
    m.base = v3(s.base_color[0], s.base_color[1], s.base_color[2]);
    m.roughness = s.roughness;
    m.metallic = s.metallic;
    m.f82 = v3(s.metallic_F82[0], s.metallic_F82[1], s.metallic_F82[2]);
    m.f90 = v3(s.metallic_F90[0], s.metallic_F90[1], s.metallic_F90[2]);
    m.f90_exponent = s.metallic_F90_falloff_exponent;
    m.anisotropy = s.anisotropy;
    m.anisotropy_rotation = s.anisotropy_rotation;
    m.second_weight = s.second_roughness_weight;
    m.second_roughness = s.second_roughness;
    m.specular = s.specular;
    m.specular_tint = s.specular_tint;
    m.specular_darkening = s.specular_darkening;
    m.specular_color = v3(s.specular_color[0], s.specular_color[1], s.specular_color[2]);
    m.coat = s.coat;
    m.coat_roughness = s.coat_roughness;
    m.coat_thickness = s.coat_medium_thickness;
    m.coat_darkening = s.coat_darkening;
    m.coat_anisotropy = s.coat_anisotropy;
    m.coat_anisotropy_rotation = s.coat_anisotropy_rotation;
    m.coat_ior = s.coat_ior;
    m.coat_absorption = v3(s.coat_medium_absorption[0], s.coat_medium_absorption[1], s.coat_medium_absorption[2]);
    m.sheen = s.sheen;
    m.ior = s.ior;
    m.transmission = s.specular_transmission;
    m.diffuse_transmission = s.diffuse_transmission;
    m.thin_walled = s.thin_walled != 0;
    // Oren-Nayar A and B from the facet-slope deviation sigma (MaterialUtils::get_oren_nayar_AB,
    // src/HostDeviceCommon/Material/MaterialUtils.h:18-23)
    m.oren_nayar = s.diffuse_lobe == GBPT_DIFFUSE_OREN_NAYAR;
    const float s2 = s.oren_nayar_sigma * s.oren_nayar_sigma;
    m.oren_a = 1.0f - s2 / (2.0f * (s2 + 0.33f));
    m.oren_b = 0.45f * s2 / (s2 + 0.09f);
    return m;
}

// Media on both sides of the interface: IOR of the medium the ray travels in (1 = air) and of
// the medium behind the surface, and whether the ray is inside the object (RayVolumeState).
// 'beer' is the Beer-Lambert attenuation of the volume the ray leaves (absorbing: not white),
// which the reference's glass and diffuse-transmission lobes apply to refracted directions
// (principled_glass_eval, Principled.h:540-546; principled_diffuse_transmission_eval, :844-851).
struct Medium
{
    float eta_incident;
    float eta_outgoing;
    bool inside;
    bool absorbing = false;
    V3 beer = V3{1.0f, 1.0f, 1.0f};
};

enum class Delta
{
    NotSmooth,      // the lobe is rough: evaluate normally
    PeakSampled,    // smooth lobe, direction came from a lobe with the same mirror peak
    PeakNotSampled  // smooth lobe, direction came from elsewhere: contributes nothing
};

GBPT_HD bool is_smooth(float roughness) { return roughness <= kSmoothRoughness; }

// MaterialUtils::is_specular_delta_reflection_sampled (MaterialUtils.h:143-177)
GBPT_HD Delta delta_state(const Material& m, float lobe_roughness, float lobe_anisotropy, int lobe)
{
    if (!is_smooth(lobe_roughness)) return Delta::NotSmooth;
    const bool base_aniso = fabsf(lobe_anisotropy - m.anisotropy) < 1.0e-3f;
    const bool coat_aniso = fabsf(lobe_anisotropy - m.coat_anisotropy) < 1.0e-3f;
    const bool smooth_base = is_smooth(m.roughness);
    if ((lobe == GBPT_LOBE_GLASS_REFLECT || lobe == GBPT_LOBE_METAL_1 || lobe == GBPT_LOBE_SPECULAR) && smooth_base &&
        base_aniso)
        return Delta::PeakSampled;
    if (lobe == GBPT_LOBE_METAL_2 && is_smooth(m.second_roughness) && base_aniso) return Delta::PeakSampled;
    if (lobe == GBPT_LOBE_COAT && coat_aniso && is_smooth(m.coat_roughness)) return Delta::PeakSampled;
    return Delta::PeakNotSampled;
}

// ---------------------------------------------------------------------------------------------
// shading frames (src/Device/includes/ONB.h)
// ---------------------------------------------------------------------------------------------
struct Frame
{
    V3 t, b, n;
    GBPT_HD V3 to_local(V3 w) const { return normalize(v3(dot(w, t), dot(w, b), dot(w, n))); }
    GBPT_HD V3 to_world(V3 w) const { return normalize(w.x * t + w.y * b + w.z * n); }
};

// Orthonormal basis around n without branches except at the south pole (Frisvad 2012 as revised
// by Nelson Max 2017)
GBPT_HD Frame make_frame(V3 n)
{
    Frame f;
    f.n = n;
    if (n.z < -0.99998796f)
    {
        f.t = v3(0.0f, -1.0f, 0.0f);
        f.b = v3(-1.0f, 0.0f, 0.0f);
        return f;
    }
    const float a = -n.x / (1.0f + n.z);
    f.t = v3(1.0f + n.x * a, a * n.y, -n.x);
    f.b = v3(f.t.y, 1.0f - n.y * n.y / (1.0f + n.z), -n.y);
    return f;
}

// Basis rotated about n by 'angle' radians (Rodrigues), for anisotropic lobes
GBPT_HD Frame make_rotated_frame(V3 n, float angle)
{
    Frame f;
    f.n = n;
    const V3 up = fabsf(n.z) < 0.9999999f ? v3(0.0f, 0.0f, 1.0f) : v3(1.0f, 0.0f, 0.0f);
    V3 t = normalize(cross(up, n));
    const float c = cosf(angle), s = sinf(angle);
    t = t * c + cross(n, t) * s + n * dot(n, t) * (1.0f - c);
    f.t = t;
    f.b = cross(n, t);
    return f;
}

// ---------------------------------------------------------------------------------------------
// Fresnel (src/Device/includes/Fresnel.h)
// ---------------------------------------------------------------------------------------------
// Unpolarised dielectric reflectance; eta = eta_transmitted / eta_incident.
GBPT_HD float fresnel_dielectric(float cos_i, float eta)
{
    if (fabsf(1.0f - eta) < 1.0e-4f) return 0.0f;
    const float sin_t2 = (1.0f - cos_i * cos_i) / (eta * eta);
    if (sin_t2 >= 1.0f) return 1.0f;  // total internal reflection
    const float cos_t = sqrtf(1.0f - sin_t2);
    const float rp = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
    const float rs = (cos_i - eta * cos_t) / (cos_i + eta * cos_t);
    return (rp * rp + rs * rs) / 2.0f;
}

// Hoffman 2023 generalisation of Adobe's F82-tint metal Fresnel (Schlick with an F90 exponent,
// minus a Lazanyi term that pins the reflectance at cos = 1/7 to F82 * Schlick)
GBPT_HD V3 fresnel_f82_tint(V3 f0, V3 f82, V3 f90, float exponent, float cos_t)
{
    const V3 schlick = f0 + (f90 - f0) * powf(1.0f - cos_t, exponent);
    if (max_comp(schlick) < 1.0e-8f) return v3(0.0f);
    constexpr float kCosMax = 1.0f / 7.0f;
    constexpr float kOneMinus = 1.0f - kCosMax;
    constexpr float kDenom = kCosMax * ((kOneMinus * kOneMinus) * (kOneMinus * kOneMinus)) * (kOneMinus * kOneMinus);
    const float lazanyi = cos_t * pow6(1.0f - cos_t);
    const V3 a = ((f0 + (f90 - f0) * powf(kOneMinus, exponent)) * (1.0f - f82)) / kDenom;
    return clamp3(0.0f, 1.0f, schlick - a * lazanyi);
}

// Hemispherical albedo of a smooth dielectric interface (d'Eon, "A Hitchhiker's Guide to
// Multiple Scattering", eq. 11.15 fit)
GBPT_HD float fresnel_hemispherical_albedo(float eta)
{
    return logf((10893.0f * eta - 1438.2f) / (-774.4f * sq(eta) + 10212.0f * eta + 1.0f));
}

// ---------------------------------------------------------------------------------------------
// GGX (src/Device/includes/BSDFs/Microfacet.h)
// ---------------------------------------------------------------------------------------------
GBPT_HD void ggx_alphas(float roughness, float anisotropy, float& ax, float& ay)
{
    const float aspect = sqrtf(1.0f - 0.9f * anisotropy);
    ax = fmaxf(kRoughnessClamp, roughness * roughness / aspect);
    ay = fmaxf(kRoughnessClamp, roughness * roughness * aspect);
}

GBPT_HD float ggx_D(float ax, float ay, V3 h)
{
    const float d = (h.x * h.x) / (ax * ax) + (h.y * h.y) / (ay * ay) + (h.z * h.z);
    return 1.0f / (kPi * ax * ay * d * d);
}

GBPT_HD float smith_lambda(float ax, float ay, V3 w)
{
    const float a = w.x * ax, b = w.y * ay;
    return (-1.0f + sqrtf(1.0f + (a * a + b * b) / (w.z * w.z))) * 0.5f;
}

GBPT_HD float smith_G1(float ax, float ay, V3 w) { return 1.0f / (1.0f + smith_lambda(ax, ay, w)); }

// Torrance-Sparrow reflection F*D*G2 / (4 NoL NoV) with VNDF-sampling pdf; smooth lobes are
// delta distributions represented by a large finite value.
GBPT_HD V3 ggx_reflection(float roughness, float anisotropy, bool height_correlated, V3 F, V3 v, V3 l, V3 h, Delta ds,
                          float& pdf)
{
    pdf = 0.0f;
    if (is_smooth(roughness))
    {
        if (ds == Delta::PeakNotSampled) return v3(0.0f);
        if (dot(reflect(v, v3(0.0f, 0.0f, 1.0f)), l) < kDeltaAlign) return v3(0.0f);
        pdf = kDeltaValue;
        return v3(kDeltaValue) * F / fabsf(l.z);
    }
    if (l.z < 0.0f) return v3(0.0f);
    float ax, ay;
    ggx_alphas(roughness, anisotropy, ax, ay);
    const float D = ggx_D(ax, ay, h);
    const float lambda_v = smith_lambda(ax, ay, v);
    const float g1v = 1.0f / (1.0f + lambda_v);
    const float d_visible = g1v * D * fmaxf(kGgxDotClamp, dot(v, h)) / v.z;
    const float nov = fmaxf(kGgxDotClamp, fabsf(v.z));
    const float nol = fmaxf(kGgxDotClamp, fabsf(l.z));
    pdf = d_visible / (4.0f * dot(v, h));
    if (pdf == 0.0f) return v3(0.0f);
    const float lambda_l = smith_lambda(ax, ay, l);
    const float g2 = height_correlated ? 1.0f / (1.0f + lambda_v + lambda_l) : g1v * (1.0f / (1.0f + lambda_l));
    return F * D * g2 / (4.0f * nol * nov);
}

// refract(d) about n (d and n in the same hemisphere, no total internal reflection)
GBPT_HD V3 refract_dir(V3 d, V3 n, float eta)
{
    const float noi = dot(d, n);
    const float cos_t = sqrtf(1.0f - (1.0f - noi * noi) / (eta * eta));
    return -d / eta + (noi / eta - cos_t) * n;
}

// Walter et al. 2007 microfacet transmission
GBPT_HD V3 ggx_refraction(const Material& m, float roughness, float eta, float F, V3 v, V3 l, V3 h, int lobe, float& pdf)
{
    const float nol = l.z, nov = v.z;
    const float hol = dot(l, h), hov = dot(v, h);
    V3 color;
    if (is_smooth(roughness))
    {
        const bool perfect = dot(refract_dir(v, v3(0.0f, 0.0f, 1.0f), eta), l) > kDeltaAlign;
        if (lobe == GBPT_LOBE_GLASS_REFRACT && perfect)
        {
            color = v3(kDeltaValue) * (1.0f - v3(F)) * m.base;
            color = color / fabsf(nol);
            pdf = kDeltaValue;
        }
        else
        {
            color = v3(0.0f);
            pdf = 0.0f;
        }
    }
    else
    {
        const float dp = hol + hov / eta;
        const float dp2 = dp * dp;
        const float denom = dp2 * nol * nov;
        float ax, ay;
        ggx_alphas(roughness, m.anisotropy, ax, ay);
        const float D = ggx_D(ax, ay, h);
        const float g1v = smith_G1(ax, ay, v);
        const float g2 = g1v * smith_G1(ax, ay, l);
        const float dwm_dwi = fabsf(hol) / dp2;
        pdf = dwm_dwi * (g1v / fabsf(nov) * D * fabsf(hov));
        color = m.base * D * (1.0f - v3(F)) * g2 * fabsf(hol * hov / denom);
    }
    return color / sq(eta);
}

// Heitz 2018 sampling of the GGX distribution of visible normals
template <typename Rng>
GBPT_HD V3 ggx_sample_visible_normal(V3 v, float ax, float ay, Rng& rng)
{
    if (ax <= kRoughnessClamp && ay <= kRoughnessClamp) return v3(0.0f, 0.0f, 1.0f);
    const float r1 = rng();
    const float r2 = rng();
    const V3 vh = normalize(v3(ax * v.x, ay * v.y, v.z));
    const float lensq = vh.x * vh.x + vh.y * vh.y;
    const V3 t1 = lensq > 0.0f ? v3(-vh.y, vh.x, 0.0f) / sqrtf(lensq) : v3(1.0f, 0.0f, 0.0f);
    const V3 t2 = cross(vh, t1);
    const float r = sqrtf(r1);
    const float phi = kTwoPi * r2;
    float sp, cp;
    sincosf(phi, &sp, &cp);
    const float p1 = r * cp;
    float p2 = r * sp;
    const float s = 0.5f * (1.0f + vh.z);
    p2 = (1.0f - s) * sqrtf(1.0f - p1 * p1) + s * p2;
    const V3 nh = p1 * t1 + p2 * t2 + sqrtf(fmaxf(0.0f, 1.0f - p1 * p1 - p2 * p2)) * vh;
    return normalize(v3(ax * nh.x, ay * nh.y, fmaxf(0.0f, nh.z)));
}

template <typename Rng>
GBPT_HD V3 ggx_sample_reflection(float roughness, float anisotropy, V3 v, Rng& rng)
{
    const float side = v.z < 0.0f ? -1.0f : 1.0f;
    float ax, ay;
    ggx_alphas(roughness, anisotropy, ax, ay);
    const V3 h = ggx_sample_visible_normal(v * side, ax, ay, rng);
    return normalize(reflect(v, h * side));
}

// normalize(n + uniform point on the unit sphere): cosine-weighted around n
// (src/Device/includes/Sampling.h:180-201)
template <typename Rng>
GBPT_HD V3 cosine_around(V3 n, Rng& rng)
{
    float r1 = rng();
    float r2 = 2.0f * rng() - 1.0f;
    if (r1 < 1.0e-8f && r2 < -0.999999f && n.z > 0.999999f)
    {
        r1 += 1.0e-7f;
        r2 += 1.0e-7f;
    }
    float st, ct;
    sincosf(kTwoPi * r1, &st, &ct);
    const float s = sqrtf(1.0f - r2 * r2);
    return normalize(n + v3(s * ct, s * st, r2));
}

// ---------------------------------------------------------------------------------------------
// lobe weights and sampling probabilities (Principled.h:1515-1618)
// ---------------------------------------------------------------------------------------------
struct Lobes
{
    float coat, sheen, metal1, metal2, specular, diffuse, glass, diffuse_transmission;
};

GBPT_HD Lobes lobe_weights(const Material& m, bool outside)
{
    const float o = outside ? 1.0f : 0.0f;
    Lobes w;
    w.coat = m.coat * o;
    w.sheen = m.sheen * o;
    const float metal = m.metallic * o;
    w.metal1 = lerp(metal, 0.0f, m.second_weight);
    w.metal2 = lerp(0.0f, metal, m.second_weight);
    const float dt = m.diffuse_transmission;
    w.glass = !outside ? (1.0f - dt) : (1.0f - m.metallic) * (1.0f - dt) * m.transmission;
    w.diffuse_transmission = !outside ? dt : (1.0f - m.metallic) * dt;
    w.specular = (1.0f - m.metallic) * (1.0f - m.transmission * (1.0f - dt)) * m.specular * o;
    w.diffuse = (1.0f - m.metallic) * (1.0f - m.transmission) * (1.0f - dt) * o;
    return w;
}

GBPT_HD Lobes lobe_probabilities(const Lobes& w)
{
    const float k = 1.0f / (w.coat + w.sheen + w.metal1 + w.metal2 + w.specular + w.diffuse + w.glass +
                            w.diffuse_transmission);
    Lobes p;
    p.coat = w.coat * k;
    p.sheen = w.sheen * k;
    p.metal1 = w.metal1 * k;
    p.metal2 = w.metal2 * k;
    p.specular = w.specular * k;
    p.diffuse = w.diffuse * k;
    p.glass = w.glass * k;
    p.diffuse_transmission = w.diffuse_transmission * k;
    return p;
}

// ---------------------------------------------------------------------------------------------
// layer helpers
// ---------------------------------------------------------------------------------------------
// IOR of the specular layer relative to what lies above it (coat or the incident medium)
GBPT_HD float specular_relative_ior(const Material& m, float incident_ior)
{
    if (m.coat == 0.0f) return m.ior;
    const float rel = m.ior / lerp(incident_ior, m.coat_ior, m.coat);
    return rel < 1.0f ? 1.0f / rel : rel;  // no TIR ring from a denser coat
}

// OpenPBR darkening of the base from light trapped under an interface (eqs. 66-68)
GBPT_HD V3 coat_darkening(const Material& m, float eta, float view_fresnel)
{
    if (m.coat_darkening == 0.0f) return v3(1.0f);
    const float kr = 1.0f - (1.0f - fresnel_hemispherical_albedo(eta)) / (eta * eta);
    const float base_roughness = lerp(1.0f, m.roughness, fmaxf(m.transmission, fmaxf(m.metallic, m.specular)));
    const float K = lerp(view_fresnel, kr, base_roughness);
    const V3 albedo = (m.base + v3(0.0f) * m.sheen) / (1.0f + m.sheen);  // sheen colour unused (sheen = 0)
    const V3 d = (1.0f - K) / (1.0f - albedo * K);
    return lerp(v3(1.0f), d, m.coat * m.coat_darkening * (1.0f - m.diffuse_transmission));
}

GBPT_HD V3 specular_darkening(const Material& m, float eta)
{
    if (m.specular_darkening == 0.0f) return v3(1.0f);
    const float K = 1.0f - (1.0f - fresnel_hemispherical_albedo(eta)) / (eta * eta);
    const V3 d = (1.0f - K) / (1.0f - m.base * K);
    return lerp(v3(1.0f), d, m.specular * m.specular_darkening * (1.0f - m.diffuse_transmission));
}

GBPT_HD float thin_walled_roughness(bool thin, float roughness, float eta)
{
    if (!thin) return roughness;
    const float r = roughness * sqrtf(3.7f * (eta - 1.0f) * sq(eta - 0.5f) / (eta * eta * eta));
    return clampf(0.0f, 1.0f, r / 1.39f);
}

// relative IOR across the glass interface, kept away from 1 (a null half vector otherwise)
GBPT_HD float glass_eta(const Medium& md)
{
    float eta = md.eta_outgoing / md.eta_incident;
    if (fabsf(eta - 1.0f) < 1.0e-5f) eta = 1.0f + 1.0e-5f;
    return eta;
}

// Fresnel of the glass interface with the thin-walled inter-reflection correction
GBPT_HD float glass_fresnel(const Material& m, float hov, float eta, float roughness)
{
    float F = fresnel_dielectric(hov, eta);
    if (m.thin_walled && F < 1.0f && roughness < 0.1f) F += sq(1.0f - F) * F / (1.0f - sq(F));
    return F;
}

// The Oren-Nayar factor A + B max(0, cos(phi_i - phi_o)) sin(alpha) tan(beta) of the diffuse lobe
// (oren_nayar_brdf_eval, src/Device/includes/BSDFs/OrenNayar.h:14-47), v and l in the unrotated
// shading frame; the azimuth difference does not depend on the frame's tangent
GBPT_HD float oren_nayar_shape(const Material& m, V3 v, V3 l)
{
    const float sin_i = sqrtf(1.0f - l.z * l.z);
    const float sin_o = sqrtf(1.0f - v.z * v.z);
    float max_cos = 0.0f;
    if (sin_i > 1.0e-4f && sin_o > 1.0e-4f)
    {
        const float sp_i = l.y / sin_i, cp_i = l.x / sin_i;
        const float sp_o = v.y / sin_o, cp_o = v.x / sin_o;
        max_cos = fmaxf(0.0f, cp_i * cp_o + sp_i * sp_o);
    }
    float sin_alpha, tan_beta;
    if (fabsf(l.z) > fabsf(v.z))
    {
        sin_alpha = sin_o;
        tan_beta = sin_i / fabsf(l.z);
    }
    else
    {
        sin_alpha = sin_i;
        tan_beta = sin_o / fabsf(v.z);
    }
    return m.oren_a + m.oren_b * max_cos * sin_alpha * tan_beta;
}

// Glass lobe (Principled.h:359-558): reflection or refraction through a GGX interface.
GBPT_HD V3 glass_eval(const Material& m, const Medium& md, bool height_correlated, V3 v, V3 l, int lobe, float& pdf)
{
    pdf = 0.0f;
    const float nov = v.z, nol = l.z;
    if (fabsf(nol) < 1.0e-8f) return v3(0.0f);
    const bool reflecting = nol * nov > 0.0f;
    const float eta = glass_eta(md);
    const float rough = thin_walled_roughness(m.thin_walled, m.roughness, eta);
    V3 h;
    if (rough <= kRoughnessClamp)
        h = v3(0.0f, 0.0f, 1.0f);
    else if (reflecting)
        h = normalize(l + v);
    else if (m.thin_walled)
        h = normalize(l * v3(1.0f, 1.0f, -1.0f) + v);
    else
        h = normalize(l * eta + v);
    if (h.z < 0.0f) h = -h;
    const float hol = dot(l, h), hov = dot(v, h);
    if (hol * nol < 0.0f || hov * nov < 0.0f) return v3(0.0f);
    const float F = glass_fresnel(m, hov, eta, rough);
    const float p_reflect = luminance(v3(F));
    if (reflecting)
    {
        const Delta ds = delta_state(m, rough, m.anisotropy, lobe);
        const V3 c = ggx_reflection(rough, m.anisotropy, height_correlated, v3(F), v, l, h, ds, pdf);
        pdf *= p_reflect;
        return c;
    }
    V3 c = ggx_refraction(m, rough, eta, F, v, l, h, lobe, pdf);
    pdf *= 1.0f - p_reflect;
    if (m.thin_walled) c = c * m.base;
    return c;
}

template <typename Rng>
GBPT_HD V3 glass_sample(const Material& m, const Medium& md, V3 v, Rng& rng, int& lobe)
{
    const float eta = glass_eta(md);
    const float rough = thin_walled_roughness(m.thin_walled, m.roughness, eta);
    float ax, ay;
    ggx_alphas(rough, m.anisotropy, ax, ay);
    V3 h = ggx_sample_visible_normal(v, ax, ay, rng);
    const float F = glass_fresnel(m, dot(v, h), eta, rough);
    if (rng() < luminance(v3(F)))
    {
        lobe = GBPT_LOBE_GLASS_REFLECT;
        return reflect(v, h);
    }
    lobe = GBPT_LOBE_GLASS_REFRACT;
    if (dot(h, v) < 0.0f) h = -h;
    if (m.thin_walled)
    {
        V3 r = reflect(v, h);  // two parallel interfaces: straight through, no bending
        r.z = -r.z;
        return r;
    }
    return refract_dir(v, h, eta);
}

// ---------------------------------------------------------------------------------------------
// the layered BSDF
// ---------------------------------------------------------------------------------------------
struct Query
{
    V3 view, ns, ng, light;
};

// f (without cosine) and pdf for light direction q.light, given the lobe it was sampled from.
GBPT_HD V3 eval(const Material& m, const Medium& md, bool height_correlated, const Query& q, int lobe, float& pdf)
{
    pdf = 0.0f;
    const bool outside = !md.inside;
    const bool refracting = dot(q.ns, q.light) < 0.0f && outside;
    const Frame F0 = make_frame(q.ns);
    const V3 v = F0.to_local(q.view), l = F0.to_local(q.light);
    const V3 h = normalize(v + l);
    const Frame FR = make_rotated_frame(q.ns, m.anisotropy_rotation * kPi);
    const V3 vr = FR.to_local(q.view), lr = FR.to_local(q.light);
    const V3 hr = normalize(vr + lr);
    const float eta_in = md.eta_incident;
    const Lobes w = lobe_weights(m, outside);
    const Lobes p = lobe_probabilities(w);

    V3 throughput = v3(1.0f);  // light left for the layers below
    V3 color = v3(0.0f);

    // coat (unrotated frame); on refraction only its attenuation applies
    if (w.coat > 0.0f && ((v.z > 0.0f && l.z > 0.0f) || refracting))
    {
        float lobe_pdf = 0.0f;
        const float eta_coat = m.coat_ior / eta_in;
        if (!refracting)
        {
            const float hol = clampf(1.0e-8f, 1.0f, dot(h, l));
            const Delta ds = delta_state(m, m.coat_roughness, m.coat_anisotropy, lobe);
            const V3 c = ggx_reflection(m.coat_roughness, m.coat_anisotropy, height_correlated,
                                        v3(fresnel_dielectric(hol, eta_coat)), v, l, h, ds, lobe_pdf);
            color = color + c * w.coat * throughput;
        }
        pdf += lobe_pdf * p.coat;
        V3 att = v3(1.0f - fresnel_dielectric(fabsf(l.z), eta_coat));
        const float view_f = fresnel_dielectric(fabsf(v.z), eta_coat);
        att = att * (1.0f - view_f);
        if (!is_white(m.coat_absorption))
        {
            // absorption along the refracted in and out paths through the coat (OpenPBR)
            const float ci = fmaxf(1.0e-6f, sqrtf(1.0f - (1.0f - l.z * l.z) / (m.coat_ior * m.coat_ior)));
            const float co = fmaxf(1.0e-6f, sqrtf(1.0f - (1.0f - v.z * v.z) / (m.coat_ior * m.coat_ior)));
            const float path = 1.0f / ci + 1.0f / co;
            att = att * exp3(-(1.0f - pow3(sqrt3(m.coat_absorption), path)) * m.coat_thickness);
        }
        att = att * coat_darkening(m, eta_coat, view_f);
        throughput = throughput * lerp(v3(1.0f), att, m.coat);
    }

    // two metal lobes (rotated frame), reflection only
    const float metal_w[2] = {w.metal1 * (refracting ? 0.0f : 1.0f), w.metal2 * (refracting ? 0.0f : 1.0f)};
    const float metal_p[2] = {p.metal1, p.metal2};
    const float metal_r[2] = {m.roughness, m.second_roughness};
#pragma unroll
    for (int k = 0; k < 2; k++)
    {
        if (!(metal_w[k] > 0.0f && vr.z > 0.0f && lr.z > 0.0f)) continue;
        float lobe_pdf = 0.0f;
        V3 c = v3(0.0f);
        const Delta ds = delta_state(m, metal_r[k], m.anisotropy, lobe);
        if (ds != Delta::PeakNotSampled)
        {
            const float hol = clampf(1.0e-8f, 1.0f, dot(hr, lr));
            const V3 F = fresnel_f82_tint(m.base, m.f82, m.f90, m.f90_exponent, hol);
            c = ggx_reflection(metal_r[k], m.anisotropy, height_correlated, F, vr, lr, hr, ds, lobe_pdf);
        }
        color = color + c * metal_w[k] * throughput;
        pdf += lobe_pdf * metal_p[k];
    }

    // glass (rotated frame), beside the glossy base rather than below it
    if (w.glass > 0.0f)
    {
        float lobe_pdf;
        const V3 c = glass_eval(m, md, height_correlated, vr, lr, lobe, lobe_pdf);
        color = color + c * w.glass * throughput;
        pdf += lobe_pdf * p.glass;
    }

    // glossy base: specular (rotated frame) over diffuse (unrotated frame)
    V3 glossy = v3(0.0f);
    if (w.specular > 0.0f && ((vr.z > 0.0f && lr.z > 0.0f) || (refracting && lobe == GBPT_LOBE_DIFFUSE_TRANSMISSION)))
    {
        const float eta_s = specular_relative_ior(m, eta_in);
        float lobe_pdf;
        const Delta ds = delta_state(m, m.roughness, m.anisotropy, lobe);
        V3 c = ggx_reflection(m.roughness, m.anisotropy, height_correlated, v3(fresnel_dielectric(dot(lr, hr), eta_s)), vr,
                              lr, hr, ds, lobe_pdf);
        c = c * lerp(v3(1.0f), m.specular_tint * m.specular_color, m.specular);
        glossy = glossy + c * w.specular * throughput;
        const float light_f = fresnel_dielectric(fabsf(lr.z), eta_s) * (1.0f - m.diffuse_transmission);
        const float view_f = fresnel_dielectric(fabsf(vr.z), eta_s);
        V3 att = v3((1.0f - light_f) * (1.0f - view_f));
        att = att * specular_darkening(m, eta_s);
        throughput = throughput * lerp(v3(1.0f), att, m.specular);
        pdf += lobe_pdf * p.specular;
    }
    const float diffuse_w = w.diffuse * (refracting ? 0.0f : 1.0f);
    if (diffuse_w > 0.0f && v.z > 0.0f && l.z > 0.0f)
    {
        const float shape = m.oren_nayar ? oren_nayar_shape(m, v, l) : 1.0f;
        glossy = glossy + m.base * kInvPi * shape * diffuse_w * throughput;
        pdf += l.z * kInvPi * p.diffuse;
    }
    color = color + glossy;

    // diffuse transmission (unrotated frame): Lambertian lobe through the surface
    if (w.diffuse_transmission > 0.0f && l.z < 0.0f)
    {
        if (!(v.z * l.z > 0.0f))
        {
            color = color + m.base * kInvPi * w.diffuse_transmission * throughput;
            pdf += fabsf(l.z * kInvPi) * p.diffuse_transmission;
        }
    }
    // a refracted direction crosses out of the volume the ray travelled in: only the glass and
    // diffuse-transmission lobes contribute there, both attenuated by its absorption
    if (md.absorbing && !(v.z * l.z > 0.0f)) color = color * md.beer;
    return color;
}

#ifdef __CUDACC__
// The same evaluation as one out-of-line function per translation unit. Kernels that evaluate the
// BSDF from several call sites (shading: the light sample, RIS candidates, BSDF-sampled light
// hits; ReSTIR reuse: the target functions) share one copy of its code instead of one inlined
// copy per site, which their instruction caches could not hold (ncu: "no instruction" was the
// shade kernel's top stall). Measured on the 1080p many-light ReSTIR frame: spatial reuse 5.23 ->
// 3.66 ms, temporal 4.17 -> 3.51, shading 11.9 -> 10.4. The initial candidates' light loop keeps
// the inlined eval (13.3 ms outlined against 10.4 inlined).
static __device__ __noinline__ V3 eval_outlined(const Material& m, const Medium& md, bool height_correlated,
                                                const Query& q, int lobe, float& pdf)
{
    return eval(m, md, height_correlated, q, lobe, pdf);
}
#define GBPT_BSDF_EVAL_CALL eval_outlined
#else
#define GBPT_BSDF_EVAL_CALL eval
#endif

// Samples a light direction (returned in world space, 'lobe' = where it came from), then
// evaluates f and pdf for it. A reflection lobe that sampled below the geometric surface
// returns f = 0, pdf = 0.
template <typename Rng, bool INLINE_EVAL = false>
GBPT_HD V3 sample(const Material& m, const Medium& md, bool height_correlated, V3 view, V3 ns, V3 ng, Rng& rng, V3& dir,
                  int& lobe, float& pdf)
{
    pdf = 0.0f;
    lobe = GBPT_LOBE_NONE;
    const Lobes w = lobe_weights(m, !md.inside);
    const Lobes p = lobe_probabilities(w);
    const float c0 = p.coat;
    const float c1 = c0 + p.sheen;
    const float c2 = c1 + p.metal1;
    const float c3 = c2 + p.metal2;
    const float c4 = c3 + p.specular;
    const float c5 = c4 + p.diffuse;
    const float c6 = c5 + p.diffuse_transmission;
    const float u = rng();
    const bool through_dt = u > c5 && u < c6;
    const bool through_glass = u > c6;
    const Frame FR = make_rotated_frame(ns, m.anisotropy_rotation * kPi);
    const V3 vr = FR.to_local(view);
    if (u < c0)
    {
        const Frame FC = make_rotated_frame(ns, m.coat_anisotropy_rotation * kPi);
        lobe = GBPT_LOBE_COAT;
        dir = FC.to_world(ggx_sample_reflection(m.coat_roughness, m.coat_anisotropy, FC.to_local(view), rng));
    }
    else if (u < c1)
    {
        dir = ns;  // sheen lobe: weight is 0 for every supported material, never reached
    }
    else if (u < c2)
    {
        lobe = GBPT_LOBE_METAL_1;
        dir = FR.to_world(ggx_sample_reflection(m.roughness, m.anisotropy, vr, rng));
    }
    else if (u < c3)
    {
        lobe = GBPT_LOBE_METAL_2;
        dir = FR.to_world(ggx_sample_reflection(m.second_roughness, m.anisotropy, vr, rng));
    }
    else if (u < c4)
    {
        lobe = GBPT_LOBE_SPECULAR;
        dir = FR.to_world(ggx_sample_reflection(m.roughness, m.anisotropy, vr, rng));
    }
    else if (u < c5)
    {
        lobe = GBPT_LOBE_DIFFUSE;
        dir = cosine_around(ns, rng);
    }
    else if (u < c6)
    {
        lobe = GBPT_LOBE_DIFFUSE_TRANSMISSION;
        dir = cosine_around(-ns, rng);
    }
    else
        dir = FR.to_world(glass_sample(m, md, vr, rng, lobe));

    if (dot(dir, ng) < 0.0f && !through_glass && !through_dt) return v3(0.0f);
    Query q;
    q.view = view;
    q.ns = ns;
    q.ng = ng;
    q.light = dir;
    // sampling's evaluation through the out-of-line copy on the device (one copy of the code per
    // translation unit) unless the caller asks for the inlined one
    if constexpr (INLINE_EVAL)
        return eval(m, md, height_correlated, q, lobe, pdf);
    else
        return GBPT_BSDF_EVAL_CALL(m, md, height_correlated, q, lobe, pdf);
}

}  // namespace bsdf
}  // namespace gbpt
