// Layered principled BSDF: eval, pdf and sampling, for the CUDA kernels and for the host build
// that the CPU tests compile (tests/native/bsdf_emu.cpp).
//
// Behaviour follows the reference's principled BSDF with energy compensation, microfacet
// regularization and sheen switched off
// (src/Device/includes/BSDFs/Principled.h:1515-1941 and the lobes it calls):
//   - lobe weights and sampling probabilities: Principled.h:1515-1618;
//   - layering (coat over sheen over metal / glass / glossy base / diffuse transmission, with the
//     fresnel transmission, coat absorption and darkening of each layer attenuating the ones
//     below): Principled.h:955-1060 (coat), 1129-1176 (metal), 1177-1218 (glass), 1219-1270
//     (diffuse transmission), 1272-1513 (specular over diffuse);
//   - GGX: anisotropic D, Smith G1/G2, Heitz 2018 visible-normal sampling, Torrance-Sparrow
//     reflection and Walter 2007 refraction: src/Device/includes/BSDFs/Microfacet.h:25-502;
//   - Fresnel: dielectric, Adobe F82-tint, d'Eon's hemispherical-albedo fit:
//     src/Device/includes/Fresnel.h:41-175; thin-film interference (Belcour and Barla 2017):
//     src/Device/includes/BSDFs/ThinFilm.h:11-226, blended into the metal (Principled.h:143-146),
//     specular (:215-240, 1363-1382) and glass (:462-483, 663-684, 758-785) Fresnel terms;
//   - dispersion: the glass lobe's IORs at the path's wavelength (Principled.h:375-380, 576-581,
//     729-734; Dispersion.h:485-499) and the wavelength's RGB weight (Dispersion.h:424-458);
//   - the Oren-Nayar diffuse lobe (OrenNayar.h:14-63);
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
    // the record itself when the material uses a lobe beyond the common ones (an Oren-Nayar
    // diffuse lobe, a thin film), else null: such materials are evaluated by a separate, out-of-line
    // instantiation that reads those parameters from here, so that the common materials' code and
    // registers stay as they are without them
    const gbpt_principled_material* ext;
};

// a glass lobe whose IOR depends on the path's wavelength (the condition under which the reference
// samples one, Intersect.h:259 and RayVolumeState.h:50)
GBPT_HD bool is_dispersive(const gbpt_principled_material& s)
{
    return s.dispersion_scale > 0.0f && s.specular_transmission > 0.0f;
}

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
    m.ext = (s.diffuse_lobe == GBPT_DIFFUSE_OREN_NAYAR || s.thin_film > 0.0f || is_dispersive(s)) ? &s : nullptr;
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
    float wavelength = 0.0f;  // the path's sampled wavelength (nm) for dispersion; 0: none yet
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

// ---------------------------------------------------------------------------------------------
// thin-film interference (Belcour and Barla, "A Practical Extension to Microfacet Theory for the
// Modeling of Varying Iridescence", 2017, and its supplemental code; ThinFilm.h:11-226): the
// Airy summation of a film between the ambient medium (eta1) and the base (eta3, kappa3), the
// first two orders of its phase terms integrated against the CIE XYZ sensitivities (Gaussian fits
// in Fourier space), both polarisations averaged, converted to CIE RGB, clamped, then rotated in
// hue about the grey axis.
// ---------------------------------------------------------------------------------------------
GBPT_HD V3 film_sensitivity(float opd, float shift)
{
    const float phase = 2.0f * kPi * opd * 1.0e-6f;
    const float val[3] = {5.4856e-13f, 4.4201e-13f, 5.2481e-13f};
    const float pos[3] = {1.6810e+06f, 1.7953e+06f, 2.2084e+06f};
    const float var[3] = {4.3278e+09f, 9.3046e+09f, 6.6121e+09f};
    float xyz[3];
#pragma unroll
    for (int c = 0; c < 3; c++)
        xyz[c] = val[c] * sqrtf(2.0f * kPi * var[c]) * cosf(pos[c] * phase + shift) * expf(-1.0f * var[c] * phase * phase);
    xyz[0] += 9.7470e-14f * sqrtf(2.0f * kPi * 4.5282e+09f) * cosf(2.2399e+06f * phase + shift) *
              expf(-4.5282e+09f * phase * phase);
    return v3(xyz[0], xyz[1], xyz[2]) / 1.0685e-7f;
}

// phase shifts of the parallel and perpendicular components reflected at an interface from eta1
// onto (eta2, kappa2)
GBPT_HD void film_phase(float cos_i, float eta1, float eta2, float kappa2, float& phi_par, float& phi_perp)
{
    const float sin2 = 1.0f - sq(cos_i);
    const float A = sq(eta2) * (1.0f - sq(kappa2)) - sq(eta1) * sin2;
    const float B = sqrtf(sq(A) + sq(2.0f * sq(eta2) * kappa2));
    const float U = sqrtf((A + B) * 0.5f);
    const float V = sqrtf((B - A) * 0.5f);
    phi_perp = atan2f(2.0f * eta1 * V * cos_i, sq(U) + sq(V) - sq(eta1 * cos_i));
    phi_par = atan2f(2.0f * eta1 * sq(eta2) * cos_i * (2.0f * kappa2 * U - (1.0f - sq(kappa2)) * V),
                     sq(sq(eta2) * (1.0f + sq(kappa2)) * cos_i) - sq(eta1) * (sq(U) + sq(V)));
}

// reflectances (parallel, perpendicular) of a conductor of relative IOR eta + i k
GBPT_HD void film_conductor(float cos_i, float eta, float k, float& rp, float& rs)
{
    const float c2 = cos_i * cos_i;
    const float s2 = 1.0f - c2;
    const float t1 = eta * eta - k * k - s2;
    const float a2pb2 = sqrtf(t1 * t1 + 4.0f * k * k * eta * eta);
    const float a = sqrtf(0.5f * (a2pb2 + t1));
    const float t2 = a2pb2 + c2;
    const float t3 = 2.0f * a * cos_i;
    rs = clampf(0.0f, 1.0f, (t2 - t3) / (t2 + t3));
    const float t4 = a2pb2 * c2 + s2 * s2;
    const float t5 = t3 * s2;
    rp = clampf(0.0f, 1.0f, rs * (t4 - t5) / (t4 + t5));
}

// rotation of an RGB colour about the grey axis by 'degrees'
GBPT_HD V3 hue_rotate(V3 c, float degrees)
{
    if (degrees == 0.0f) return c;
    const float ca = cosf(degrees / 180.0f * kPi);
    const float sa = sinf(degrees / 180.0f * kPi);
    constexpr float kS = 0.57735026918962576451f;  // sqrt(1/3)
    constexpr float kT = 1.0f / 3.0f;
    const float d = ca + (1.0f - ca) / 3.0f;
    const float p = kT * (1.0f - ca) - kS * sa;
    const float q = kT * (1.0f - ca) + kS * sa;
    const float d2 = ca + kT * (1.0f - ca);
    const V3 r = v3(c.x * d + c.y * p + c.z * q, c.x * q + c.y * d2 + c.z * p, c.x * p + c.y * q + c.z * d2);
    return clamp3(0.0f, 1.0f, r);
}

// RGB reflectance of the film seen from a medium of IOR ambient_ior at cosine cos_i (out of line
// on the device: only film materials take it)
GBPT_HD_OUTLINE V3 thin_film_fresnel(const gbpt_principled_material& e, float ambient_ior, float cos_i)
{
    if (e.thin_film == 0.0f) return v3(0.0f);
    // the base under the film: the override, else the material's own IOR with no extinction
    const float eta1 = ambient_ior, eta2 = e.thin_film_ior;
    const float eta3 = e.thin_film_do_ior_override ? e.thin_film_base_ior_override : e.ior;
    const float kappa3 = e.thin_film_do_ior_override ? e.thin_film_kappa_3 : 0.0f;
    float r12p = 1.0f, r12s = 1.0f, r23p = 0.0f, r23s = 0.0f, t121p = 0.0f, t121s = 0.0f, cos2 = 0.0f;
    const float cos_t2 = 1.0f - (1.0f - sq(cos_i)) * sq(eta1 / eta2);
    if (cos_t2 > 0.0f)
    {
        cos2 = sqrtf(cos_t2);
        film_conductor(cos_i, eta2 / eta1, 0.0f, r12p, r12s);
        film_conductor(cos2, eta3 / eta2, kappa3, r23p, r23s);
        t121p = 1.0f - r12p;
        t121s = 1.0f - r12s;
    }
    const float D = e.thin_film_thickness / 1000.0f * cos2;  // optical path difference, micrometres
    float phi21p, phi21s, phi23p, phi23s;
    film_phase(cos_i, eta1, eta2, 0.0f, phi21p, phi21s);
    film_phase(cos2, eta2, eta3, kappa3, phi23p, phi23s);
    phi21p = kPi - phi21p;
    phi21s = kPi - phi21s;
    const float r123[2] = {sqrtf(r12p * r23p), sqrtf(r12s * r23s)};
    const float r12[2] = {r12p, r12s}, r23[2] = {r23p, r23s}, t121[2] = {t121p, t121s};
    const float phi[2] = {phi23p + phi21p, phi23s + phi21s};
    V3 I = v3(0.0f);
#pragma unroll
    for (int pol = 0; pol < 2; pol++)
    {
        const float Rs = (sq(t121[pol]) * r23[pol]) / (1.0f - r12[pol] * r23[pol]);
        I = I + v3(r12[pol] + Rs);
        float Cm = Rs - t121[pol];
#pragma unroll
        for (int k = 1; k <= 2; k++)
        {
            Cm *= r123[pol];
            I = I + Cm * (2.0f * film_sensitivity(k * D, k * phi[pol]));
        }
    }
    I = I * 0.5f;
    // CIE XYZ (1931) to CIE RGB
    const V3 rgb = v3(2.3646381f * I.x - 0.8965361f * I.y - 0.4680737f * I.z,
                      -0.5151664f * I.x + 1.4264000f * I.y + 0.0887608f * I.z,
                      0.0052037f * I.x - 0.0144081f * I.y + 1.0092106f * I.z);
    return hue_rotate(clamp3(0.0f, 1.0f, rgb), e.thin_film_hue_shift * 360.0f);
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

// refract(d) about n (d and n in the same hemisphere); the zero vector under total internal
// reflection. Without a film the glass lobe never refracts there (its Fresnel term is 1); with a
// film the blended Fresnel term can be below 1 at a totally reflecting interface, where the
// reference's refraction returns NaN directions: sampling returns f = 0, pdf = 0 instead.
GBPT_HD V3 refract_dir(V3 d, V3 n, float eta)
{
    const float noi = dot(d, n);
    const float k = 1.0f - (1.0f - noi * noi) / (eta * eta);
    if (k < 0.0f) return v3(0.0f);
    const float cos_t = sqrtf(k);
    return -d / eta + (noi / eta - cos_t) * n;
}

// Walter et al. 2007 microfacet transmission
GBPT_HD V3 ggx_refraction(const Material& m, float roughness, float eta, V3 F, V3 v, V3 l, V3 h, int lobe, float& pdf)
{
    const float nol = l.z, nov = v.z;
    const float hol = dot(l, h), hov = dot(v, h);
    V3 color;
    if (is_smooth(roughness))
    {
        const bool perfect = dot(refract_dir(v, v3(0.0f, 0.0f, 1.0f), eta), l) > kDeltaAlign;
        if (lobe == GBPT_LOBE_GLASS_REFRACT && perfect)
        {
            color = v3(kDeltaValue) * (1.0f - F) * m.base;
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
        color = m.base * D * (1.0f - F) * g2 * fabsf(hol * hov / denom);
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

// IOR at 'wavelength' (nm) of a medium whose IOR at 587.6 nm is base_ior, from the Abbe number
// scaled by 1 / scale (Cauchy's two-term fit through the Fraunhofer F and C lines, as OpenPBR
// specifies; compute_dispersion_ior, src/Device/includes/Dispersion.h:485-499)
GBPT_HD float dispersion_ior(float abbe_number, float scale, float base_ior, float wavelength)
{
    if (scale == 0.0f) return base_ior;
    constexpr float kD2 = 334777.96f;                  // 587.6^2
    constexpr float kFC = 0.00000191038851931481f;     // 486.1^-2 - 656.3^-2
    const float abbe = abbe_number / scale;
    const float B = (base_ior - 1.0f) / (abbe * kFC);
    const float A = base_ior - B / kD2;
    return A + B / (wavelength * wavelength);
}

// RGB weight of a wavelength (nm, in [360, 830]) for the path's colour filter, averaging (1, 1, 1)
// over that range: the reference's closed-form fit of its CIE-based conversion
// (wavelength_to_RGB_fit, src/Device/includes/Dispersion.h:424-458, the default
// WavelengthToRGBMethod); its coefficients are kept as the reference has them so that dispersive
// paths carry the same colours.
GBPT_HD V3 wavelength_rgb(float wl)
{
    V3 c;
    if (wl < 463.0f)
        c.x = -1.2776028240727566e-01f / (1.0f + expf((wl - 4.2680623367293401e+02f) / 8.2197460736637176e+00f)) +
              -1.3925673552505122e-11f * expf((wl - 45.0f) / 1.8175459086411596e+01f) + 1.2898689750552100e-01f;
    else if (wl > 553.0f)
        c.x = 1.7963649137825513e+01f * (1.0f / 2.6577826611702449e+01f) *
                  expf(-0.5f * sq((wl - 6.0625724092824566e+02f) * (1.0f / 2.6577826611702449e+01f))) +
              2.5574660155104657e-03f;
    else
        c.x = 0.0f;
    c.y = 3.4962267376163049e+02f * expf(-0.5f * sq((wl - 5.4209217455705152e+02f) / -2.9598170255834638e+01f)) / wl;
    c.z = expf(3.2987659944421112e+03f + (-2.0975839709372405e+05f / wl) - 4.6368268395094020e+02f * logf(wl));
    return c * 10.0f;
}

// relative IOR across the glass interface, kept away from 1 (a null half vector otherwise); both
// sides' IORs taken at the path's wavelength for a dispersive material. eta_i: the incident side's
// IOR (what a film on the glass sees).
GBPT_HD float glass_eta(const Material& m, const Medium& md, float& eta_i)
{
    eta_i = md.eta_incident;
    float eta_t = md.eta_outgoing;
    if (m.ext && m.ext->dispersion_scale > 0.0f && md.wavelength > 0.0f)
    {
        eta_i = dispersion_ior(m.ext->dispersion_abbe_number, m.ext->dispersion_scale, eta_i, md.wavelength);
        eta_t = dispersion_ior(m.ext->dispersion_abbe_number, m.ext->dispersion_scale, eta_t, md.wavelength);
    }
    float eta = eta_t / eta_i;
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

// The glass Fresnel term blended with the film's, seen from the incident medium (no thin-walled
// correction with a film)
GBPT_HD V3 glass_fresnel_film(const gbpt_principled_material& e, float hov, float eta, float eta_incident)
{
    const V3 F_film = thin_film_fresnel(e, eta_incident, hov);
    return lerp(e.thin_film < 1.0f ? v3(fresnel_dielectric(hov, eta)) : v3(0.0f), F_film, e.thin_film);
}

// Fresnel of the specular layer (relative IOR eta_s), blended with the film's seen from the layer
// above it when the material has one (principled_specular_fresnel)
template <bool EXT>
GBPT_HD V3 specular_fresnel(const Material& m, float eta_s, float cos_i)
{
    const float F = fresnel_dielectric(cos_i, eta_s);
    if constexpr (!EXT) return v3(F);
    else if (m.ext->thin_film == 0.0f) return v3(F);
    else return lerp(m.ext->thin_film < 1.0f ? v3(F) : v3(0.0f), thin_film_fresnel(*m.ext, m.ior / eta_s, cos_i),
                     m.ext->thin_film);
}

// The Oren-Nayar factor A + B max(0, cos(phi_i - phi_o)) sin(alpha) tan(beta) of the diffuse lobe
// (oren_nayar_brdf_eval, src/Device/includes/BSDFs/OrenNayar.h:14-47), v and l in the unrotated
// shading frame; the azimuth difference does not depend on the frame's tangent
GBPT_HD float oren_nayar_shape(float sigma, V3 v, V3 l)
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
    // A and B from the facet-slope deviation (MaterialUtils::get_oren_nayar_AB,
    // src/HostDeviceCommon/Material/MaterialUtils.h:18-23)
    const float s2 = sigma * sigma;
    const float A = 1.0f - s2 / (2.0f * (s2 + 0.33f));
    const float B = 0.45f * s2 / (s2 + 0.09f);
    return A + B * max_cos * sin_alpha * tan_beta;
}

// Glass lobe (Principled.h:359-558): reflection or refraction through a GGX interface.
template <bool EXT>
GBPT_HD V3 glass_eval(const Material& m, const Medium& md, bool height_correlated, V3 v, V3 l, int lobe, float& pdf)
{
    pdf = 0.0f;
    const float nov = v.z, nol = l.z;
    if (fabsf(nol) < 1.0e-8f) return v3(0.0f);
    const bool reflecting = nol * nov > 0.0f;
    float eta_i;
    const float eta = glass_eta(m, md, eta_i);
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
    V3 F;
    if (EXT && m.ext->thin_film > 0.0f) F = glass_fresnel_film(*m.ext, hov, eta, eta_i);
    else F = v3(glass_fresnel(m, hov, eta, rough));
    const float p_reflect = luminance(F);
    if (reflecting)
    {
        const Delta ds = delta_state(m, rough, m.anisotropy, lobe);
        const V3 c = ggx_reflection(rough, m.anisotropy, height_correlated, F, v, l, h, ds, pdf);
        pdf *= p_reflect;
        return c;
    }
    V3 c = ggx_refraction(m, rough, eta, F, v, l, h, lobe, pdf);
    pdf *= 1.0f - p_reflect;
    if (m.thin_walled) c = c * m.base;
    return c;
}

// the glass lobe's reflection probability with a film (out of line on the device)
GBPT_HD_OUTLINE float glass_reflect_probability_film(const gbpt_principled_material& e, float hov, float eta,
                                                     float eta_incident)
{
    return luminance(glass_fresnel_film(e, hov, eta, eta_incident));
}

template <typename Rng>
GBPT_HD V3 glass_sample(const Material& m, const Medium& md, V3 v, Rng& rng, int& lobe)
{
    float eta_i;
    const float eta = glass_eta(m, md, eta_i);
    const float rough = thin_walled_roughness(m.thin_walled, m.roughness, eta);
    float ax, ay;
    ggx_alphas(rough, m.anisotropy, ax, ay);
    V3 h = ggx_sample_visible_normal(v, ax, ay, rng);
    const float hov = dot(v, h);
    const float p_reflect = (m.ext && m.ext->thin_film > 0.0f) ? glass_reflect_probability_film(*m.ext, hov, eta, eta_i)
                                               : luminance(v3(glass_fresnel(m, hov, eta, rough)));
    if (rng() < p_reflect)
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

// f (without cosine) and pdf for light direction q.light, given the lobe it was sampled from;
// EXT: the material uses an Oren-Nayar diffuse lobe or a thin film (a separate instantiation, so
// that the common materials run code without those terms)
template <bool EXT>
GBPT_HD V3 eval_layers(const Material& m, const Medium& md, bool height_correlated, const Query& q, int lobe, float& pdf)
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
            V3 F = fresnel_f82_tint(m.base, m.f82, m.f90, m.f90_exponent, hol);
            if constexpr (EXT)
                if (m.ext->thin_film > 0.0f) F = lerp(F, thin_film_fresnel(*m.ext, eta_in, hol), m.ext->thin_film);
            c = ggx_reflection(metal_r[k], m.anisotropy, height_correlated, F, vr, lr, hr, ds, lobe_pdf);
        }
        color = color + c * metal_w[k] * throughput;
        pdf += lobe_pdf * metal_p[k];
    }

    // glass (rotated frame), beside the glossy base rather than below it
    if (w.glass > 0.0f)
    {
        float lobe_pdf;
        const V3 c = glass_eval<EXT>(m, md, height_correlated, vr, lr, lobe, lobe_pdf);
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
        V3 c = ggx_reflection(m.roughness, m.anisotropy, height_correlated, specular_fresnel<EXT>(m, eta_s, dot(lr, hr)),
                              vr, lr, hr, ds, lobe_pdf);
        c = c * lerp(v3(1.0f), m.specular_tint * m.specular_color, m.specular);
        glossy = glossy + c * w.specular * throughput;
        V3 att;
        if (!EXT || m.ext->thin_film == 0.0f)
        {
            const float light_f = fresnel_dielectric(fabsf(lr.z), eta_s) * (1.0f - m.diffuse_transmission);
            const float view_f = fresnel_dielectric(fabsf(vr.z), eta_s);
            att = v3((1.0f - light_f) * (1.0f - view_f));
        }
        else
        {
            const V3 light_f = specular_fresnel<true>(m, eta_s, fabsf(lr.z)) * (1.0f - m.diffuse_transmission);
            att = (1.0f - light_f) * (1.0f - specular_fresnel<true>(m, eta_s, fabsf(vr.z)));
        }
        att = att * specular_darkening(m, eta_s);
        throughput = throughput * lerp(v3(1.0f), att, m.specular);
        pdf += lobe_pdf * p.specular;
    }
    const float diffuse_w = w.diffuse * (refracting ? 0.0f : 1.0f);
    if (diffuse_w > 0.0f && v.z > 0.0f && l.z > 0.0f)
    {
        float shape = 1.0f;
        if constexpr (EXT)
            if (m.ext->diffuse_lobe == GBPT_DIFFUSE_OREN_NAYAR) shape = oren_nayar_shape(m.ext->oren_nayar_sigma, v, l);
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

// the instantiation for materials with extension lobes, out of line on the device
GBPT_HD_OUTLINE V3 eval_ext(const Material& m, const Medium& md, bool height_correlated, const Query& q, int lobe,
                             float& pdf)
{
    return eval_layers<true>(m, md, height_correlated, q, lobe, pdf);
}

GBPT_HD V3 eval(const Material& m, const Medium& md, bool height_correlated, const Query& q, int lobe, float& pdf)
{
    if (m.ext) return eval_ext(m, md, height_correlated, q, lobe, pdf);
    return eval_layers<false>(m, md, height_correlated, q, lobe, pdf);
}

#ifdef __CUDACC__
// The same evaluation as one out-of-line function per translation unit. Kernels that evaluate the
// BSDF from several call sites (shading: the light sample, RIS candidates, BSDF-sampled light
// hits; ReSTIR reuse: the target functions) share one copy of its code instead of one inlined
// copy per site, which their instruction caches could not hold (ncu: "no instruction" was the
// shade kernel's top stall). Measured on the 1080p many-light ReSTIR frame: spatial reuse 5.23 ->
// 3.66 ms, temporal 4.17 -> 3.51, shading 11.9 -> 10.4. The initial candidates' light loop keeps
// the inlined eval (13.3 ms outlined against 10.4 inlined).
// Materials with extension lobes go to eval_ext, its own out-of-line function: the choice is made
// here, at the call site, so that neither copy calls the other (a call inside the evaluation, or
// inside a kernel's candidate loop, cost 4-5% of a ReSTIR frame through the calling convention).
static __device__ __noinline__ V3 eval_common(const Material& m, const Medium& md, bool height_correlated,
                                              const Query& q, int lobe, float& pdf)
{
    return eval_layers<false>(m, md, height_correlated, q, lobe, pdf);
}
__device__ __forceinline__ V3 eval_outlined(const Material& m, const Medium& md, bool height_correlated,
                                            const Query& q, int lobe, float& pdf)
{
    return m.ext ? eval_ext(m, md, height_correlated, q, lobe, pdf) : eval_common(m, md, height_correlated, q, lobe, pdf);
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
    {
        const V3 d = glass_sample(m, md, vr, rng, lobe);
        if (d.x == 0.0f && d.y == 0.0f && d.z == 0.0f)
        {
            dir = ns;  // refraction under total internal reflection: no direction
            return v3(0.0f);
        }
        dir = FR.to_world(d);
    }

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
