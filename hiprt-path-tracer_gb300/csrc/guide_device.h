// Device math of the guiding network: hash-grid encoding, spherical-harmonic encoding, the
// vMF-mixture head (pdf, loss gradient, sampling), shared by the training / inference kernels
// (guide.cu) and the path tracer's guided sampling (render.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gbpt_guide.h"
#include "hd_math.h"

namespace gbpt {
namespace guide {

using namespace hd;

constexpr int kLevels = GBPT_GUIDE_LEVELS;
constexpr int kTable = GBPT_GUIDE_TABLE;
constexpr int kFeat = GBPT_GUIDE_FEATURES;
constexpr int kIn = GBPT_GUIDE_IN;
constexpr int kHid = GBPT_GUIDE_HIDDEN;
constexpr int kOut = GBPT_GUIDE_OUT;
constexpr int kLobes = GBPT_GUIDE_LOBES;
constexpr int kRow = GBPT_GUIDE_ROW;
constexpr int kGridFeatures = kLevels * kFeat;  // inputs 0..31
constexpr int kNormalIn = kGridFeatures;        // inputs 32..34
constexpr int kShIn = kNormalIn + 3;            // inputs 35..50
constexpr int kAlphaOut = kLobes * 5;           // raw output 40
constexpr float kKappaMin = 0.1f;
constexpr float kKappaMax = 500.0f;
constexpr float kAlphaMin = 0.05f;

// resolutions floor(16 * 256^(l / 15)): 16 .. 4096, geometric
__host__ __device__ __forceinline__ int level_res(int l)
{
    const int r[16] = {16, 23, 33, 48, 70, 101, 147, 212, 307, 445, 645, 933, 1351, 1955, 2830, 4096};
    return r[l];
}

// table slot of grid vertex (x, y, z) at a level of resolution res: dense when the level fits
__host__ __device__ __forceinline__ uint32_t grid_slot(int res, uint32_t x, uint32_t y, uint32_t z)
{
    const uint32_t side = (uint32_t)res + 1u;
    if (side * side * side <= (uint32_t)kTable) return x + side * (y + side * z);
    return (x * 1u ^ y * 2654435761u ^ z * 805459861u) & (uint32_t)(kTable - 1);
}

struct Domain
{
    float lo[3], inv_ext[3];
};

// Cell of point u (unit-box coordinates) at a level: lower corner and fractional position
__device__ __forceinline__ void level_cell(const float* u, int res, uint32_t* i0, float* f)
{
#pragma unroll
    for (int a = 0; a < 3; a++)
    {
        const float x = u[a] * (float)res;
        int xi = (int)floorf(x);
        xi = xi < 0 ? 0 : (xi > res - 1 ? res - 1 : xi);
        i0[a] = (uint32_t)xi;
        f[a] = x - (float)xi;
    }
}

__device__ __forceinline__ void unit_coords(const Domain& d, V3 p, float* u)
{
    u[0] = clampf(0.0f, 1.0f, (p.x - d.lo[0]) * d.inv_ext[0]);
    u[1] = clampf(0.0f, 1.0f, (p.y - d.lo[1]) * d.inv_ext[1]);
    u[2] = clampf(0.0f, 1.0f, (p.z - d.lo[2]) * d.inv_ext[2]);
}

__device__ __forceinline__ float corner_weight(int c, const float* f)
{
    return ((c & 1) ? f[0] : 1.0f - f[0]) * ((c & 2) ? f[1] : 1.0f - f[1]) * ((c & 4) ? f[2] : 1.0f - f[2]);
}

// Trilinear hash-grid lookup through the BF16 copy of the features (2 per entry in one 32-bit
// word, feature 0 in the low half): 32 features of point p (scene coordinates)
__device__ __forceinline__ void encode(const Domain& d, const uint32_t* __restrict__ grid_bf16, V3 p, float* feat)
{
    float u[3];
    unit_coords(d, p, u);
    // fully unrolled: the level resolutions and the dense / hashed choice become constants and
    // the 128 gathers can be issued together
#pragma unroll
    for (int l = 0; l < kLevels; l++)
    {
        const int res = level_res(l);
        uint32_t i0[3];
        float f[3];
        level_cell(u, res, i0, f);
        float f0 = 0.0f, f1 = 0.0f;
        const uint32_t* g = grid_bf16 + (size_t)l * kTable;
#pragma unroll
        for (int c = 0; c < 8; c++)
        {
            const float w = corner_weight(c, f);
            const uint32_t s = grid_slot(res, i0[0] + (c & 1), i0[1] + ((c >> 1) & 1), i0[2] + ((c >> 2) & 1));
            const uint32_t v = __ldg(g + s);
            f0 += w * __uint_as_float(v << 16);
            f1 += w * __uint_as_float(v & 0xFFFF0000u);
        }
        feat[2 * l] = f0;
        feat[2 * l + 1] = f1;
    }
}

// Scatters d(loss)/d(features) to the FP32 grid gradient with the same trilinear weights
__device__ __forceinline__ void encode_backward(const Domain& d, float* __restrict__ grad_grid, V3 p, const float* dfeat)
{
    float u[3];
    unit_coords(d, p, u);
    for (int l = 0; l < kLevels; l++)
    {
        if (dfeat[2 * l] == 0.0f && dfeat[2 * l + 1] == 0.0f) continue;
        const int res = level_res(l);
        uint32_t i0[3];
        float f[3];
        level_cell(u, res, i0, f);
        float* gl = grad_grid + (size_t)l * kTable * kFeat;
        for (int c = 0; c < 8; c++)
        {
            const float w = corner_weight(c, f);
            const uint32_t s = grid_slot(res, i0[0] + (c & 1), i0[1] + ((c >> 1) & 1), i0[2] + ((c >> 2) & 1));
            atomicAdd(gl + 2 * s, w * dfeat[2 * l]);
            atomicAdd(gl + 2 * s + 1, w * dfeat[2 * l + 1]);
        }
    }
}

// Real spherical harmonics of bands 0..3 (16 values) of a unit vector, orthonormal on the sphere:
// normalisation sqrt((2l+1)/(4 pi) (l-|m|)!/(l+|m|)!), times sqrt(2) for m != 0, no
// Condon-Shortley phase; the polynomials are the Cartesian forms of the associated Legendre
// functions of z times cos / sin of m phi.
__host__ __device__ __forceinline__ void sh16(float x, float y, float z, float* o)
{
    const float xx = x * x, yy = y * y, zz = z * z;
    o[0] = 0.28209479177387814f;
    o[1] = 0.48860251190291992f * y;
    o[2] = 0.48860251190291992f * z;
    o[3] = 0.48860251190291992f * x;
    o[4] = 1.0925484305920792f * x * y;
    o[5] = 1.0925484305920792f * y * z;
    o[6] = 0.31539156525252005f * (3.0f * zz - 1.0f);
    o[7] = 1.0925484305920792f * x * z;
    o[8] = 0.54627421529603959f * (xx - yy);
    o[9] = 0.59004358992664352f * y * (3.0f * xx - yy);
    o[10] = 2.8906114426405538f * x * y * z;
    o[11] = 0.45704579946446572f * y * (5.0f * zz - 1.0f);
    o[12] = 0.37317633259011546f * z * (5.0f * zz - 3.0f);
    o[13] = 0.45704579946446572f * x * (5.0f * zz - 1.0f);
    o[14] = 1.4453057213202769f * z * (xx - yy);
    o[15] = 0.59004358992664352f * x * (xx - 3.0f * yy);
}

// Network input row: 32 grid features, the normal, SH16 of the view direction, zeros
__device__ __forceinline__ void input_row(const float* feat, V3 n, V3 view, float* x)
{
#pragma unroll
    for (int i = 0; i < kGridFeatures; i++) x[i] = feat[i];
    x[kNormalIn] = n.x;
    x[kNormalIn + 1] = n.y;
    x[kNormalIn + 2] = n.z;
    sh16(view.x, view.y, view.z, x + kShIn);
#pragma unroll
    for (int i = kShIn + 16; i < kIn; i++) x[i] = 0.0f;
}

__host__ __device__ __forceinline__ float softplus(float x) { return x > 20.0f ? x : log1pf(expf(x)); }
__host__ __device__ __forceinline__ float sigmoid(float x) { return 1.0f / (1.0f + expf(-x)); }

struct Lobe
{
    V3 mu;
    float kappa, weight;
};

// Mixture from the raw outputs: lobe i from raw[5i..5i+4] (direction xyz, concentration, weight
// logit); also the norms of the raw directions (for the backward pass) and the probability of
// sampling the mixture.
__device__ __forceinline__ void head(const float* raw, Lobe* lobes, float* dir_len, float& alpha)
{
    float mx = -1e30f;
#pragma unroll
    for (int i = 0; i < kLobes; i++) mx = fmaxf(mx, raw[5 * i + 4]);
    float sum = 0.0f;
#pragma unroll
    for (int i = 0; i < kLobes; i++)
    {
        const V3 a = v3(raw[5 * i], raw[5 * i + 1], raw[5 * i + 2]);
        const float len = sqrtf(dot(a, a) + 1e-12f);
        dir_len[i] = len;
        lobes[i].mu = a / len;
        lobes[i].kappa = fminf(softplus(raw[5 * i + 3]) + kKappaMin, kKappaMax);
        lobes[i].weight = expf(raw[5 * i + 4] - mx);
        sum += lobes[i].weight;
    }
#pragma unroll
    for (int i = 0; i < kLobes; i++) lobes[i].weight /= sum;
    alpha = kAlphaMin + (1.0f - 2.0f * kAlphaMin) * sigmoid(raw[kAlphaOut]);
}

// log of the vMF density kappa / (2 pi (1 - e^{-2 kappa})) exp(kappa (mu.w - 1))
__host__ __device__ __forceinline__ float log_vmf(float kappa, float c)
{
    return logf(kappa) - 1.8378770664093453f - log1pf(-expf(-2.0f * kappa)) + kappa * (c - 1.0f);
}

__device__ __forceinline__ float mixture_pdf(const Lobe* lobes, V3 w)
{
    float q = 0.0f;
    for (int i = 0; i < kLobes; i++) q += lobes[i].weight * expf(log_vmf(lobes[i].kappa, dot(lobes[i].mu, w)));
    return q;
}

// Gradient of the sample's loss with respect to the 48 raw outputs, scale = w / sum(w):
//   -scale log q(w)                                    -> lobe outputs 0..39
//   -scale log(alpha q + (1 - alpha) p_bsdf), q fixed  -> output 40 (only when p_bsdf >= 0)
// Returns the sample's loss.
__device__ __forceinline__ float head_backward(const float* raw, const Lobe* lobes, const float* dir_len, float alpha, V3 w,
                                               float scale, float p_bsdf, float* draw)
{
    float lv[kLobes];
    float mx = -1e30f;
    for (int i = 0; i < kLobes; i++)
    {
        lv[i] = logf(fmaxf(lobes[i].weight, 1e-30f)) + log_vmf(lobes[i].kappa, dot(lobes[i].mu, w));
        mx = fmaxf(mx, lv[i]);
    }
    float s = 0.0f;
    for (int i = 0; i < kLobes; i++) s += expf(lv[i] - mx);
    const float logq = mx + logf(s);
    for (int i = 0; i < kOut; i++) draw[i] = 0.0f;
    for (int i = 0; i < kLobes; i++)
    {
        const float resp = expf(lv[i] - logq);  // pi_i v_i / q
        const float k = lobes[i].kappa;
        const float c = dot(lobes[i].mu, w);
        // weight logits (softmax): d log q / d l_i = resp_i - pi_i
        draw[5 * i + 4] = -scale * (resp - lobes[i].weight);
        // concentration: d log v / d kappa = 1/k - 2e^{-2k}/(1-e^{-2k}) + c - 1, times softplus'
        const float e2 = expf(-2.0f * k);
        const float dlogv = 1.0f / k - 2.0f * e2 / (1.0f - e2) + c - 1.0f;
        const bool clamped = softplus(raw[5 * i + 3]) + kKappaMin >= kKappaMax;
        draw[5 * i + 3] = clamped ? 0.0f : -scale * resp * dlogv * sigmoid(raw[5 * i + 3]);
        // direction: d log v / d mu = kappa w; mu = a / |a|
        const V3 gm = (w - c * lobes[i].mu) * (resp * k / dir_len[i]);
        draw[5 * i] = -scale * gm.x;
        draw[5 * i + 1] = -scale * gm.y;
        draw[5 * i + 2] = -scale * gm.z;
    }
    float loss = -scale * logq;
    if (p_bsdf >= 0.0f && scale > 0.0f)
    {
        const float q = expf(logq);
        const float c = alpha * q + (1.0f - alpha) * p_bsdf;
        if (c > 0.0f)
        {
            const float sg = sigmoid(raw[kAlphaOut]);
            draw[kAlphaOut] = -scale * (q - p_bsdf) / c * (1.0f - 2.0f * kAlphaMin) * sg * (1.0f - sg);
            loss += -scale * logf(c);
        }
    }
    return loss;
}

// Samples a vMF lobe with two uniforms (Jakob's numerically stable inversion of the cosine to
// the mean, "Numerically stable sampling of the von Mises Fisher distribution on S2", 2012)
__device__ __forceinline__ V3 sample_vmf(V3 mu, float k, float u1, float u2)
{
    const float wz = fminf(1.0f, fmaxf(-1.0f, 1.0f + logf(u1 + (1.0f - u1) * expf(-2.0f * k)) / k));
    const float r = sqrtf(fmaxf(0.0f, 1.0f - wz * wz));
    float sn, cs;
    sincosf(kTwoPi * u2, &sn, &cs);
    // frame around mu (Frisvad, "Building an orthonormal basis from a 3D unit vector without
    // normalization", 2012)
    const V3 n = mu;
    V3 t, b;
    if (n.z < -0.99998796f)
    {
        t = v3(0.0f, -1.0f, 0.0f);
        b = v3(-1.0f, 0.0f, 0.0f);
    }
    else
    {
        const float a = -n.x / (1.0f + n.z);
        t = v3(1.0f + n.x * a, a * n.y, -n.x);
        b = v3(t.y, 1.0f - n.y * n.y / (1.0f + n.z), -n.y);
    }
    return normalize(t * (r * cs) + b * (r * sn) + n * wz);
}

// Mixture of one inferred row read from global memory one lobe at a time (the path tracer's
// per-entry rows: 8 x (mu xyz, kappa, weight), alpha); keeps the values out of registers.
__device__ __forceinline__ float mixture_pdf_at(const float* __restrict__ L, V3 w)
{
    float q = 0.0f;
#pragma unroll 2
    for (int i = 0; i < kLobes; i++)
    {
        const float* l = L + 5 * i;
        const float wt = __ldg(l + 4);
        if (wt > 0.0f) q += wt * expf(log_vmf(__ldg(l + 3), dot(v3(__ldg(l), __ldg(l + 1), __ldg(l + 2)), w)));
    }
    return q;
}

// Samples the row's mixture with three uniforms: the lobe by u0, then the lobe's vMF
__device__ __forceinline__ V3 sample_mixture_at(const float* __restrict__ L, float u0, float u1, float u2)
{
    int pick = kLobes - 1;
    float acc = 0.0f;
    for (int i = 0; i < kLobes; i++)
    {
        acc += __ldg(L + 5 * i + 4);
        if (u0 < acc)
        {
            pick = i;
            break;
        }
    }
    const float* l = L + 5 * pick;
    return sample_vmf(v3(__ldg(l), __ldg(l + 1), __ldg(l + 2)), __ldg(l + 3), u1, u2);
}

__device__ __forceinline__ float alpha_at(const float* __restrict__ L) { return __ldg(L + kAlphaOut); }

}  // namespace guide
}  // namespace gbpt
