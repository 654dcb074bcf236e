// Device math of the guiding network: hash-grid encoding, the vMF-mixture head (pdf, log-pdf
// gradient, sampling), shared by the training / inference kernels (guide.cu) and the path
// tracer's guided sampling (render.cu).
#pragma once

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
constexpr float kKappaMin = 0.1f;
constexpr float kKappaMax = 500.0f;

// resolutions floor(4 * 1.5^l)
__host__ __device__ __forceinline__ int level_res(int l)
{
    const int r[8] = {4, 6, 9, 13, 20, 30, 45, 68};
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

// Trilinear hash-grid lookup: 16 features of point p (in scene coordinates)
__device__ __forceinline__ void encode(const Domain& d, const float* __restrict__ grid, V3 p, float* feat)
{
    const float u[3] = {clampf(0.0f, 1.0f, (p.x - d.lo[0]) * d.inv_ext[0]), clampf(0.0f, 1.0f, (p.y - d.lo[1]) * d.inv_ext[1]),
                        clampf(0.0f, 1.0f, (p.z - d.lo[2]) * d.inv_ext[2])};
#pragma unroll
    for (int l = 0; l < kLevels; l++)
    {
        const int res = level_res(l);
        uint32_t i0[3];
        float f[3];
#pragma unroll
        for (int a = 0; a < 3; a++)
        {
            const float x = u[a] * (float)res;
            int xi = (int)floorf(x);
            xi = xi < 0 ? 0 : (xi > res - 1 ? res - 1 : xi);
            i0[a] = (uint32_t)xi;
            f[a] = x - (float)xi;
        }
        float f0 = 0.0f, f1 = 0.0f;
#pragma unroll
        for (int c = 0; c < 8; c++)
        {
            const float w = ((c & 1) ? f[0] : 1.0f - f[0]) * ((c & 2) ? f[1] : 1.0f - f[1]) * ((c & 4) ? f[2] : 1.0f - f[2]);
            const uint32_t s = grid_slot(res, i0[0] + (c & 1), i0[1] + ((c >> 1) & 1), i0[2] + ((c >> 2) & 1));
            const float2 g = *reinterpret_cast<const float2*>(grid + ((size_t)l * kTable + s) * kFeat);
            f0 += w * g.x;
            f1 += w * g.y;
        }
        feat[2 * l] = f0;
        feat[2 * l + 1] = f1;
    }
}

// Scatters d(loss)/d(features) back to the grid with the same trilinear weights
__device__ __forceinline__ void encode_backward(const Domain& d, float* __restrict__ grad_grid, V3 p, const float* dfeat)
{
    const float u[3] = {clampf(0.0f, 1.0f, (p.x - d.lo[0]) * d.inv_ext[0]), clampf(0.0f, 1.0f, (p.y - d.lo[1]) * d.inv_ext[1]),
                        clampf(0.0f, 1.0f, (p.z - d.lo[2]) * d.inv_ext[2])};
    for (int l = 0; l < kLevels; l++)
    {
        if (dfeat[2 * l] == 0.0f && dfeat[2 * l + 1] == 0.0f) continue;
        const int res = level_res(l);
        uint32_t i0[3];
        float f[3];
        for (int a = 0; a < 3; a++)
        {
            const float x = u[a] * (float)res;
            int xi = (int)floorf(x);
            xi = xi < 0 ? 0 : (xi > res - 1 ? res - 1 : xi);
            i0[a] = (uint32_t)xi;
            f[a] = x - (float)xi;
        }
        for (int c = 0; c < 8; c++)
        {
            const float w = ((c & 1) ? f[0] : 1.0f - f[0]) * ((c & 2) ? f[1] : 1.0f - f[1]) * ((c & 4) ? f[2] : 1.0f - f[2]);
            const uint32_t s = grid_slot(res, i0[0] + (c & 1), i0[1] + ((c >> 1) & 1), i0[2] + ((c >> 2) & 1));
            float* g = grad_grid + ((size_t)l * kTable + s) * kFeat;
            atomicAdd(g, w * dfeat[2 * l]);
            atomicAdd(g + 1, w * dfeat[2 * l + 1]);
        }
    }
}

// Network input row: 16 grid features, the normal, a constant 1 (the bias input), the direction
// towards the viewer (outgoing direction of the shading point), zeros
__device__ __forceinline__ void input_row(const float* feat, V3 n, V3 view, float* x)
{
#pragma unroll
    for (int i = 0; i < 16; i++) x[i] = feat[i];
    x[16] = n.x;
    x[17] = n.y;
    x[18] = n.z;
    x[19] = 1.0f;
    x[20] = view.x;
    x[21] = view.y;
    x[22] = view.z;
#pragma unroll
    for (int i = 23; i < kIn; i++) x[i] = 0.0f;
}

__device__ __forceinline__ float softplus(float x) { return x > 20.0f ? x : log1pf(expf(x)); }
__device__ __forceinline__ float sigmoid(float x) { return 1.0f / (1.0f + expf(-x)); }

struct Lobe
{
    V3 mu;
    float kappa, weight;
};

// Mixture from the 48 raw outputs: lobe i from raw[5i..5i+4] (direction xyz, concentration,
// weight logit). Also returns the norms of the raw directions (for the backward pass).
__device__ __forceinline__ void head(const float* raw, Lobe* lobes, float* dir_len)
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
}

// log of the vMF density kappa / (2 pi (1 - e^{-2 kappa})) exp(kappa (mu.w - 1))
__device__ __forceinline__ float log_vmf(float kappa, float c)
{
    return logf(kappa) - 1.8378770664093453f - log1pf(-expf(-2.0f * kappa)) + kappa * (c - 1.0f);
}

__device__ __forceinline__ float mixture_pdf(const Lobe* lobes, V3 w)
{
    float q = 0.0f;
    for (int i = 0; i < kLobes; i++) q += lobes[i].weight * expf(log_vmf(lobes[i].kappa, dot(lobes[i].mu, w)));
    return q;
}

// d(-scale * log q(w))/d(raw) for the 48 raw outputs; returns log q.
__device__ __forceinline__ float head_backward(const float* raw, const Lobe* lobes, const float* dir_len, V3 w, float scale,
                                               float* draw)
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
    return logq;
}

// Samples a vMF lobe with two uniforms (Jakob's numerically stable inversion of the cosine to
// the mean, "Numerically stable sampling of the von Mises Fisher distribution on S2", 2012)
__device__ __forceinline__ V3 sample_vmf(V3 mu, float k, float u1, float u2)
{
    const float wz = fminf(1.0f, fmaxf(-1.0f, 1.0f + logf(u1 + (1.0f - u1) * expf(-2.0f * k)) / k));
    const float r = sqrtf(fmaxf(0.0f, 1.0f - wz * wz));
    float sn, cs;
    sincosf(kTwoPi * u2, &sn, &cs);
    // frame around mu (Frisvad / Max)
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

// Samples a direction from the mixture with three uniforms: the lobe by u0, then the lobe's vMF
__device__ __forceinline__ V3 sample_mixture(const Lobe* lobes, float u0, float u1, float u2)
{
    int pick = kLobes - 1;
    float acc = 0.0f;
    for (int i = 0; i < kLobes; i++)
    {
        acc += lobes[i].weight;
        if (u0 < acc)
        {
            pick = i;
            break;
        }
    }
    return sample_vmf(lobes[pick].mu, lobes[pick].kappa, u1, u2);
}

// Mixture read from global memory one lobe at a time (the path tracer's per-entry lobes,
// 8 x (mu xyz, kappa, weight)); keeps the 40 values out of registers.
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

}  // namespace guide
}  // namespace gbpt
