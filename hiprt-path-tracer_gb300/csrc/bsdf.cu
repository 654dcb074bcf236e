// Batched principled-BSDF entry points (declared in include/gbpt_bsdf.h): one thread per query,
// materials gathered by index, queries read as five 16-byte words.
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/gbpt_bsdf.h"
#include "handles.h"
#include "principled.h"

namespace gbpt {
namespace {

using namespace bsdf;

struct LoadedQuery
{
    Query q;
    Medium md;
    int lobe;
};

__device__ __forceinline__ LoadedQuery load_query(const gbpt_bsdf_query* qs, int64_t i)
{
    const float4* p = reinterpret_cast<const float4*>(qs + i);
    const float4 a = p[0], b = p[1], c = p[2], d = p[3], e = p[4];
    LoadedQuery r;
    r.q.view = v3(a.x, a.y, a.z);
    r.q.ns = v3(a.w, b.x, b.y);
    r.q.ng = v3(b.z, b.w, c.x);
    r.q.light = v3(c.y, c.z, c.w);
    r.md.eta_incident = d.x;
    r.md.eta_outgoing = d.y;
    r.md.inside = __float_as_int(d.z) != 0;
    r.lobe = __float_as_int(d.w);
    r.md.wavelength = fabsf(e.x);
    return r;
}

// A query whose material index is out of range returns zeros (and lobe NONE when sampling).
__global__ void __launch_bounds__(256) bsdf_eval_kernel(const gbpt_principled_material* __restrict__ mats, int n_mats,
                                                        const int32_t* __restrict__ mat_index,
                                                        const gbpt_bsdf_query* __restrict__ qs, int64_t n,
                                                        bool height_correlated, float4* __restrict__ out_f,
                                                        float* __restrict__ out_pdf)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    {
        const int mi = mat_index[i];
        float pdf = 0.0f;
        V3 f = v3(0.0f);
        if (mi >= 0 && mi < n_mats)
        {
            const LoadedQuery lq = load_query(qs, i);
            const Material m = load_material(mats[mi]);
            f = eval(m, lq.md, height_correlated, lq.q, lq.lobe, pdf);
        }
        if (out_f) out_f[i] = make_float4(f.x, f.y, f.z, pdf);
        if (out_pdf) out_pdf[i] = pdf;
    }
}

__global__ void __launch_bounds__(256) bsdf_sample_kernel(const gbpt_principled_material* __restrict__ mats,
                                                          int n_mats, const int32_t* __restrict__ mat_index,
                                                          const gbpt_bsdf_query* __restrict__ qs,
                                                          const uint32_t* __restrict__ seeds, int64_t n,
                                                          bool height_correlated, float4* __restrict__ out,
                                                          int32_t* __restrict__ out_lobe, uint32_t* __restrict__ out_rng)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    {
        const int mi = mat_index[i];
        Xorshift32 rng{seeds[i]};
        float pdf = 0.0f;
        V3 f = v3(0.0f), dir = v3(0.0f);
        int lobe = GBPT_LOBE_NONE;
        if (mi >= 0 && mi < n_mats)
        {
            const LoadedQuery lq = load_query(qs, i);
            const Material m = load_material(mats[mi]);
            f = sample(m, lq.md, height_correlated, lq.q.view, lq.q.ns, lq.q.ng, rng, dir, lobe, pdf);
        }
        out[2 * i] = make_float4(dir.x, dir.y, dir.z, f.x);
        out[2 * i + 1] = make_float4(f.y, f.z, pdf, 0.0f);
        if (out_lobe) out_lobe[i] = lobe;
        if (out_rng) out_rng[i] = rng.state;
    }
}

int grid_for(int64_t n)
{
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t want = (n + 255) / 256;
    const int64_t cap = (int64_t)sms * 8;
    return (int)(want < 1 ? 1 : (want > cap ? cap : want));
}

gbpt_status check_common(const gbpt_principled_material* mats, int32_t n_mats, const int32_t* mat_index,
                         const gbpt_bsdf_query* qs, int64_t n)
{
    if (n < 0) return set_error(GBPT_ERROR_INVALID_ARG, "n is negative");
    if (n > 0 && (!mats || n_mats <= 0 || !mat_index || !qs))
        return set_error(GBPT_ERROR_INVALID_ARG, "materials, material_index and queries must be device pointers");
    if ((reinterpret_cast<uintptr_t>(qs) & 15u) != 0)
        return set_error(GBPT_ERROR_INVALID_ARG, "queries must be 16-byte aligned");
    return GBPT_OK;
}

}  // namespace
}  // namespace gbpt

extern "C" {

gbpt_status gbpt_bsdf_eval(const gbpt_principled_material* materials, int32_t n_materials, const int32_t* material_index,
                           const gbpt_bsdf_query* queries, int64_t n, const gbpt_bsdf_options* options,
                           float* out_rgb_pdf, void* stream)
{
    gbpt_status st = gbpt::check_common(materials, n_materials, material_index, queries, n);
    if (st != GBPT_OK) return st;
    if (n == 0) return GBPT_OK;
    if (!out_rgb_pdf || (reinterpret_cast<uintptr_t>(out_rgb_pdf) & 15u) != 0)
        return gbpt::set_error(GBPT_ERROR_INVALID_ARG, "out_rgb_pdf must be a 16-byte aligned device pointer");
    const bool hc = options && options->ggx_height_correlated;
    gbpt::bsdf_eval_kernel<<<gbpt::grid_for(n), 256, 0, (cudaStream_t)stream>>>(
        materials, n_materials, material_index, queries, n, hc, reinterpret_cast<float4*>(out_rgb_pdf), nullptr);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GBPT_OK : gbpt::cuda_error(e, "bsdf eval launch");
}

gbpt_status gbpt_bsdf_pdf(const gbpt_principled_material* materials, int32_t n_materials, const int32_t* material_index,
                          const gbpt_bsdf_query* queries, int64_t n, const gbpt_bsdf_options* options, float* out_pdf,
                          void* stream)
{
    gbpt_status st = gbpt::check_common(materials, n_materials, material_index, queries, n);
    if (st != GBPT_OK) return st;
    if (n == 0) return GBPT_OK;
    if (!out_pdf) return gbpt::set_error(GBPT_ERROR_INVALID_ARG, "out_pdf is NULL");
    const bool hc = options && options->ggx_height_correlated;
    gbpt::bsdf_eval_kernel<<<gbpt::grid_for(n), 256, 0, (cudaStream_t)stream>>>(materials, n_materials, material_index,
                                                                                 queries, n, hc, nullptr, out_pdf);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GBPT_OK : gbpt::cuda_error(e, "bsdf pdf launch");
}

gbpt_status gbpt_bsdf_sample(const gbpt_principled_material* materials, int32_t n_materials,
                             const int32_t* material_index, const gbpt_bsdf_query* queries, const uint32_t* seeds,
                             int64_t n, const gbpt_bsdf_options* options, float* out, int32_t* out_lobe,
                             uint32_t* out_rng_state, void* stream)
{
    gbpt_status st = gbpt::check_common(materials, n_materials, material_index, queries, n);
    if (st != GBPT_OK) return st;
    if (n == 0) return GBPT_OK;
    if (!seeds) return gbpt::set_error(GBPT_ERROR_INVALID_ARG, "seeds is NULL");
    if (!out || (reinterpret_cast<uintptr_t>(out) & 15u) != 0)
        return gbpt::set_error(GBPT_ERROR_INVALID_ARG, "out must be a 16-byte aligned device pointer");
    const bool hc = options && options->ggx_height_correlated;
    gbpt::bsdf_sample_kernel<<<gbpt::grid_for(n), 256, 0, (cudaStream_t)stream>>>(
        materials, n_materials, material_index, queries, seeds, n, hc, reinterpret_cast<float4*>(out), out_lobe,
        out_rng_state);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GBPT_OK : gbpt::cuda_error(e, "bsdf sample launch");
}

}  // extern "C"
