// Environment-map table build on the device (sm_103a): RGB9E5 packing with the per-texel
// luminance, then the FP64 running sum over texels in row-major order (the binary-search CDF) and
// the FP64 total that normalises the alias table.
//
// Restates RendererEnvmap's texel packing (RGBE9995Packed::pack,
// src/HostDeviceCommon/Packing.h:441-475) and Image32Bit::compute_cdf / luminance_of_pixel
// (src/Image/Image.cpp:526-549,625-645); the reference sums in float on the host, this build in
// FP64 on the device, rounding each running sum to float once.
#include <cuda_runtime.h>
#include <stdint.h>

#include "render_common.h"
#include "render_kernels.h"

namespace gbpt {
namespace {

// R9G9B9E5 shared-exponent packing. The shared exponent comes from the largest channel (at least
// 2^-16, at most 65408 = 511 * 2^7) after rounding it to 9 significant bits: bias = 2^(e + 15)
// where 2^e bounds that channel. Adding the bias to a channel shifts its value, rounded to nearest
// even in units of 2^(e - 8), into the low 9 bits of the sum's mantissa; the 5-bit exponent field
// holds e + 16 (mod 32), so that unpacking scales the mantissas by 2^(field - 24) = 2^(e - 8).
// Same steps as the reference's packing so that texels agree bit for bit.
__device__ __forceinline__ uint32_t rgb9e5_pack(float r, float g, float b)
{
    const float hi = __uint_as_float(0x477F8000u);
    const float lo = __uint_as_float(0x37800000u);
    r = fminf(fmaxf(r, 0.0f), hi);
    g = fminf(fmaxf(g, 0.0f), hi);
    b = fminf(fmaxf(b, 0.0f), hi);
    const float m = fmaxf(fmaxf(lo, r), fmaxf(g, b));
    const float bias = __uint_as_float((__float_as_uint(m) + 0x07804000u) & 0x7F800000u);
    const uint32_t R = __float_as_uint(__fadd_rn(r, bias));
    const uint32_t G = __float_as_uint(__fadd_rn(g, bias));
    const uint32_t B = __float_as_uint(__fadd_rn(b, bias));
    const uint32_t E = (__float_as_uint(bias) << 4) + 0x10000000u;
    return E | (B << 18) | (G << 9) | (R & 0x1FFu);
}

__global__ void __launch_bounds__(256) env_pack_kernel(const float* __restrict__ rgb, int64_t n,
                                                        uint32_t* __restrict__ texels, float* __restrict__ lum)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    {
        const float r = rgb[3 * i], g = rgb[3 * i + 1], b = rgb[3 * i + 2];
        texels[i] = rgb9e5_pack(r, g, b);
        // luminance_of_pixel: weights applied channel by channel to the float texel
        lum[i] = __fadd_rn(__fadd_rn(__fmul_rn(r, 0.3086f), __fmul_rn(g, 0.6094f)), __fmul_rn(b, 0.0820f));
    }
}

// FP64 running sum in tiles of kScanThreads * kScanItems texels: per-tile totals, an exclusive scan
// of the totals in one block, then each tile rescans itself from its offset. Every sum has a fixed
// association, so the tables are the same on every run.
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ double thread_items_sum(const float* __restrict__ x, int64_t n, int64_t base)
{
    double acc = 0.0;
    for (int k = 0; k < kScanItems; k++)
    {
        const int64_t i = base + k;
        if (i < n) acc += (double)x[i];
    }
    return acc;
}

// inclusive scan of one double per thread over the block (Hillis-Steele in shared memory)
__device__ __forceinline__ double block_inclusive_scan(double v, double* sh)
{
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < kScanThreads; off <<= 1)
    {
        const double add = threadIdx.x >= (unsigned)off ? sh[threadIdx.x - off] : 0.0;
        __syncthreads();
        v += add;
        sh[threadIdx.x] = v;
        __syncthreads();
    }
    return v;
}

__global__ void __launch_bounds__(kScanThreads) tile_total_kernel(const float* __restrict__ x, int64_t n,
                                                                  double* __restrict__ tile_total)
{
    __shared__ double sh[kScanThreads];
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    const double v = block_inclusive_scan(thread_items_sum(x, n, base), sh);
    if (threadIdx.x == kScanThreads - 1) tile_total[blockIdx.x] = v;
}

__global__ void __launch_bounds__(kScanThreads) tile_offset_kernel(const double* __restrict__ tile_total, int n_tiles,
                                                                   double* __restrict__ tile_offset,
                                                                   double* __restrict__ sum64)
{
    __shared__ double sh[kScanThreads];
    double carry = 0.0;
    for (int b0 = 0; b0 < n_tiles; b0 += kScanThreads)
    {
        const int b = b0 + threadIdx.x;
        const double t = b < n_tiles ? tile_total[b] : 0.0;
        const double inc = block_inclusive_scan(t, sh);
        if (b < n_tiles) tile_offset[b] = carry + (inc - t);
        const double chunk = sh[kScanThreads - 1];
        __syncthreads();
        carry += chunk;
    }
    if (threadIdx.x == 0) *sum64 = carry;
}

__global__ void __launch_bounds__(kScanThreads) tile_scan_kernel(const float* __restrict__ x, int64_t n,
                                                                 const double* __restrict__ tile_offset,
                                                                 float* __restrict__ cdf)
{
    __shared__ double sh[kScanThreads];
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    const double own = thread_items_sum(x, n, base);
    const double inc = block_inclusive_scan(own, sh);
    double run = tile_offset[blockIdx.x] + (inc - own);
    for (int k = 0; k < kScanItems; k++)
    {
        const int64_t i = base + k;
        if (i < n)
        {
            run += (double)x[i];
            cdf[i] = (float)run;
        }
    }
}

}  // namespace

int envmap_scan_tiles(int64_t n) { return (int)((n + kScanTile - 1) / kScanTile); }

cudaError_t launch_envmap_tables(const float* rgb, int64_t n, uint32_t* texels, float* lum, float* cdf,
                                 double* tile_total, double* tile_offset, double* sum64, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    const int n_tiles = envmap_scan_tiles(n);
    int64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    env_pack_kernel<<<(int)blocks, 256, 0, st>>>(rgb, n, texels, lum);
    tile_total_kernel<<<n_tiles, kScanThreads, 0, st>>>(lum, n, tile_total);
    tile_offset_kernel<<<1, kScanThreads, 0, st>>>(tile_total, n_tiles, tile_offset, sum64);
    tile_scan_kernel<<<n_tiles, kScanThreads, 0, st>>>(lum, n, tile_offset, cdf);
    return cudaGetLastError();
}

}  // namespace gbpt
