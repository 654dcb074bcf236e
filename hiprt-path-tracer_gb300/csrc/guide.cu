// Guiding network kernels (sm_103a): hash-grid encoding, the 32-64-64-48 MLP on tcgen05 tensor
// cores (BF16 operands in shared memory, FP32 accumulators in TMEM), the vMF-mixture head and its
// loss, the backward pass, Adam and the BF16 weight packing.
//
// One CTA of 128 threads processes tiles of 128 samples (M = 128, one sample per thread and per
// TMEM lane). Per tile: encode -> X; D1 = X W1 -> ReLU -> H1; D2 = H1 W2 -> ReLU -> H2;
// D3 = H2 W3 -> head. Training continues with dY (loss gradient of the 48 raw outputs) ->
// dH2 = dY W3^T (masked by ReLU') -> dH1 = dH2 W2^T (masked) -> dX = dH1 W1^T -> hash-grid scatter;
// the weight gradients dW3 = H2^T dY, dW2 = H1^T dH2, dW1 = X^T dH1 are reduced over the tile in
// shared memory by the CUDA cores and flushed once per CTA. The MMAs are issued by thread 0 and
// completed through an mbarrier; every wait is bounded and reports through an error flag.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "guide_device.h"
#include "guide_kernels.h"
#include "umma.h"

namespace gbpt {
namespace guide {
namespace {

constexpr int kTile = 128;
constexpr int kWaitLimit = 1 << 24;
constexpr uint32_t kTmemCols = 256;
// TMEM columns (accumulators start on multiples of 64): forward D1 @0, D2 @64, D3 @128 (48 wide);
// backward dH2 @192, dH1 @0, dX @64 (32 wide)

struct Smem
{
    uint64_t mbar;
    uint32_t tmem;
    uint32_t pad;
    __nv_bfloat16 w[kPackedWeights];
    __nv_bfloat16 x[kTile * kIn];
    __nv_bfloat16 h1[kTile * kHid];
    __nv_bfloat16 h2[kTile * kHid];
    __nv_bfloat16 dy[kTile * kOut];
    __nv_bfloat16 dh2[kTile * kHid];
    __nv_bfloat16 dh1[kTile * kHid];
    float dw[kNumWeights];
};
constexpr size_t kSmemTrain = sizeof(Smem);
// inference needs the weights and the forward activations only
constexpr size_t kSmemInfer = offsetof(Smem, dy);

__device__ __forceinline__ int kmo(int r, int k, int K) { return umma::kmajor_offset(r, k, K); }

__device__ __forceinline__ V3 load3(const float* __restrict__ a, int64_t row)
{
    return v3(a[3 * row], a[3 * row + 1], a[3 * row + 2]);
}

// rows in the batch: the device count when there is one (capped by n_max), else n_max
__device__ __forceinline__ int64_t batch_size(const Batch& b)
{
    if (!b.count) return b.n_max;
    const int64_t c = *b.count;
    return c < 0 ? 0 : (c < b.n_max ? c : b.n_max);
}

__device__ __forceinline__ void copy_weights(Smem& sm, const uint16_t* packed)
{
    const uint4* src = reinterpret_cast<const uint4*>(packed);
    uint4* dst = reinterpret_cast<uint4*>(sm.w);
    for (int i = threadIdx.x; i < kPackedWeights / 8; i += blockDim.x) dst[i] = src[i];
}

// makes this thread's shared-memory writes visible to the tensor core, then syncs the CTA
__device__ __forceinline__ void publish_smem()
{
    umma::fence_async_smem();
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
}

// issue (thread 0) + wait (all) one GEMM; false if the wait gave up
__device__ __forceinline__ bool run_gemm(Smem& sm, uint32_t col, const __nv_bfloat16* A, const __nv_bfloat16* B, int N,
                                         int K, uint32_t& phase)
{
    if (threadIdx.x == 0) umma::gemm_commit(sm.tmem + col, A, B, N, K, &sm.mbar);
    const bool ok = umma::mbar_wait(&sm.mbar, phase, kWaitLimit);
    phase ^= 1u;
    umma::fence_after();
    return __syncthreads_and(ok ? 1 : 0) != 0;  // every thread takes the same branch
}

__device__ __forceinline__ void load_cols(const Smem& sm, int col, int count, float* out)
{
    const int warp = threadIdx.x >> 5;
    for (int c = 0; c < count; c += 16) umma::tmem_ld16(umma::lane_addr(sm.tmem, warp, col + c), out + c);
}

__device__ __forceinline__ void setup(Smem& sm)
{
    if (threadIdx.x < 32) umma::tmem_alloc(&sm.tmem, kTmemCols);
    if (threadIdx.x == 0) umma::mbar_init(&sm.mbar);
}

__device__ __forceinline__ void teardown(Smem& sm)
{
    umma::fence_before();
    __syncthreads();
    if (threadIdx.x < 32) umma::tmem_dealloc(sm.tmem, kTmemCols);
}

// Forward of one tile up to the 48 raw outputs of this thread's row; h1/h2 keep the ReLU'd
// activations in shared memory and m1/m2 their positivity bits. False if a wait gave up.
__device__ bool forward_tile(Smem& sm, const Net& net, bool valid, V3 p, V3 n, V3 view, float* raw, uint32_t* m1,
                             uint32_t* m2, uint32_t& phase)
{
    const int t = threadIdx.x;
    {
        float feat[16], x[kIn];
        const Domain d = {{net.lo[0], net.lo[1], net.lo[2]}, {net.inv_ext[0], net.inv_ext[1], net.inv_ext[2]}};
        if (valid)
            encode(d, net.params + kNumWeights, p, feat);
        else
            for (int i = 0; i < 16; i++) feat[i] = 0.0f;
        input_row(feat, valid ? n : v3(0.0f), valid ? view : v3(0.0f), x);
        if (!valid) x[19] = 0.0f;
        for (int k = 0; k < kIn; k++) sm.x[kmo(t, k, kIn)] = __float2bfloat16(x[k]);
    }
    publish_smem();
    if (!run_gemm(sm, 0, sm.x, sm.w + kW1f, kHid, kIn, phase)) return false;
    float h[kHid];
    load_cols(sm, 0, kHid, h);
    m1[0] = m1[1] = 0u;
    for (int k = 0; k < kHid; k++)
    {
        const float v = fmaxf(h[k], 0.0f);
        if (h[k] > 0.0f) m1[k >> 5] |= 1u << (k & 31);
        sm.h1[kmo(t, k, kHid)] = __float2bfloat16(v);
    }
    publish_smem();
    if (!run_gemm(sm, 64, sm.h1, sm.w + kW2f, kHid, kHid, phase)) return false;
    load_cols(sm, 64, kHid, h);
    m2[0] = m2[1] = 0u;
    for (int k = 0; k < kHid; k++)
    {
        const float v = fmaxf(h[k], 0.0f);
        if (h[k] > 0.0f) m2[k >> 5] |= 1u << (k & 31);
        sm.h2[kmo(t, k, kHid)] = __float2bfloat16(v);
    }
    publish_smem();
    if (!run_gemm(sm, 128, sm.h2, sm.w + kW3f, kOut, kHid, phase)) return false;
    load_cols(sm, 128, kOut, raw);
    return true;
}

// out[o] += sum over the tile's rows of A[r][i] * B[r][j], o = i * NB + j (A: K-major with KA
// columns, B: K-major with NB columns); the tile's 128 threads split the outputs
__device__ __forceinline__ void accumulate_outer(float* out, const __nv_bfloat16* A, int KA, const __nv_bfloat16* B, int NB)
{
    for (int o = threadIdx.x; o < KA * NB; o += blockDim.x)
    {
        const int i = o / NB, j = o - i * NB;
        float acc = 0.0f;
        for (int r = 0; r < kTile; r++)
            acc += __bfloat162float(A[kmo(r, i, KA)]) * __bfloat162float(B[kmo(r, j, NB)]);
        out[o] += acc;
    }
}

// ---------------------------------------------------------------------------------------------
// training: forward + loss + backward, persistent over tiles
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kTile) train_kernel(Net net, Batch b, const float* __restrict__ weight_sum,
                                                      float* __restrict__ grads, float* __restrict__ loss, int* err)
{
    const int64_t n = batch_size(b);
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Smem& sm = *reinterpret_cast<Smem*>(smem_raw);
    const int t = threadIdx.x;
    copy_weights(sm, net.packed);
    for (int i = t; i < kNumWeights; i += blockDim.x) sm.dw[i] = 0.0f;
    setup(sm);
    publish_smem();
    const float inv_wsum = *weight_sum > 0.0f ? 1.0f / *weight_sum : 0.0f;
    const Domain d = {{net.lo[0], net.lo[1], net.lo[2]}, {net.inv_ext[0], net.inv_ext[1], net.inv_ext[2]}};
    uint32_t phase = 0;
    float loss_acc = 0.0f;
    bool ok = true;
    const int64_t n_tiles = (n + kTile - 1) / kTile;
    for (int64_t tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x)
    {
        const int64_t row = tile * kTile + t;
        const bool valid = row < n;
        V3 p = v3(0.0f), nn = v3(0.0f), vw = v3(0.0f), w = v3(0.0f, 0.0f, 1.0f);
        float ws = 0.0f;
        if (valid)
        {
            p = load3(b.pos, row);
            nn = load3(b.nrm, row);
            vw = load3(b.view, row);
            w = load3(b.dir, row);
            ws = fmaxf(b.weight[row], 0.0f);
        }
        float raw[kOut];
        uint32_t m1[2], m2[2];
        ok = forward_tile(sm, net, valid, p, nn, vw, raw, m1, m2, phase);
        if (!ok) break;
        // head, loss and its gradient for this row
        float draw[kOut];
        {
            Lobe lobes[kLobes];
            float len[kLobes];
            head(raw, lobes, len);
            const float scale = valid ? ws * inv_wsum : 0.0f;
            const float logq = head_backward(raw, lobes, len, w, scale, draw);
            if (scale > 0.0f) loss_acc += -scale * logq;
        }
        for (int k = 0; k < kOut; k++) sm.dy[kmo(t, k, kOut)] = __float2bfloat16(draw[k]);
        publish_smem();
        accumulate_outer(sm.dw + kOffW3, sm.h2, kHid, sm.dy, kOut);  // dW3 = H2^T dY
        ok = run_gemm(sm, 192, sm.dy, sm.w + kW3b, kHid, kOut, phase);  // dH2 = dY W3^T
        if (!ok) break;
        float g[kHid];
        load_cols(sm, 192, kHid, g);
        for (int k = 0; k < kHid; k++)
            sm.dh2[kmo(t, k, kHid)] = __float2bfloat16((m2[k >> 5] >> (k & 31)) & 1u ? g[k] : 0.0f);
        publish_smem();
        accumulate_outer(sm.dw + kOffW2, sm.h1, kHid, sm.dh2, kHid);  // dW2 = H1^T dH2
        ok = run_gemm(sm, 0, sm.dh2, sm.w + kW2b, kHid, kHid, phase);  // dH1 = dH2 W2^T
        if (!ok) break;
        load_cols(sm, 0, kHid, g);
        for (int k = 0; k < kHid; k++)
            sm.dh1[kmo(t, k, kHid)] = __float2bfloat16((m1[k >> 5] >> (k & 31)) & 1u ? g[k] : 0.0f);
        publish_smem();
        accumulate_outer(sm.dw + kOffW1, sm.x, kIn, sm.dh1, kHid);  // dW1 = X^T dH1
        ok = run_gemm(sm, 64, sm.dh1, sm.w + kW1b, kIn, kHid, phase);  // dX = dH1 W1^T
        if (!ok) break;
        float dx[kIn];
        load_cols(sm, 64, kIn, dx);
        if (valid) encode_backward(d, grads + kNumWeights, p, dx);
        __syncthreads();  // the next tile overwrites the shared tiles
    }
    if (!ok && t == 0) atomicExch(err, 1);
    __syncthreads();
    for (int i = t; i < kNumWeights; i += blockDim.x)
        if (sm.dw[i] != 0.0f) atomicAdd(grads + i, sm.dw[i]);
    for (int o = 16; o > 0; o >>= 1) loss_acc += __shfl_xor_sync(0xffffffffu, loss_acc, o);
    if ((t & 31) == 0 && loss_acc != 0.0f) atomicAdd(loss, loss_acc);
    teardown(sm);
}

// ---------------------------------------------------------------------------------------------
// inference: mixture per query (8 x (mu xyz, kappa, weight))
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kTile) infer_kernel(Net net, Batch b, float* __restrict__ lobes_out, int* err)
{
    const int64_t n = batch_size(b);
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Smem& sm = *reinterpret_cast<Smem*>(smem_raw);
    const int t = threadIdx.x;
    copy_weights(sm, net.packed);
    setup(sm);
    publish_smem();
    uint32_t phase = 0;
    bool ok = true;
    const int64_t n_tiles = (n + kTile - 1) / kTile;
    for (int64_t tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x)
    {
        const int64_t row = tile * kTile + t;
        const bool valid = row < n;
        V3 p = v3(0.0f), nn = v3(0.0f), vw = v3(0.0f);
        if (valid)
        {
            p = load3(b.pos, row);
            nn = load3(b.nrm, row);
            vw = load3(b.view, row);
        }
        float raw[kOut];
        uint32_t m1[2], m2[2];
        ok = forward_tile(sm, net, valid, p, nn, vw, raw, m1, m2, phase);
        if (!ok) break;
        if (valid)
        {
            Lobe L[kLobes];
            float len[kLobes];
            head(raw, L, len);
            float* o = lobes_out + 40 * row;
            for (int i = 0; i < kLobes; i++)
            {
                o[5 * i] = L[i].mu.x;
                o[5 * i + 1] = L[i].mu.y;
                o[5 * i + 2] = L[i].mu.z;
                o[5 * i + 3] = L[i].kappa;
                o[5 * i + 4] = L[i].weight;
            }
        }
        __syncthreads();
    }
    if (!ok && t == 0) atomicExch(err, 1);
    teardown(sm);
}

// ---------------------------------------------------------------------------------------------
// parameters: initialisation, BF16 packing, Adam, weight sum
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ float hash_uniform(uint32_t i, uint32_t seed)
{
    uint32_t x = i * 0x9E3779B1u ^ (seed * 0x85EBCA77u + 0x165667B1u);
    x ^= x >> 16;
    x *= 0x7FEB352Du;
    x ^= x >> 15;
    x *= 0x846CA68Bu;
    x ^= x >> 16;
    return (float)(x >> 8) * (1.0f / 16777216.0f);
}

// Glorot-uniform weights, grid features uniform in [-1e-4, 1e-4]
__global__ void init_kernel(float* params, uint32_t seed)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kNumParams; i += gridDim.x * blockDim.x)
    {
        const float u = 2.0f * hash_uniform((uint32_t)i, seed) - 1.0f;
        float s;
        if (i < kOffW2)
            s = sqrtf(6.0f / (kIn + kHid));
        else if (i < kOffW3)
            s = sqrtf(6.0f / (kHid + kHid));
        else if (i < kNumWeights)
            s = sqrtf(6.0f / (kHid + kOut));
        else
            s = 1.0e-4f;
        params[i] = u * s;
    }
}

__global__ void pack_kernel(const float* __restrict__ params, __nv_bfloat16* __restrict__ packed)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kNumWeights; i += gridDim.x * blockDim.x)
    {
        const __nv_bfloat16 v = __float2bfloat16(params[i]);
        if (i < kOffW2)
        {
            const int a = i / kHid, b = i % kHid;  // W1[a in 32][b out 64]
            packed[kW1f + kmo(b, a, kIn)] = v;
            packed[kW1b + kmo(a, b, kHid)] = v;
        }
        else if (i < kOffW3)
        {
            const int j = i - kOffW2, a = j / kHid, b = j % kHid;  // W2[a][b]
            packed[kW2f + kmo(b, a, kHid)] = v;
            packed[kW2b + kmo(a, b, kHid)] = v;
        }
        else
        {
            const int j = i - kOffW3, a = j / kOut, b = j % kOut;  // W3[a in 64][b out 48]
            packed[kW3f + kmo(b, a, kHid)] = v;
            packed[kW3b + kmo(a, b, kOut)] = v;
        }
    }
}

__global__ void adam_kernel(float* __restrict__ params, const float* __restrict__ grads, float* __restrict__ m,
                            float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kNumParams; i += gridDim.x * blockDim.x)
    {
        const float g = grads[i];
        const float mi = b1 * m[i] + (1.0f - b1) * g;
        const float vi = b2 * v[i] + (1.0f - b2) * g * g;
        m[i] = mi;
        v[i] = vi;
        params[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

__global__ void weight_sum_kernel(Batch b, float* __restrict__ out)
{
    const float* __restrict__ w = b.weight;
    const int64_t n = batch_size(b);
    float acc = 0.0f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        acc += fmaxf(w[i], 0.0f);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0 && acc != 0.0f) atomicAdd(out, acc);
}

}  // namespace

cudaError_t launch_guide_init(float* params, uint32_t seed, cudaStream_t st)
{
    init_kernel<<<512, 256, 0, st>>>(params, seed);
    return cudaGetLastError();
}

cudaError_t launch_guide_pack(const float* params, uint16_t* packed, cudaStream_t st)
{
    pack_kernel<<<(kNumWeights + 255) / 256, 256, 0, st>>>(params, reinterpret_cast<__nv_bfloat16*>(packed));
    return cudaGetLastError();
}

cudaError_t launch_guide_weight_sum(const Batch& b, float* out_sum, cudaStream_t st)
{
    cudaError_t e = cudaMemsetAsync(out_sum, 0, sizeof(float), st);
    if (e != cudaSuccess) return e;
    int64_t blocks = (b.n_max + 255) / 256;
    if (blocks < 1) blocks = 1;
    if (blocks > 1024) blocks = 1024;
    weight_sum_kernel<<<(int)blocks, 256, 0, st>>>(b, out_sum);
    return cudaGetLastError();
}

cudaError_t launch_guide_train(const Net& net, const Batch& b, const float* weight_sum, float* grads, float* loss, int* err,
                               int n_sm, cudaStream_t st)
{
    static bool attr_set = false;
    if (!attr_set)
    {
        cudaError_t e = cudaFuncSetAttribute(train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemTrain);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    const int64_t tiles = (b.n_max + kTile - 1) / kTile;
    const int grid = (int)(tiles < n_sm ? (tiles < 1 ? 1 : tiles) : n_sm);
    train_kernel<<<grid, kTile, kSmemTrain, st>>>(net, b, weight_sum, grads, loss, err);
    return cudaGetLastError();
}

cudaError_t launch_guide_infer(const Net& net, const Batch& b, float* lobes, int* err, int n_sm, cudaStream_t st)
{
    static bool attr_set = false;
    if (!attr_set)
    {
        cudaError_t e = cudaFuncSetAttribute(infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemInfer);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    const int64_t tiles = (b.n_max + kTile - 1) / kTile;
    const int64_t cap = (int64_t)n_sm * 2;
    const int grid = (int)(tiles < cap ? (tiles < 1 ? 1 : tiles) : cap);
    infer_kernel<<<grid, kTile, kSmemInfer, st>>>(net, b, lobes, err);
    return cudaGetLastError();
}

cudaError_t launch_guide_adam(float* params, const float* grads, float* m, float* v, float lr, float beta1, float beta2,
                              float eps, int step, cudaStream_t st)
{
    const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
    adam_kernel<<<1024, 256, 0, st>>>(params, grads, m, v, lr, beta1, beta2, eps, c1, c2);
    return cudaGetLastError();
}

}  // namespace guide
}  // namespace gbpt
