// Guiding network kernels (sm_103a): hash-grid + spherical-harmonic encoding, the 64-64-64-64-48
// MLP on the tcgen05 tensor cores (BF16 operands in shared memory, FP32 accumulators in TMEM), the
// vMF-mixture head and its loss, the backward pass, Adam and the BF16 packing of weights and grid.
//
// One CTA of 128 threads processes tiles of 128 samples (M = 128, one sample per thread and per
// TMEM lane). Forward: X -> H1 = ReLU(X W1) -> H2 -> H3 -> raw = H3 W4 -> head. Training continues
// with the loss gradient dY of the raw outputs and, per layer l = 4..1,
//   dH_{l-1} = (dH_l W_l^T) masked by ReLU'    (M = 128 samples, tensor core)
//   dW_l    += H_{l-1}^T dH_l                   (M = the layer's 64 inputs, K = the tile's samples)
// The weight gradients accumulate in TMEM across all tiles of the CTA and are flushed once. Their
// A operand H^T is 64 rows: the MMA runs with M = 128 and the upper 64 rows of D (read from the
// next 16 KB of shared memory) are ignored. MMAs are issued by thread 0 and completed through an
// mbarrier; every wait is bounded and reports through an error flag.
#include <cstddef>

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
// TMEM columns. Training (512 allocated): F @0 (forward D / backward dH, up to 64 wide), the
// weight-gradient accumulators dW1 @128, dW2 @192, dW3 @256 (64 wide), dW4 @320 (48 wide).
// Inference: F only (64 allocated).
constexpr uint32_t kTmemTrain = 512;
constexpr uint32_t kTmemInfer = 64;
constexpr uint32_t kColF = 0;
__device__ __forceinline__ uint32_t col_dw(int l) { return 128u + 64u * (uint32_t)l; }

using bf16 = __nv_bfloat16;

// Operand arrays start on 16-byte boundaries: the weights are copied and the activations stored in
// 16-byte words, and the shared-memory matrix descriptors address 16-byte units.
struct SmemTrain
{
    uint64_t mbar;
    uint32_t tmem;
    uint32_t pad;
    alignas(16) bf16 w[kPackedWeights];
    // transposed layer inputs X^T, H1^T, H2^T, H3^T (64 rows x K = 128 samples): the A operands
    // of dW1..dW4; each is followed by 16 KB of shared memory that the M = 128 MMA reads as rows
    // 64..127 (results ignored)
    bf16 tr[4][kHid * kTile];
    bf16 act[2][kTile * kHid];  // K-major activations / output gradients (A operands), ping-pong
    bf16 gt[2][kHid * kTile];   // transposed output gradients (B operands of dW), ping-pong
};

// Inference keeps one operand buffer: every MMA has completed (its mbarrier wait) before the
// epilogue overwrites its input with the next layer's, so 47 KB per CTA and four CTAs per SM.
struct SmemInfer
{
    uint64_t mbar;
    uint32_t tmem;
    uint32_t pad;
    alignas(16) bf16 w[kFwdWeights];
    alignas(16) bf16 act[kTile * kHid];
};
constexpr int kInferCtasPerSm = 4;
static_assert(offsetof(SmemInfer, w) % 16 == 0 && offsetof(SmemInfer, act) % 16 == 0,
              "inference operands must start on 16-byte boundaries");
static_assert(sizeof(SmemInfer) * kInferCtasPerSm <= 227 * 1024 && kTmemInfer * kInferCtasPerSm <= 512,
              "four inference CTAs per SM");
static_assert(offsetof(SmemTrain, w) % 16 == 0 && offsetof(SmemTrain, tr) % 16 == 0 &&
                  offsetof(SmemTrain, act) % 16 == 0 && offsetof(SmemTrain, gt) % 16 == 0,
              "training operands must start on 16-byte boundaries");


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

__device__ __forceinline__ void copy_weights(bf16* dst, const uint16_t* packed, int count)
{
    const uint4* src = reinterpret_cast<const uint4*>(packed);
    uint4* d = reinterpret_cast<uint4*>(dst);
    for (int i = threadIdx.x; i < count / 8; i += blockDim.x) d[i] = src[i];
}

// makes this thread's shared-memory writes visible to the tensor core, then syncs the CTA
__device__ __forceinline__ void publish_smem()
{
    umma::fence_async_smem();
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
}

// all threads: wait (at most 'limit' polls) for the MMAs committed to the mbarrier; false (on every
// thread) if a thread gave up. A thread that gave up still waits, bounded by kWaitLimit, for that
// phase to complete: the kernel then stops with no tensor-core work of its own in flight, so that
// it can free the TMEM those MMAs write.
__device__ __forceinline__ bool wait_mma(uint64_t* mbar, uint32_t& phase, int limit)
{
    const bool ok = umma::mbar_wait(mbar, phase, limit);
    if (!ok) umma::mbar_wait(mbar, phase, kWaitLimit);
    phase ^= 1u;
    umma::fence_after();
    return __syncthreads_and(ok ? 1 : 0) != 0;
}

// issue (thread 0) + wait (all) one forward GEMM into F
__device__ __forceinline__ bool run_gemm(uint64_t* mbar, uint32_t tmem, const bf16* A, const bf16* B, int N, int K,
                                         uint32_t& phase, int limit)
{
    if (threadIdx.x == 0) umma::gemm_commit(tmem + kColF, A, B, N, K, mbar);
    return wait_mma(mbar, phase, limit);
}

__device__ __forceinline__ void load_cols(uint32_t tmem, uint32_t col, int count, float* out)
{
    const int warp = threadIdx.x >> 5;
    for (int c = 0; c < count; c += 16) umma::tmem_ld16(umma::lane_addr(tmem, warp, (int)col + c), out + c);
}

// stores this thread's row of n values (n a multiple of 8) as BF16, rounded to nearest even:
// K-major into 'a' (row t, K = n), eight values per 16-byte store (8 consecutive k of a row are 16
// contiguous bytes of a core matrix), and, when 't_out' is given, transposed into it (row k,
// K = 128 samples)
__device__ __forceinline__ void store_row(bf16* a, bf16* t_out, const float* v, int n)
{
    const int t = threadIdx.x;
    for (int k0 = 0; k0 < n; k0 += 8)
    {
        uint32_t w[4];
        for (int j = 0; j < 4; j++)
        {
            const __nv_bfloat162 h = __floats2bfloat162_rn(v[k0 + 2 * j], v[k0 + 2 * j + 1]);
            w[j] = *reinterpret_cast<const uint32_t*>(&h);
        }
        *reinterpret_cast<uint4*>(a + kmo(t, k0, n)) = make_uint4(w[0], w[1], w[2], w[3]);
        if (t_out)
            for (int j = 0; j < 8; j++) t_out[kmo(k0 + j, t, kTile)] = __float2bfloat16(v[k0 + j]);
    }
}

// ReLU of the 64 accumulator columns with their positivity mask bits
__device__ __forceinline__ void relu(float* h, uint32_t* mask)
{
    mask[0] = mask[1] = 0u;
    for (int k = 0; k < kHid; k++)
    {
        if (h[k] > 0.0f)
            mask[k >> 5] |= 1u << (k & 31);
        else
            h[k] = 0.0f;
    }
}

// gradient of a hidden layer's output masked by ReLU'
__device__ __forceinline__ void mask_grad(float* g, const uint32_t* mask)
{
    for (int k = 0; k < kHid; k++)
        if (!((mask[k >> 5] >> (k & 31)) & 1u)) g[k] = 0.0f;
}

// Forward of one tile up to the 48 raw outputs of this thread's row. act0 / act1: the K-major
// operand buffers of even / odd layers (one buffer may serve both); 'tr' (training only, else
// null) receives the transposed inputs of every layer and 'masks' the three ReLU masks. False if
// a wait gave up.
__device__ bool forward_tile(uint64_t* mbar, uint32_t tmem, const bf16* w, bf16* act0, bf16* act1,
                             bf16 (*tr)[kHid * kTile], const Net& net, bool valid, V3 p, V3 n, V3 view, float* raw,
                             uint32_t (*masks)[2], uint32_t& phase)
{
    bf16* const act[2] = {act0, act1};
    {
        float feat[kGridFeatures], x[kIn];
        const Domain d = {{net.lo[0], net.lo[1], net.lo[2]}, {net.inv_ext[0], net.inv_ext[1], net.inv_ext[2]}};
        if (valid)
        {
            encode(d, net.grid_bf16, p, feat);
            input_row(feat, n, view, x);
        }
        else
            for (int k = 0; k < kIn; k++) x[k] = 0.0f;
        store_row(act[0], tr ? tr[0] : nullptr, x, kIn);
    }
    publish_smem();
    const int wf[3] = {kW1f, kW2f, kW3f};
    float h[kHid];
    for (int l = 0; l < 3; l++)
    {
        if (!run_gemm(mbar, tmem, act[l & 1], w + wf[l], kHid, kHid, phase, net.wait_limit)) return false;
        load_cols(tmem, kColF, kHid, h);
        uint32_t scratch[2];
        relu(h, masks ? masks[l] : scratch);
        store_row(act[(l + 1) & 1], tr ? tr[l + 1] : nullptr, h, kHid);
        publish_smem();
    }
    if (!run_gemm(mbar, tmem, act[1], w + kW4f, kOut, kHid, phase, net.wait_limit)) return false;
    load_cols(tmem, kColF, kOut, raw);
    return true;
}

// ---------------------------------------------------------------------------------------------
// training: forward + loss + backward, persistent over tiles
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kTile) train_kernel(Net net, Batch b, const float* __restrict__ weight_sum,
                                                      float* __restrict__ grads, float* __restrict__ loss, int* err)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    SmemTrain& sm = *reinterpret_cast<SmemTrain*>(smem_raw);
    const int t = threadIdx.x;
    const int64_t n = batch_size(b);
    copy_weights(sm.w, net.packed, kPackedWeights);
    if (t < 32) umma::tmem_alloc(&sm.tmem, kTmemTrain);
    if (t == 0) umma::mbar_init(&sm.mbar);
    publish_smem();
    const uint32_t tmem = sm.tmem;
    const float inv_wsum = *weight_sum > 0.0f ? 1.0f / *weight_sum : 0.0f;
    const Domain d = {{net.lo[0], net.lo[1], net.lo[2]}, {net.inv_ext[0], net.inv_ext[1], net.inv_ext[2]}};
    uint32_t phase = 0;
    float loss_acc = 0.0f;
    bool ok = true, first = true;
    const int64_t n_tiles = (n + kTile - 1) / kTile;
    for (int64_t tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x)
    {
        const int64_t row = tile * kTile + t;
        const bool valid = row < n;
        V3 p = v3(0.0f), nn = v3(0.0f), vw = v3(0.0f), w = v3(0.0f, 0.0f, 1.0f);
        float ws = 0.0f, pb = -1.0f;
        if (valid)
        {
            p = load3(b.pos, row);
            nn = load3(b.nrm, row);
            vw = load3(b.view, row);
            w = load3(b.dir, row);
            ws = fmaxf(b.weight[row], 0.0f);
            if (b.bsdf_pdf) pb = fmaxf(b.bsdf_pdf[row], 0.0f);
        }
        float raw[kOut];
        uint32_t masks[3][2];
        ok = forward_tile(&sm.mbar, tmem, sm.w, sm.act[0], sm.act[1], sm.tr, net, valid, p, nn, vw, raw, masks, phase);
        if (!ok) break;
        // head, loss and its gradient for this row -> dY (K-major, K = 48) and dY^T
        {
            float draw[kOut];
            Lobe lobes[kLobes];
            float len[kLobes], alpha;
            head(raw, lobes, len, alpha);
            const float scale = valid ? ws * inv_wsum : 0.0f;
            const float l = head_backward(raw, lobes, len, alpha, w, scale, pb, draw);
            if (scale > 0.0f) loss_acc += l;
            store_row(sm.act[0], sm.gt[0], draw, kOut);
        }
        publish_smem();
        // layers 4..1: dH_{l-1} = dH_l W_l^T into F and dW_l += H_{l-1}^T dH_l, one commit
        const int wb[4] = {kW1b, kW2b, kW3b, kW4b};
        float g[kHid];
        for (int l = 3; l >= 0 && ok; l--)
        {
            const int n_out = l == 3 ? kOut : kHid;  // width of dH_l
            const int cur = (3 - l) & 1;             // buffers holding dH_l
            if (t == 0)
            {
                umma::gemm_issue(tmem + kColF, sm.act[cur], sm.w + wb[l], l == 0 ? kGridFeatures : kHid, n_out, false);
                umma::gemm_issue(tmem + col_dw(l), sm.tr[l], sm.gt[cur], n_out, kTile, !first);
                umma::commit(&sm.mbar);
            }
            ok = wait_mma(&sm.mbar, phase, net.wait_limit);
            if (!ok) break;
            if (l > 0)
            {
                load_cols(tmem, kColF, kHid, g);
                mask_grad(g, masks[l - 1]);
                store_row(sm.act[cur ^ 1], sm.gt[cur ^ 1], g, kHid);
                publish_smem();
            }
            else
            {
                load_cols(tmem, kColF, kGridFeatures, g);
                if (valid) encode_backward(d, grads + kNumWeights, p, g);
            }
        }
        first = false;
        __syncthreads();  // the next tile overwrites the shared tiles
    }
    if (!ok && t == 0) atomicExch(err, 1);
    // flush the weight-gradient accumulators: rows 0..63 (lanes of warps 0 and 1) = input units
    if (ok && !first && t < 64)
    {
        const int offs[4] = {kOffW1, kOffW2, kOffW3, kOffW4};
        for (int l = 0; l < 4; l++)
        {
            const int n_out = l == 3 ? kOut : kHid;
            float v[16];
            for (int c = 0; c < n_out; c += 16)
            {
                umma::tmem_ld16(umma::lane_addr(tmem, t >> 5, (int)col_dw(l) + c), v);
                for (int j = 0; j < 16; j++)
                    if (v[j] != 0.0f) atomicAdd(grads + offs[l] + t * n_out + c + j, v[j]);
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) loss_acc += __shfl_xor_sync(0xffffffffu, loss_acc, o);
    if ((t & 31) == 0 && loss_acc != 0.0f) atomicAdd(loss, loss_acc);
    umma::fence_before();
    __syncthreads();
    if (t < 32) umma::tmem_dealloc(tmem, kTmemTrain);
}

// ---------------------------------------------------------------------------------------------
// inference: mixture per query (8 x (mu xyz, kappa, weight), alpha, 3 zeros)
// ---------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kTile) infer_kernel(Net net, Batch b, float* __restrict__ out, int* err)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    SmemInfer& sm = *reinterpret_cast<SmemInfer*>(smem_raw);
    const int t = threadIdx.x;
    const int64_t n = batch_size(b);
    copy_weights(sm.w, net.packed, kFwdWeights);
    if (t < 32) umma::tmem_alloc(&sm.tmem, kTmemInfer);
    if (t == 0) umma::mbar_init(&sm.mbar);
    publish_smem();
    const uint32_t tmem = sm.tmem;
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
        ok = forward_tile(&sm.mbar, tmem, sm.w, sm.act, sm.act, nullptr, net, valid, p, nn, vw, raw, nullptr, phase);
        if (!ok) break;
        if (valid)
        {
            Lobe L[kLobes];
            float len[kLobes], alpha;
            head(raw, L, len, alpha);
            float4* o = reinterpret_cast<float4*>(out + (int64_t)kRow * row);
            for (int i = 0; i < kLobes; i += 4)
            {
                // lobes i..i+3 = 20 floats = 5 float4
                float v[20];
                for (int j = 0; j < 4; j++)
                {
                    v[5 * j] = L[i + j].mu.x;
                    v[5 * j + 1] = L[i + j].mu.y;
                    v[5 * j + 2] = L[i + j].mu.z;
                    v[5 * j + 3] = L[i + j].kappa;
                    v[5 * j + 4] = L[i + j].weight;
                }
                for (int q = 0; q < 5; q++) o[(5 * i) / 4 + q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
            }
            o[10] = make_float4(alpha, 0.0f, 0.0f, 0.0f);
        }
        __syncthreads();
    }
    if (!ok && t == 0) atomicExch(err, 1);
    umma::fence_before();
    __syncthreads();
    if (t < 32) umma::tmem_dealloc(tmem, kTmemInfer);
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
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < kNumParams; i += (int64_t)gridDim.x * blockDim.x)
    {
        const float u = 2.0f * hash_uniform((uint32_t)i, seed) - 1.0f;
        float s;
        if (i < kOffW4)
            s = sqrtf(6.0f / (kHid + kHid));
        else if (i < kNumWeights)
            s = sqrtf(6.0f / (kHid + kOut));
        else
            s = 1.0e-4f;
        params[i] = u * s;
    }
}

__global__ void pack_kernel(const float* __restrict__ params, bf16* __restrict__ packed, uint32_t* __restrict__ grid_bf16)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < kNumWeights; i += stride)
    {
        const bf16 v = __float2bfloat16(params[i]);
        const int l = i < kOffW4 ? (int)(i / (kHid * kHid)) : 3;
        const int base = l == 3 ? kOffW4 : l * kHid * kHid;
        const int n_out = l == 3 ? kOut : kHid;
        const int j = (int)i - base, a = j / n_out, o = j % n_out;  // W_l[a = input][o = output]
        const int fwd[4] = {kW1f, kW2f, kW3f, kW4f}, bwd[4] = {kW1b, kW2b, kW3b, kW4b};
        packed[fwd[l] + kmo(o, a, kHid)] = v;   // W^T: row = output, K = input (64)
        packed[bwd[l] + kmo(a, o, n_out)] = v;  // W: row = input, K = output
    }
    const float2* g = reinterpret_cast<const float2*>(params + kNumWeights);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (int64_t)kLevels * kTable; i += stride)
    {
        const float2 v = g[i];
        const uint32_t lo = (uint32_t)__bfloat16_as_ushort(__float2bfloat16(v.x));
        const uint32_t hi = (uint32_t)__bfloat16_as_ushort(__float2bfloat16(v.y));
        grid_bf16[i] = lo | (hi << 16);
    }
}

__global__ void adam_kernel(float* __restrict__ params, const float* __restrict__ grads, float* __restrict__ m,
                            float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < kNumParams; i += (int64_t)gridDim.x * blockDim.x)
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
    init_kernel<<<2048, 256, 0, st>>>(params, seed);
    return cudaGetLastError();
}

cudaError_t launch_guide_pack(const float* params, uint16_t* packed, uint32_t* grid_bf16, cudaStream_t st)
{
    pack_kernel<<<2048, 256, 0, st>>>(params, reinterpret_cast<bf16*>(packed), grid_bf16);
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
        cudaError_t e = cudaFuncSetAttribute(train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SmemTrain));
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    const int64_t tiles = (b.n_max + kTile - 1) / kTile;
    const int grid = (int)(tiles < n_sm ? (tiles < 1 ? 1 : tiles) : n_sm);
    train_kernel<<<grid, kTile, sizeof(SmemTrain), st>>>(net, b, weight_sum, grads, loss, err);
    return cudaGetLastError();
}

cudaError_t launch_guide_infer(const Net& net, const Batch& b, float* lobes, int* err, int n_sm, cudaStream_t st)
{
    static bool attr_set = false;
    if (!attr_set)
    {
        cudaError_t e = cudaFuncSetAttribute(infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SmemInfer));
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    const int64_t tiles = (b.n_max + kTile - 1) / kTile;
    const int64_t cap = (int64_t)n_sm * kInferCtasPerSm;
    const int grid = (int)(tiles < cap ? (tiles < 1 ? 1 : tiles) : cap);
    infer_kernel<<<grid, kTile, sizeof(SmemInfer), st>>>(net, b, lobes, err);
    return cudaGetLastError();
}

cudaError_t launch_guide_adam(float* params, const float* grads, float* m, float* v, float lr, float beta1, float beta2,
                              float eps, int step, cudaStream_t st)
{
    const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
    adam_kernel<<<2048, 256, 0, st>>>(params, grads, m, v, lr, beta1, beta2, eps, c1, c2);
    return cudaGetLastError();
}

}  // namespace guide
}  // namespace gbpt
