// C ABI of the guiding network (include/gbpt_guide.h): parameter buffers, Adam state, training and
// inference launches.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <new>
#include <string>

#include "../../include/gbpt_guide.h"
#include "guide_kernels.h"
#include "handles.h"

using gbpt::cuda_error;
using gbpt::set_error;
namespace G = gbpt::guide;

struct gbpt_guide
{
    gbpt_guide_params p;
    float* params = nullptr;  // [weights | grid]
    float* grads = nullptr;
    float* m = nullptr;
    float* v = nullptr;
    uint16_t* packed = nullptr;
    uint32_t* grid_bf16 = nullptr;
    float* scratch = nullptr;  // [weight sum, loss]
    int* err = nullptr;
    int step = 0;
    int n_sm = 1;
};

namespace {

G::Net net_of(const gbpt_guide* g)
{
    G::Net n;
    n.params = g->params;
    n.packed = g->packed;
    n.grid_bf16 = g->grid_bf16;
    n.wait_limit = g->p.wait_limit > 0 ? g->p.wait_limit : (g->p.wait_limit == 0 ? (1 << 24) : 0);
    for (int a = 0; a < 3; a++)
    {
        n.lo[a] = g->p.scene_min[a];
        const float ext = g->p.scene_max[a] - g->p.scene_min[a];
        n.inv_ext[a] = ext > 0.0f ? 1.0f / ext : 0.0f;
    }
    return n;
}

void release(gbpt_guide* g)
{
    cudaFree(g->params);
    cudaFree(g->grads);
    cudaFree(g->m);
    cudaFree(g->v);
    cudaFree(g->packed);
    cudaFree(g->grid_bf16);
    cudaFree(g->scratch);
    cudaFree(g->err);
}

gbpt_status check_err(gbpt_guide* g, cudaStream_t cs)
{
    int err = 0;
    cudaError_t e = cudaMemcpyAsync(&err, g->err, sizeof(int), cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
    if (e != cudaSuccess) return cuda_error(e, "guide status read-back");
    if (err) return set_error(GBPT_ERROR_TIMEOUT, "a tensor-core wait of the guiding network gave up");
    return GBPT_OK;
}

G::Batch host_batch(const float* pos, const float* nrm, const float* view, const float* dir, const float* w,
                    const float* bsdf_pdf, int64_t n)
{
    G::Batch b;
    b.pos = pos;
    b.nrm = nrm;
    b.view = view;
    b.dir = dir;
    b.weight = w;
    b.bsdf_pdf = bsdf_pdf;
    b.count = nullptr;
    b.n_max = n;
    return b;
}

// forward + backward into g->grads (zeroed here); loss into g->scratch[1]
gbpt_status compute_gradients(gbpt_guide* g, const G::Batch& b, cudaStream_t cs)
{
    if (b.n_max < 0 || b.n_max > g->p.max_batch) return set_error(GBPT_ERROR_INVALID_ARG, "n must be in 0..max_batch");
    if (b.n_max > 0 && (!b.pos || !b.nrm || !b.view || !b.dir || !b.weight))
        return set_error(GBPT_ERROR_INVALID_ARG, "training arrays must be device pointers");
    cudaError_t e = cudaMemsetAsync(g->grads, 0, sizeof(float) * G::kNumParams, cs);
    if (e == cudaSuccess) e = cudaMemsetAsync(g->scratch + 1, 0, sizeof(float), cs);
    if (e == cudaSuccess) e = G::launch_guide_weight_sum(b, g->scratch, cs);
    if (e == cudaSuccess && b.n_max > 0)
        e = G::launch_guide_train(net_of(g), b, g->scratch, g->grads, g->scratch + 1, g->err, g->n_sm, cs);
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "guide training launch");
}

gbpt_status adam_step(gbpt_guide* g, cudaStream_t cs)
{
    g->step++;
    cudaError_t e = G::launch_guide_adam(g->params, g->grads, g->m, g->v, g->p.learning_rate, g->p.beta1, g->p.beta2,
                                         g->p.epsilon, g->step, cs);
    if (e == cudaSuccess) e = G::launch_guide_pack(g->params, g->packed, g->grid_bf16, cs);
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "guide update");
}

}  // namespace

extern "C" {

gbpt_status gbpt_guide_default_params(gbpt_guide_params* p)
{
    if (!p) return set_error(GBPT_ERROR_INVALID_ARG, "params is NULL");
    std::memset(p, 0, sizeof(*p));
    for (int a = 0; a < 3; a++)
    {
        p->scene_min[a] = 0.0f;
        p->scene_max[a] = 1.0f;
    }
    p->learning_rate = 1.0e-2f;
    p->beta1 = 0.9f;
    p->beta2 = 0.99f;
    p->epsilon = 1.0e-8f;
    p->seed = 1;
    p->max_batch = 1 << 18;
    return GBPT_OK;
}

gbpt_status gbpt_guide_create(const gbpt_guide_params* p, gbpt_guide** out)
{
    if (!p || !out) return set_error(GBPT_ERROR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    if (p->max_batch < 1 || p->max_batch > (1 << 26)) return set_error(GBPT_ERROR_INVALID_ARG, "max_batch out of range");
    for (int a = 0; a < 3; a++)
        if (!(p->scene_max[a] > p->scene_min[a])) return set_error(GBPT_ERROR_INVALID_ARG, "empty scene box");
    gbpt_guide* g = new (std::nothrow) gbpt_guide();
    if (!g) return set_error(GBPT_ERROR_OOM, "host allocation failed");
    g->p = *p;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g->n_sm, cudaDevAttrMultiProcessorCount, dev);
    const size_t np = sizeof(float) * G::kNumParams;
    cudaError_t e = cudaMalloc(&g->params, np);
    if (e == cudaSuccess) e = cudaMalloc(&g->grads, np);
    if (e == cudaSuccess) e = cudaMalloc(&g->m, np);
    if (e == cudaSuccess) e = cudaMalloc(&g->v, np);
    if (e == cudaSuccess) e = cudaMalloc(&g->packed, sizeof(uint16_t) * G::kPackedWeights);
    if (e == cudaSuccess) e = cudaMalloc(&g->grid_bf16, sizeof(uint32_t) * GBPT_GUIDE_LEVELS * GBPT_GUIDE_TABLE);
    if (e == cudaSuccess) e = cudaMalloc(&g->scratch, 2 * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&g->err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(g->m, 0, np);
    if (e == cudaSuccess) e = cudaMemset(g->v, 0, np);
    if (e == cudaSuccess) e = cudaMemset(g->err, 0, sizeof(int));
    if (e == cudaSuccess) e = G::launch_guide_init(g->params, p->seed, nullptr);
    if (e == cudaSuccess) e = G::launch_guide_pack(g->params, g->packed, g->grid_bf16, nullptr);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess)
    {
        release(g);
        delete g;
        return e == cudaErrorMemoryAllocation ? set_error(GBPT_ERROR_OOM, "guide allocation") : cuda_error(e, "guide create");
    }
    *out = g;
    return GBPT_OK;
}

gbpt_status gbpt_guide_destroy(gbpt_guide* g)
{
    if (!g) return GBPT_OK;
    release(g);
    delete g;
    return GBPT_OK;
}

gbpt_status gbpt_guide_train(gbpt_guide* g, const float* position, const float* normal, const float* view,
                             const float* direction, const float* weight, const float* bsdf_pdf, int64_t n, float* loss,
                             void* stream)
{
    if (!g) return set_error(GBPT_ERROR_INVALID_ARG, "guide is NULL");
    cudaStream_t cs = (cudaStream_t)stream;
    gbpt_status st = compute_gradients(g, host_batch(position, normal, view, direction, weight, bsdf_pdf, n), cs);
    if (st != GBPT_OK) return st;
    if (loss)
    {
        cudaError_t e = cudaMemcpyAsync(loss, g->scratch + 1, sizeof(float), cudaMemcpyDeviceToHost, cs);
        if (e != cudaSuccess) return cuda_error(e, "loss read-back");
    }
    st = adam_step(g, cs);
    if (st != GBPT_OK) return st;
    if (loss) return check_err(g, cs);
    return GBPT_OK;
}

gbpt_status gbpt_guide_gradients(gbpt_guide* g, const float* position, const float* normal, const float* view,
                                 const float* direction, const float* weight, const float* bsdf_pdf, int64_t n,
                                 float* grad_weights, float* grad_grid, float* loss, void* stream)
{
    if (!g) return set_error(GBPT_ERROR_INVALID_ARG, "guide is NULL");
    cudaStream_t cs = (cudaStream_t)stream;
    gbpt_status st = compute_gradients(g, host_batch(position, normal, view, direction, weight, bsdf_pdf, n), cs);
    if (st != GBPT_OK) return st;
    cudaError_t e = cudaSuccess;
    if (grad_weights)
        e = cudaMemcpyAsync(grad_weights, g->grads, sizeof(float) * G::kNumWeights, cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess && grad_grid)
        e = cudaMemcpyAsync(grad_grid, g->grads + G::kNumWeights, sizeof(float) * GBPT_GUIDE_GRID_PARAMS,
                            cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess && loss) e = cudaMemcpyAsync(loss, g->scratch + 1, sizeof(float), cudaMemcpyDeviceToHost, cs);
    if (e != cudaSuccess) return cuda_error(e, "gradient read-back");
    return check_err(g, cs);
}

gbpt_status gbpt_guide_infer(gbpt_guide* g, const float* position, const float* normal, const float* view, int64_t n,
                             float* lobes, void* stream)
{
    if (!g) return set_error(GBPT_ERROR_INVALID_ARG, "guide is NULL");
    if (n < 0) return set_error(GBPT_ERROR_INVALID_ARG, "n is negative");
    if (n == 0) return GBPT_OK;
    if (!position || !normal || !view || !lobes) return set_error(GBPT_ERROR_INVALID_ARG, "arrays must be device pointers");
    cudaError_t e = G::launch_guide_infer(net_of(g), host_batch(position, normal, view, nullptr, nullptr, nullptr, n), lobes, g->err,
                                          g->n_sm, (cudaStream_t)stream);
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "guide inference launch");
}

gbpt_status gbpt_guide_error_flag(gbpt_guide* g, int32_t* flag)
{
    if (!g || !flag) return set_error(GBPT_ERROR_INVALID_ARG, "NULL argument");
    cudaError_t e = cudaMemcpy(flag, g->err, sizeof(int), cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "guide status read-back");
}

gbpt_status gbpt_guide_get_params(gbpt_guide* g, float* weights, float* grid)
{
    if (!g) return set_error(GBPT_ERROR_INVALID_ARG, "guide is NULL");
    cudaError_t e = cudaSuccess;
    if (weights) e = cudaMemcpy(weights, g->params, sizeof(float) * G::kNumWeights, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && grid)
        e = cudaMemcpy(grid, g->params + G::kNumWeights, sizeof(float) * GBPT_GUIDE_GRID_PARAMS, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "guide parameter read-back");
}

gbpt_status gbpt_guide_set_params(gbpt_guide* g, const float* weights, const float* grid)
{
    if (!g) return set_error(GBPT_ERROR_INVALID_ARG, "guide is NULL");
    cudaError_t e = cudaSuccess;
    if (weights) e = cudaMemcpy(g->params, weights, sizeof(float) * G::kNumWeights, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && grid)
        e = cudaMemcpy(g->params + G::kNumWeights, grid, sizeof(float) * GBPT_GUIDE_GRID_PARAMS, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = G::launch_guide_pack(g->params, g->packed, g->grid_bf16, nullptr);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "guide parameter upload");
}

}  // extern "C"

namespace gbpt {
namespace guide {

gbpt_status render_infer(gbpt_guide* g, const Batch& b, float* lobes, cudaStream_t cs)
{
    cudaError_t e = launch_guide_infer(net_of(g), b, lobes, g->err, g->n_sm, cs);
    return e == cudaSuccess ? GBPT_OK : cuda_error(e, "guide inference launch");
}

gbpt_status render_train(gbpt_guide* g, const Batch& b, cudaStream_t cs)
{
    Batch c = b;
    if (c.n_max > g->p.max_batch) c.n_max = g->p.max_batch;
    gbpt_status st = compute_gradients(g, c, cs);
    return st == GBPT_OK ? adam_step(g, cs) : st;
}

int64_t max_batch(const gbpt_guide* g) { return g->p.max_batch; }

}  // namespace guide
}  // namespace gbpt
