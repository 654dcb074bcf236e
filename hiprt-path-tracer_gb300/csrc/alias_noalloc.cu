// gbpt_alias_table_build_noalloc: the emitter power alias table built without any device
// allocation, for callers that cannot call cudaMalloc (declared in include/gbpt_render.h).
//
// The kernels are the ones gbpt_scene_create uses (FP64 sum, normalisation, Vose partition;
// render.cu). Their scratch (block partial sums, the normalised FP64 list and the two Vose queues)
// lives in one file-scope __device__ array of fixed size, which every device that loads libgbpt
// holds until the process exits. Host code cannot pass that array's name to a kernel: in host
// code the name is only a host-side stand-in. Its device address is looked up with
// cudaGetSymbolAddress, with the device current, on the first call made in each CUDA context
// (the address belongs to the context: after cudaDeviceReset, or in another context on the same
// device, it is looked up again).
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/gbpt_render.h"
#include "handles.h"
#include "render_kernels.h"

namespace {

constexpr int kMaxEmitters = GBPT_ALIAS_NOALLOC_MAX_EMITTERS;
constexpr int kPartials = 64;  // block partial sums of the FP64 reduction
// Layout in doubles: partials [0, 64), normalised list [64, 64 + n_max),
// then the small and large queues as int32 (n_max each = n_max / 2 doubles each).
constexpr size_t kScratchDoubles = (size_t)kPartials + (size_t)kMaxEmitters + (size_t)kMaxEmitters;
static_assert(kMaxEmitters % 2 == 0, "queue area must be a whole number of doubles");

static __device__ __align__(256) double g_alias_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double* g_scratch_addr[kMaxDevices] = {};
CUcontext g_scratch_ctx[kMaxDevices] = {};  // the context each cached address belongs to

using CtxGetCurrentFn = CUresult (*)(CUcontext*);

// cuCtxGetCurrent through the runtime's driver entry point (no link against the driver library)
CtxGetCurrentFn ctx_get_current()
{
    static const CtxGetCurrentFn fn = []() -> CtxGetCurrentFn {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return nullptr;
        return reinterpret_cast<CtxGetCurrentFn>(p);
    }();
    return fn;
}

// Device address of g_alias_scratch in the current context (looked up again when the context of
// the current device is not the one the cached address was taken in).
gbpt_status scratch_for_current_device(double** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return gbpt::cuda_error(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices)
        return gbpt::set_error(GBPT_ERROR_UNSUPPORTED, "device ordinal " + std::to_string(dev) + " is beyond the " +
                                                           std::to_string(kMaxDevices) + " devices this entry point tracks");
    const CtxGetCurrentFn get_ctx = ctx_get_current();
    if (!get_ctx) return gbpt::set_error(GBPT_ERROR_UNSUPPORTED, "cuCtxGetCurrent is unavailable");
    CUcontext ctx = nullptr;
    if (get_ctx(&ctx) != CUDA_SUCCESS) return gbpt::set_error(GBPT_ERROR_CUDA, "cuCtxGetCurrent failed");
    if (!ctx)
    {
        // no context current on this thread yet: the runtime makes the device's primary one current
        e = cudaFree(nullptr);
        if (e != cudaSuccess) return gbpt::cuda_error(e, "context initialisation");
        if (get_ctx(&ctx) != CUDA_SUCCESS || !ctx) return gbpt::set_error(GBPT_ERROR_CUDA, "no current CUDA context");
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev] || g_scratch_ctx[dev] != ctx)
    {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_alias_scratch);
        if (e != cudaSuccess) return gbpt::cuda_error(e, "cudaGetSymbolAddress of the alias-table scratch");
        g_scratch_addr[dev] = static_cast<double*>(p);
        g_scratch_ctx[dev] = ctx;
    }
    *out = g_scratch_addr[dev];
    return GBPT_OK;
}

}  // namespace

extern "C" {

gbpt_status gbpt_alias_table_build_noalloc(const float* power, int32_t n, float* probas, int32_t* alias,
                                           double* power_sum64, void* stream)
{
    if (n < 0) return gbpt::set_error(GBPT_ERROR_INVALID_ARG, "n is negative");
    if (n > kMaxEmitters)
        return gbpt::set_error(GBPT_ERROR_INVALID_ARG, "n = " + std::to_string(n) +
                                                           " emitters exceeds the no-allocation maximum of " +
                                                           std::to_string(kMaxEmitters));
    if (n == 0) return GBPT_OK;
    if (!power || !probas || !alias || !power_sum64)
        return gbpt::set_error(GBPT_ERROR_INVALID_ARG, "power, probas, alias and power_sum64 must be device pointers");
    double* scratch = nullptr;
    gbpt_status st = scratch_for_current_device(&scratch);
    if (st != GBPT_OK) return st;
    double* partial = scratch;
    double* q = scratch + kPartials;
    int32_t* smalls = reinterpret_cast<int32_t*>(scratch + kPartials + kMaxEmitters);
    int32_t* larges = smalls + kMaxEmitters;
    // Every scratch word the kernels read is written earlier in the same call (partials by the
    // sum, q by the normalisation, the queues by the Vose pass), so nothing needs clearing.
    cudaError_t e = gbpt::launch_alias_table(power, n, partial, kPartials, power_sum64, q, probas, alias, smalls,
                                             larges, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? GBPT_OK : gbpt::cuda_error(e, "alias table launch");
}

}  // extern "C"
