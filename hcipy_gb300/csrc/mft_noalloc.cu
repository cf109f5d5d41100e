// hx_mft_execute_noalloc: the matrix Fourier transform for callers that cannot
// allocate device memory while they run.
//
// Who needs it: code that drives the propagation from a context where calling
// cudaMalloc (or any allocator that may call it, torch's included) is not
// allowed or not possible -- a real-time control loop that must not stall on
// the allocator, a host framework that owns all device memory and hands out
// only input and output buffers, a plugin ABI that passes plain pointers and
// no allocator.  hx_mft_execute needs a caller-provided workspace for the
// intermediate product of its two GEMMs; this entry point takes that scratch
// from a fixed device array compiled into the library instead.
//
// The scratch is `g_mft_scratch` below: HX_MFT_NOALLOC_SCRATCH_BYTES (16 MiB),
// 256-byte aligned, one copy per GPU that loads this library, kept until the
// process exits.  Host code must not pass the array's name to a kernel -- on the
// host it is only a stand-in symbol -- so on its first call on each device this
// entry point asks the runtime for the array's device address
// (cudaGetSymbolAddress, with that device current) and caches it.  That first
// call per device should therefore come before any stream capture.  The cache
// is keyed on the device and its current CUDA context: after cudaDeviceReset
// (or any teardown that gives the device a new primary context) the module is
// loaded again at a new address, and the next call looks the address up again
// instead of using a stale one.
//
// Every call uses the same array and it keeps the previous call's contents.
// The MFT overwrites every scratch element it reads (the whole intermediate is
// written by the first GEMM before the second reads it), so nothing has to
// start at zero.  Two calls whose kernels overlap on the GPU (different
// streams, or different host threads without ordering) race on the array.
#include "hx_common.cuh"

#include <cuda.h>

#include <mutex>

namespace {

__device__ __align__(256) unsigned char g_mft_scratch[HX_MFT_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
void* g_scratch_ptr[kMaxDevices] = {};
CUcontext g_scratch_ctx[kMaxDevices] = {};
std::mutex g_scratch_mutex;

using CtxGetCurrent = CUresult (*)(CUcontext*);

// cuCtxGetCurrent from the driver, looked up once through the runtime (the library does not link libcuda).
CtxGetCurrent ctx_get_current() {
    static CtxGetCurrent fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<CtxGetCurrent>(p);
    });
    return fn;
}

int scratch_for_current_device(void** out) {
    int dev = 0;
    HX_TRY(hx::cuda_status(cudaGetDevice(&dev), "hx_mft_execute_noalloc: cudaGetDevice"));
    if (dev < 0 || dev >= kMaxDevices) {
        hx::set_error("hx_mft_execute_noalloc: device %d out of range", dev);
        return HX_ERR_UNSUPPORTED;
    }
    CtxGetCurrent get = ctx_get_current();
    CUcontext ctx = nullptr;
    if (!get || get(&ctx) != CUDA_SUCCESS) {
        hx::set_error("hx_mft_execute_noalloc: cuCtxGetCurrent is not available from the driver");
        return HX_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (g_scratch_ptr[dev] == nullptr || ctx == nullptr || g_scratch_ctx[dev] != ctx) {
        // The lookup makes the device's primary context current if none was, so the context is read again after
        // it: that is the context this call's kernels run in.
        void* p = nullptr;
        HX_TRY(hx::cuda_status(cudaGetSymbolAddress(&p, g_mft_scratch),
                               "hx_mft_execute_noalloc: cudaGetSymbolAddress(scratch)"));
        if (get(&ctx) != CUDA_SUCCESS) {
            hx::set_error("hx_mft_execute_noalloc: cuCtxGetCurrent failed");
            return HX_ERR_CUDA;
        }
        g_scratch_ptr[dev] = p;
        g_scratch_ctx[dev] = ctx;
    }
    *out = g_scratch_ptr[dev];
    return HX_OK;
}

}  // namespace

extern "C" {

int hx_mft_execute_noalloc(const hx_mft_plan* plan, int direction, int batch, const void* in, void* out,
                           double alpha_re, double alpha_im, void* stream) {
    HX_CHECK_ARG(plan != nullptr, "hx_mft_execute_noalloc: plan is NULL");
    HX_CHECK_ARG(batch >= 1, "hx_mft_execute_noalloc: batch must be >= 1 (got %d)", batch);
    const size_t need = hx_mft_workspace_bytes(plan, direction, batch);
    HX_CHECK_ARG(need <= (size_t)HX_MFT_NOALLOC_SCRATCH_BYTES,
                 "hx_mft_execute_noalloc: this transform needs %zu bytes of scratch for batch %d, more than the "
                 "%d-byte static scratch; use hx_mft_execute with a workspace, or a smaller batch",
                 need, batch, HX_MFT_NOALLOC_SCRATCH_BYTES);
    void* scratch = nullptr;
    HX_TRY(scratch_for_current_device(&scratch));
    return hx_mft_execute(plan, direction, batch, in, out, alpha_re, alpha_im, scratch,
                          (size_t)HX_MFT_NOALLOC_SCRATCH_BYTES, stream);
}

}  // extern "C"
