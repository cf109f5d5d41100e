// Split-operand tensor-core MFT: not built yet in this version.
#include "mft_tc.cuh"

namespace hx {

struct SplitMftPlan {};

int split_mft_create(int, int, int, int, const float2*, const float2*, const float2*, const float2*, const float2*,
                     const float2*, cudaStream_t, SplitMftPlan** out) {
    *out = nullptr;
    set_error("the split tensor-core MFT is not available in this build");
    return HX_ERR_UNSUPPORTED;
}

size_t split_mft_workspace_bytes(const SplitMftPlan*, int, int) { return 0; }

int split_mft_execute(const SplitMftPlan*, int, int, const float2*, float2*, double, double, int, const float2*,
                      const float2*, void*, size_t, cudaStream_t) {
    set_error("the split tensor-core MFT is not available in this build");
    return HX_ERR_UNSUPPORTED;
}

void split_mft_destroy(SplitMftPlan* p) { delete p; }

}  // namespace hx
