// Split-operand tensor-core form of the matrix Fourier transform (tcgen05 on sm_103a).
#pragma once

#include "hx_common.cuh"

namespace hx {

struct SplitMftPlan;

int split_mft_create(int nx, int ny, int nu, int nv, const float2* m1f, const float2* m2f, const float2* m1b,
                     const float2* m2b, const float2* m1a, const float2* m2a, cudaStream_t stream, SplitMftPlan** out);
size_t split_mft_workspace_bytes(const SplitMftPlan* p, int direction, int batch);
int split_mft_execute(const SplitMftPlan* p, int direction, int batch, const float2* in, float2* out, double are,
                      double aim, int epilogue, const float2* mask, const float2* src, void* ws, size_t ws_bytes,
                      cudaStream_t stream);
void split_mft_destroy(SplitMftPlan* p);

}  // namespace hx
