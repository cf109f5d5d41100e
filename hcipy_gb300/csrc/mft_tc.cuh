// Split-operand tensor-core form of the matrix Fourier transform (tcgen05 on sm_103a).
#pragma once

#include "hx_common.cuh"

namespace hx {

struct SplitMftPlan;

// Builds the sliced phase matrices from device coordinate and weight arrays (weights may be NULL).
int split_mft_create(int nx, int ny, int nu, int nv, const double* x, const double* y, const double* u,
                     const double* v, const double* wx, const double* wy, const double* wu, const double* wv,
                     cudaStream_t stream, SplitMftPlan** out);
size_t split_mft_workspace_bytes(const SplitMftPlan* p, int direction, int batch);
int split_mft_execute(const SplitMftPlan* p, int direction, int batch, const float2* in, float2* out, double are,
                      double aim, int epilogue, const float2* mask, const float2* src, void* ws, size_t ws_bytes,
                      cudaStream_t stream);
// Status word of the bounded device waits (HX_OK or HX_ERR_TIMEOUT); synchronizes with the device.
int split_mft_status(const SplitMftPlan* p, int reset);
void split_mft_destroy(SplitMftPlan* p);

}  // namespace hx
