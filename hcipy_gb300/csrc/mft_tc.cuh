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
// Fields are complex64 or complex128 (dtype HX_C64 / HX_C128), independently for input, output and the
// Babinet source; the mask is complex64.
int split_mft_execute(const SplitMftPlan* p, int direction, int batch, const void* in, int in_dtype, void* out,
                      int out_dtype, double are, double aim, int epilogue, const float2* mask, const void* src,
                      int src_dtype, void* ws, size_t ws_bytes, cudaStream_t stream);
// Forward transform of complex64 fields times exp(i scale screen), the phase applied while slicing (screen: the
// plan's ny x nx float32 values, shared by the batch).
int split_mft_execute_phase(const SplitMftPlan* p, int batch, const void* in, const float* screen, double scale,
                            void* out, int out_dtype, double are, double aim, void* ws, cudaStream_t stream);
// Lyot coronagraph and (if img != NULL) its final image, with the focal-plane and Lyot-plane fields in
// float-float between the transforms.
size_t split_lyot_workspace_bytes(const SplitMftPlan* fpm, const SplitMftPlan* img, int batch);
int split_lyot_execute(const SplitMftPlan* fpm, const SplitMftPlan* img, int batch, const void* e, int e_dtype,
                       const float2* one_minus_fpm, const float2* stop, double af_re, double af_im, double ab_re,
                       double ab_im, double ai_re, double ai_im, void* lyot_out, int lyot_dtype, void* img_out,
                       int img_dtype, void* ws, cudaStream_t stream);
// Status word of the bounded device waits (HX_OK or HX_ERR_TIMEOUT); synchronizes with the device.
int split_mft_status(const SplitMftPlan* p, int reset);
void split_mft_destroy(SplitMftPlan* p);
// Tile policy of the plan's GEMMs: HX_SCHEDULE_LATENCY or HX_SCHEDULE_THROUGHPUT.
void split_mft_set_schedule(SplitMftPlan* p, int schedule);
// Autotuner of the split GEMM tiles (process-wide): on/off, number of measured shapes, forget them.
void split_autotune(int on);
int split_autotune_entries();
// Entry i: shape {m_tiles, N, grid_z, ktiles}, n candidates with their tile width, K split and time (<= 8).
int split_autotune_entry(int i, long long* shape, int* n, int* bn, int* ksplit, float* ms);
void split_autotune_clear();
// Weighted intensity sums sum_p w[p] |E_b[p]|^2 per field (w may be NULL) in compensated float-float
// arithmetic, and their gradient 2 g_b w E_b; fields are complex64 or complex128.
size_t intensity_sums_workspace_bytes(long long n, int batch);
int intensity_sums(const void* field, int dtype, long long n, int batch, const float* w, double* sums, void* ws,
                   cudaStream_t stream);
int intensity_sums_grad(const void* field, int dtype, long long n, int batch, const float* w, const double* g,
                        void* out, cudaStream_t stream);

}  // namespace hx
