// Deformable-mirror surfaces and phase screens on the device.
//
//  * hx_influence_apply: S[v, p] = sum_a Phi[p, a] A[v, a] for a batch of command vectors
//    (DeformableMirror.surface = ModeBasis.linear_combination, hcipy/optics/deformable_mirror.py:251-262,
//    hcipy/mode_basis/mode_basis.py:239-258).  Phi is sparse (Gaussian pokes cut off at 3 actuator pitches,
//    ~23 actuators per pupil pixel), stored CSR over pupil pixels.  One thread per pixel walks its row and
//    keeps VC accumulators; consecutive pixels touch nearly the same actuators, so the gathers of A hit L1.
//  * hx_influence_apply_transpose: G_a[v, a] = sum_p Phi[p, a] G[v, p] (the gradient of the surface with
//    respect to the actuators), from the CSC form.  One CTA per (actuator, vector group) walks the
//    actuator's pixels and reduces in a fixed order, so the result is deterministic.
//  * hx_phase_apply / hx_phase_apply_grad: out = e exp(i c s) with broadcasting over a leading batch
//    (DeformableMirror.forward/backward with c = +-2k, deformable_mirror.py:200-238; AtmosphericLayer
//    forward/backward with c = +-1/lambda, hcipy/atmosphere/atmospheric_model.py:143-151), and its gradient
//    for real s: g_s = c Im(conj(out) g_out), g_e = g_out exp(-i c s) summed over broadcast copies.
#include "hx_common.cuh"

#include <cmath>

namespace {

constexpr int VC = 8;  // command vectors per thread (forward) / per CTA (transpose)

template <typename T>
__global__ void influence_apply_kernel(int npix, int nact, const int* __restrict__ row_ptr,
                                       const int* __restrict__ col_idx, const T* __restrict__ vals, int nvec,
                                       const T* __restrict__ act, T* __restrict__ surf) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int v0 = blockIdx.y * VC;
    if (p >= npix) return;
    T acc[VC];
#pragma unroll
    for (int v = 0; v < VC; ++v) acc[v] = T(0);
    const int j1 = row_ptr[p + 1];
    for (int j = row_ptr[p]; j < j1; ++j) {
        const int a = col_idx[j];
        const T w = vals[j];
#pragma unroll
        for (int v = 0; v < VC; ++v)
            if (v0 + v < nvec) acc[v] += w * __ldg(&act[(long long)(v0 + v) * nact + a]);
    }
#pragma unroll
    for (int v = 0; v < VC; ++v)
        if (v0 + v < nvec) surf[(long long)(v0 + v) * npix + p] = acc[v];
}

template <typename T>
__global__ void influence_transpose_kernel(int npix, int nact, const int* __restrict__ col_ptr,
                                           const int* __restrict__ row_idx, const T* __restrict__ vals, int nvec,
                                           const T* __restrict__ g, T* __restrict__ g_act) {
    const int a = blockIdx.x;
    const int v0 = blockIdx.y * VC;
    __shared__ T red[VC][256 / 32];
    T acc[VC];
#pragma unroll
    for (int v = 0; v < VC; ++v) acc[v] = T(0);
    const int j1 = col_ptr[a + 1];
    for (int j = col_ptr[a] + threadIdx.x; j < j1; j += blockDim.x) {
        const int p = row_idx[j];
        const T w = vals[j];
#pragma unroll
        for (int v = 0; v < VC; ++v)
            if (v0 + v < nvec) acc[v] += w * __ldg(&g[(long long)(v0 + v) * npix + p]);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int v = 0; v < VC; ++v) {
        T x = acc[v];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) red[v][warp] = x;
    }
    __syncthreads();
    if (threadIdx.x < VC && v0 + threadIdx.x < nvec) {
        T x = T(0);
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) x += red[threadIdx.x][w];
        g_act[(long long)(v0 + threadIdx.x) * nact + a] = x;
    }
}

__device__ __forceinline__ void sincos_t(float x, float* s, float* c) { sincosf(x, s, c); }
__device__ __forceinline__ void sincos_t(double x, double* s, double* c) { sincos(x, s, c); }

template <typename T>
__global__ void phase_apply_kernel(long long n, int batch, int batch_e, int batch_s,
                                   const typename hx::cplx<T>::type* __restrict__ e, const T* __restrict__ s, T scale,
                                   typename hx::cplx<T>::type* __restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int b = blockIdx.y;
    if (i >= n) return;
    T sn, cs;
    sincos_t(scale * s[(long long)(b % batch_s) * n + i], &sn, &cs);
    const auto x = e[(long long)(b % batch_e) * n + i];
    out[(long long)b * n + i] = hx::make_c<T>(x.x * cs - x.y * sn, x.x * sn + x.y * cs);
}

// One thread per pixel, looping over the batch: g_s for every output, g_e summed over the copies that share
// an input field (batch_e == 1 or batch_e == batch).
template <typename T>
__global__ void phase_grad_kernel(long long n, int batch, int batch_e, int batch_s,
                                  const typename hx::cplx<T>::type* __restrict__ e, const T* __restrict__ s, T scale,
                                  const typename hx::cplx<T>::type* __restrict__ g_out, T* __restrict__ g_s,
                                  typename hx::cplx<T>::type* __restrict__ g_e) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    T ge_re = T(0), ge_im = T(0);
    for (int b = 0; b < batch; ++b) {
        T sn, cs;
        sincos_t(scale * s[(long long)(b % batch_s) * n + i], &sn, &cs);
        const auto x = e[(long long)(b % batch_e) * n + i];
        const auto g = g_out[(long long)b * n + i];
        // out = x exp(i c s); conj(out) g = conj(x) exp(-i c s) g
        const T gr = g.x * cs + g.y * sn;  // g exp(-i c s)
        const T gi = g.y * cs - g.x * sn;
        if (g_s) {
            const T im = x.x * gi - x.y * gr;  // Im(conj(x) * (g exp(-i c s)))
            if (batch_s == batch) g_s[(long long)b * n + i] = scale * im;
            else if (b == 0) g_s[i] = scale * im;
            else g_s[i] += scale * im;
        }
        if (g_e) {
            if (batch_e == batch) {
                g_e[(long long)b * n + i] = hx::make_c<T>(gr, gi);
            } else {
                ge_re += gr;
                ge_im += gi;
            }
        }
    }
    if (g_e && batch_e != batch) g_e[i] = hx::make_c<T>(ge_re, ge_im);
}

}  // namespace

extern "C" {

int hx_influence_apply(int npix, int nact, const int* row_ptr, const int* col_idx, const void* vals, int dtype,
                       int nvec, const void* actuators, void* surface, void* stream) {
    HX_CHECK_ARG(npix > 0 && nact > 0 && nvec > 0, "hx_influence_apply: sizes must be positive");
    HX_CHECK_ARG(row_ptr && col_idx && vals && actuators && surface, "hx_influence_apply: NULL pointer");
    HX_CHECK_ARG(dtype == HX_F32 || dtype == HX_F64, "hx_influence_apply: dtype must be HX_F32 or HX_F64");
    HX_CHECK_ARG(nvec <= 65535 * VC, "hx_influence_apply: too many command vectors (%d)", nvec);
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    dim3 grid(hx::ceil_div(npix, 256), hx::ceil_div(nvec, VC));
    cudaStream_t st = (cudaStream_t)stream;
    const double esz = dtype == HX_F32 ? 4.0 : 8.0;
    hx::TraceScope trace(HX_TRACE_DM, esz * ((double)nvec * (npix + nact)) + 4.0 * (npix + 1), st);
    if (dtype == HX_F32)
        influence_apply_kernel<float><<<grid, 256, 0, st>>>(npix, nact, row_ptr, col_idx, (const float*)vals, nvec,
                                                            (const float*)actuators, (float*)surface);
    else
        influence_apply_kernel<double><<<grid, 256, 0, st>>>(npix, nact, row_ptr, col_idx, (const double*)vals,
                                                             nvec, (const double*)actuators, (double*)surface);
    return hx::launch_status("influence_apply_kernel");
}

int hx_influence_apply_transpose(int npix, int nact, const int* col_ptr, const int* row_idx, const void* vals,
                                 int dtype, int nvec, const void* g_surface, void* g_actuators, void* stream) {
    HX_CHECK_ARG(npix > 0 && nact > 0 && nvec > 0, "hx_influence_apply_transpose: sizes must be positive");
    HX_CHECK_ARG(col_ptr && row_idx && vals && g_surface && g_actuators, "hx_influence_apply_transpose: NULL pointer");
    HX_CHECK_ARG(dtype == HX_F32 || dtype == HX_F64, "hx_influence_apply_transpose: dtype must be HX_F32 or HX_F64");
    HX_CHECK_ARG(nact <= 2147483647 && nvec <= 65535 * VC, "hx_influence_apply_transpose: grid too large");
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    dim3 grid(nact, hx::ceil_div(nvec, VC));
    cudaStream_t st = (cudaStream_t)stream;
    const double esz = dtype == HX_F32 ? 4.0 : 8.0;
    hx::TraceScope trace(HX_TRACE_DM, esz * ((double)nvec * (npix + nact)) + 4.0 * (nact + 1), st);
    if (dtype == HX_F32)
        influence_transpose_kernel<float><<<grid, 256, 0, st>>>(npix, nact, col_ptr, row_idx, (const float*)vals,
                                                                nvec, (const float*)g_surface, (float*)g_actuators);
    else
        influence_transpose_kernel<double><<<grid, 256, 0, st>>>(npix, nact, col_ptr, row_idx, (const double*)vals,
                                                                 nvec, (const double*)g_surface,
                                                                 (double*)g_actuators);
    return hx::launch_status("influence_transpose_kernel");
}

int hx_phase_apply(long long n, int batch, int batch_e, int batch_s, const void* e, int dtype, const void* s,
                   double scale, void* out, void* stream) {
    HX_CHECK_ARG(n > 0 && batch > 0 && batch_e > 0 && batch_s > 0, "hx_phase_apply: sizes must be positive");
    HX_CHECK_ARG((batch_e == 1 || batch_e == batch) && (batch_s == 1 || batch_s == batch),
                 "hx_phase_apply: field and screen batches must be 1 or %d", batch);
    HX_CHECK_ARG(e && s && out, "hx_phase_apply: NULL pointer");
    HX_CHECK_ARG(dtype == HX_C64 || dtype == HX_C128, "hx_phase_apply: dtype must be HX_C64 or HX_C128");
    HX_CHECK_ARG(batch <= 65535, "hx_phase_apply: batch too large (%d)", batch);
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    dim3 grid(hx::ceil_div(n, 256), batch);
    cudaStream_t st = (cudaStream_t)stream;
    const double csz = dtype == HX_C64 ? 8.0 : 16.0;
    hx::TraceScope trace(HX_TRACE_DM, (double)n * (csz * (batch_e + batch) + csz / 2 * batch_s), st);
    if (dtype == HX_C64)
        phase_apply_kernel<float><<<grid, 256, 0, st>>>(n, batch, batch_e, batch_s, (const float2*)e, (const float*)s,
                                                        (float)scale, (float2*)out);
    else
        phase_apply_kernel<double><<<grid, 256, 0, st>>>(n, batch, batch_e, batch_s, (const double2*)e,
                                                         (const double*)s, scale, (double2*)out);
    return hx::launch_status("phase_apply_kernel");
}

int hx_phase_apply_grad(long long n, int batch, int batch_e, int batch_s, const void* e, int dtype, const void* s,
                        double scale, const void* g_out, void* g_s, void* g_e, void* stream) {
    HX_CHECK_ARG(n > 0 && batch > 0 && batch_e > 0 && batch_s > 0, "hx_phase_apply_grad: sizes must be positive");
    HX_CHECK_ARG((batch_e == 1 || batch_e == batch) && (batch_s == 1 || batch_s == batch),
                 "hx_phase_apply_grad: field and screen batches must be 1 or %d", batch);
    HX_CHECK_ARG(e && s && g_out && (g_s || g_e), "hx_phase_apply_grad: NULL pointer");
    HX_CHECK_ARG(dtype == HX_C64 || dtype == HX_C128, "hx_phase_apply_grad: dtype must be HX_C64 or HX_C128");
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    dim3 grid(hx::ceil_div(n, 256));
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == HX_C64)
        phase_grad_kernel<float><<<grid, 256, 0, st>>>(n, batch, batch_e, batch_s, (const float2*)e, (const float*)s,
                                                       (float)scale, (const float2*)g_out, (float*)g_s, (float2*)g_e);
    else
        phase_grad_kernel<double><<<grid, 256, 0, st>>>(n, batch, batch_e, batch_s, (const double2*)e,
                                                        (const double*)s, scale, (const double2*)g_out,
                                                        (double*)g_s, (double2*)g_e);
    return hx::launch_status("phase_grad_kernel");
}

}  // extern "C"
