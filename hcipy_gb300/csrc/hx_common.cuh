// Shared helpers of the hcipy_gb300 CUDA library: status codes, error text,
// launch accounting and small complex-arithmetic utilities.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <cstdio>
#include <cstring>

#include "../../include/hcipy_gb300.h"

namespace hx {

// Records the message of the last failure on this host thread (read back by hx_last_error()).
void set_error(const char* fmt, ...);

// Counts every kernel this library launches (hx_launch_count()).
void count_launch(int n = 1);

// Host-side fault injection: when HX_FAULT names `site` ("alloc", "plan" or
// "launch"), the entry point returns HX_ERR_INJECTED before touching the GPU.
bool fault_injected(const char* site);

// Kernel timing (hx_trace_enable): a scope records a CUDA event on `stream` when it opens and another when it
// closes, so a launch issued inside the scope is timed on its own stream.  Free when tracing is off.
bool trace_on();
int trace_begin(int kind, double work, cudaStream_t stream);
void trace_end(int record, cudaStream_t stream);
struct TraceScope {
    int record = -1;
    cudaStream_t stream;
    TraceScope(int kind, double work, cudaStream_t st, bool enabled = true) : stream(st) {
        if (enabled && trace_on()) record = trace_begin(kind, work, st);
    }
    ~TraceScope() {
        if (record >= 0) trace_end(record, stream);
    }
};

inline int cuda_status(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return HX_OK;
    set_error("%s: %s", what, cudaGetErrorString(e));
    return HX_ERR_CUDA;
}

// Checks the launch that was just issued.
inline int launch_status(const char* what) {
    count_launch();
    return cuda_status(cudaGetLastError(), what);
}

inline unsigned ceil_div(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

// SMs of the current device (cached per device).
inline int num_sms() {
    static int cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
    if (cache[dev] == 0) {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        cache[dev] = n > 0 ? n : 148;
    }
    return cache[dev];
}

template <typename T> struct cplx;
template <> struct cplx<float> { using type = float2; };
template <> struct cplx<double> { using type = double2; };

template <typename T> __host__ __device__ inline typename cplx<T>::type make_c(T re, T im);
template <> __host__ __device__ inline float2 make_c<float>(float re, float im) { return make_float2(re, im); }
template <> __host__ __device__ inline double2 make_c<double>(double re, double im) { return make_double2(re, im); }

template <typename C> __host__ __device__ inline C cmul(C a, C b) {
    C r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}

// x exp(i ph) for a complex64 value with the products and sums rounded one by one (no contraction into FMAs),
// so that every kernel that applies a phase screen to complex64 fields gives the same bits.
__device__ __forceinline__ float2 phase_rotate(float2 x, float ph) {
    float sn, cs;
    sincosf(ph, &sn, &cs);
    return make_float2(__fsub_rn(__fmul_rn(x.x, cs), __fmul_rn(x.y, sn)),
                       __fadd_rn(__fmul_rn(x.x, sn), __fmul_rn(x.y, cs)));
}

}  // namespace hx

#define HX_TRY(expr)                  \
    do {                              \
        int _hx_rc = (expr);          \
        if (_hx_rc != HX_OK) return _hx_rc; \
    } while (0)

#define HX_CHECK_ARG(cond, ...)                 \
    do {                                        \
        if (!(cond)) {                          \
            hx::set_error(__VA_ARGS__);         \
            return HX_ERR_INVALID;              \
        }                                       \
    } while (0)
