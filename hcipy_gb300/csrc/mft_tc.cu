// Split-operand tensor-core form of the matrix Fourier transform on tcgen05 (sm_103a): plans (the sliced phase
// matrices), the slicing kernels, tile choice and autotuner, the Lyot chain with its row passes, and the
// compensated dark-hole intensity sums.  The GEMM kernel and the numerics of the split form are described in
// split_gemm.cuh; split_gemm_bn*.cu instantiate it per tile width.
#include "hx_common.cuh"
#include "mft_tc.cuh"
#include "split_gemm.cuh"
#include "tc_ptx.cuh"

#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <atomic>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

namespace hx {
using namespace sg;
namespace {

// ---- slicing (FP32 only) ------------------------------------------------------------------------------

// Power of two strictly above the largest magnitude of a row/column (1 for zero rows).
__device__ __forceinline__ float pow2_above(float mx) {
    if (!(mx > 0.0f) || !isfinite(mx)) return 1.0f;
    int e;
    frexpf(mx, &e);  // mx = f 2^e, f in [0.5, 1)
    return ldexpf(1.0f, e);
}

// hi + lo scaled into [-1, 1) -> a0 + 2^-11 a1 + 2^-22 a2 (times 2^-6); every step is exact except the
// single addition of the scaled low word, whose rounding is below 2^-31 of the scale.
__device__ __forceinline__ void slice3(ff x, float inv, __half& h0, __half& h1, __half& h2) {
    const float th = x.hi * inv * 64.0f;
    const float tl = x.lo * inv * 64.0f;
    const float a0 = rintf(th);
    const float r = __fadd_rn(__fsub_rn(th, a0), tl) * 2048.0f;
    const float a1 = rintf(r);
    const float a2 = rintf(__fsub_rn(r, a1) * 2048.0f);
    h0 = __float2half_rn(a0);
    h1 = __float2half_rn(a1);
    h2 = __float2half_rn(a2);
}

// One CTA per complex row m of X (M x K, row stride ld): writes the Cr and Ci rows of A' (EMB = 0), or the one
// row [Re | Im] of A (EMB = 1).
template <int EMB>
__global__ void slice_rows_kernel(FieldIO src, long long ld, int K, int Kp, const unsigned int* rowmax,
                                  __half* planes, long long plane_stride, int kpitch, float* scale_out) {
    const int m = blockIdx.x;
    __shared__ float red[32];
    __shared__ float s_scale;
    float mx = 0.0f;
    if (rowmax) {
        mx = __uint_as_float(rowmax[m]);
    } else {
        for (int k0 = 4 * threadIdx.x; k0 < K; k0 += 4 * blockDim.x) {
            cff v[4];
            if (k0 + 4 <= K) {
                load4_field(src, (long long)m * ld + k0, v);
            } else {
#pragma unroll
                for (int j = 0; j < 4; ++j) v[j] = k0 + j < K ? load_field(src, (long long)m * ld + k0 + j) : cff{};
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) mx = fmaxf(mx, fmaxf(fabsf(v[j].re.hi), fabsf(v[j].im.hi)));
        }
        for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
        __syncthreads();
        if (threadIdx.x < 32) {
            mx = threadIdx.x < (int)(blockDim.x >> 5) ? red[threadIdx.x] : 0.0f;
            for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        }
    }
    if (threadIdx.x == 0) {
        s_scale = pow2_above(mx);
        scale_out[m] = s_scale;
    }
    __syncthreads();
    const float inv = 1.0f / s_scale;
    const long long r_cr = EMB ? (long long)m : (long long)(m / 64) * 128 + (m % 64);
    const long long r_ci = r_cr + 64;
    // Four consecutive K-elements per thread: 8-byte stores into each plane (Kp and kpitch are multiples of 32).
    for (int k0 = 4 * threadIdx.x; k0 < Kp; k0 += 4 * blockDim.x) {
        __half rs[3][4], is[3][4];
        cff v[4];
        if (k0 + 4 <= K) {
            load4_field(src, (long long)m * ld + k0, v);
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) v[j] = k0 + j < K ? load_field(src, (long long)m * ld + k0 + j) : cff{};
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            slice3(v[j].re, inv, rs[0][j], rs[1][j], rs[2][j]);
            slice3(v[j].im, inv, is[0][j], is[1][j], is[2][j]);
        }
#pragma unroll
        for (int p = 0; p < 3; ++p) {
            __half* pl = planes + p * plane_stride;
            __half2 re01 = __halves2half2(rs[p][0], rs[p][1]), re23 = __halves2half2(rs[p][2], rs[p][3]);
            __half2 im01 = __halves2half2(is[p][0], is[p][1]), im23 = __halves2half2(is[p][2], is[p][3]);
            __half2 ni01 = __hneg2(im01), ni23 = __hneg2(im23);
            *reinterpret_cast<uint2*>(pl + r_cr * kpitch + k0) =
                make_uint2(*reinterpret_cast<uint32_t*>(&re01), *reinterpret_cast<uint32_t*>(&re23));
            if (EMB) {
                *reinterpret_cast<uint2*>(pl + r_cr * kpitch + Kp + k0) =
                    make_uint2(*reinterpret_cast<uint32_t*>(&im01), *reinterpret_cast<uint32_t*>(&im23));
                continue;
            }
            *reinterpret_cast<uint2*>(pl + r_cr * kpitch + Kp + k0) =
                make_uint2(*reinterpret_cast<uint32_t*>(&ni01), *reinterpret_cast<uint32_t*>(&ni23));
            *reinterpret_cast<uint2*>(pl + r_ci * kpitch + k0) =
                make_uint2(*reinterpret_cast<uint32_t*>(&im01), *reinterpret_cast<uint32_t*>(&im23));
            *reinterpret_cast<uint2*>(pl + r_ci * kpitch + Kp + k0) =
                make_uint2(*reinterpret_cast<uint32_t*>(&re01), *reinterpret_cast<uint32_t*>(&re23));
        }
    }
}

// slice_rows_kernel<1> for a row whose maximum is not known yet and that fits in registers (Kp <= 1024 G): the
// CTA reads the row once into registers (G groups of four consecutive points per thread), takes its maximum and
// slices from the registers, where slice_rows_kernel reads the row twice.  Same slices, same scales.
// PHASE: the row is a complex64 field times exp(i scale screen) (a phase screen of screen_rows x K values shared by
// the stacked fields), applied here as hx::phase_rotate does, so the phase-screened field is never stored.
template <int G, bool PHASE>
__global__ void __launch_bounds__(256) slice_rows_reg_kernel(FieldIO src, long long ld, int K, int Kp, __half* planes,
                                                             long long plane_stride, int kpitch, float* scale_out,
                                                             const float* __restrict__ screen, int screen_rows,
                                                             float phase_scale) {
    const long long m = blockIdx.x;
    __shared__ float red[8];
    __shared__ float s_scale;
    cff v[G][4];
    float mx = 0.0f;
#pragma unroll
    for (int gi = 0; gi < G; ++gi) {
        const int k0 = 4 * ((int)threadIdx.x + gi * 256);
        if constexpr (PHASE) {
            const float* srow = screen + (m % screen_rows) * (long long)K;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                cff x = {};
                if (k0 + j < K) {
                    const float2 e = hx::phase_rotate(src.c64[m * ld + k0 + j], __fmul_rn(phase_scale, srow[k0 + j]));
                    x = {{e.x, 0.0f}, {e.y, 0.0f}};
                }
                v[gi][j] = x;
            }
        } else if (k0 + 4 <= K) {
            load4_field(src, m * ld + k0, v[gi]);
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) v[gi][j] = k0 + j < K ? load_field(src, m * ld + k0 + j) : cff{};
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) mx = fmaxf(mx, fmaxf(fabsf(v[gi][j].re.hi), fabsf(v[gi][j].im.hi)));
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < 8; ++i) mx = fmaxf(mx, red[i]);
        s_scale = pow2_above(mx);
        scale_out[m] = s_scale;
    }
    __syncthreads();
    const float inv = 1.0f / s_scale;
#pragma unroll
    for (int gi = 0; gi < G; ++gi) {
        const int k0 = 4 * ((int)threadIdx.x + gi * 256);
        if (k0 >= Kp) continue;
        __half rs[3][4], is[3][4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            slice3(v[gi][j].re, inv, rs[0][j], rs[1][j], rs[2][j]);
            slice3(v[gi][j].im, inv, is[0][j], is[1][j], is[2][j]);
        }
#pragma unroll
        for (int p = 0; p < 3; ++p) {
            __half* pl = planes + p * plane_stride + m * kpitch;
            __half2 re01 = __halves2half2(rs[p][0], rs[p][1]), re23 = __halves2half2(rs[p][2], rs[p][3]);
            __half2 im01 = __halves2half2(is[p][0], is[p][1]), im23 = __halves2half2(is[p][2], is[p][3]);
            *reinterpret_cast<uint2*>(pl + k0) =
                make_uint2(*reinterpret_cast<uint32_t*>(&re01), *reinterpret_cast<uint32_t*>(&re23));
            *reinterpret_cast<uint2*>(pl + Kp + k0) =
                make_uint2(*reinterpret_cast<uint32_t*>(&im01), *reinterpret_cast<uint32_t*>(&im23));
        }
    }
}

// Column maxima max(|Re|, |Im|) of per-field K x N matrices (fields along grid z), as float bits.
__global__ void colmax_kernel(FieldIO src, int K, int N, long long field_stride, unsigned int* colmax,
                              long long colmax_stride) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const int z = blockIdx.z;
    if (n >= N) return;
    const int k0 = blockIdx.y * 64;
    const int k1 = min(K, k0 + 64);
    float mx = 0.0f;
    for (int k = k0; k < k1; ++k) {
        const cff v = load_field(src, z * field_stride + (long long)k * N + n);
        mx = fmaxf(mx, fmaxf(fabsf(v.re.hi), fabsf(v.im.hi)));
    }
    atomicMax(&colmax[z * colmax_stride + n], __float_as_uint(mx));
}

// Per-field K x N matrix Y -> B' rows (z*n_rows_per_field + n): [slices of Re Y[:, n] | slices of Im Y[:, n]].
// emb (plan-time phase matrices that carry the embedding, see the file comment): two rows per column n, in
// blocks of 8 columns, row (n/8)*16 + n%8 = [Re | -Im] and row (n/8)*16 + 8 + n%8 = [Im | Re].
__global__ void slice_cols_kernel(FieldIO src, int K, int N, int Kp, long long field_stride,
                                  const unsigned int* colmax, long long colmax_stride, __half* planes,
                                  long long plane_stride, int kpitch, int n_rows_per_field, float* scale_out,
                                  int emb) {
    __shared__ ff tr[32][33], ti[32][33];
    __shared__ float sc[32];
    const int n0 = blockIdx.x * 32, k0 = blockIdx.y * 32, z = blockIdx.z;
    const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
    if (ty == 0) {
        const int n = n0 + tx;
        const float mx = n < N ? __uint_as_float(colmax[z * colmax_stride + n]) : 0.0f;
        sc[tx] = pow2_above(mx);
        if (k0 == 0 && n < N) scale_out[(long long)z * n_rows_per_field + n] = sc[tx];
    }
    for (int r = ty; r < 32; r += 8) {
        const int k = k0 + r, n = n0 + tx;
        cff v = {{0.0f, 0.0f}, {0.0f, 0.0f}};
        if (k < K && n < N) v = load_field(src, z * field_stride + (long long)k * N + n);
        tr[r][tx] = v.re;
        ti[r][tx] = v.im;
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
        const int n = n0 + r, k = k0 + tx;
        if (n >= N || k >= Kp) continue;
        const float inv = 1.0f / sc[r];
        __half r0, r1, r2, i0, i1, i2;
        slice3(tr[tx][r], inv, r0, r1, r2);
        slice3(ti[tx][r], inv, i0, i1, i2);
        const __half rs[3] = {r0, r1, r2};
        const __half is[3] = {i0, i1, i2};
        if (emb) {
            const long long row = (long long)z * n_rows_per_field + (n >> 3) * 16 + (n & 7);
#pragma unroll
            for (int p = 0; p < 3; ++p) {
                __half* pl = planes + p * plane_stride;
                pl[row * kpitch + k] = rs[p];
                pl[row * kpitch + Kp + k] = __hneg(is[p]);
                pl[(row + 8) * kpitch + k] = is[p];
                pl[(row + 8) * kpitch + Kp + k] = rs[p];
            }
            continue;
        }
        const long long row = (long long)z * n_rows_per_field + n;
#pragma unroll
        for (int p = 0; p < 3; ++p) {
            __half* pl = planes + p * plane_stride;
            pl[row * kpitch + k] = rs[p];
            pl[row * kpitch + Kp + k] = is[p];
        }
    }
}

// Phase matrix as float-float planes: M[r, c] = wr[r] wc[c] exp(sign i a[r] b[c]), evaluated in float64
// once per plan.
__global__ void phase_planes_kernel(int rows, int cols, const double* a, const double* b, double sign,
                                    const double* wr, const double* wc, float* re_hi, float* re_lo, float* im_hi,
                                    float* im_lo) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)rows * cols) return;
    const int r = (int)(idx / cols), c = (int)(idx % cols);
    double s, co;
    sincos(a[r] * b[c], &s, &co);
    double w = 1.0;
    if (wr) w *= wr[r];
    if (wc) w *= wc[c];
    const double re = w * co, im = w * sign * s;
    re_hi[idx] = (float)re;
    re_lo[idx] = (float)(re - (double)(float)re);
    im_hi[idx] = (float)im;
    im_lo[idx] = (float)(im - (double)(float)im);
}

// Copy between field formats (float-float planes -> complex64 / complex128), two elements per thread.
__global__ void field_copy_kernel(FieldIO src, FieldIO dst, long long n) {
    const long long i = 2 * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
    if (i + 1 < n) {
        const cff a = load_field(src, i), b = load_field(src, i + 1);
        store_field(dst, i, a);
        store_field(dst, i + 1, b);
    } else if (i < n) {
        store_field(dst, i, load_field(src, i));
    }
}

// L = S (E - alpha T) for one row per CTA, T the inverse transform of the focal-plane field in float-float: the
// Babinet subtraction and the Lyot stop of the coronagraph (hcipy/coronagraphy/lyot.py:79-90) as a pass of its
// own.  In the GEMM's epilogue the same arithmetic ran on the epilogue warps of one CTA per SM while the tensor
// cores idled; here it runs at full occupancy and streams the fields once.  rowmax (optional): the row maximum
// of max(|Re|, |Im|) as float bits, for the slicing of the next transform.
template <int SRC, int OUT>
__global__ void babinet_rows_kernel(FieldIO t, FieldIO src, const float2* __restrict__ stop, cff alpha, int ny, int nx,
                                    FieldIO out, unsigned int* rowmax) {
    const long long row = blockIdx.x;
    const long long base = row * nx;
    const float2* srow = stop ? stop + (row % ny) * nx : nullptr;
    const bool real_alpha = alpha.im.hi == 0.0f && alpha.im.lo == 0.0f;
    const bool imag_alpha = alpha.re.hi == 0.0f && alpha.re.lo == 0.0f;
    float mx = 0.0f;
    // U columns per thread per round, all loads issued before the arithmetic
    constexpr int U = 4;
    for (int c0 = threadIdx.x; c0 < nx; c0 += U * blockDim.x) {
        cff v[U], e[U];
        float2 mk[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int c = c0 + u * blockDim.x;
            if (c < nx) {
                v[u] = load_fmt<FMT_FF>(t, base + c);
                e[u] = load_fmt<SRC>(src, base + c);
                mk[u] = srow ? __ldg(&srow[c]) : make_float2(1.0f, 0.0f);
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int c = c0 + u * blockDim.x;
            if (c >= nx) continue;
            cff w = real_alpha   ? cff{ff_mul(v[u].re, alpha.re), ff_mul(v[u].im, alpha.re)}
                    : imag_alpha ? cff{ff_neg(ff_mul(v[u].im, alpha.im)), ff_mul(v[u].re, alpha.im)}
                                 : cff_mul(v[u], alpha);
            w = {ff_add(e[u].re, ff_neg(w.re)), ff_add(e[u].im, ff_neg(w.im))};
            if (srow) w = mk[u].y == 0.0f ? cff{ff_mulf(w.re, mk[u].x), ff_mulf(w.im, mk[u].x)} : cff_mul_c64(w, mk[u]);
            store_fmt<OUT>(out, base + c, w);
            mx = fmaxf(mx, fmaxf(fabsf(w.re.hi), fabsf(w.im.hi)));
        }
    }
    if (!rowmax) return;
    __shared__ float red[32];
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) mx = fmaxf(mx, red[w]);
        rowmax[row] = __float_as_uint(mx);
    }
}

// The same row pass when the Lyot plane only feeds the image transform: the CTA keeps its row in registers (G
// groups of four consecutive points per thread, Kp <= 1024 G), takes the row maximum, and writes the three fp16
// slice planes of the row ([Re | Im], zero-padded to Kp) and its scale straight into the image transform's first
// GEMM operand.  The slices are those slice_rows_kernel<1> makes from the float-float row with that maximum, so
// the result is unchanged; the float-float Lyot plane is neither written nor read back.
template <int SRC, int G>
__global__ void __launch_bounds__(256) babinet_slice_rows_kernel(FieldIO t, FieldIO src, const float2* __restrict__ stop,
                                                                 cff alpha, int ny, int nx, int Kp, __half* planes,
                                                                 long long plane_stride, int kpitch, float* scale_out) {
    const long long row = blockIdx.x;
    const long long base = row * nx;
    const float2* srow = stop ? stop + (row % ny) * nx : nullptr;
    const bool real_alpha = alpha.im.hi == 0.0f && alpha.im.lo == 0.0f;
    const bool imag_alpha = alpha.re.hi == 0.0f && alpha.re.lo == 0.0f;
    __shared__ float red[8];
    __shared__ float s_scale;
    cff w[G][4];
    float mx = 0.0f;
#pragma unroll
    for (int gi = 0; gi < G; ++gi) {
        const int k0 = 4 * ((int)threadIdx.x + gi * 256);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int c = k0 + j;
            cff x = {};
            if (c < nx) {
                const cff v = load_fmt<FMT_FF>(t, base + c);
                const cff e = load_fmt<SRC>(src, base + c);
                x = real_alpha   ? cff{ff_mul(v.re, alpha.re), ff_mul(v.im, alpha.re)}
                    : imag_alpha ? cff{ff_neg(ff_mul(v.im, alpha.im)), ff_mul(v.re, alpha.im)}
                                 : cff_mul(v, alpha);
                x = {ff_add(e.re, ff_neg(x.re)), ff_add(e.im, ff_neg(x.im))};
                if (srow) {
                    const float2 mk = __ldg(&srow[c]);
                    x = mk.y == 0.0f ? cff{ff_mulf(x.re, mk.x), ff_mulf(x.im, mk.x)} : cff_mul_c64(x, mk);
                }
                mx = fmaxf(mx, fmaxf(fabsf(x.re.hi), fabsf(x.im.hi)));
            }
            w[gi][j] = x;
        }
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < 8; ++i) mx = fmaxf(mx, red[i]);
        s_scale = pow2_above(mx);
        scale_out[row] = s_scale;
    }
    __syncthreads();
    const float inv = 1.0f / s_scale;
#pragma unroll
    for (int gi = 0; gi < G; ++gi) {
        const int k0 = 4 * ((int)threadIdx.x + gi * 256);
        if (k0 >= Kp) continue;
        __half rs[3][4], is[3][4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            slice3(w[gi][j].re, inv, rs[0][j], rs[1][j], rs[2][j]);
            slice3(w[gi][j].im, inv, is[0][j], is[1][j], is[2][j]);
        }
#pragma unroll
        for (int p = 0; p < 3; ++p) {
            __half* pl = planes + p * plane_stride + row * kpitch;
            __half2 re01 = __halves2half2(rs[p][0], rs[p][1]), re23 = __halves2half2(rs[p][2], rs[p][3]);
            __half2 im01 = __halves2half2(is[p][0], is[p][1]), im23 = __halves2half2(is[p][2], is[p][3]);
            *reinterpret_cast<uint2*>(pl + k0) =
                make_uint2(*reinterpret_cast<uint32_t*>(&re01), *reinterpret_cast<uint32_t*>(&re23));
            *reinterpret_cast<uint2*>(pl + Kp + k0) =
                make_uint2(*reinterpret_cast<uint32_t*>(&im01), *reinterpret_cast<uint32_t*>(&im23));
        }
    }
}

template <int SRC>
int launch_babinet_src(FieldIO t, FieldIO src, const float2* stop, cff alpha, long long rows, int ny, int nx,
                       FieldIO out, int out_fmt, unsigned int* rowmax, cudaStream_t st) {
    if (rows > 2147483647LL) {
        set_error("Lyot plane too large");
        return HX_ERR_UNSUPPORTED;
    }
    const dim3 grid((unsigned)rows);
    if (out_fmt == FMT_FF) babinet_rows_kernel<SRC, FMT_FF><<<grid, 256, 0, st>>>(t, src, stop, alpha, ny, nx, out, rowmax);
    else if (out_fmt == FMT_C128)
        babinet_rows_kernel<SRC, FMT_C128><<<grid, 256, 0, st>>>(t, src, stop, alpha, ny, nx, out, rowmax);
    else babinet_rows_kernel<SRC, FMT_C64><<<grid, 256, 0, st>>>(t, src, stop, alpha, ny, nx, out, rowmax);
    return launch_status("babinet_rows_kernel");
}

// ---- host side ------------------------------------------------------------------------------------

inline long long round_up(long long x, long long m) { return (x + m - 1) / m * m; }

PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, []() {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// A sliced operand in global memory: three fp16 planes of rows x kpitch (K-major) and one scale per logical row.
struct SliceMat {
    __half* planes = nullptr;
    float* scale = nullptr;
    long long rows = 0;
    int kpitch = 0;
    int Kp = 0;
    long long plane_stride() const { return rows * kpitch; }
    size_t plane_bytes() const { return 3 * (size_t)rows * kpitch * sizeof(__half); }
};

int encode_map(CUtensorMap* map, const SliceMat& s, int box_rows) {
    auto enc = get_encode();
    if (!enc) {
        set_error("cuTensorMapEncodeTiled is not available from the driver");
        return HX_ERR_UNSUPPORTED;
    }
    cuuint64_t dims[3] = {(cuuint64_t)s.kpitch, (cuuint64_t)s.rows, 3};
    cuuint64_t strides[2] = {(cuuint64_t)s.kpitch * 2, (cuuint64_t)s.rows * s.kpitch * 2};
    cuuint32_t box[3] = {BK, (cuuint32_t)box_rows, 3};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, s.planes, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (%d) for %lld rows x %d", (int)r, s.rows, s.kpitch);
        return HX_ERR_CUDA;
    }
    return HX_OK;
}

// Carves 256-byte aligned pieces out of a workspace (or, with base == nullptr, only counts bytes).
struct Carver {
    uint8_t* base;
    size_t off = 0;
    explicit Carver(void* b) : base((uint8_t*)b) {}
    void* take(size_t bytes) {
        off = (size_t)round_up((long long)off, 256);
        void* p = base ? base + off : nullptr;
        off += bytes;
        return p;
    }
};

void carve_slices(Carver& c, SliceMat& s, long long rows, int K, long long scales) {
    s.Kp = (int)round_up(K, 32);
    s.kpitch = 2 * s.Kp;
    s.rows = rows;
    s.planes = (__half*)c.take(s.plane_bytes());
    s.scale = (float*)c.take(sizeof(float) * scales);
}

FieldIO carve_ff(Carver& c, long long n) {
    FieldIO f;
    f.re_hi = (float*)c.take(sizeof(float) * n);
    f.re_lo = (float*)c.take(sizeof(float) * n);
    f.im_hi = (float*)c.take(sizeof(float) * n);
    f.im_lo = (float*)c.take(sizeof(float) * n);
    return f;
}

// phase (optional, emb rows of a complex64 field only): the rows are the field times exp(i phase->scale screen).
struct RowPhase {
    const float* screen;
    int rows;
    float scale;
};

int launch_slice_rows(const FieldIO& src, long long ld, long long M, int K, const unsigned int* rowmax,
                      SliceMat& s, cudaStream_t st, bool emb = false, const RowPhase* phase = nullptr) {
    if (M > 2147483647LL) return HX_ERR_UNSUPPORTED;
    if (phase && (!emb || rowmax || s.Kp > 4096 || !src.c64 || src.c128 || src.re_hi)) {
        set_error("a phase screen is applied only while slicing complex64 rows of at most 4096 points");
        return HX_ERR_UNSUPPORTED;
    }
    if (emb && !rowmax && s.Kp <= 4096) {
        const unsigned grid = (unsigned)M;
        const long long ps = s.plane_stride();
        const float* scr = phase ? phase->screen : nullptr;
        const int sr = phase ? phase->rows : 1;
        const float sc = phase ? phase->scale : 0.0f;
        auto run = [&](auto g_tag, auto p_tag) {
            constexpr int G = decltype(g_tag)::value;
            constexpr bool P = decltype(p_tag)::value;
            slice_rows_reg_kernel<G, P><<<grid, 256, 0, st>>>(src, ld, K, s.Kp, s.planes, ps, s.kpitch, s.scale, scr,
                                                              sr, sc);
        };
        auto by_g = [&](auto p_tag) {
            switch ((s.Kp + 1023) / 1024) {
                case 1: run(std::integral_constant<int, 1>(), p_tag); break;
                case 2: run(std::integral_constant<int, 2>(), p_tag); break;
                case 3: run(std::integral_constant<int, 3>(), p_tag); break;
                default: run(std::integral_constant<int, 4>(), p_tag);
            }
        };
        if (phase) by_g(std::true_type());
        else by_g(std::false_type());
        return launch_status("slice_rows_reg_kernel");
    }
    if (emb)
        slice_rows_kernel<1><<<(unsigned)M, 256, 0, st>>>(src, ld, K, s.Kp, rowmax, s.planes, s.plane_stride(),
                                                          s.kpitch, s.scale);
    else
        slice_rows_kernel<0><<<(unsigned)M, 256, 0, st>>>(src, ld, K, s.Kp, rowmax, s.planes, s.plane_stride(),
                                                          s.kpitch, s.scale);
    return launch_status("slice_rows_kernel");
}

int launch_colmax(const FieldIO& src, int K, int N, int fields, long long field_stride, unsigned int* colmax,
                  long long colmax_stride, cudaStream_t st) {
    dim3 grid(ceil_div(N, 128), ceil_div(K, 64), fields);
    colmax_kernel<<<grid, 128, 0, st>>>(src, K, N, field_stride, colmax, colmax_stride);
    return launch_status("colmax_kernel");
}

int launch_slice_cols(const FieldIO& src, int K, int N, int fields, long long field_stride,
                      const unsigned int* colmax, long long colmax_stride, SliceMat& s, int n_rows_per_field,
                      cudaStream_t st, bool emb = false) {
    dim3 grid(ceil_div(N, 32), ceil_div(s.Kp, 32), fields);
    slice_cols_kernel<<<grid, dim3(32, 8), 0, st>>>(src, K, N, s.Kp, field_stride, colmax, colmax_stride, s.planes,
                                                    s.plane_stride(), s.kpitch, n_rows_per_field, s.scale,
                                                    emb ? 1 : 0);
    return launch_status("slice_cols_kernel");
}

void set_alpha(GemmArgs& g, double re, double im) {
    g.alpha[0] = (float)re;
    g.alpha[1] = (float)(re - (double)g.alpha[0]);
    g.alpha[2] = (float)im;
    g.alpha[3] = (float)(im - (double)g.alpha[2]);
}

int sm_count() {
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

// Tile width and K split of one GEMM.
struct TileChoice {
    int bn = 128;
    int ksplit = 1;
    int n_tiles = 1;
    long long tiles = 0;  // output tiles over all grid z
    size_t partial_floats() const { return ksplit > 1 ? (size_t)tiles * ksplit * 2 * bn * BM : 0; }
};

void forced_tiles(int* bn, int* ks) {
    static int forced_bn = 0, forced_split = 0;
    static std::once_flag once;
    std::call_once(once, [] {
        const char* e = getenv("HX_SPLIT_TILE");
        int b = 0, k = 0;
        const int n = e ? sscanf(e, "%d,%d", &b, &k) : 0;
        if (n >= 1 && (b == 64 || b == 112 || b == 128)) forced_bn = b;
        if (n == 2 && k >= 1) forced_split = k;
    });
    *bn = forced_bn;
    *ks = forced_split;
}

// HX_SPLIT_CLUSTER=0 turns the cluster reduction of a split K off (tuning and comparisons).
bool clusters_allowed() {
    static int allowed = -1;
    static std::once_flag once;
    std::call_once(once, [] {
        const char* e = getenv("HX_SPLIT_CLUSTER");
        allowed = (e && e[0] == '0') ? 0 : 1;
    });
    return allowed == 1;
}

// A CTA sums at most MAX_SPLIT_KTILES K-steps (its level-0 FP32 sum stays exact), so a longer K is always split
// across CTAs, whose float-float partials the last CTA of the tile adds.
TileChoice make_choice(long long m_tiles, int N, int grid_z, int ktiles, int bn, int ksplit) {
    TileChoice c;
    c.bn = bn;
    c.n_tiles = (int)ceil_div(N, bn);
    c.tiles = m_tiles * c.n_tiles * grid_z;
    const int min_split = (int)ceil_div(ktiles, MAX_SPLIT_KTILES);
    c.ksplit = std::max(min_split, std::max(1, std::min(ksplit, std::max(1, ktiles / 4))));
    return c;
}

// K split that fills the GPU with a given tile count.
int fill_split(long long tiles, int sms) { return tiles < sms ? (int)(sms / tiles) : 1; }

// Candidate tiles of one GEMM: BN 128 and 64, each unsplit and split to fill the GPU.
std::vector<TileChoice> tile_candidates(long long m_tiles, int N, int grid_z, int ktiles) {
    std::vector<TileChoice> v;
    const int sms = sm_count();
    for (int bn : {128, 112, 64}) {
        if (bn > 64 && N <= 64) continue;
        const TileChoice c1 = make_choice(m_tiles, N, grid_z, ktiles, bn, 1);
        v.push_back(c1);
        const TileChoice c2 = make_choice(m_tiles, N, grid_z, ktiles, bn, fill_split(c1.tiles, sms));
        if (c2.ksplit > c1.ksplit) v.push_back(c2);
    }
    return v;
}

// BN = 128 halves the A traffic per product against BN = 64 and is taken when its tiles fill at least 3/4 of
// the SMs.  Smaller GEMMs take BN = 64 and split K so that the grid fills the GPU (at least four K-steps per
// CTA): more CTAs share the epilogue and the last CTA of a tile reads fewer partial bytes.
// HX_SPLIT_TILE="bn[,ksplit]" overrides the choice (tuning); with the autotuner on, a measured choice for the
// same GEMM shape takes precedence (see launch_gemm).
// Under HX_SCHEDULE_THROUGHPUT the GEMM shares the GPU with concurrent ones (other streams or graph branches
// fill the SMs), so no K split is taken (its partial sums and fix-up are extra work once the GPU is full) and the
// wider tile that pads the output columns least is used.
TileChoice choose_tile(long long m_tiles, int N, int grid_z, int ktiles, int schedule) {
    int fbn, fks;
    forced_tiles(&fbn, &fks);
    if (schedule == HX_SCHEDULE_THROUGHPUT && !fbn && !fks) {
        const int bn = N <= 64 ? 64 : (round_up(N, 112) < round_up(N, 128) ? 112 : 128);
        return make_choice(m_tiles, N, grid_z, ktiles, bn, 1);
    }
    const int sms = sm_count();
    const long long tiles128 = m_tiles * (long long)ceil_div(N, 128) * grid_z;
    const int bn = fbn ? fbn : (N > 64 && 4 * tiles128 >= 3LL * sms ? 128 : 64);
    const long long tiles = m_tiles * (long long)ceil_div(N, bn) * grid_z;
    return make_choice(m_tiles, N, grid_z, ktiles, bn, fks ? fks : fill_split(tiles, sms));
}

// ---- autotuner: the fastest candidate per GEMM shape, measured once on the caller's stream -------------

struct GemmShape {
    long long m_tiles;
    int N, grid_z, ktiles, sms, dev, emb;
    bool operator<(const GemmShape& o) const {
        return std::tie(m_tiles, N, grid_z, ktiles, sms, dev, emb) <
               std::tie(o.m_tiles, o.N, o.grid_z, o.ktiles, o.sms, o.dev, o.emb);
    }
};

struct TunedEntry {
    int n = 0;                 // candidates measured
    TileChoice cand[8];
    float ms[8];               // best of two timed launches each
};

// The kept candidate of a measured shape.  Latency: the fastest.  Throughput: the least SM time, the duration
// times the SMs its CTAs occupy (one resident CTA per SM), which is what it takes from concurrent GEMMs.
TileChoice pick_tuned(const TunedEntry& e, int schedule) {
    const int sms = sm_count();
    int best = 0;
    double best_cost = 1e300;
    for (int k = 0; k < e.n; ++k) {
        double cost = e.ms[k];
        if (schedule == HX_SCHEDULE_THROUGHPUT)
            cost *= (double)std::min<long long>(e.cand[k].tiles * e.cand[k].ksplit, (long long)sms);
        if (cost < best_cost) {
            best_cost = cost;
            best = k;
        }
    }
    return e.cand[best];
}

std::atomic<int> g_autotune{0};
std::mutex g_tune_mu;
std::map<GemmShape, TunedEntry> g_tuned;

// One launch with a given tile choice.  partial / counters: split-K workspace (unused when c.ksplit == 1).
int launch_choice(GemmArgs& g, const SliceMat& A, const SliceMat& B, const TileChoice& c, int grid_z,
                  float* partial, unsigned int* counters, double cmacs, bool traced, cudaStream_t st) {
    const long long m_tiles = ceil_div(A.rows, BM);
    if (m_tiles > 65535 || grid_z > 65535 || (long long)c.n_tiles * c.ksplit > 2147483647LL) {
        set_error("split GEMM grid too large");
        return HX_ERR_UNSUPPORTED;
    }
    HX_TRY(encode_map(&g.tmap_a, A, BM));
    HX_TRY(encode_map(&g.tmap_b, B, c.bn));
    g.ktiles = A.kpitch / BK;
    g.ksplit = c.ksplit;
    g.n_tiles = c.n_tiles;
    g.partial = partial;
    g.counters = counters;
    // A split K reduces inside a thread-block cluster when the split allows it (see cluster_ok), else through
    // float-float partials in the workspace that the last CTA of each tile adds.
    g.cluster = c.ksplit > 1 && clusters_allowed() &&
                (c.bn == 64 ? cluster_ok_bn64(c.ksplit) : c.bn == 112 ? cluster_ok_bn112(c.ksplit)
                                                                      : cluster_ok_bn128(c.ksplit));
    if (c.ksplit > 1 && !g.cluster)
        HX_TRY(cuda_status(cudaMemsetAsync(counters, 0, sizeof(unsigned int) * c.tiles, st), "memset counters"));
    dim3 grid((unsigned)(c.n_tiles * c.ksplit), (unsigned)m_tiles, grid_z);
    const int out = output_fmt(g.out);
    const int src = g.epi == HX_EPI_BABINET ? input_fmt(g.src) : FMT_NONE;
    TraceScope trace(HX_TRACE_SPLIT_GEMM, cmacs, st, traced);
    if (c.bn == 64) return launch_bn64(g, grid, out, src, st);
    if (c.bn == 112) return launch_bn112(g, grid, out, src, st);
    return launch_bn128(g, grid, out, src, st);
}

// Times every candidate (one warm-up launch, then the best of two timed launches) with CUDA events on the
// stream and keeps the fastest.  The launches write the same result each time (the epilogue maxima are
// idempotent).
int tune(GemmArgs& g, const SliceMat& A, const SliceMat& B, const GemmShape& key, int grid_z, float* partial,
         unsigned int* counters, cudaStream_t st, TunedEntry* out) {
    const std::vector<TileChoice> cands = tile_candidates(key.m_tiles, key.N, key.grid_z, key.ktiles);
    cudaEvent_t ev[3];
    for (int i = 0; i < 3; ++i) {
        if (cudaEventCreate(&ev[i]) != cudaSuccess) {
            for (int j = 0; j < i; ++j) cudaEventDestroy(ev[j]);
            set_error("autotune: cudaEventCreate failed");
            return HX_ERR_CUDA;
        }
    }
    TunedEntry entry;
    int rc = HX_OK;
    for (const TileChoice& c : cands) {
        if ((rc = launch_choice(g, A, B, c, grid_z, partial, counters, 0.0, false, st)) != HX_OK) break;
        cudaEventRecord(ev[0], st);
        if ((rc = launch_choice(g, A, B, c, grid_z, partial, counters, 0.0, false, st)) != HX_OK) break;
        cudaEventRecord(ev[1], st);
        if ((rc = launch_choice(g, A, B, c, grid_z, partial, counters, 0.0, false, st)) != HX_OK) break;
        cudaEventRecord(ev[2], st);
        if ((rc = cuda_status(cudaEventSynchronize(ev[2]), "autotune sync")) != HX_OK) break;
        float t1 = 0.0f, t2 = 0.0f;
        cudaEventElapsedTime(&t1, ev[0], ev[1]);
        cudaEventElapsedTime(&t2, ev[1], ev[2]);
        const float ms = std::min(t1, t2);
        if (entry.n < 8) {
            entry.cand[entry.n] = c;
            entry.ms[entry.n] = ms;
            ++entry.n;
        }
    }
    for (int i = 0; i < 3; ++i) cudaEventDestroy(ev[i]);
    if (rc != HX_OK) return rc;
    if (entry.n == 0) {
        set_error("autotune: no tile candidate");
        return HX_ERR_INVALID;
    }
    *out = entry;
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tuned[key] = entry;
    return HX_OK;
}

// partial / counters are sized for every candidate (carve_ws), so the autotuner may pick any of them.
int launch_gemm(GemmArgs& g, const SliceMat& A, const SliceMat& B, TileChoice c, int grid_z, float* partial,
                unsigned int* counters, double cmacs, int schedule, cudaStream_t st) {
    if (A.kpitch != B.kpitch) {
        set_error("internal: split GEMM K mismatch (%d vs %d)", A.kpitch, B.kpitch);
        return HX_ERR_INVALID;
    }
    int fbn, fks;
    forced_tiles(&fbn, &fks);
    if (g_autotune.load(std::memory_order_relaxed) && !fbn && !fks) {
        int dev = 0;
        cudaGetDevice(&dev);
        // with the embedding on B, a complex column is two B' rows
        const GemmShape key{ceil_div(A.rows, BM), g.emb ? 2 * g.N : g.N, grid_z, A.kpitch / BK, sm_count(), dev,
                            g.emb};
        bool found = false;
        {
            std::lock_guard<std::mutex> lock(g_tune_mu);
            auto it = g_tuned.find(key);
            if (it != g_tuned.end()) {
                c = pick_tuned(it->second, schedule);
                found = true;
            }
        }
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        cudaStreamIsCapturing(st, &cap);
        if (!found && cap == cudaStreamCaptureStatusNone) {
            TunedEntry entry;
            HX_TRY(tune(g, A, B, key, grid_z, partial, counters, st, &entry));
            c = pick_tuned(entry, schedule);
        }
    }
    return launch_choice(g, A, B, c, grid_z, partial, counters, cmacs, true, st);
}

GemmArgs base_args(int* status) {
    GemmArgs g;
    memset(&g, 0, sizeof(g));
    set_alpha(g, 1.0, 0.0);
    g.rows_per_field = 1;
    g.status = status;
    return g;
}

}  // namespace

// =================================================================================================

struct SplitMftPlan {
    int nx, ny, nu, nv;
    void* mem = nullptr;     // one allocation for all sliced matrices
    SliceMat m2f, m1f;       // forward: B of G1 (rows nu64, K nx), A of G2 (rows 2 nv64, K ny)
    SliceMat m1b, m2b;       // backward: A of G1 (rows 2 ny64, K nv), B of G2 (rows nx64, K nu)
    SliceMat m1a, m2a;       // adjoint (own copies only for non-uniform weights)
    int* status = nullptr;
    int schedule = HX_SCHEDULE_LATENCY;  // tile policy of its GEMMs
};

namespace {

// Slice a phase matrix (rows x cols, evaluated on the device) as an A (row) or B (column) operand; emb: a B operand
// that carries the complex embedding (two rows per column, see the file comment).
int slice_phase(int rows, int cols, const double* a, const double* b, double sign, const double* wr,
                const double* wc, bool as_rows, SliceMat& out, cudaStream_t st, bool emb = false) {
    void* tmp = nullptr;
    const long long n = (long long)rows * cols;
    Carver count(nullptr);
    carve_ff(count, n);
    count.take(sizeof(unsigned int) * round_up(cols, 64));
    int rc = cuda_status(cudaMalloc(&tmp, count.off), "cudaMalloc(phase matrix)");
    if (rc == HX_OK) {
        Carver c(tmp);
        FieldIO f = carve_ff(c, n);
        unsigned int* mx = (unsigned int*)c.take(sizeof(unsigned int) * round_up(cols, 64));
        phase_planes_kernel<<<ceil_div(n, 256), 256, 0, st>>>(rows, cols, a, b, sign, wr, wc, f.re_hi, f.re_lo,
                                                              f.im_hi, f.im_lo);
        rc = launch_status("phase_planes_kernel");
        if (rc == HX_OK) {
            if (as_rows) {
                rc = launch_slice_rows(f, cols, rows, cols, nullptr, out, st);
            } else {
                rc = cuda_status(cudaMemsetAsync(mx, 0, sizeof(unsigned int) * round_up(cols, 64), st), "memset");
                if (rc == HX_OK) rc = launch_colmax(f, rows, cols, 1, 0, mx, 0, st);
                if (rc == HX_OK) rc = launch_slice_cols(f, rows, cols, 1, 0, mx, 0, out, 0, st, emb);
            }
        }
    }
    cudaStreamSynchronize(st);
    cudaFree(tmp);
    return rc;
}

// Workspace of one direction: operand slices, the float-float intermediate, the max arrays and the split-K
// partials (shared by the two GEMMs, which run one after the other on the stream).
struct Ws {
    unsigned int* in_max = nullptr;  // input column maxima (backward only)
    SliceMat s1;                     // sliced input operand of the first GEMM
    FieldIO t;                       // float-float intermediate
    unsigned int* t_max = nullptr;   // its column (forward) or row (backward) maxima
    SliceMat s2;                     // sliced intermediate for the second GEMM
    TileChoice c1, c2;               // tiles of the two GEMMs
    float* partial = nullptr;
    unsigned int* counters = nullptr;
};

// The GEMMs whose A operand is the per-call field (the forward transform's first, the backward transform's
// second) carry the embedding on their constant B operand: the field is sliced once as [Re | Im] rows, and the
// tile logic counts two B' rows per complex output column.
void carve_ws(Carver& c, const SplitMftPlan* p, int direction, int batch, Ws& w) {
    long long g1_rows, g2_rows;
    int g1_n, g1_z, g1_kt, g2_n, g2_z, g2_kt;
    const long long rows = (long long)batch * p->ny;
    const long long nu64 = round_up(p->nu, 64);
    const long long b_rows = round_up(batch * nu64, 128);
    if (direction == HX_FORWARD) {
        carve_slices(c, w.s1, round_up(rows, BM), p->nx, rows);  // rows past the field: discarded tile rows
        w.t = carve_ff(c, rows * p->nu);
        w.t_max = (unsigned int*)c.take(sizeof(unsigned int) * batch * nu64);
        carve_slices(c, w.s2, b_rows, p->ny, b_rows);
        g1_rows = w.s1.rows, g1_n = 2 * p->nu, g1_z = 1, g1_kt = w.s1.kpitch / BK;
        g2_rows = p->m1f.rows, g2_n = p->nu, g2_z = batch, g2_kt = p->m1f.kpitch / BK;
    } else {
        w.in_max = (unsigned int*)c.take(sizeof(unsigned int) * batch * nu64);
        carve_slices(c, w.s1, b_rows, p->nv, b_rows);
        w.t = carve_ff(c, rows * p->nu);
        w.t_max = (unsigned int*)c.take(sizeof(unsigned int) * rows);
        carve_slices(c, w.s2, round_up(rows, BM), p->nu, rows);
        g1_rows = p->m1b.rows, g1_n = p->nu, g1_z = batch, g1_kt = p->m1b.kpitch / BK;
        g2_rows = w.s2.rows, g2_n = 2 * p->nx, g2_z = 1, g2_kt = w.s2.kpitch / BK;
    }
    w.c1 = choose_tile(ceil_div(g1_rows, BM), g1_n, g1_z, g1_kt, p->schedule);
    w.c2 = choose_tile(ceil_div(g2_rows, BM), g2_n, g2_z, g2_kt, p->schedule);
    // split-K workspace for every candidate tile of both GEMMs, so the layout does not depend on the choice
    size_t part = 0;
    long long tiles = 0;
    for (const TileChoice* t : {&w.c1, &w.c2}) {
        const long long m_tiles = t == &w.c1 ? ceil_div(g1_rows, BM) : ceil_div(g2_rows, BM);
        for (const TileChoice& cand : tile_candidates(m_tiles, t == &w.c1 ? g1_n : g2_n, t == &w.c1 ? g1_z : g2_z,
                                                      t == &w.c1 ? g1_kt : g2_kt)) {
            part = std::max(part, cand.partial_floats());
            tiles = std::max(tiles, cand.tiles);
        }
        part = std::max(part, t->partial_floats());
        tiles = std::max(tiles, t->tiles);
    }
    w.partial = (float*)c.take(sizeof(float) * part);
    w.counters = (unsigned int*)c.take(sizeof(unsigned int) * tiles);
}

// The sliced operand of a forward run's first GEMM in workspace ws: the first piece carve_ws takes.
SliceMat forward_input_slices(const SplitMftPlan* p, int batch, void* ws) {
    Carver c(ws);
    SliceMat s;
    const long long rows = (long long)batch * p->ny;
    carve_slices(c, s, round_up(rows, BM), p->nx, rows);
    return s;
}

// in/out: c64 or float-float fields.  in_max: optional precomputed maxima of the input in the orientation the
// first GEMM slices it (forward: per stacked row; backward: per field and column, stride nu64).  out_rowmax /
// out_colmax: optional maxima of the output for a following transform (zeroed by the caller).  in_sliced
// (forward only): the caller has already written the first GEMM's sliced operand into the workspace (the first
// piece carve_ws takes, see forward_input_slices), and `in` is not read.
int split_mft_run(const SplitMftPlan* p, int direction, int batch, const FieldIO& in, const unsigned int* in_max,
                  const FieldIO& out, double are, double aim, int epilogue, const float2* mask, const FieldIO& src,
                  unsigned int* out_rowmax, unsigned int* out_colmax, void* ws, cudaStream_t st,
                  bool in_sliced = false, const RowPhase* in_phase = nullptr) {
    const int nx = p->nx, ny = p->ny, nu = p->nu, nv = p->nv;
    const long long nu64 = round_up(nu, 64);
    const long long rows = (long long)batch * ny;
    Carver c(ws);
    Ws w;
    carve_ws(c, p, direction, batch, w);
    if (direction == HX_FORWARD) {
        HX_TRY(cuda_status(cudaMemsetAsync(w.t_max, 0, sizeof(unsigned int) * batch * nu64, st), "memset"));
        // G1: T = E . M2f, stacked over the batch (embedding on M2f); column maxima of T per field for the next
        // slicing.
        if (!in_sliced) HX_TRY(launch_slice_rows(in, nx, rows, nx, in_max, w.s1, st, true, in_phase));
        GemmArgs g1 = base_args(p->status);
        g1.emb = 1;
        g1.M = (int)rows;
        g1.N = nu;
        g1.row_scale = w.s1.scale;
        g1.col_scale = p->m2f.scale;
        g1.out = w.t;
        g1.ldo = nu;
        g1.colmax = w.t_max;
        g1.colmax_rows_per_field = ny;
        g1.colmax_field_stride = nu64;
        HX_TRY(launch_gemm(g1, w.s1, p->m2f, w.c1, 1, w.partial, w.counters, (double)rows * nu * nx, p->schedule, st));
        // G2: out[b] = alpha M1f . T[b] with the fused epilogue.
        HX_TRY(launch_slice_cols(w.t, ny, nu, batch, (long long)ny * nu, w.t_max, nu64, w.s2, (int)nu64, st));
        GemmArgs g2 = base_args(p->status);
        g2.M = nv;
        g2.N = nu;
        g2.b_rows_per_z = (int)nu64;
        g2.row_scale = p->m1f.scale;
        g2.col_scale = w.s2.scale;
        g2.col_scale_z = nu64;
        set_alpha(g2, are, aim);
        g2.out = out;
        g2.ldo = nu;
        g2.out_z = (long long)nv * nu;
        g2.epi = epilogue;
        g2.mask = mask;
        g2.src = src;
        g2.rows_per_field = nv;
        g2.rowmax = out_rowmax;
        g2.rowmax_z = nv;
        g2.colmax = out_colmax;
        g2.colmax_z = nu64;
        return launch_gemm(g2, p->m1f, w.s2, w.c2, batch, w.partial, w.counters, (double)nv * nu * ny * batch, p->schedule, st);
    }
    const SliceMat& m1 = direction == HX_BACKWARD ? p->m1b : p->m1a;
    const SliceMat& m2 = direction == HX_BACKWARD ? p->m2b : p->m2a;
    HX_TRY(cuda_status(cudaMemsetAsync(w.t_max, 0, sizeof(unsigned int) * rows, st), "memset"));
    // G1: T[b] = M1 . F[b]  (F sliced by columns), row maxima of T for the next slicing.
    const unsigned int* fmax = in_max;
    if (!fmax) {
        HX_TRY(cuda_status(cudaMemsetAsync(w.in_max, 0, sizeof(unsigned int) * batch * nu64, st), "memset"));
        HX_TRY(launch_colmax(in, nv, nu, batch, (long long)nv * nu, w.in_max, nu64, st));
        fmax = w.in_max;
    }
    HX_TRY(launch_slice_cols(in, nv, nu, batch, (long long)nv * nu, fmax, nu64, w.s1, (int)nu64, st));
    GemmArgs g1 = base_args(p->status);
    g1.M = ny;
    g1.N = nu;
    g1.b_rows_per_z = (int)nu64;
    g1.row_scale = m1.scale;
    g1.col_scale = w.s1.scale;
    g1.col_scale_z = nu64;
    g1.out = w.t;
    g1.ldo = nu;
    g1.out_z = (long long)ny * nu;
    g1.rowmax = w.t_max;
    g1.rowmax_z = ny;
    HX_TRY(launch_gemm(g1, m1, w.s1, w.c1, batch, w.partial, w.counters, (double)ny * nu * nv * batch, p->schedule, st));
    // G2: out = alpha T . M2, stacked over the batch (embedding on M2), with the fused epilogue.
    HX_TRY(launch_slice_rows(w.t, nu, rows, nu, w.t_max, w.s2, st, true));
    GemmArgs g2 = base_args(p->status);
    g2.emb = 1;
    g2.M = (int)rows;
    g2.N = nx;
    g2.row_scale = w.s2.scale;
    g2.col_scale = m2.scale;
    set_alpha(g2, are, aim);
    g2.out = out;
    g2.ldo = nx;
    g2.epi = epilogue;
    g2.mask = mask;
    g2.src = src;
    g2.rows_per_field = ny;
    g2.rowmax = out_rowmax;
    g2.colmax = out_colmax;
    g2.colmax_rows_per_field = ny;
    g2.colmax_field_stride = round_up(nx, 64);
    return launch_gemm(g2, w.s2, m2, w.c2, 1, w.partial, w.counters, (double)rows * nx * nu, p->schedule, st);
}

}  // namespace

int split_mft_create(int nx, int ny, int nu, int nv, const double* x, const double* y, const double* u,
                     const double* v, const double* wx, const double* wy, const double* wu, const double* wv,
                     cudaStream_t st, SplitMftPlan** out) {
    *out = nullptr;
    if (std::max(std::max(nx, ny), std::max(nu, nv)) > MAX_GRID_POINTS) {
        set_error("the split tensor-core MFT takes grids of at most %d points per axis", MAX_GRID_POINTS);
        return HX_ERR_UNSUPPORTED;
    }
    SplitMftPlan* p = new SplitMftPlan();
    p->nx = nx; p->ny = ny; p->nu = nu; p->nv = nv;
    const bool own_adj = wx || wy || wu || wv;
    // m2f, m2b, m2a are the B operands of GEMMs whose A is the field: they carry the embedding (two rows per
    // column, blocks of 8 columns); the padding rows are zero, and rows past them read as zeros through the TMA
    // bounds.
    auto layout = [&](Carver& c) {
        carve_slices(c, p->m2f, round_up(2LL * nu, 128), nx, round_up(nu, 64));
        carve_slices(c, p->m1f, 2 * round_up(nv, 64), ny, nv);
        carve_slices(c, p->m1b, 2 * round_up(ny, 64), nv, ny);
        carve_slices(c, p->m2b, round_up(2LL * nx, 128), nu, round_up(nx, 64));
        if (own_adj) {
            carve_slices(c, p->m1a, 2 * round_up(ny, 64), nv, ny);
            carve_slices(c, p->m2a, round_up(2LL * nx, 128), nu, round_up(nx, 64));
        }
        p->status = (int*)c.take(sizeof(int));
    };
    Carver count(nullptr);
    layout(count);
    int rc = cuda_status(cudaMalloc(&p->mem, count.off), "cudaMalloc(split MFT plan)");
    if (rc == HX_OK) rc = cuda_status(cudaMemsetAsync(p->mem, 0, count.off, st), "memset split plan");
    if (rc == HX_OK) {
        Carver c(p->mem);
        layout(c);
        if (!own_adj) {
            p->m1a = p->m1b;
            p->m2a = p->m2b;
        }
        // forward: M2f[x,u] = wx exp(-i x u) as B (K = x rows, N = u); M1f[v,y] = exp(-i v y) wy as A
        rc = slice_phase(nx, nu, x, u, -1.0, wx, nullptr, false, p->m2f, st, true);
        if (rc == HX_OK) rc = slice_phase(nv, ny, v, y, -1.0, nullptr, wy, true, p->m1f, st);
        // backward: M1b[y,v] = exp(+i y v) wv as A; M2b[u,x] = wu exp(+i u x) as B
        if (rc == HX_OK) rc = slice_phase(ny, nv, y, v, +1.0, nullptr, wv, true, p->m1b, st);
        if (rc == HX_OK) rc = slice_phase(nu, nx, u, x, +1.0, wu, nullptr, false, p->m2b, st, true);
        if (rc == HX_OK && own_adj) {
            rc = slice_phase(ny, nv, y, v, +1.0, wy, nullptr, true, p->m1a, st);
            if (rc == HX_OK) rc = slice_phase(nu, nx, u, x, +1.0, nullptr, wx, false, p->m2a, st, true);
        }
    }
    if (rc != HX_OK) {
        split_mft_destroy(p);
        return rc;
    }
    *out = p;
    return HX_OK;
}

size_t split_mft_workspace_bytes(const SplitMftPlan* p, int direction, int batch) {
    if (!p || batch <= 0) return 0;
    Carver c(nullptr);
    Ws w;
    carve_ws(c, p, direction, batch, w);
    return c.off + 256;
}

namespace {
FieldIO input_field(const void* p, int dtype) {
    FieldIO f;
    if (dtype == HX_C128) f.c128 = (const double2*)p;
    else f.c64 = (const float2*)p;
    return f;
}
FieldIO output_field(void* p, int dtype) {
    FieldIO f;
    if (dtype == HX_C128) f.c128_out = (double2*)p;
    else f.c64_out = (float2*)p;
    return f;
}
}  // namespace

int split_mft_execute(const SplitMftPlan* p, int direction, int batch, const void* in, int in_dtype, void* out,
                      int out_dtype, double are, double aim, int epilogue, const float2* mask, const void* src,
                      int src_dtype, void* ws, size_t ws_bytes, cudaStream_t st) {
    if (!p) {
        set_error("the split tensor-core MFT plan is missing");
        return HX_ERR_INVALID;
    }
    return split_mft_run(p, direction, batch, input_field(in, in_dtype), nullptr, output_field(out, out_dtype), are,
                         aim, epilogue, mask, input_field(src, src_dtype), nullptr, nullptr, ws, st);
}

// Forward transform of complex64 fields times exp(i scale screen) (screen: ny x nx float32, shared by the batch):
// the phase is applied while the first GEMM's operand is sliced.
int split_mft_execute_phase(const SplitMftPlan* p, int batch, const void* in, const float* screen, double scale,
                            void* out, int out_dtype, double are, double aim, void* ws, cudaStream_t st) {
    if (!p) {
        set_error("the split tensor-core MFT plan is missing");
        return HX_ERR_INVALID;
    }
    const RowPhase ph{screen, p->ny, (float)scale};
    FieldIO none;
    return split_mft_run(p, HX_FORWARD, batch, input_field(in, HX_C64), nullptr, output_field(out, out_dtype), are,
                         aim, HX_EPI_NONE, nullptr, none, nullptr, nullptr, ws, st, false, &ph);
}

// Lyot coronagraph (and final image) with float-float fields between the transforms.
size_t split_lyot_workspace_bytes(const SplitMftPlan* fpm, const SplitMftPlan* img, int batch) {
    const long long pupil = (long long)fpm->nx * fpm->ny, focal = (long long)fpm->nu * fpm->nv;
    Carver c(nullptr);
    carve_ff(c, batch * focal);
    carve_ff(c, batch * pupil);
    c.take(sizeof(unsigned int) * batch * round_up(fpm->nu, 64));
    c.take(sizeof(unsigned int) * batch * fpm->ny);
    const size_t own = c.off + 256;
    size_t inner = std::max(split_mft_workspace_bytes(fpm, HX_FORWARD, batch),
                            split_mft_workspace_bytes(fpm, HX_BACKWARD, batch));
    if (img) inner = std::max(inner, split_mft_workspace_bytes(img, HX_FORWARD, batch));
    return own + inner + 256;
}

int split_lyot_execute(const SplitMftPlan* fpm, const SplitMftPlan* img, int batch, const void* e, int e_dtype,
                       const float2* one_minus_fpm, const float2* stop, double af_re, double af_im, double ab_re,
                       double ab_im, double ai_re, double ai_im, void* lyot_out, int lyot_dtype, void* img_out,
                       int img_dtype, void* ws, cudaStream_t st) {
    const long long pupil = (long long)fpm->nx * fpm->ny, focal = (long long)fpm->nu * fpm->nv;
    Carver c(ws);
    FieldIO ef = carve_ff(c, batch * focal);
    FieldIO lp = carve_ff(c, batch * pupil);
    const long long nu64 = round_up(fpm->nu, 64);
    unsigned int* ef_colmax = (unsigned int*)c.take(sizeof(unsigned int) * batch * nu64);
    unsigned int* lp_rowmax = (unsigned int*)c.take(sizeof(unsigned int) * batch * fpm->ny);
    void* inner = c.take(0);
    HX_TRY(cuda_status(cudaMemsetAsync(ef_colmax, 0, sizeof(unsigned int) * batch * nu64, st), "memset"));
    HX_TRY(cuda_status(cudaMemsetAsync(lp_rowmax, 0, sizeof(unsigned int) * batch * fpm->ny, st), "memset"));
    FieldIO fe = input_field(e, e_dtype), none;
    // E_f = P(E) (1 - M), kept in float-float with its column maxima.
    HX_TRY(split_mft_run(fpm, HX_FORWARD, batch, fe, nullptr, ef, af_re, af_im, HX_EPI_MUL, one_minus_fpm, none,
                         nullptr, ef_colmax, inner, st));
    // T = P^-1(E_f) in float-float (a plain epilogue: the GEMM's epilogue warps are few), then
    // L = S (E - alpha T) in a row pass: straight into the caller's Lyot-plane buffer when no image follows,
    // else in float-float (in place) with its row maxima for the image transform.
    const bool direct = lyot_out && !img;
    HX_TRY(split_mft_run(fpm, HX_BACKWARD, batch, ef, ef_colmax, lp, 1.0, 0.0, HX_EPI_NONE, nullptr, none, nullptr,
                         nullptr, inner, st));
    // With only the image wanted, the row pass slices the Lyot plane for the image transform itself.
    const long long rows = (long long)batch * fpm->ny;
    const int kp_img = img ? (int)round_up(fpm->nx, 32) : 0;
    const bool fused = img && !lyot_out && kp_img <= 4096 && rows <= 2147483647LL;
    if (fused) {
        GemmArgs ga;
        set_alpha(ga, ab_re, ab_im);
        const cff alpha = {{ga.alpha[0], ga.alpha[1]}, {ga.alpha[2], ga.alpha[3]}};
        SliceMat s1 = forward_input_slices(img, batch, inner);
        const int groups = (kp_img + 1023) / 1024;
        auto run = [&](auto src_tag, auto g_tag) {
            constexpr int SRC = decltype(src_tag)::value, G = decltype(g_tag)::value;
            babinet_slice_rows_kernel<SRC, G><<<(unsigned)rows, 256, 0, st>>>(
                lp, fe, stop, alpha, fpm->ny, fpm->nx, s1.Kp, s1.planes, s1.plane_stride(), s1.kpitch, s1.scale);
        };
        using I = std::integral_constant<int, FMT_C128>;
        using J = std::integral_constant<int, FMT_C64>;
        using G1 = std::integral_constant<int, 1>;
        using G2 = std::integral_constant<int, 2>;
        using G3 = std::integral_constant<int, 3>;
        using G4 = std::integral_constant<int, 4>;
        if (e_dtype == HX_C128) {
            if (groups == 1) run(I(), G1()); else if (groups == 2) run(I(), G2());
            else if (groups == 3) run(I(), G3()); else run(I(), G4());
        } else {
            if (groups == 1) run(J(), G1()); else if (groups == 2) run(J(), G2());
            else if (groups == 3) run(J(), G3()); else run(J(), G4());
        }
        HX_TRY(launch_status("babinet_slice_rows_kernel"));
        return split_mft_run(img, HX_FORWARD, batch, lp, nullptr, output_field(img_out, img_dtype), ai_re, ai_im,
                             HX_EPI_NONE, nullptr, none, nullptr, nullptr, inner, st, true);
    }
    {
        GemmArgs ga;
        set_alpha(ga, ab_re, ab_im);
        const cff alpha = {{ga.alpha[0], ga.alpha[1]}, {ga.alpha[2], ga.alpha[3]}};
        const FieldIO dst = direct ? output_field(lyot_out, lyot_dtype) : lp;
        const int out_fmt = direct ? output_fmt(dst) : FMT_FF;
        if (e_dtype == HX_C128)
            HX_TRY(launch_babinet_src<FMT_C128>(lp, fe, stop, alpha, rows, fpm->ny, fpm->nx, dst, out_fmt,
                                                direct ? nullptr : lp_rowmax, st));
        else
            HX_TRY(launch_babinet_src<FMT_C64>(lp, fe, stop, alpha, rows, fpm->ny, fpm->nx, dst, out_fmt,
                                               direct ? nullptr : lp_rowmax, st));
    }
    if (lyot_out && !direct) {
        const long long n = batch * pupil;
        field_copy_kernel<<<ceil_div(n, 512), 256, 0, st>>>(lp, output_field(lyot_out, lyot_dtype), n);
        HX_TRY(launch_status("field_copy_kernel"));
    }
    if (img) {
        HX_TRY(split_mft_run(img, HX_FORWARD, batch, lp, lp_rowmax, output_field(img_out, img_dtype), ai_re, ai_im,
                             HX_EPI_NONE, nullptr, none, nullptr, nullptr, inner, st));
    }
    return HX_OK;
}

int split_mft_status(const SplitMftPlan* p, int reset) {
    if (!p || !p->status) return HX_OK;
    int h = 0;
    HX_TRY(cuda_status(cudaMemcpy(&h, p->status, sizeof(int), cudaMemcpyDeviceToHost), "read split status"));
    if (reset && h != 0) cudaMemset(p->status, 0, sizeof(int));
    if (h != 0) set_error("a bounded wait in the split tensor-core GEMM gave up");
    return h;
}

void split_mft_set_schedule(SplitMftPlan* p, int schedule) {
    if (p) p->schedule = schedule;
}

void split_autotune(int on) { g_autotune.store(on ? 1 : 0, std::memory_order_relaxed); }

int split_autotune_entries() {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    return (int)g_tuned.size();
}

int split_autotune_entry(int i, long long* shape, int* n, int* bn, int* ksplit, float* ms) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    if (i < 0 || i >= (int)g_tuned.size()) return HX_ERR_INVALID;
    auto it = g_tuned.begin();
    std::advance(it, i);
    shape[0] = it->first.m_tiles;
    shape[1] = it->first.N;
    shape[2] = it->first.grid_z;
    shape[3] = it->first.ktiles;
    *n = it->second.n;
    for (int k = 0; k < it->second.n; ++k) {
        bn[k] = it->second.cand[k].bn;
        ksplit[k] = it->second.cand[k].ksplit;
        ms[k] = it->second.ms[k];
    }
    return HX_OK;
}

void split_autotune_clear() {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tuned.clear();
}

void split_mft_destroy(SplitMftPlan* p) {
    if (!p) return;
    cudaFree(p->mem);
    delete p;
}

// ---- weighted intensity sums (the dark-hole contrast) -------------------------------------------------
//
// sums[b] = sum_p w[p] |E_b[p]|^2 with float-float products and a compensated (float-float) accumulation on the
// FP32 pipe: per-chunk partials in a fixed reduction order, then one warp per field adds its chunks in order,
// so the result does not depend on scheduling.  Its gradient (torch's convention for a real loss of complex
// fields) is 2 g_b w[p] E_b[p].

namespace {

constexpr int INT_THREADS = 256;
constexpr int INT_CHUNK = INT_THREADS * 32;  // pixels per CTA of the partial pass

__device__ __forceinline__ ff warp_sum_ff(ff v) {
    for (int o = 16; o > 0; o >>= 1)
        v = ff_add(v, ff{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)});
    return v;
}

template <int SRC>
__global__ void __launch_bounds__(INT_THREADS) intensity_partial_kernel(FieldIO f, long long n,
                                                                        const float* __restrict__ w,
                                                                        float2* partial) {
    const int b = blockIdx.y;
    const long long p0 = (long long)blockIdx.x * INT_CHUNK;
    const long long p1 = min(n, p0 + INT_CHUNK);
    ff acc = {0.0f, 0.0f};
    for (long long p = p0 + threadIdx.x; p < p1; p += INT_THREADS) {
        const cff v = load_fmt<SRC>(f, (long long)b * n + p);
        ff s = ff_add(ff_mul(v.re, v.re), ff_mul(v.im, v.im));
        if (w) s = ff_mulf(s, __ldg(&w[p]));
        acc = ff_add(acc, s);
    }
    __shared__ float2 red[INT_THREADS / 32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    acc = warp_sum_ff(acc);
    if (lane == 0) red[warp] = make_float2(acc.hi, acc.lo);
    __syncthreads();
    if (warp == 0) {
        acc = lane < INT_THREADS / 32 ? ff{red[lane].x, red[lane].y} : ff{0.0f, 0.0f};
        acc = warp_sum_ff(acc);
        if (lane == 0) partial[(long long)b * gridDim.x + blockIdx.x] = make_float2(acc.hi, acc.lo);
    }
}

__global__ void intensity_final_kernel(const float2* __restrict__ partial, int nchunks, int batch,
                                       double* sums) {
    const int b = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (b >= batch) return;
    ff acc = {0.0f, 0.0f};
    for (int c = lane; c < nchunks; c += 32) {
        const float2 q = partial[(long long)b * nchunks + c];
        acc = ff_add(acc, ff{q.x, q.y});
    }
    acc = warp_sum_ff(acc);
    if (lane == 0) sums[b] = ff_to_double(acc);
}

template <int FMT>
__global__ void __launch_bounds__(INT_THREADS) intensity_grad_kernel(FieldIO f, long long n,
                                                                     const float* __restrict__ w,
                                                                     const double* __restrict__ g, FieldIO out) {
    const int b = blockIdx.y;
    __shared__ ff s_scale;
    if (threadIdx.x == 0) {
        const ff gb = double_to_ff(g[b]);
        s_scale = {2.0f * gb.hi, 2.0f * gb.lo};  // exact doubling
    }
    __syncthreads();
    const ff scale = s_scale;
    for (long long p = (long long)blockIdx.x * INT_THREADS + threadIdx.x; p < n;
         p += (long long)gridDim.x * INT_THREADS) {
        const long long i = (long long)b * n + p;
        const cff v = load_fmt<FMT>(f, i);
        const ff c = w ? ff_mulf(scale, __ldg(&w[p])) : scale;
        store_fmt<FMT>(out, i, cff{ff_mul(v.re, c), ff_mul(v.im, c)});
    }
}

}  // namespace

size_t intensity_sums_workspace_bytes(long long n, int batch) {
    if (n <= 0 || batch <= 0) return 0;
    return sizeof(float2) * (size_t)batch * ceil_div(n, INT_CHUNK);
}

int intensity_sums(const void* field, int dtype, long long n, int batch, const float* w, double* sums, void* ws,
                   cudaStream_t st) {
    const unsigned nchunks = ceil_div(n, INT_CHUNK);
    if (batch > 65535) {
        set_error("hx_intensity_sums: at most 65535 fields per call");
        return HX_ERR_UNSUPPORTED;
    }
    float2* partial = (float2*)ws;
    const dim3 grid(nchunks, (unsigned)batch);
    if (dtype == HX_C128)
        intensity_partial_kernel<FMT_C128><<<grid, INT_THREADS, 0, st>>>(input_field(field, dtype), n, w, partial);
    else
        intensity_partial_kernel<FMT_C64><<<grid, INT_THREADS, 0, st>>>(input_field(field, dtype), n, w, partial);
    HX_TRY(launch_status("intensity_partial_kernel"));
    intensity_final_kernel<<<ceil_div(batch, 8), 256, 0, st>>>(partial, (int)nchunks, batch, sums);
    return launch_status("intensity_final_kernel");
}

int intensity_sums_grad(const void* field, int dtype, long long n, int batch, const float* w, const double* g,
                        void* out, cudaStream_t st) {
    if (batch > 65535) {
        set_error("hx_intensity_sums_grad: at most 65535 fields per call");
        return HX_ERR_UNSUPPORTED;
    }
    const unsigned bx = std::min<unsigned>(ceil_div(n, INT_THREADS), 4096u);
    const dim3 grid(bx, (unsigned)batch);
    if (dtype == HX_C128)
        intensity_grad_kernel<FMT_C128><<<grid, INT_THREADS, 0, st>>>(input_field(field, dtype), n, w, g,
                                                                     output_field(out, dtype));
    else
        intensity_grad_kernel<FMT_C64><<<grid, INT_THREADS, 0, st>>>(input_field(field, dtype), n, w, g,
                                                                    output_field(out, dtype));
    return launch_status("intensity_grad_kernel");
}

}  // namespace hx
