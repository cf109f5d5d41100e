// Split-operand tensor-core form of the matrix Fourier transform on tcgen05 (sm_103a).
//
// Numerics.  Every complex GEMM C = A.B runs as one real GEMM on the embedding
//     A' = [[Ar, -Ai], [Ai, Ar]] (2M x 2K),  B' = [Br; Bi] (2K x N),  C' = [Cr; Ci].
// Each row of A' (column of B') is scaled by a power of two s >= its largest
// magnitude and cut into three fixed-point slices,
//     x = s (2^-6 a0 + 2^-17 a1 + 2^-28 a2),  a0 in [-64, 64], a1, a2 in [-1024, 1024],
// all exact in fp16.  Products are grouped by level (a0 b0 | a0 b1 + a1 b0 |
// a0 b2 + a1 b1 + a2 b0 | a1 b2 + a2 b1) into four FP32 accumulators in TMEM;
// the dropped level (a2 b2) weighs at most 2^-36, so ~29 bits of each operand
// survive.  The level-0 products are integers of magnitude <= 2^12, so their
// FP32 sum is exact up to 4096 terms (K' = 2K <= 4096); the other levels carry
// 2^-11, 2^-22 and 2^-33 of the weight, so their FP32 rounding sits far below
// 2^-29.  The epilogue combines the levels in float64.  This removes the FP32
// accumulation error of the plain path, which dominates a coronagraph's dark
// hole (its normalized-intensity error is ~1e-10 in FP32).
//
// Kernel.  One CTA computes 64 complex rows x 64 columns of C: a 128-row tile of
// A' (the 64 Cr rows then their 64 Ci rows) times a 64-row tile of B'.
// warp 0 issues TMA loads (one 3-D box per operand per stage: three slice
// planes of 64 K-elements, 128-byte swizzle), warp 1 issues tcgen05.mma
// (8 slice products x 4 K16 steps per stage) into four TMEM accumulators of
// 128 lanes x 64 columns, warps 2-5 read TMEM, combine the levels in float64,
// apply the row/column scales, alpha and the fused epilogue, and write the
// result.  Three pipeline stages of 72 KiB.  All waits are bounded: a wait that
// runs out records HX_ERR_TIMEOUT in the plan's status word, the CTA drains its
// own copies and MMAs, frees its TMEM and returns.  A wait is bounded by the
// global timer (2 s), not by a poll count.
#include "hx_common.cuh"
#include "mft_tc.cuh"
#include "tc_ptx.cuh"

#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <mutex>

namespace hx {
namespace {

constexpr int BM = 128;  // A' rows per tile (64 complex rows)
constexpr int BN = 64;   // output columns per tile
constexpr int BK = 64;   // K' elements per stage (128 bytes of fp16)
constexpr int STAGES = 3;
constexpr int NSLICE = 3;
constexpr int A_PLANE_BYTES = BM * BK * 2;
constexpr int B_PLANE_BYTES = BN * BK * 2;
constexpr int A_STAGE_BYTES = NSLICE * A_PLANE_BYTES;
constexpr int B_STAGE_BYTES = NSLICE * B_PLANE_BYTES;
constexpr int STAGE_BYTES = A_STAGE_BYTES + B_STAGE_BYTES;
constexpr int EPI_PITCH = BN + 1;  // float64 staging row pitch (bank spread)
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;
constexpr int TMEM_COLS = 256;  // four level accumulators of BN columns
constexpr int NUM_THREADS = 192;
constexpr uint64_t WAIT_LIMIT = 2000000000ull;  // 2 s per wait
constexpr int MAX_KPITCH = 4096;  // exact level-0 sums need K' <= 4096

static_assert(BM * EPI_PITCH * 8 <= STAGES * STAGE_BYTES, "epilogue staging must fit the pipeline buffers");

enum { OUT_F64_PLANES = 0, OUT_C64 = 1 };

struct __align__(64) GemmArgs {
    CUtensorMap tmap_a;
    CUtensorMap tmap_b;
    int m_tiles, n_tiles, ktiles;
    int a_rows_per_z;      // A' row offset per grid z (0: shared A)
    int b_rows_per_z;      // B' row offset per grid z (0: shared B)
    int M, N;              // valid complex rows / columns of the output (per z)
    const double* row_scale;
    long long row_scale_z;
    const double* col_scale;
    long long col_scale_z;
    double alpha_re, alpha_im;
    int out_mode;
    double* out_re;
    double* out_im;
    float2* out_c64;
    long long ldo, out_z;
    int epi;
    const float2* mask;
    const float2* src;
    int rows_per_field;    // mask index = (m % rows_per_field) * N + n
    unsigned long long* colmax;
    long long colmax_z;
    int colmax_rows_per_field;  // colmax field = m / colmax_rows_per_field (stacked rows), plus z
    long long colmax_field_stride;
    unsigned long long* rowmax;
    long long rowmax_z;
    int* status;
};

__device__ __forceinline__ void raise_status(int* status, volatile int* abort_flag) {
    *abort_flag = 1;
    if (status) atomicExch(status, HX_ERR_TIMEOUT);
}

__global__ void __launch_bounds__(NUM_THREADS, 1) split_gemm_kernel(const __grid_constant__ GemmArgs g) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    const uint32_t raw_addr = ptx::smem_addr(smem_raw);
    uint8_t* smem = smem_raw + ((1024 - (raw_addr & 1023)) & 1023);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE_BYTES);
    // bars[0..S): full, bars[S..2S): empty, bars[2S]: accumulators ready
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 2);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int n_tile = blockIdx.x, m_tile = blockIdx.y, z = blockIdx.z;

    auto bar_full = [&](int s) { return ptx::smem_addr(&bars[s]); };
    auto bar_empty = [&](int s) { return ptx::smem_addr(&bars[STAGES + s]); };
    const uint32_t bar_accum = ptx::smem_addr(&bars[2 * STAGES]);

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            ptx::mbar_init(bar_full(s), 1);
            ptx::mbar_init(bar_empty(s), 1);
        }
        ptx::mbar_init(bar_accum, 1);
        *abort_flag = 0;
        ptx::fence_mbar_init();
    }
    if (warp == 1) {
        ptx::tmem_alloc(ptx::smem_addr(tmem_slot), TMEM_COLS);
        ptx::tmem_relinquish();
    }
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            int last_use[STAGES];
            for (int s = 0; s < STAGES; ++s) last_use[s] = -1;
            const int a_row0 = m_tile * BM + z * g.a_rows_per_z;
            const int b_row0 = n_tile * BN + z * g.b_rows_per_z;
            for (int kt = 0; kt < g.ktiles; ++kt) {
                if (*abort_flag) break;
                const int s = kt % STAGES;
                const int u = kt / STAGES;
                if (u > 0 && !ptx::mbar_wait_bounded(bar_empty(s), (u - 1) & 1, WAIT_LIMIT)) {
                    raise_status(g.status, abort_flag);
                    break;
                }
                uint8_t* sa = smem + s * STAGE_BYTES;
                uint8_t* sb = sa + A_STAGE_BYTES;
                ptx::mbar_arrive_expect_tx(bar_full(s), STAGE_BYTES);
                ptx::tma_load_3d(ptx::smem_addr(sa), &g.tmap_a, kt * BK, a_row0, 0, bar_full(s));
                ptx::tma_load_3d(ptx::smem_addr(sb), &g.tmap_b, kt * BK, b_row0, 0, bar_full(s));
                last_use[s] = u;
            }
            // No copy may land in shared memory after this CTA exits.
            for (int s = 0; s < STAGES; ++s)
                if (last_use[s] >= 0 && !ptx::mbar_wait_bounded(bar_full(s), last_use[s] & 1, WAIT_LIMIT))
                    raise_status(g.status, abort_flag);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = ptx::umma_idesc_f16(BM, BN);
            // (A slice, B slice, level) of the kept products; the first product of a level starts it.
            constexpr int NPROD = 8;
            const int pa[NPROD] = {0, 0, 1, 0, 1, 2, 1, 2};
            const int pb[NPROD] = {0, 1, 0, 2, 1, 0, 2, 1};
            const int pl[NPROD] = {0, 1, 1, 2, 2, 2, 3, 3};
            const int first[NPROD] = {1, 1, 0, 1, 0, 0, 1, 0};
            for (int kt = 0; kt < g.ktiles; ++kt) {
                if (*abort_flag) break;
                const int s = kt % STAGES;
                const int u = kt / STAGES;
                if (!ptx::mbar_wait_bounded(bar_full(s), u & 1, WAIT_LIMIT)) {
                    raise_status(g.status, abort_flag);
                    break;
                }
                ptx::tc_fence_after();
                const uint32_t a0 = ptx::smem_addr(smem + s * STAGE_BYTES);
                const uint32_t b0 = a0 + A_STAGE_BYTES;
#pragma unroll
                for (int kk = 0; kk < BK / 16; ++kk) {
#pragma unroll
                    for (int p = 0; p < NPROD; ++p) {
                        const uint64_t ad = ptx::umma_desc_sw128(a0 + pa[p] * A_PLANE_BYTES + kk * 32);
                        const uint64_t bd = ptx::umma_desc_sw128(b0 + pb[p] * B_PLANE_BYTES + kk * 32);
                        const uint32_t acc = (kt > 0 || kk > 0 || !first[p]) ? 1u : 0u;
                        ptx::umma_f16(tmem + pl[p] * BN, ad, bd, idesc, acc);
                    }
                }
                ptx::umma_commit(bar_empty(s));
            }
            // Arrives once every MMA issued above has completed (at once if none was issued); TMEM is
            // released only after that.
            ptx::umma_commit(bar_accum);
            if (!ptx::mbar_wait_bounded(bar_accum, 0, WAIT_LIMIT)) raise_status(g.status, abort_flag);
        }
    } else {
        // ---- epilogue: warps 2..5 ----
        const int et = threadIdx.x - 64;           // 0..127
        const int quarter = warp & 3;              // TMEM lane quarter this warp may access
        const int row = quarter * 32 + lane;       // A' row within the tile = TMEM lane
        double* stage = reinterpret_cast<double*>(smem);
        if (!ptx::mbar_wait_bounded(bar_accum, 0, WAIT_LIMIT)) raise_status(g.status, abort_flag);
        ptx::tc_fence_after();
        // Warp-uniform decision: the TMEM loads below are .sync.aligned.
        const bool live = __shfl_sync(0xffffffffu, (int)(*abort_flag == 0), 0) != 0;
        if (live) {
            const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
#pragma unroll 1
            for (int c = 0; c < BN / 16; ++c) {
                float v0[16], v1[16], v2[16], v3[16];
                ptx::tmem_ld_16(tmem + lane_base + 0 * BN + c * 16, v0);
                ptx::tmem_ld_16(tmem + lane_base + 1 * BN + c * 16, v1);
                ptx::tmem_ld_16(tmem + lane_base + 2 * BN + c * 16, v2);
                ptx::tmem_ld_16(tmem + lane_base + 3 * BN + c * 16, v3);
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const double v = (double)v0[j] * 0x1p-12 + (double)v1[j] * 0x1p-23 + (double)v2[j] * 0x1p-34 +
                                     (double)v3[j] * 0x1p-45;
                    stage[row * EPI_PITCH + c * 16 + j] = v;
                }
            }
        }
        ptx::named_barrier(1, 128);
        if (live && !*abort_flag) {
#pragma unroll 1
            for (int i = 0; i < (64 * BN) / 128; ++i) {
                const int idx = et + 128 * i;
                const int ml = idx / BN, nl = idx % BN;
                const int m = m_tile * 64 + ml;
                const int n = n_tile * BN + nl;
                if (m >= g.M || n >= g.N) continue;
                const double sc = g.row_scale[z * g.row_scale_z + m] * g.col_scale[z * g.col_scale_z + n];
                const double cr = stage[ml * EPI_PITCH + nl] * sc;
                const double ci = stage[(64 + ml) * EPI_PITCH + nl] * sc;
                double re = g.alpha_re * cr - g.alpha_im * ci;
                double im = g.alpha_re * ci + g.alpha_im * cr;
                const long long o = z * g.out_z + (long long)m * g.ldo + n;
                if (g.epi == HX_EPI_MUL) {
                    const float2 mk = g.mask[(long long)(m % g.rows_per_field) * g.N + n];
                    const double r2 = re * mk.x - im * mk.y;
                    im = re * mk.y + im * mk.x;
                    re = r2;
                } else if (g.epi == HX_EPI_BABINET) {
                    const float2 e = g.src[o];
                    re = (double)e.x - re;
                    im = (double)e.y - im;
                    if (g.mask) {
                        const float2 mk = g.mask[(long long)(m % g.rows_per_field) * g.N + n];
                        const double r2 = re * mk.x - im * mk.y;
                        im = re * mk.y + im * mk.x;
                        re = r2;
                    }
                }
                if (g.out_mode == OUT_F64_PLANES) {
                    g.out_re[o] = re;
                    g.out_im[o] = im;
                } else {
                    g.out_c64[o] = make_float2((float)re, (float)im);
                }
                const double mag = fmax(fabs(re), fabs(im));
                if (g.colmax) {
                    const long long f = g.colmax_rows_per_field > 0 ? m / g.colmax_rows_per_field : 0;
                    atomicMax(&g.colmax[z * g.colmax_z + f * g.colmax_field_stride + n],
                              (unsigned long long)__double_as_longlong(mag));
                }
                if (g.rowmax)
                    atomicMax(&g.rowmax[z * g.rowmax_z + m], (unsigned long long)__double_as_longlong(mag));
            }
        }
    }
    ptx::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        ptx::tc_fence_after();
        ptx::tmem_dealloc(tmem, TMEM_COLS);
    }
}

// ---- slicing --------------------------------------------------------------------------------------

__device__ __forceinline__ double pow2_scale(double mx) {
    if (!(mx > 0.0) || !isfinite(mx)) return 1.0;
    int e;
    frexp(mx, &e);  // mx = f 2^e, f in [0.5, 1)
    return ldexp(1.0, e);
}

// x in [-1, 1] -> a0 + 2^-11 a1 + 2^-22 a2 (times 2^-6), rounded to nearest at each step.
__device__ __forceinline__ void slice3(double t, __half& h0, __half& h1, __half& h2) {
    double u = t * 64.0;
    const double a0 = rint(u);
    u = (u - a0) * 2048.0;
    const double a1 = rint(u);
    u = (u - a1) * 2048.0;
    const double a2 = rint(u);
    h0 = __double2half(a0);
    h1 = __double2half(a1);
    h2 = __double2half(a2);
}

__device__ __forceinline__ void load_cplx(const float2* c64, const double* re, const double* im, long long i,
                                          double& xr, double& xi) {
    if (c64) {
        const float2 v = c64[i];
        xr = v.x;
        xi = v.y;
    } else {
        xr = re[i];
        xi = im[i];
    }
}

// One CTA per complex row m of X (M x K, row stride ld): writes the Cr and Ci rows of A'.
__global__ void slice_rows_kernel(const float2* src_c64, const double* src_re, const double* src_im, long long ld,
                                  int K, int Kp, const unsigned long long* rowmax, __half* planes,
                                  long long plane_stride, int kpitch, double* scale_out) {
    const int m = blockIdx.x;
    __shared__ double red[32];
    __shared__ double s_scale;
    double mx = 0.0;
    if (rowmax) {
        mx = __longlong_as_double((long long)rowmax[m]);
    } else {
        for (int k = threadIdx.x; k < K; k += blockDim.x) {
            double xr, xi;
            load_cplx(src_c64, src_re, src_im, (long long)m * ld + k, xr, xi);
            mx = fmax(mx, fmax(fabs(xr), fabs(xi)));
        }
        for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
        __syncthreads();
        if (threadIdx.x < 32) {
            mx = threadIdx.x < (int)(blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
            for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        }
    }
    if (threadIdx.x == 0) {
        s_scale = pow2_scale(mx);
        scale_out[m] = s_scale;
    }
    __syncthreads();
    const double inv = 1.0 / s_scale;
    const long long r_cr = (long long)(m / 64) * 128 + (m % 64);
    const long long r_ci = r_cr + 64;
    for (int k = threadIdx.x; k < Kp; k += blockDim.x) {
        double xr = 0.0, xi = 0.0;
        if (k < K) load_cplx(src_c64, src_re, src_im, (long long)m * ld + k, xr, xi);
        __half r0, r1, r2, i0, i1, i2;
        slice3(xr * inv, r0, r1, r2);
        slice3(xi * inv, i0, i1, i2);
        const __half rs[3] = {r0, r1, r2};
        const __half is[3] = {i0, i1, i2};
#pragma unroll
        for (int p = 0; p < 3; ++p) {
            __half* pl = planes + p * plane_stride;
            pl[r_cr * kpitch + k] = rs[p];
            pl[r_cr * kpitch + Kp + k] = __hneg(is[p]);
            pl[r_ci * kpitch + k] = is[p];
            pl[r_ci * kpitch + Kp + k] = rs[p];
        }
    }
}

// Column maxima max(|Re|, |Im|) of per-field K x N matrices (fields along grid z), as float64 bits.
__global__ void colmax_kernel(const float2* src_c64, const double* src_re, const double* src_im, int K, int N,
                              long long field_stride, unsigned long long* colmax, long long colmax_stride) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    const int z = blockIdx.z;
    if (n >= N) return;
    const int k0 = blockIdx.y * 64;
    const int k1 = min(K, k0 + 64);
    double mx = 0.0;
    for (int k = k0; k < k1; ++k) {
        double xr, xi;
        load_cplx(src_c64, src_re, src_im, z * field_stride + (long long)k * N + n, xr, xi);
        mx = fmax(mx, fmax(fabs(xr), fabs(xi)));
    }
    atomicMax(&colmax[z * colmax_stride + n], (unsigned long long)__double_as_longlong(mx));
}

// Per-field K x N matrix Y -> B' rows (z*n_rows_per_field + n): [slices of Re Y[:, n] | slices of Im Y[:, n]].
__global__ void slice_cols_kernel(const float2* src_c64, const double* src_re, const double* src_im, int K, int N,
                                  int Kp, long long field_stride, const unsigned long long* colmax,
                                  long long colmax_stride, __half* planes, long long plane_stride, int kpitch,
                                  int n_rows_per_field, double* scale_out) {
    __shared__ double tr[32][33], ti[32][33];
    __shared__ double sc[32];
    const int n0 = blockIdx.x * 32, k0 = blockIdx.y * 32, z = blockIdx.z;
    const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
    if (ty == 0) {
        const int n = n0 + tx;
        const double mx = n < N ? __longlong_as_double((long long)colmax[z * colmax_stride + n]) : 0.0;
        sc[tx] = pow2_scale(mx);
        if (k0 == 0 && n < N) scale_out[(long long)z * n_rows_per_field + n] = sc[tx];
    }
    for (int r = ty; r < 32; r += 8) {
        const int k = k0 + r, n = n0 + tx;
        double xr = 0.0, xi = 0.0;
        if (k < K && n < N) load_cplx(src_c64, src_re, src_im, z * field_stride + (long long)k * N + n, xr, xi);
        tr[r][tx] = xr;
        ti[r][tx] = xi;
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
        const int n = n0 + r, k = k0 + tx;
        if (n >= N || k >= Kp) continue;
        const double inv = 1.0 / sc[r];
        __half r0, r1, r2, i0, i1, i2;
        slice3(tr[tx][r] * inv, r0, r1, r2);
        slice3(ti[tx][r] * inv, i0, i1, i2);
        const __half rs[3] = {r0, r1, r2};
        const __half is[3] = {i0, i1, i2};
        const long long row = (long long)z * n_rows_per_field + n;
#pragma unroll
        for (int p = 0; p < 3; ++p) {
            __half* pl = planes + p * plane_stride;
            pl[row * kpitch + k] = rs[p];
            pl[row * kpitch + Kp + k] = is[p];
        }
    }
}

// Phase matrix in float64 planes: M[r, c] = wr[r] wc[c] exp(sign i a[r] b[c]).
__global__ void phase_planes_kernel(int rows, int cols, const double* a, const double* b, double sign,
                                    const double* wr, const double* wc, double* re, double* im) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)rows * cols) return;
    const int r = (int)(idx / cols), c = (int)(idx % cols);
    double s, co;
    sincos(a[r] * b[c], &s, &co);
    double w = 1.0;
    if (wr) w *= wr[r];
    if (wc) w *= wc[c];
    re[idx] = w * co;
    im[idx] = w * sign * s;
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
    double* scale = nullptr;
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
    s.scale = (double*)c.take(sizeof(double) * scales);
}

int launch_slice_rows(const float2* c64, const double* re, const double* im, long long ld, long long M, int K,
                      const unsigned long long* rowmax, SliceMat& s, cudaStream_t st) {
    if (M > 2147483647LL) return HX_ERR_UNSUPPORTED;
    slice_rows_kernel<<<(unsigned)M, 256, 0, st>>>(c64, re, im, ld, K, s.Kp, rowmax, s.planes, s.plane_stride(),
                                                   s.kpitch, s.scale);
    return launch_status("slice_rows_kernel");
}

int launch_colmax(const float2* c64, const double* re, const double* im, int K, int N, int fields,
                  long long field_stride, unsigned long long* colmax, long long colmax_stride, cudaStream_t st) {
    dim3 grid(ceil_div(N, 128), ceil_div(K, 64), fields);
    colmax_kernel<<<grid, 128, 0, st>>>(c64, re, im, K, N, field_stride, colmax, colmax_stride);
    return launch_status("colmax_kernel");
}

int launch_slice_cols(const float2* c64, const double* re, const double* im, int K, int N, int fields,
                      long long field_stride, const unsigned long long* colmax, long long colmax_stride,
                      SliceMat& s, int n_rows_per_field, cudaStream_t st) {
    dim3 grid(ceil_div(N, 32), ceil_div(s.Kp, 32), fields);
    slice_cols_kernel<<<grid, dim3(32, 8), 0, st>>>(c64, re, im, K, N, s.Kp, field_stride, colmax, colmax_stride,
                                                    s.planes, s.plane_stride(), s.kpitch, n_rows_per_field, s.scale);
    return launch_status("slice_cols_kernel");
}

int launch_gemm(GemmArgs& g, const SliceMat& A, const SliceMat& B, long long a_tiles_rows, int grid_z,
                cudaStream_t st) {
    if (A.kpitch != B.kpitch) {
        set_error("internal: split GEMM K mismatch (%d vs %d)", A.kpitch, B.kpitch);
        return HX_ERR_INVALID;
    }
    HX_TRY(encode_map(&g.tmap_a, A, BM));
    HX_TRY(encode_map(&g.tmap_b, B, BN));
    g.ktiles = A.kpitch / BK;
    g.m_tiles = (int)(a_tiles_rows / BM);
    g.n_tiles = ceil_div(g.N, BN);
    static bool configured = false;
    if (!configured) {
        HX_TRY(cuda_status(cudaFuncSetAttribute(split_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                SMEM_BYTES),
                           "cudaFuncSetAttribute(split_gemm_kernel)"));
        configured = true;
    }
    if (g.m_tiles > 65535 || grid_z > 65535) {
        set_error("split GEMM grid too large");
        return HX_ERR_UNSUPPORTED;
    }
    dim3 grid(g.n_tiles, g.m_tiles, grid_z);
    split_gemm_kernel<<<grid, NUM_THREADS, SMEM_BYTES, st>>>(g);
    return launch_status("split_gemm_kernel");
}

GemmArgs base_args(int* status) {
    GemmArgs g;
    memset(&g, 0, sizeof(g));
    g.alpha_re = 1.0;
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
};

namespace {

// Slice a float64 phase matrix (rows x cols, generated on the device) as an A (row) or B (column) operand.
int slice_phase(int rows, int cols, const double* a, const double* b, double sign, const double* wr,
                const double* wc, bool as_rows, SliceMat& out, cudaStream_t st) {
    double *re = nullptr, *im = nullptr;
    unsigned long long* mx = nullptr;
    const long long n = (long long)rows * cols;
    int rc = cuda_status(cudaMalloc(&re, sizeof(double) * n), "cudaMalloc(phase re)");
    if (rc == HX_OK) rc = cuda_status(cudaMalloc(&im, sizeof(double) * n), "cudaMalloc(phase im)");
    if (rc == HX_OK) {
        phase_planes_kernel<<<ceil_div(n, 256), 256, 0, st>>>(rows, cols, a, b, sign, wr, wc, re, im);
        rc = launch_status("phase_planes_kernel");
    }
    if (rc == HX_OK) {
        if (as_rows) {
            rc = launch_slice_rows(nullptr, re, im, cols, rows, cols, nullptr, out, st);
        } else {
            rc = cuda_status(cudaMalloc(&mx, sizeof(unsigned long long) * round_up(cols, 64)), "cudaMalloc(colmax)");
            if (rc == HX_OK)
                rc = cuda_status(cudaMemsetAsync(mx, 0, sizeof(unsigned long long) * round_up(cols, 64), st),
                                 "memset colmax");
            if (rc == HX_OK) rc = launch_colmax(nullptr, re, im, rows, cols, 1, 0, mx, 0, st);
            if (rc == HX_OK) rc = launch_slice_cols(nullptr, re, im, rows, cols, 1, 0, mx, 0, out, 0, st);
        }
    }
    cudaStreamSynchronize(st);
    cudaFree(re);
    cudaFree(im);
    cudaFree(mx);
    return rc;
}

}  // namespace

int split_mft_create(int nx, int ny, int nu, int nv, const double* x, const double* y, const double* u,
                     const double* v, const double* wx, const double* wy, const double* wu, const double* wv,
                     cudaStream_t st, SplitMftPlan** out) {
    *out = nullptr;
    if (2 * round_up(std::max(std::max(nx, ny), std::max(nu, nv)), 32) > MAX_KPITCH) {
        set_error("the split tensor-core MFT takes grids of at most %d points per axis", MAX_KPITCH / 2);
        return HX_ERR_UNSUPPORTED;
    }
    SplitMftPlan* p = new SplitMftPlan();
    p->nx = nx; p->ny = ny; p->nu = nu; p->nv = nv;
    const bool own_adj = wx || wy || wu || wv;
    // Layout pass (sizes), then one allocation, then the real pass.
    auto layout = [&](Carver& c) {
        carve_slices(c, p->m2f, round_up(nu, 64), nx, round_up(nu, 64));
        carve_slices(c, p->m1f, 2 * round_up(nv, 64), ny, nv);
        carve_slices(c, p->m1b, 2 * round_up(ny, 64), nv, ny);
        carve_slices(c, p->m2b, round_up(nx, 64), nu, round_up(nx, 64));
        if (own_adj) {
            carve_slices(c, p->m1a, 2 * round_up(ny, 64), nv, ny);
            carve_slices(c, p->m2a, round_up(nx, 64), nu, round_up(nx, 64));
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
        rc = slice_phase(nx, nu, x, u, -1.0, wx, nullptr, false, p->m2f, st);
        if (rc == HX_OK) rc = slice_phase(nv, ny, v, y, -1.0, nullptr, wy, true, p->m1f, st);
        // backward: M1b[y,v] = exp(+i y v) wv as A; M2b[u,x] = wu exp(+i u x) as B
        if (rc == HX_OK) rc = slice_phase(ny, nv, y, v, +1.0, nullptr, wv, true, p->m1b, st);
        if (rc == HX_OK) rc = slice_phase(nu, nx, u, x, +1.0, wu, nullptr, false, p->m2b, st);
        if (rc == HX_OK && own_adj) {
            rc = slice_phase(ny, nv, y, v, +1.0, wy, nullptr, true, p->m1a, st);
            if (rc == HX_OK) rc = slice_phase(nu, nx, u, x, +1.0, nullptr, wx, false, p->m2a, st);
        }
    }
    if (rc != HX_OK) {
        split_mft_destroy(p);
        return rc;
    }
    *out = p;
    return HX_OK;
}

namespace {

struct FwdWs {
    SliceMat a1;            // input rows (batch*ny) x K nx
    double *t_re, *t_im;    // (batch*ny) x nu
    unsigned long long* tmax;  // batch x nu64
    SliceMat b2;            // batch*nu64 rows, K ny
};
struct BwdWs {
    unsigned long long* fmax;  // batch x nu64
    SliceMat b1;            // batch*nu64 rows, K nv
    double *t_re, *t_im;    // batch x ny x nu
    unsigned long long* tmax;  // batch*ny
    SliceMat a2;            // rows 2 (batch*ny)64, K nu
};

void carve_fwd(Carver& c, const SplitMftPlan* p, int batch, FwdWs& w) {
    const long long rows = (long long)batch * p->ny;
    const long long nu64 = round_up(p->nu, 64);
    carve_slices(c, w.a1, 2 * round_up(rows, 64), p->nx, rows);
    w.t_re = (double*)c.take(sizeof(double) * rows * p->nu);
    w.t_im = (double*)c.take(sizeof(double) * rows * p->nu);
    w.tmax = (unsigned long long*)c.take(sizeof(unsigned long long) * batch * nu64);
    carve_slices(c, w.b2, (long long)batch * nu64, p->ny, (long long)batch * nu64);
}

void carve_bwd(Carver& c, const SplitMftPlan* p, int batch, BwdWs& w) {
    const long long rows = (long long)batch * p->ny;
    const long long nu64 = round_up(p->nu, 64);
    w.fmax = (unsigned long long*)c.take(sizeof(unsigned long long) * batch * nu64);
    carve_slices(c, w.b1, (long long)batch * nu64, p->nv, (long long)batch * nu64);
    w.t_re = (double*)c.take(sizeof(double) * rows * p->nu);
    w.t_im = (double*)c.take(sizeof(double) * rows * p->nu);
    w.tmax = (unsigned long long*)c.take(sizeof(unsigned long long) * rows);
    carve_slices(c, w.a2, 2 * round_up(rows, 64), p->nu, rows);
}

}  // namespace

size_t split_mft_workspace_bytes(const SplitMftPlan* p, int direction, int batch) {
    if (!p || batch <= 0) return 0;
    Carver c(nullptr);
    if (direction == HX_FORWARD) {
        FwdWs w;
        carve_fwd(c, p, batch, w);
    } else {
        BwdWs w;
        carve_bwd(c, p, batch, w);
    }
    return c.off + 256;
}

int split_mft_execute(const SplitMftPlan* p, int direction, int batch, const float2* in, float2* out, double are,
                      double aim, int epilogue, const float2* mask, const float2* src, void* ws, size_t ws_bytes,
                      cudaStream_t st) {
    if (!p) {
        set_error("the split tensor-core MFT plan is missing");
        return HX_ERR_INVALID;
    }
    const int nx = p->nx, ny = p->ny, nu = p->nu, nv = p->nv;
    const long long nu64 = round_up(nu, 64);
    if (direction == HX_FORWARD) {
        Carver c(ws);
        FwdWs w;
        carve_fwd(c, p, batch, w);
        const long long rows = (long long)batch * ny;
        HX_TRY(cuda_status(cudaMemsetAsync(w.tmax, 0, sizeof(unsigned long long) * batch * nu64, st), "memset"));
        // G1: T = E . M2f, stacked over the batch; column maxima of T per field for the next slicing.
        HX_TRY(launch_slice_rows(in, nullptr, nullptr, nx, rows, nx, nullptr, w.a1, st));
        GemmArgs g1 = base_args(p->status);
        g1.M = (int)rows;
        g1.N = nu;
        g1.row_scale = w.a1.scale;
        g1.col_scale = p->m2f.scale;
        g1.out_mode = OUT_F64_PLANES;
        g1.out_re = w.t_re;
        g1.out_im = w.t_im;
        g1.ldo = nu;
        g1.colmax = w.tmax;
        g1.colmax_rows_per_field = ny;
        g1.colmax_field_stride = nu64;
        HX_TRY(launch_gemm(g1, w.a1, p->m2f, w.a1.rows, 1, st));
        // G2: out[b] = alpha M1f . T[b]
        HX_TRY(launch_slice_cols(nullptr, w.t_re, w.t_im, ny, nu, batch, (long long)ny * nu, w.tmax, nu64, w.b2,
                                 (int)nu64, st));
        GemmArgs g2 = base_args(p->status);
        g2.M = nv;
        g2.N = nu;
        g2.b_rows_per_z = (int)nu64;
        g2.row_scale = p->m1f.scale;
        g2.col_scale = w.b2.scale;
        g2.col_scale_z = nu64;
        g2.alpha_re = are;
        g2.alpha_im = aim;
        g2.out_mode = OUT_C64;
        g2.out_c64 = out;
        g2.ldo = nu;
        g2.out_z = (long long)nv * nu;
        g2.epi = epilogue;
        g2.mask = mask;
        g2.src = src;
        g2.rows_per_field = nv;
        return launch_gemm(g2, p->m1f, w.b2, p->m1f.rows, batch, st);
    }
    const SliceMat& m1 = direction == HX_BACKWARD ? p->m1b : p->m1a;
    const SliceMat& m2 = direction == HX_BACKWARD ? p->m2b : p->m2a;
    Carver c(ws);
    BwdWs w;
    carve_bwd(c, p, batch, w);
    const long long rows = (long long)batch * ny;
    HX_TRY(cuda_status(cudaMemsetAsync(w.fmax, 0, sizeof(unsigned long long) * batch * nu64, st), "memset"));
    HX_TRY(cuda_status(cudaMemsetAsync(w.tmax, 0, sizeof(unsigned long long) * rows, st), "memset"));
    // G1: T[b] = M1 . F[b]  (F sliced by columns), row maxima of T for the next slicing.
    HX_TRY(launch_colmax(in, nullptr, nullptr, nv, nu, batch, (long long)nv * nu, w.fmax, nu64, st));
    HX_TRY(launch_slice_cols(in, nullptr, nullptr, nv, nu, batch, (long long)nv * nu, w.fmax, nu64, w.b1, (int)nu64,
                             st));
    GemmArgs g1 = base_args(p->status);
    g1.M = ny;
    g1.N = nu;
    g1.b_rows_per_z = (int)nu64;
    g1.row_scale = m1.scale;
    g1.col_scale = w.b1.scale;
    g1.col_scale_z = nu64;
    g1.out_mode = OUT_F64_PLANES;
    g1.out_re = w.t_re;
    g1.out_im = w.t_im;
    g1.ldo = nu;
    g1.out_z = (long long)ny * nu;
    g1.rowmax = w.tmax;
    g1.rowmax_z = ny;
    HX_TRY(launch_gemm(g1, m1, w.b1, m1.rows, batch, st));
    // G2: out = alpha T . M2, stacked over the batch, with the fused epilogue.
    HX_TRY(launch_slice_rows(nullptr, w.t_re, w.t_im, nu, rows, nu, w.tmax, w.a2, st));
    GemmArgs g2 = base_args(p->status);
    g2.M = (int)rows;
    g2.N = nx;
    g2.row_scale = w.a2.scale;
    g2.col_scale = m2.scale;
    g2.alpha_re = are;
    g2.alpha_im = aim;
    g2.out_mode = OUT_C64;
    g2.out_c64 = out;
    g2.ldo = nx;
    g2.epi = epilogue;
    g2.mask = mask;
    g2.src = src;
    g2.rows_per_field = ny;
    return launch_gemm(g2, w.a2, m2, w.a2.rows, 1, st);
}

int split_mft_status(const SplitMftPlan* p, int reset) {
    if (!p || !p->status) return HX_OK;
    int h = 0;
    HX_TRY(cuda_status(cudaMemcpy(&h, p->status, sizeof(int), cudaMemcpyDeviceToHost), "read split status"));
    if (reset && h != 0) cudaMemset(p->status, 0, sizeof(int));
    if (h != 0) set_error("a bounded wait in the split tensor-core GEMM gave up");
    return h;
}

void split_mft_destroy(SplitMftPlan* p) {
    if (!p) return;
    cudaFree(p->mem);
    delete p;
}

}  // namespace hx
