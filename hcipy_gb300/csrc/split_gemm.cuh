// The split-operand tcgen05 GEMM kernel of the matrix Fourier transform and its launch templates.
//
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
// FP32 sum is exact up to 4096 terms: a CTA sums at most K' = 4096, and a
// longer K' is split across CTAs (see split K below); the other levels carry
// 2^-11, 2^-22 and 2^-33 of the weight, so their FP32 rounding sits far below
// 2^-29.  This removes the FP32 accumulation error of the plain path, which
// dominates a coronagraph's dark hole (its normalized-intensity error is
// ~1e-9 in FP32).
//
// All arithmetic around the tensor cores is FP32: the GB300's float64 rate is a
// small fraction of its FP32 rate.  The epilogue combines the levels into a
// float-float pair (hi + lo, ~46 bits) with error-free TwoSum/TwoProduct steps,
// and applies the scales, alpha, the focal-plane mask and the Babinet
// subtraction in float-float.  Intermediate fields travel between the two GEMMs
// of an MFT, and between the MFTs of a coronagraph, as float-float planes
// (hi and lo of Re and Im); slicing reads them with FP32 operations only.
//
// Where the embedding lives.  When A is a plan constant (a phase matrix) the
// embedding above is used (EMB = 0): A' holds 64-row blocks of Cr rows then Ci
// rows and B' is the field, [Br; Bi] per column.  When A is the per-call field
// (EMB = 1) the embedding moves to the constant B instead, so that the field is
// sliced once as [Ar | Ai] (M x 2K) and never duplicated:
//     B' = [[Br, Bi], [-Bi, Br]] (2K x 2N),  C = [Cr | Ci],
// stored as B' rows (one per output column, K' = 2K long) in blocks of 8 complex
// columns: the 8 Cr rows [Br | -Bi] then the 8 Ci rows [Bi | Br].  A tile is then
// 128 complex rows x BN/2 complex columns, and TMEM lane = complex row.
//
// Kernel.  One CTA computes 64 complex rows x BN columns of C (BN = 64 or 128):
// a 128-row tile of A' (the 64 Cr rows then their 64 Ci rows) times a BN-row
// tile of B' (EMB = 0; with EMB = 1, 128 complex rows x BN/2 complex columns).
// warp 0 issues TMA loads (one 3-D box per operand per stage:
// three slice planes of 64 K-elements, 128-byte swizzle), warp 1 issues
// tcgen05.mma (8 slice products x 4 K16 steps per stage) into four TMEM
// accumulators of 128 lanes x BN columns, warps 2-9 read TMEM, combine and
// finish the result.  Three stages of 72 KiB (BN = 64) or two of 96 KiB
// (BN = 128).  GEMMs with too few tiles to fill the GPU split K across CTAs:
// each CTA combines its levels into a float-float partial (level 0 exactly),
// and the partials are added in split order with float-float additions (error
// ~2^-47 of a partial, far below the 2^-29 slice truncation).  Where the split
// allows it (at most 8 CTAs, 16-column slices) the splits of a tile form a
// thread-block cluster: each CTA sends the column slices of its partial to
// their owners through distributed shared memory, and every CTA adds and
// finishes one slice.  Otherwise each split writes its partial to the
// workspace and the last CTA of the tile (counted with an atomic) adds them
// and runs the epilogue.  All waits are
// bounded by the global timer: a wait that runs out records HX_ERR_TIMEOUT in
// the plan's status word, the CTA drains its own copies and MMAs, frees its
// TMEM and returns.
#pragma once

#include "hx_common.cuh"
#include "tc_ptx.cuh"

#include <cuda_fp16.h>
#include <cudaTypedefs.h>

#include <type_traits>

namespace hx {
namespace sg {

constexpr int BM = 128;  // A' rows per tile (64 complex rows)
constexpr int BK = 64;   // K' elements per stage (128 bytes of fp16)
constexpr int NSLICE = 3;
constexpr int A_PLANE_BYTES = BM * BK * 2;
constexpr int A_STAGE_BYTES = NSLICE * A_PLANE_BYTES;
constexpr int NUM_THREADS = 320;  // TMA warp, MMA warp, 8 epilogue warps
constexpr uint64_t WAIT_LIMIT = 2000000000ull;  // 2 s per wait
constexpr int MAX_SPLIT_K = 4096;               // exact level-0 sums need at most 4096 K' per CTA
constexpr int MAX_SPLIT_KTILES = MAX_SPLIT_K / BK;
constexpr int MAX_GRID_POINTS = 8192;           // points per axis of a split plan
constexpr int EXTRA_BYTES = 1024 + 3712;        // alignment slack, barriers, flags, per-row tables

// Tile of BN output columns: four level accumulators of BN TMEM columns each, so BN = 128 takes all
// 512 columns of the SM.  Stage count fills the shared memory.
template <int BN> struct Tile {
    static_assert(BN % 16 == 0 && 4 * BN <= 512, "four level accumulators of BN columns must fit TMEM");
    static constexpr int B_PLANE_BYTES = BN * BK * 2;
    static constexpr int STAGE_BYTES = A_STAGE_BYTES + NSLICE * B_PLANE_BYTES;
    static constexpr int STAGES = BN == 64 ? 3 : 2;
    static constexpr int PIPE_BYTES = STAGES * STAGE_BYTES;
    static constexpr int SMEM_BYTES = PIPE_BYTES + EXTRA_BYTES;
    static constexpr int TMEM_COLS = 4 * BN <= 256 ? 256 : 512;  // allocation: a power of two >= 4 BN
    static constexpr int PITCH = BN + 1;  // epilogue staging row pitch in floats (bank spread)
    static_assert((2 * BM + 64) * PITCH * 4 <= PIPE_BYTES, "epilogue staging must fit the pipeline buffers");
    static_assert(SMEM_BYTES <= 227 * 1024, "shared memory per CTA");
};

// ---- float-float arithmetic (error-free transformations in FP32) -------------------------------------

struct ff {
    float hi, lo;
};

__device__ __forceinline__ ff two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

__device__ __forceinline__ ff two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ ff ff_add(ff a, ff b) {
    const ff s = two_sum(a.hi, b.hi);
    const float t = __fadd_rn(__fadd_rn(a.lo, b.lo), s.lo);
    return two_sum(s.hi, t);
}

__device__ __forceinline__ ff ff_neg(ff a) { return {-a.hi, -a.lo}; }

__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    const ff p = two_prod(a.hi, b.hi);
    const float t = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo));
    return two_sum(p.hi, t);
}

__device__ __forceinline__ ff ff_mulf(ff a, float b) {
    const ff p = two_prod(a.hi, b);
    return two_sum(p.hi, __fmaf_rn(a.lo, b, p.lo));
}

// Complex float-float: (a + ib).
struct cff {
    ff re, im;
};

__device__ __forceinline__ cff cff_mul(cff a, cff b) {
    return {ff_add(ff_mul(a.re, b.re), ff_neg(ff_mul(a.im, b.im))), ff_add(ff_mul(a.re, b.im), ff_mul(a.im, b.re))};
}

__device__ __forceinline__ cff cff_mul_c64(cff a, float2 b) {
    return {ff_add(ff_mulf(a.re, b.x), ff_neg(ff_mulf(a.im, b.y))), ff_add(ff_mulf(a.re, b.y), ff_mulf(a.im, b.x))};
}

// ---- field formats ----------------------------------------------------------------------------------

// A batch of complex values as interleaved complex64, interleaved complex128, or four float-float planes.
struct FieldIO {
    const float2* c64 = nullptr;
    float2* c64_out = nullptr;
    const double2* c128 = nullptr;
    double2* c128_out = nullptr;
    float* re_hi = nullptr;
    float* re_lo = nullptr;
    float* im_hi = nullptr;
    float* im_lo = nullptr;
};

// Field formats as compile-time tags of the GEMM epilogue.
enum : int { FMT_NONE = 0, FMT_C64 = 1, FMT_C128 = 2, FMT_FF = 3 };

// float64 -> float-float with integer operations only (the GB300's float64 pipe is narrow): hi is x truncated
// to 24 bits, lo the remainder rounded to float (|lo| < ulp(hi)).  Magnitudes below 2^-126 read as zero;
// infinities and NaNs go to hi.
__device__ __forceinline__ ff double_to_ff(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned int sign = (unsigned int)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7ff);
    const unsigned long long mant = b & 0xFFFFFFFFFFFFFull;
    const int ef = e - 896;  // biased float exponent
    if (e == 0x7ff) return {__uint_as_float(sign | 0x7f800000u | (mant ? 0x400000u : 0u)), 0.0f};
    if (ef >= 255) return {__uint_as_float(sign | 0x7f800000u), 0.0f};
    if (ef <= 0) return {__uint_as_float(sign), 0.0f};
    const float hi = __uint_as_float(sign | ((unsigned int)ef << 23) | (unsigned int)(mant >> 29));
    // remainder = rem * 2^(ef - 179) = (rem * 2^-64) * 2^(ef - 115): both powers of two are normal floats, and
    // the product underflows gradually for the smallest hi.
    float lo = __uint2float_rn((unsigned int)(mant & 0x1FFFFFFFull)) * 0x1p-64f *
               __uint_as_float((unsigned int)(ef + 12) << 23);
    if (sign) lo = -lo;
    return {hi, lo};
}

// Exact float -> float64 by bit placement (subnormal floats are normalised).
__device__ __forceinline__ unsigned long long float_bits_to_double_bits(unsigned int fb) {
    const unsigned long long sign = (unsigned long long)(fb & 0x80000000u) << 32;
    const unsigned int e = (fb >> 23) & 0xff;
    unsigned int m = fb & 0x7fffffu;
    if (e == 0xff) return sign | 0x7ff0000000000000ull | ((unsigned long long)m << 29);
    if (e == 0) {
        if (m == 0) return sign;
        const int sh = __clz(m) - 8;  // bring the leading one to bit 23
        m = (m << sh) & 0x7fffffu;
        return sign | ((unsigned long long)(1 - sh + 896) << 52) | ((unsigned long long)m << 29);
    }
    return sign | ((unsigned long long)(e + 896) << 52) | ((unsigned long long)m << 29);
}

// hi + lo as float64: each float is placed exactly into float64 bits (integer operations), then one float64
// addition rounds the sum.
__device__ __forceinline__ double ff_to_double(ff v) {
    return __dadd_rn(__longlong_as_double((long long)float_bits_to_double_bits(__float_as_uint(v.hi))),
                     __longlong_as_double((long long)float_bits_to_double_bits(__float_as_uint(v.lo))));
}

template <int FMT> __device__ __forceinline__ cff load_fmt(const FieldIO& f, long long i) {
    if constexpr (FMT == FMT_FF) {
        return {{f.re_hi[i], f.re_lo[i]}, {f.im_hi[i], f.im_lo[i]}};
    } else if constexpr (FMT == FMT_C128) {
        const double2 v = f.c128[i];
        return {double_to_ff(v.x), double_to_ff(v.y)};
    } else {
        const float2 v = f.c64[i];
        return {{v.x, 0.0f}, {v.y, 0.0f}};
    }
}

template <int FMT> __device__ __forceinline__ void store_fmt(const FieldIO& f, long long i, cff v) {
    if constexpr (FMT == FMT_FF) {
        f.re_hi[i] = v.re.hi;
        f.re_lo[i] = v.re.lo;
        f.im_hi[i] = v.im.hi;
        f.im_lo[i] = v.im.lo;
    } else if constexpr (FMT == FMT_C128) {
        f.c128_out[i] = make_double2(ff_to_double(v.re), ff_to_double(v.im));
    } else {
        f.c64_out[i] = make_float2(__fadd_rn(v.re.hi, v.re.lo), __fadd_rn(v.im.hi, v.im.lo));
    }
}

inline int input_fmt(const FieldIO& f) { return f.re_hi ? FMT_FF : f.c128 ? FMT_C128 : f.c64 ? FMT_C64 : FMT_NONE; }
inline int output_fmt(const FieldIO& f) { return f.re_hi ? FMT_FF : f.c128_out ? FMT_C128 : FMT_C64; }

// Runtime-format forms for the slicing and copy kernels (one format per launch, so the branches are uniform).
__device__ __forceinline__ cff load_field(const FieldIO& f, long long i) {
    if (f.re_hi) return load_fmt<FMT_FF>(f, i);
    if (f.c128) return load_fmt<FMT_C128>(f, i);
    return load_fmt<FMT_C64>(f, i);
}

// Elements i .. i+3 of a field, with 16-byte loads where the addresses allow them.
__device__ __forceinline__ void load4_field(const FieldIO& f, long long i, cff* v) {
    if (f.re_hi) {
        const float* p[4] = {f.re_hi + i, f.re_lo + i, f.im_hi + i, f.im_lo + i};
        if (((reinterpret_cast<uintptr_t>(p[0]) | reinterpret_cast<uintptr_t>(p[1]) | reinterpret_cast<uintptr_t>(p[2]) |
              reinterpret_cast<uintptr_t>(p[3])) & 15) == 0) {
            const float4 rh = *reinterpret_cast<const float4*>(p[0]), rl = *reinterpret_cast<const float4*>(p[1]);
            const float4 ih = *reinterpret_cast<const float4*>(p[2]), il = *reinterpret_cast<const float4*>(p[3]);
            v[0] = {{rh.x, rl.x}, {ih.x, il.x}};
            v[1] = {{rh.y, rl.y}, {ih.y, il.y}};
            v[2] = {{rh.z, rl.z}, {ih.z, il.z}};
            v[3] = {{rh.w, rl.w}, {ih.w, il.w}};
            return;
        }
    } else if (!f.c128) {
        if ((reinterpret_cast<uintptr_t>(f.c64 + i) & 15) == 0) {
            const float4 a = reinterpret_cast<const float4*>(f.c64 + i)[0];
            const float4 b = reinterpret_cast<const float4*>(f.c64 + i)[1];
            v[0] = {{a.x, 0.0f}, {a.y, 0.0f}};
            v[1] = {{a.z, 0.0f}, {a.w, 0.0f}};
            v[2] = {{b.x, 0.0f}, {b.y, 0.0f}};
            v[3] = {{b.z, 0.0f}, {b.w, 0.0f}};
            return;
        }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) v[j] = load_field(f, i + j);
}

__device__ __forceinline__ void store_field(const FieldIO& f, long long i, cff v) {
    if (f.re_hi) store_fmt<FMT_FF>(f, i, v);
    else if (f.c128_out) store_fmt<FMT_C128>(f, i, v);
    else store_fmt<FMT_C64>(f, i, v);
}

// ---- the tensor-core GEMM ----------------------------------------------------------------------------

struct __align__(64) GemmArgs {
    CUtensorMap tmap_a;
    CUtensorMap tmap_b;
    int ktiles;            // K' / BK
    int ksplit;            // CTAs along K per output tile
    int n_tiles;           // output column tiles (grid x = n_tiles * ksplit)
    int a_rows_per_z;      // A' row offset per grid z (0: shared A)
    int b_rows_per_z;      // B' row offset per grid z (0: shared B)
    int M, N;              // valid complex rows / columns of the output (per z)
    const float* row_scale;
    long long row_scale_z;
    const float* col_scale;
    long long col_scale_z;
    float alpha[4];        // Re hi, Re lo, Im hi, Im lo
    FieldIO out;
    long long ldo, out_z;
    int epi;
    const float2* mask;
    FieldIO src;           // Babinet source, same indexing as the output
    int emb;               // 1: the embedding is on B (A = [Ar | Ai]), see the file comment
    int cluster;           // 1: the ksplit CTAs of a tile form a thread-block cluster (see the kernel)
    int rows_per_field;    // mask index = (m % rows_per_field) * N + n
    unsigned int* colmax;  // max(|Re|, |Im|) of the output as float bits, per (field, column)
    long long colmax_z;
    int colmax_rows_per_field;  // field of a stacked row = m / colmax_rows_per_field (0: one field)
    long long colmax_field_stride;
    unsigned int* rowmax;  // per output row
    long long rowmax_z;
    float* partial;        // split K: float-float partial of every split of every tile
    unsigned int* counters;  // split K: finished splits per tile (zero before the launch)
    int* status;
};

__device__ __forceinline__ void raise_status(int* status, volatile int* abort_flag) {
    *abort_flag = 1;
    if (status) atomicExch(status, HX_ERR_TIMEOUT);
}

// The four level sums of one element as float-float: level 0 is an exact integer and the level weights are
// powers of two, so only the additions round.
__device__ __forceinline__ ff combine_levels(float v0, float v1, float v2, float v3) {
    const ff s = two_sum(v0 * 0x1p-12f, v1 * 0x1p-23f);
    return two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(v2 * 0x1p-34f, v3 * 0x1p-45f)));
}

// OUT: format of the result; SRC: format of the Babinet source (FMT_NONE for other epilogues); EMB: where the
// complex embedding lives (0: on A, 1: on B).
template <int BN, int OUT, int SRC, int EMB>
__global__ void __launch_bounds__(NUM_THREADS, 1) split_gemm_kernel(const __grid_constant__ GemmArgs g) {
    using T = Tile<BN>;
    constexpr int STAGES = T::STAGES;
    constexpr int TM = EMB ? 128 : 64;     // complex rows of a tile
    constexpr int TN = EMB ? BN / 2 : BN;  // complex columns of a tile
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    const uint32_t raw_addr = ptx::smem_addr(smem_raw);
    uint8_t* smem = smem_raw + ((1024 - (raw_addr & 1023)) & 1023);
    uint8_t* extra = smem + T::PIPE_BYTES;
    // bars[0..S): full, bars[S..2S): empty, bars[2S]: accumulators ready
    uint64_t* bars = reinterpret_cast<uint64_t*>(extra);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(extra + 64);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(extra + 68);
    volatile int* last_flag = reinterpret_cast<volatile int*>(extra + 72);
    float* s_rscale = reinterpret_cast<float*>(extra + 128);               // per tile row (TM): row scale
    int* s_field = reinterpret_cast<int*>(extra + 640);                    // m / colmax_rows_per_field
    long long* s_rowoff = reinterpret_cast<long long*>(extra + 1152);      // output offset of the row
    long long* s_maskoff = reinterpret_cast<long long*>(extra + 2176);     // mask offset of the row
    unsigned int* s_rowmax = reinterpret_cast<unsigned int*>(extra + 3200);  // EMB: row maxima of the tile

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    // the K-splits of a tile are consecutive CTAs when they form a cluster, else n_tiles apart
    const int n_tile = g.cluster ? blockIdx.x / g.ksplit : blockIdx.x % g.n_tiles;
    const int ks = g.cluster ? blockIdx.x % g.ksplit : blockIdx.x / g.n_tiles;
    const int m_tile = blockIdx.y, z = blockIdx.z;
    const int kt0 = (int)((long long)g.ktiles * ks / g.ksplit);
    const int nkt = (int)((long long)g.ktiles * (ks + 1) / g.ksplit) - kt0;

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
        *last_flag = 0;
        ptx::fence_mbar_init();
    }
    if (threadIdx.x >= 64 && threadIdx.x < 64 + TM) {
        const int r = threadIdx.x - 64;
        const int m = m_tile * TM + r;
        const bool ok = m < g.M;
        s_rscale[r] = ok ? g.row_scale[z * g.row_scale_z + m] : 0.0f;
        s_field[r] = (ok && g.colmax_rows_per_field > 0) ? m / g.colmax_rows_per_field : 0;
        s_rowoff[r] = z * g.out_z + (long long)m * g.ldo;
        s_maskoff[r] = ok ? (long long)(m % g.rows_per_field) * g.N : 0;
        if (EMB) s_rowmax[r] = 0u;
    }
    if (warp == 1) {
        ptx::tmem_alloc(ptx::smem_addr(tmem_slot), T::TMEM_COLS);
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
            for (int i = 0; i < nkt; ++i) {
                if (*abort_flag) break;
                const int s = i % STAGES;
                const int u = i / STAGES;
                if (u > 0 && !ptx::mbar_wait_bounded(bar_empty(s), (u - 1) & 1, WAIT_LIMIT)) {
                    raise_status(g.status, abort_flag);
                    break;
                }
                uint8_t* sa = smem + s * T::STAGE_BYTES;
                uint8_t* sb = sa + A_STAGE_BYTES;
                ptx::mbar_arrive_expect_tx(bar_full(s), T::STAGE_BYTES);
                ptx::tma_load_3d(ptx::smem_addr(sa), &g.tmap_a, (kt0 + i) * BK, a_row0, 0, bar_full(s));
                ptx::tma_load_3d(ptx::smem_addr(sb), &g.tmap_b, (kt0 + i) * BK, b_row0, 0, bar_full(s));
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
            for (int i = 0; i < nkt; ++i) {
                if (*abort_flag) break;
                const int s = i % STAGES;
                const int u = i / STAGES;
                if (!ptx::mbar_wait_bounded(bar_full(s), u & 1, WAIT_LIMIT)) {
                    raise_status(g.status, abort_flag);
                    break;
                }
                ptx::tc_fence_after();
                const uint32_t a0 = ptx::smem_addr(smem + s * T::STAGE_BYTES);
                const uint32_t b0 = a0 + A_STAGE_BYTES;
#pragma unroll
                for (int kk = 0; kk < BK / 16; ++kk) {
#pragma unroll
                    for (int p = 0; p < NPROD; ++p) {
                        const uint64_t ad = ptx::umma_desc_sw128(a0 + pa[p] * A_PLANE_BYTES + kk * 32);
                        const uint64_t bd = ptx::umma_desc_sw128(b0 + pb[p] * T::B_PLANE_BYTES + kk * 32);
                        const uint32_t acc = (i > 0 || kk > 0 || !first[p]) ? 1u : 0u;
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
    }
    // ---- epilogue: warps 2..9, two per TMEM lane quarter (each takes every other 16-column chunk) ----------
    constexpr int EPI = NUM_THREADS - 64;
    const bool epi_warp = warp >= 2;
    const int et = threadIdx.x - 64;         // 0..EPI-1 on the epilogue warps
    const int quarter = warp & 3;            // TMEM lane quarter this warp may access
    const int half = (warp - 2) >> 2;        // 0 or 1
    const int row = quarter * 32 + lane;     // A' row within the tile = TMEM lane
    const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
    bool live = false;
    if (epi_warp) {
        if (!ptx::mbar_wait_bounded(bar_accum, 0, WAIT_LIMIT)) raise_status(g.status, abort_flag);
        ptx::tc_fence_after();
        // Warp-uniform decision: the TMEM loads below are .sync.aligned.
        live = __shfl_sync(0xffffffffu, (int)(*abort_flag == 0), 0) != 0;
    }
    auto own_chunk = [&](int c, ff* r) {
        float v0[16], v1[16], v2[16], v3[16];
        ptx::tmem_ld_16(tmem + lane_base + 0 * BN + c * 16, v0);
        ptx::tmem_ld_16(tmem + lane_base + 1 * BN + c * 16, v1);
        ptx::tmem_ld_16(tmem + lane_base + 2 * BN + c * 16, v2);
        ptx::tmem_ld_16(tmem + lane_base + 3 * BN + c * 16, v3);
#pragma unroll
        for (int j = 0; j < 16; ++j) r[j] = combine_levels(v0[j], v1[j], v2[j], v3[j]);
    };
    // The slice of the tile this CTA finishes: all of it, or with a cluster of S splits the q-th of S column
    // slices (W = BN / S TMEM columns, TNs complex columns; W is a multiple of 16, so with EMB = 1 a slice holds
    // whole 8-column Cr / Ci blocks).
    const int S = g.cluster ? g.ksplit : 1;
    const int q = g.cluster ? ks : 0;
    const int W = BN / S;
    const int TNs = TN / S;
    float* fin_hi = nullptr;
    float* fin_lo = nullptr;
    int fpitch = 0;
    float* s_mag = nullptr;  // magnitudes of the slice for the row maxima (EMB = 0)
    bool finish = true;
    if (g.cluster) {
        // Every CTA of the cluster holds [split][hi, lo][128 rows][W + 4] float-float partials of its slice in its
        // pipeline buffers; each CTA sends the other slices of its partial to their owners through distributed
        // shared memory (16-byte stores), then adds the S partials of its own slice in split order and finishes it.
        const int WP = W + 4;
        const int PSZ = 2 * BM * WP;
        float* part_s = reinterpret_cast<float*>(smem);
        __syncwarp();
        ptx::cluster_sync();  // every CTA's copies and MMAs are complete: its pipeline buffers are free
        if (epi_warp && live) {
#pragma unroll 1
            for (int c = half; c < BN / 16; c += 2) {
                ff r[16];
                own_chunk(c, r);
                const int dst = (c * 16) / W;
                const int col0 = c * 16 - dst * W;
                float* base = part_s + ks * PSZ + row * WP + col0;
                if (dst == ks) {
#pragma unroll
                    for (int j = 0; j < 16; j += 4) {
                        *reinterpret_cast<float4*>(base + j) = make_float4(r[j].hi, r[j + 1].hi, r[j + 2].hi, r[j + 3].hi);
                        *reinterpret_cast<float4*>(base + BM * WP + j) =
                            make_float4(r[j].lo, r[j + 1].lo, r[j + 2].lo, r[j + 3].lo);
                    }
                } else {
                    const uint32_t a_hi = ptx::map_shared_rank(ptx::smem_addr(base), (uint32_t)dst);
                    const uint32_t a_lo = ptx::map_shared_rank(ptx::smem_addr(base + BM * WP), (uint32_t)dst);
#pragma unroll
                    for (int j = 0; j < 16; j += 4) {
                        ptx::st_cluster_v4(a_hi + 4 * j, make_float4(r[j].hi, r[j + 1].hi, r[j + 2].hi, r[j + 3].hi));
                        ptx::st_cluster_v4(a_lo + 4 * j, make_float4(r[j].lo, r[j + 1].lo, r[j + 2].lo, r[j + 3].lo));
                    }
                }
            }
        }
        __syncwarp();
        ptx::cluster_sync();  // every partial slice is in place
        if (epi_warp && live) {
#pragma unroll 1
            for (int e = et; e < BM * W; e += EPI) {
                const int r_ = e / W, c_ = e - (e / W) * W;
                const int o = r_ * WP + c_;
                ff acc = {part_s[o], part_s[BM * WP + o]};
                for (int sp = 1; sp < S; ++sp) acc = ff_add(acc, ff{part_s[sp * PSZ + o], part_s[sp * PSZ + BM * WP + o]});
                part_s[o] = acc.hi;
                part_s[BM * WP + o] = acc.lo;
            }
        }
        fin_hi = part_s;
        fin_lo = part_s + BM * WP;
        fpitch = WP;
        s_mag = part_s + S * PSZ;
    } else if (epi_warp) {
        float* st_hi = reinterpret_cast<float*>(smem);
        float* st_lo = st_hi + BM * T::PITCH;
        fin_hi = st_hi;
        fin_lo = st_lo;
        fpitch = T::PITCH;
        s_mag = st_lo + BM * T::PITCH;
        // Split K: float-float partial per split, [split][hi/lo][column / 4][row][column % 4] (float4 per thread).
        constexpr long long PART = 2LL * BN * BM;
        const long long tile = ((long long)z * gridDim.y + m_tile) * g.n_tiles + n_tile;
        float* part_base = g.ksplit > 1 ? g.partial + tile * g.ksplit * PART : nullptr;
        auto part_at = [&](int s, int plane, int c4) {
            return reinterpret_cast<float4*>(part_base + s * PART + ((long long)(plane * (BN / 4) + c4) * BM + row) * 4);
        };
        if (g.ksplit > 1) {
            if (live) {
#pragma unroll 1
                for (int c = half; c < BN / 16; c += 2) {
                    ff r[16];
                    own_chunk(c, r);
#pragma unroll
                    for (int qq = 0; qq < 4; ++qq) {
                        __stcg(part_at(ks, 0, c * 4 + qq), make_float4(r[4 * qq].hi, r[4 * qq + 1].hi, r[4 * qq + 2].hi, r[4 * qq + 3].hi));
                        __stcg(part_at(ks, 1, c * 4 + qq), make_float4(r[4 * qq].lo, r[4 * qq + 1].lo, r[4 * qq + 2].lo, r[4 * qq + 3].lo));
                    }
                }
            }
            __threadfence();
            ptx::named_barrier(1, EPI);
            if (et == 0) *last_flag = atomicAdd(&g.counters[tile], 1u) == (unsigned)(g.ksplit - 1) ? 1 : 0;
            ptx::named_barrier(1, EPI);
            finish = *last_flag != 0;
            if (finish && live) {
                __threadfence();
#pragma unroll 1
                for (int c = half; c < BN / 16; c += 2) {
                    ff own[16], acc[16];
                    own_chunk(c, own);
                    // Splits in index order (the sum does not depend on which CTA finishes last); two at a time.
#pragma unroll 1
                    for (int s0 = 0; s0 < g.ksplit; s0 += 2) {
                        float4 ph[2][4], pl[2][4];
#pragma unroll
                        for (int d = 0; d < 2; ++d) {
                            const int sp = s0 + d;
                            if (sp < g.ksplit && sp != ks) {
#pragma unroll
                                for (int qq = 0; qq < 4; ++qq) {
                                    ph[d][qq] = __ldcg(part_at(sp, 0, c * 4 + qq));
                                    pl[d][qq] = __ldcg(part_at(sp, 1, c * 4 + qq));
                                }
                            }
                        }
#pragma unroll
                        for (int d = 0; d < 2; ++d) {
                            const int sp = s0 + d;
                            if (sp >= g.ksplit) continue;
#pragma unroll
                            for (int j = 0; j < 16; ++j) {
                                ff p = own[j];
                                if (sp != ks) {
                                    const float4 h = ph[d][j >> 2], l = pl[d][j >> 2];
                                    const int w = j & 3;
                                    p = {w == 0 ? h.x : w == 1 ? h.y : w == 2 ? h.z : h.w,
                                         w == 0 ? l.x : w == 1 ? l.y : w == 2 ? l.z : l.w};
                                }
                                acc[j] = sp == 0 ? p : ff_add(acc[j], p);
                            }
                        }
                    }
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        st_hi[row * T::PITCH + c * 16 + j] = acc[j].hi;
                        st_lo[row * T::PITCH + c * 16 + j] = acc[j].lo;
                    }
                }
            }
        } else if (live) {
#pragma unroll 1
            for (int c = half; c < BN / 16; c += 2) {
                ff r[16];
                own_chunk(c, r);
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    st_hi[row * T::PITCH + c * 16 + j] = r[j].hi;
                    st_lo[row * T::PITCH + c * 16 + j] = r[j].lo;
                }
            }
        }
    }
    if (epi_warp) {
        ptx::named_barrier(1, EPI);
        const bool run = finish && live && !*abort_flag;
        const int ncol0 = n_tile * TN + q * TNs;  // first complex column of the slice
        // The rows of the slice: with the whole tile (no cluster) its width is a compile-time constant.
        auto rows_pass = [&](auto tns_c) {
            constexpr int TNC = decltype(tns_c)::value;
            const int TNS = TNC > 0 ? TNC : TNs;
            const cff alpha = {{g.alpha[0], g.alpha[1]}, {g.alpha[2], g.alpha[3]}};
            const bool real_alpha = g.alpha[2] == 0.0f && g.alpha[3] == 0.0f;
            const bool imag_alpha = g.alpha[0] == 0.0f && g.alpha[1] == 0.0f;  // e.g. Fraunhofer's 1/(i f lambda)
            const bool unit_alpha = real_alpha && g.alpha[0] == 1.0f && g.alpha[1] == 0.0f;
            const float2* mask = (g.epi == HX_EPI_MUL || g.epi == HX_EPI_BABINET) ? g.mask : nullptr;
            // Each thread keeps one complex column of the slice; a warp covers consecutive columns of one row.
            const int nl = et % TNS;
            const int n = ncol0 + nl;
            const bool nok = n < g.N;
            const float csc = nok ? g.col_scale[z * g.col_scale_z + n] : 0.0f;
            // staged position of the real and imaginary parts: EMB = 0, rows ml and 64 + ml of column nl;
            // EMB = 1, row ml, columns of the 8-column Cr / Ci blocks
            const int c_re = EMB ? (nl >> 3) * 16 + (nl & 7) : nl;
            const int c_im = EMB ? c_re + 8 : nl;
            constexpr int R_IM = EMB ? 0 : 64;
            const int RSTEP = EPI / TNS;          // rows per iteration
            const int ITER = TM / RSTEP;          // a multiple of U for every tile and slice width in use
            constexpr int U = 4;                  // rows per batch: loads issued before any store
            // With TNs not dividing the epilogue threads (BN = 112) the last EPI - RSTEP * TNs threads have no
            // column; they skip the loop so that no row beyond the tile's TM is touched.
            const bool has_col = et < RSTEP * TNS;
            const int r0 = et / TNS;
            const int mlim = g.M - m_tile * TM;   // valid rows of this tile
            int cfield = -1;
            float cmax = 0.0f;
#pragma unroll 1
            for (int i0 = 0; i0 < (has_col ? ITER : 0); i0 += U) {
                cff e[U];
                float2 mk[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int ml = r0 + RSTEP * (i0 + u);
                    const bool ok = nok && ml < mlim;
                    e[u] = {{0.0f, 0.0f}, {0.0f, 0.0f}};
                    mk[u] = make_float2(1.0f, 0.0f);
                    if constexpr (SRC != FMT_NONE) {
                        if (ok) e[u] = load_fmt<SRC>(g.src, s_rowoff[ml] + n);
                    }
                    if (ok && mask) mk[u] = __ldg(&mask[s_maskoff[ml] + n]);
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int ml = r0 + RSTEP * (i0 + u);
                    float mag = 0.0f;
                    if (nok && ml < mlim) {
                        const float sc = s_rscale[ml] * csc;  // product of powers of two: exact
                        cff v = {ff{fin_hi[ml * fpitch + c_re] * sc, fin_lo[ml * fpitch + c_re] * sc},
                                 ff{fin_hi[(R_IM + ml) * fpitch + c_im] * sc, fin_lo[(R_IM + ml) * fpitch + c_im] * sc}};
                        if (!unit_alpha)
                            v = real_alpha   ? cff{ff_mul(v.re, alpha.re), ff_mul(v.im, alpha.re)}
                                : imag_alpha ? cff{ff_neg(ff_mul(v.im, alpha.im)), ff_mul(v.re, alpha.im)}
                                             : cff_mul(v, alpha);
                        if constexpr (SRC != FMT_NONE) v = {ff_add(e[u].re, ff_neg(v.re)), ff_add(e[u].im, ff_neg(v.im))};
                        if (mask) v = mk[u].y == 0.0f ? cff{ff_mulf(v.re, mk[u].x), ff_mulf(v.im, mk[u].x)}
                                                      : cff_mul_c64(v, mk[u]);
                        store_fmt<OUT>(g.out, s_rowoff[ml] + n, v);
                        mag = fmaxf(fabsf(v.re.hi), fabsf(v.im.hi));
                        if (g.colmax) {
                            const int f = s_field[ml];
                            if (f != cfield) {
                                if (cfield >= 0 && cmax > 0.0f)
                                    atomicMax(&g.colmax[z * g.colmax_z + cfield * g.colmax_field_stride + n],
                                              __float_as_uint(cmax));
                                cfield = f;
                                cmax = 0.0f;
                            }
                            cmax = fmaxf(cmax, mag);
                        }
                    }
                    if (g.rowmax) {
                        if (EMB) {
                            if (mag > 0.0f) atomicMax(&s_rowmax[ml], __float_as_uint(mag));
                        } else {
                            s_mag[ml * fpitch + nl] = mag;
                        }
                    }
                }
            }
            if (g.colmax && cfield >= 0 && cmax > 0.0f)
                atomicMax(&g.colmax[z * g.colmax_z + cfield * g.colmax_field_stride + n], __float_as_uint(cmax));
        };
        if (run) {
            if (S == 1) rows_pass(std::integral_constant<int, TN>{});
            else rows_pass(std::integral_constant<int, 0>{});
        }
        ptx::named_barrier(1, EPI);
        if (run && g.rowmax && et < TM && et < g.M - m_tile * TM) {
            float mx = 0.0f;
            if (EMB) {
                mx = __uint_as_float(s_rowmax[et]);
            } else {
                const int nmax = min(TNs, g.N - ncol0);
                for (int c = 0; c < nmax; ++c) mx = fmaxf(mx, s_mag[et * fpitch + c]);
            }
            if (mx > 0.0f) atomicMax(&g.rowmax[z * g.rowmax_z + m_tile * TM + et], __float_as_uint(mx));
        }
    }
    ptx::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        ptx::tc_fence_after();
        ptx::tmem_dealloc(tmem, T::TMEM_COLS);
    }
}

// ---- launches (instantiated per tile width in split_gemm_bn*.cu) --------------------------------

template <int BN, int OUT, int SRC, int EMB> int launch_tile(const GemmArgs& g, dim3 grid, cudaStream_t st) {
    static bool configured[64];
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64 || !configured[dev]) {
        HX_TRY(cuda_status(cudaFuncSetAttribute(split_gemm_kernel<BN, OUT, SRC, EMB>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize, Tile<BN>::SMEM_BYTES),
                           "cudaFuncSetAttribute(split_gemm_kernel)"));
        if (dev >= 0 && dev < 64) configured[dev] = true;
    }
    if (!g.cluster) {
        split_gemm_kernel<BN, OUT, SRC, EMB><<<grid, NUM_THREADS, Tile<BN>::SMEM_BYTES, st>>>(g);
        return launch_status("split_gemm_kernel");
    }
    // the ksplit CTAs of a tile (consecutive along x) form one cluster
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(NUM_THREADS);
    cfg.dynamicSmemBytes = Tile<BN>::SMEM_BYTES;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)g.ksplit;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    HX_TRY(cuda_status(cudaLaunchKernelEx(&cfg, split_gemm_kernel<BN, OUT, SRC, EMB>, g), "split_gemm_kernel (cluster)"));
    return launch_status("split_gemm_kernel");
}

template <int BN, int OUT, int SRC> int launch_emb(const GemmArgs& g, dim3 grid, cudaStream_t st) {
    return g.emb ? launch_tile<BN, OUT, SRC, 1>(g, grid, st) : launch_tile<BN, OUT, SRC, 0>(g, grid, st);
}

template <int BN, int OUT> int launch_src(const GemmArgs& g, dim3 grid, int src, cudaStream_t st) {
    switch (src) {
        case FMT_NONE: return launch_emb<BN, OUT, FMT_NONE>(g, grid, st);
        case FMT_C64: return launch_emb<BN, OUT, FMT_C64>(g, grid, st);
        case FMT_C128: return launch_emb<BN, OUT, FMT_C128>(g, grid, st);
        default:
            set_error("internal: unsupported Babinet source format");
            return HX_ERR_INVALID;
    }
}

template <int BN> int launch_out(const GemmArgs& g, dim3 grid, int out, int src, cudaStream_t st) {
    switch (out) {
        case FMT_FF: return launch_src<BN, FMT_FF>(g, grid, src, st);
        case FMT_C128: return launch_src<BN, FMT_C128>(g, grid, src, st);
        default: return launch_src<BN, FMT_C64>(g, grid, src, st);
    }
}

// Whether the ksplit K-splits of a BN-column tile can reduce as one thread-block cluster: at most 8 CTAs, column
// slices of whole 16-column chunks, and at least one such cluster resident on this device.
int cluster_ok_bn64(int ksplit);
int cluster_ok_bn112(int ksplit);
int cluster_ok_bn128(int ksplit);

template <int BN> int cluster_ok(int ksplit) {
    if (ksplit < 2 || ksplit > 8 || (BN / 16) % ksplit != 0) return 0;
    static int cache[64][9];  // per device and split: 0 unknown, 1 yes, 2 no
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
    if (cache[dev][ksplit] == 0) {
        auto kern = split_gemm_kernel<BN, FMT_FF, FMT_NONE, 0>;
        int n = 0;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)ksplit, 1, 1);
        cfg.blockDim = dim3(NUM_THREADS);
        cfg.dynamicSmemBytes = Tile<BN>::SMEM_BYTES;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)ksplit;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        const bool ok = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             Tile<BN>::SMEM_BYTES) == cudaSuccess &&
                        cudaOccupancyMaxActiveClusters(&n, kern, &cfg) == cudaSuccess && n > 0;
        cudaGetLastError();  // a refused query leaves no error behind
        cache[dev][ksplit] = ok ? 1 : 2;
    }
    return cache[dev][ksplit] == 1;
}

// One launch of the kernel with BN = 64, 112 or 128 columns per tile; out and src are field formats (FMT_*).
int launch_bn64(const GemmArgs& g, dim3 grid, int out, int src, cudaStream_t st);
int launch_bn112(const GemmArgs& g, dim3 grid, int out, int src, cudaStream_t st);
int launch_bn128(const GemmArgs& g, dim3 grid, int out, int src, cudaStream_t st);

}  // namespace sg
}  // namespace hx
