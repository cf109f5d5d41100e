// Complex GEMM on the CUDA cores: C = alpha * A . B (all row-major, strided batch).
//
// This is the plain drop-in arithmetic of the matrix Fourier transform
// (the reference calls BLAS cgemm/zgemm, hcipy/fourier/matrix_fourier_transform.py:154-172):
// complex64 operands with float32 accumulation, or complex128 with float64.
//
// Tiling: a CTA computes a BM x BN tile of C with 256 threads; each thread
// owns TM x TN complex accumulators at rows ty + i*NTY and columns
// tx + j*NTX (so a warp's B reads are 128-byte contiguous and its A reads are
// broadcasts).  K advances BK complex elements per stage through two shared
// memory stages; the next stage is fetched into registers while the current
// one is multiplied.  All edges are guarded, so any M, N, K and any leading
// dimension work (8-byte / 16-byte element alignment only).
#pragma once

#include "hx_common.cuh"

namespace hx {

// Fused epilogue of the last GEMM of a Fourier operator.
//   EPI_NONE   : C = alpha * acc
//   EPI_MUL    : C = alpha * acc * mask[f]          (focal-plane mask, apodizer)
//   EPI_BABINET: C = mask[f] * (src[i] - alpha*acc) (Babinet subtraction and Lyot stop;
//                                                    mask may be NULL = no stop)
// i is the element's own index in C, f its index inside one field:
// f = (row % rows_per_field) * ldc + col.
enum { EPI_NONE = 0, EPI_MUL = 1, EPI_BABINET = 2 };

template <typename Cx>
struct Epilogue {
    int kind = EPI_NONE;
    const Cx* mask = nullptr;
    const Cx* src = nullptr;
    long long rows_per_field = 1;
};

template <typename T, int BM, int BN, int BK, int TM, int TN>
struct SimtGemmCfg {
    static constexpr int NTX = BN / TN;
    static constexpr int NTY = BM / TM;
    static constexpr int THREADS = NTX * NTY;
    static_assert(THREADS == 256, "tile must map to 256 threads");
    static constexpr int A_PER_THREAD = BM * BK / THREADS;
    static constexpr int B_PER_THREAD = BK * BN / THREADS;
    static_assert(A_PER_THREAD >= 1 && B_PER_THREAD >= 1, "tile too small");
};

template <typename T, int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__(256)
cgemm_nn_simt(int M, int N, int K, typename cplx<T>::type alpha,
              const typename cplx<T>::type* __restrict__ A, long long lda, long long strideA,
              const typename cplx<T>::type* __restrict__ B, long long ldb, long long strideB,
              typename cplx<T>::type* __restrict__ C, long long ldc, long long strideC,
              Epilogue<typename cplx<T>::type> epi) {
    using Cx = typename cplx<T>::type;
    using Cfg = SimtGemmCfg<T, BM, BN, BK, TM, TN>;
    constexpr int NTX = Cfg::NTX;
    constexpr int NTY = Cfg::NTY;
    constexpr int AP = Cfg::A_PER_THREAD;
    constexpr int BP = Cfg::B_PER_THREAD;

    __shared__ Cx As[2][BK][BM];
    __shared__ Cx Bs[2][BK][BN];

    const int tid = threadIdx.x;
    const int tx = tid % NTX;
    const int ty = tid / NTX;
    const long long m0 = (long long)blockIdx.y * BM;
    const long long n0 = (long long)blockIdx.x * BN;

    A += strideA * blockIdx.z;
    B += strideB * blockIdx.z;
    C += strideC * blockIdx.z;

    // Global-load mapping: A tile (BM x BK) read row-wise, AP consecutive k per thread.
    constexpr int A_THREADS_PER_ROW = BK / AP;
    const int a_row = tid / A_THREADS_PER_ROW;
    const int a_col = (tid % A_THREADS_PER_ROW) * AP;
    // B tile (BK x BN) read row-wise, BP consecutive n per thread.
    constexpr int B_THREADS_PER_ROW = BN / BP;
    const int b_row = tid / B_THREADS_PER_ROW;
    const int b_col = (tid % B_THREADS_PER_ROW) * BP;

    const Cx zero = make_c<T>(T(0), T(0));
    Cx ra[AP];
    Cx rb[BP];

    auto load_tile = [&](int k0) {
        const long long gm = m0 + a_row;
#pragma unroll
        for (int i = 0; i < AP; ++i) {
            const int gk = k0 + a_col + i;
            ra[i] = (gm < M && gk < K) ? A[gm * lda + gk] : zero;
        }
        const int gk = k0 + b_row;
#pragma unroll
        for (int j = 0; j < BP; ++j) {
            const long long gn = n0 + b_col + j;
            rb[j] = (gk < K && gn < N) ? B[(long long)gk * ldb + gn] : zero;
        }
    };
    auto store_tile = [&](int s) {
#pragma unroll
        for (int i = 0; i < AP; ++i) As[s][a_col + i][a_row] = ra[i];
#pragma unroll
        for (int j = 0; j < BP; ++j) Bs[s][b_row][b_col + j] = rb[j];
    };

    Cx acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = zero;

    const int ktiles = (K + BK - 1) / BK;
    load_tile(0);
    store_tile(0);
    __syncthreads();

    for (int kt = 0; kt < ktiles; ++kt) {
        const int s = kt & 1;
        if (kt + 1 < ktiles) load_tile((kt + 1) * BK);
#pragma unroll
        for (int k = 0; k < BK; ++k) {
            Cx a[TM];
            Cx b[TN];
#pragma unroll
            for (int i = 0; i < TM; ++i) a[i] = As[s][k][ty + i * NTY];
#pragma unroll
            for (int j = 0; j < TN; ++j) b[j] = Bs[s][k][tx + j * NTX];
#pragma unroll
            for (int i = 0; i < TM; ++i)
#pragma unroll
                for (int j = 0; j < TN; ++j) {
                    acc[i][j].x = fma(a[i].x, b[j].x, acc[i][j].x);
                    acc[i][j].x = fma(-a[i].y, b[j].y, acc[i][j].x);
                    acc[i][j].y = fma(a[i].x, b[j].y, acc[i][j].y);
                    acc[i][j].y = fma(a[i].y, b[j].x, acc[i][j].y);
                }
        }
        if (kt + 1 < ktiles) {
            store_tile(s ^ 1);
        }
        __syncthreads();
    }

    const long long cbase = strideC * blockIdx.z;
#pragma unroll
    for (int i = 0; i < TM; ++i) {
        const long long gm = m0 + ty + i * NTY;
        if (gm >= M) continue;
        const long long frow = (gm % epi.rows_per_field) * ldc;
#pragma unroll
        for (int j = 0; j < TN; ++j) {
            const long long gn = n0 + tx + j * NTX;
            if (gn >= N) continue;
            Cx r = cmul(alpha, acc[i][j]);
            if (epi.kind == EPI_MUL) {
                r = cmul(r, epi.mask[frow + gn]);
            } else if (epi.kind == EPI_BABINET) {
                const Cx e = epi.src[cbase + gm * ldc + gn];
                r.x = e.x - r.x;
                r.y = e.y - r.y;
                if (epi.mask) r = cmul(r, epi.mask[frow + gn]);
            }
            C[gm * ldc + gn] = r;
        }
    }
}

// C[b] = alpha * A[b] . B[b] for b < batch, with A: M x K (lda), B: K x N (ldb), C: M x N (ldc).
template <typename T>
int cgemm_nn(int M, int N, int K, typename cplx<T>::type alpha,
             const typename cplx<T>::type* A, long long lda, long long strideA,
             const typename cplx<T>::type* B, long long ldb, long long strideB,
             typename cplx<T>::type* C, long long ldc, long long strideC,
             int batch, cudaStream_t stream, Epilogue<typename cplx<T>::type> epi = {}, bool throughput = false);

// Tile of C per CTA: the widest tile whose grid still gives every SM two CTAs, since a small transform on the
// widest tile would leave most of the 152 SMs idle (a 256^2 -> 128^2 MFT is 4 CTAs of 128 x 64).  Narrow tiles
// read more shared memory per FMA but occupy the GPU.  With throughput = true (concurrent transforms fill the GPU)
// the widest tile is kept.
inline int simt_tile_level(int M, int N, int batch, int levels, const int* bm, const int* bn) {
    const long long want = 2LL * num_sms();
    for (int l = 0; l < levels; ++l)
        if ((long long)ceil_div(N, bn[l]) * ceil_div(M, bm[l]) * batch >= want) return l;
    return levels - 1;
}

template <typename T, int BM, int BN, int BK, int TM, int TN>
int launch_simt(int M, int N, int K, typename cplx<T>::type alpha, const typename cplx<T>::type* A, long long lda,
                long long sA, const typename cplx<T>::type* B, long long ldb, long long sB,
                typename cplx<T>::type* C, long long ldc, long long sC, int batch, cudaStream_t stream,
                Epilogue<typename cplx<T>::type> epi) {
    dim3 grid(ceil_div(N, BN), ceil_div(M, BM), batch);
    if (grid.y > 65535u || batch > 65535) {
        set_error("cgemm: problem too large for one launch (M=%d, batch=%d)", M, batch);
        return HX_ERR_UNSUPPORTED;
    }
    TraceScope trace(HX_TRACE_SIMT_GEMM, (double)M * N * K * batch, stream);
    cgemm_nn_simt<T, BM, BN, BK, TM, TN><<<grid, 256, 0, stream>>>(M, N, K, alpha, A, lda, sA, B, ldb, sB, C, ldc,
                                                                   sC, epi);
    return launch_status(sizeof(T) == 4 ? "cgemm_nn_simt<float>" : "cgemm_nn_simt<double>");
}

template <>
inline int cgemm_nn<float>(int M, int N, int K, float2 alpha, const float2* A, long long lda, long long sA,
                           const float2* B, long long ldb, long long sB, float2* C, long long ldc, long long sC,
                           int batch, cudaStream_t stream, Epilogue<float2> epi, bool throughput) {
    static const int bm[3] = {128, 64, 32}, bn[3] = {64, 32, 32};
    switch (throughput ? 0 : simt_tile_level(M, N, batch, 3, bm, bn)) {
        case 0: return launch_simt<float, 128, 64, 8, 8, 4>(M, N, K, alpha, A, lda, sA, B, ldb, sB, C, ldc, sC, batch,
                                                             stream, epi);
        case 1: return launch_simt<float, 64, 32, 8, 4, 2>(M, N, K, alpha, A, lda, sA, B, ldb, sB, C, ldc, sC, batch,
                                                           stream, epi);
        default: return launch_simt<float, 32, 32, 8, 2, 2>(M, N, K, alpha, A, lda, sA, B, ldb, sB, C, ldc, sC, batch,
                                                            stream, epi);
    }
}

template <>
inline int cgemm_nn<double>(int M, int N, int K, double2 alpha, const double2* A, long long lda, long long sA,
                            const double2* B, long long ldb, long long sB, double2* C, long long ldc, long long sC,
                            int batch, cudaStream_t stream, Epilogue<double2> epi, bool throughput) {
    static const int bm[2] = {64, 32}, bn[2] = {64, 32};
    if (throughput || simt_tile_level(M, N, batch, 2, bm, bn) == 0)
        return launch_simt<double, 64, 64, 8, 4, 4>(M, N, K, alpha, A, lda, sA, B, ldb, sB, C, ldc, sC, batch, stream,
                                                    epi);
    return launch_simt<double, 32, 32, 8, 2, 2>(M, N, K, alpha, A, lda, sA, B, ldb, sB, C, ldc, sC, batch, stream,
                                                epi);
}

}  // namespace hx
