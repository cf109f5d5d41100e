// One step of electric-field conjugation in one launch: the dark-zone gather of the focal-plane field, the
// product of the EFC matrix with [Re E_dz, Im E_dz] and the actuator update a - gain * (M . x), as in the loop of
// the reference's EFC tutorial (the update that util/matrix_inversion.py's Tikhonov inverse feeds).
//
// The work is split over thread-block clusters of kEfcSplit CTAs: a cluster updates kEfcRows actuators (rows of M,
// nact x 2 n_dz float64, row-major), each of its CTAs one slice of the dark-zone pixels.  The matrix is the
// traffic (952 x 6702 x 8 B = 51 MB for the 952-actuator, 3351-pixel dark zone) and streams from HBM once per
// step; each CTA gathers its slice of the field into shared memory as float-float pairs, so the scattered loads
// of the gather are shared by the cluster's rows and the row stream is plain coalesced loads.  The CTAs' partial
// sums meet in the first CTA's shared memory (distributed shared memory) and are added there in rank order.
// Products and sums run in float-float arithmetic on the FP32 pipe (the float64 inputs are split into hi + lo
// with integer operations), each thread adding its strided terms in order and each CTA combining its threads in
// a fixed tree, so the step is deterministic and keeps ~46 bits.
#include <cstdlib>

#include "hx_common.cuh"
#include "split_gemm.cuh"
#include "tc_ptx.cuh"

namespace {

using hx::sg::ff;
using hx::sg::ff_add;
using hx::sg::ff_mul;
using hx::sg::double_to_ff;
using hx::sg::ff_to_double;

constexpr int kEfcThreads = 128;
constexpr int kEfcRows = 4;
constexpr int kEfcSplit = 8;     // CTAs per cluster (pixel slices)
constexpr int kEfcChunk = 1024;  // pixels per shared-memory chunk: 1024 x 16 B = 16 KB

template <typename Cx>
__device__ __forceinline__ float4 field_ff(const Cx* e, int p);

template <>
__device__ __forceinline__ float4 field_ff<float2>(const float2* e, int p) {
    const float2 v = e[p];
    return make_float4(v.x, 0.0f, v.y, 0.0f);
}

template <>
__device__ __forceinline__ float4 field_ff<double2>(const double2* e, int p) {
    const double2 v = e[p];
    const ff re = double_to_ff(v.x), im = double_to_ff(v.y);
    return make_float4(re.hi, re.lo, im.hi, im.lo);
}

// SPLIT: CTAs per cluster (kEfcSplit, or 1 where clusters cannot be launched).
template <typename Cx, int SPLIT>
__global__ void __launch_bounds__(kEfcThreads) efc_step_kernel(const double* __restrict__ m, int nact, int n_dz,
                                                               const Cx* __restrict__ field,
                                                               const int* __restrict__ dz_index,
                                                               const double* __restrict__ act, ff gain,
                                                               double* __restrict__ act_out) {
    __shared__ float4 xs[kEfcChunk];
    __shared__ ff red[kEfcRows][kEfcThreads / 32];
    __shared__ __align__(16) ff part[SPLIT][kEfcRows];
    const int rank = (int)blockIdx.x % SPLIT;
    const int row0 = ((int)blockIdx.x / SPLIT) * kEfcRows;
    const int nrows = min(kEfcRows, nact - row0);
    const long long ld = 2LL * n_dz;
    const int p0 = (int)((long long)n_dz * rank / SPLIT), p1 = (int)((long long)n_dz * (rank + 1) / SPLIT);
    if constexpr (SPLIT > 1) hx::ptx::cluster_arrive_relaxed();  // first phase of the cluster barrier
    ff acc[kEfcRows];
#pragma unroll
    for (int q = 0; q < kEfcRows; ++q) acc[q] = {0.0f, 0.0f};
    for (int c0 = p0; c0 < p1; c0 += kEfcChunk) {
        const int clen = min(kEfcChunk, p1 - c0);
        if (c0 > p0) __syncthreads();  // the previous chunk is consumed
        for (int i = threadIdx.x; i < clen; i += kEfcThreads) xs[i] = field_ff<Cx>(field, __ldg(&dz_index[c0 + i]));
        __syncthreads();
#pragma unroll 2
        for (int i = threadIdx.x; i < clen; i += kEfcThreads) {
            double mre[kEfcRows], mim[kEfcRows];
#pragma unroll
            for (int q = 0; q < kEfcRows; ++q) {
                const double* mr = m + (long long)(row0 + min(q, nrows - 1)) * ld + c0 + i;
                mre[q] = __ldg(mr);
                mim[q] = __ldg(mr + n_dz);
            }
            const float4 x = xs[i];
            const ff xr = {x.x, x.y}, xi = {x.z, x.w};
#pragma unroll
            for (int q = 0; q < kEfcRows; ++q) {
                acc[q] = ff_add(acc[q], ff_mul(double_to_ff(mre[q]), xr));
                acc[q] = ff_add(acc[q], ff_mul(double_to_ff(mim[q]), xi));
            }
        }
    }
    // fixed tree: warps by shuffles, then the warp sums in order
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int q = 0; q < kEfcRows; ++q) {
        ff v = acc[q];
        for (int o = 16; o > 0; o >>= 1)
            v = ff_add(v, ff{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)});
        if (lane == 0) red[q][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < kEfcRows) {
        const int q = threadIdx.x;
        ff s = red[q][0];
        for (int w = 1; w < kEfcThreads / 32; ++w) s = ff_add(s, red[q][w]);
        red[q][0] = s;
    }
    if constexpr (SPLIT > 1) {
        // every CTA of the cluster has started (its shared memory exists) before the first remote store: the
        // barrier phase opened at the kernel's start; the CTA barrier orders red[] for thread 0
        __syncthreads();
        hx::ptx::cluster_wait();
        if (threadIdx.x == 0) {
            static_assert(kEfcRows == 4, "two 16-byte stores carry the four partial sums");
            const uint32_t dst = hx::ptx::map_shared_rank(hx::ptx::smem_addr(&part[rank][0]), 0);
            hx::ptx::st_cluster_v4(dst, make_float4(red[0][0].hi, red[0][0].lo, red[1][0].hi, red[1][0].lo));
            hx::ptx::st_cluster_v4(dst + 16, make_float4(red[2][0].hi, red[2][0].lo, red[3][0].hi, red[3][0].lo));
        }
        hx::ptx::cluster_sync();
        if (rank != 0) return;
    } else {
        __syncthreads();
        if (threadIdx.x < kEfcRows) part[0][threadIdx.x] = red[threadIdx.x][0];
        __syncthreads();
    }
    if (threadIdx.x < nrows) {
        const int q = threadIdx.x;
        ff s = part[0][q];
        for (int r = 1; r < SPLIT; ++r) s = ff_add(s, part[r][q]);
        const ff g = ff_mul(gain, s);
        const ff a = double_to_ff(act[row0 + q]);
        act_out[row0 + q] = ff_to_double(ff_add(a, ff{-g.hi, -g.lo}));
    }
}

template <typename Cx>
bool clusters_ok() {
    static int ok[64];  // per device: 0 unknown, 1 yes, 2 no
    static const bool off = [] {  // HX_NO_CLUSTERS=1: the one-CTA form (tests of that path)
        const char* e = getenv("HX_NO_CLUSTERS");
        return e && e[0] == '1';
    }();
    int dev = 0;
    if (off || cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
    if (!ok[dev]) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(kEfcSplit, 1, 1);
        cfg.blockDim = dim3(kEfcThreads);
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = kEfcSplit;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int n = 0;
        const bool good =
            cudaOccupancyMaxActiveClusters(&n, efc_step_kernel<Cx, kEfcSplit>, &cfg) == cudaSuccess && n > 0;
        cudaGetLastError();
        ok[dev] = good ? 1 : 2;
    }
    return ok[dev] == 1;
}

template <typename Cx>
int launch(const double* m, int nact, int n_dz, const void* field, const int* idx, const double* act, ff g,
           double* out, cudaStream_t st) {
    const unsigned blocks = (unsigned)hx::ceil_div(nact, kEfcRows);
    if (clusters_ok<Cx>()) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(blocks * kEfcSplit, 1, 1);
        cfg.blockDim = dim3(kEfcThreads);
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = kEfcSplit;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        HX_TRY(hx::cuda_status(cudaLaunchKernelEx(&cfg, efc_step_kernel<Cx, kEfcSplit>, m, nact, n_dz,
                                                  (const Cx*)field, idx, act, g, out),
                               "efc_step_kernel"));
    } else {
        efc_step_kernel<Cx, 1><<<blocks, kEfcThreads, 0, st>>>(m, nact, n_dz, (const Cx*)field, idx, act, g, out);
    }
    return hx::launch_status("efc_step_kernel");
}

}  // namespace

extern "C" {

int hx_efc_step(const double* efc_matrix, int nact, int n_dz, const void* field, int dtype, const int* dz_index,
                const double* actuators, double gain, double* actuators_out, void* stream) {
    HX_CHECK_ARG(nact >= 0 && n_dz >= 0, "hx_efc_step: sizes must not be negative (%d actuators, %d pixels)", nact,
                 n_dz);
    HX_CHECK_ARG(dtype == HX_C64 || dtype == HX_C128, "hx_efc_step: dtype must be HX_C64 or HX_C128");
    HX_CHECK_ARG(nact == 0 || (actuators && actuators_out), "hx_efc_step: NULL actuator pointer");
    HX_CHECK_ARG(n_dz == 0 || (efc_matrix && field && dz_index), "hx_efc_step: NULL matrix, field or index");
    if (nact == 0) return HX_OK;
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    cudaStream_t st = (cudaStream_t)stream;
    const float ghi = (float)gain;
    const ff g = {ghi, (float)(gain - (double)ghi)};
    hx::TraceScope trace(HX_TRACE_DM, (double)nact * 2.0 * n_dz * sizeof(double), st);
    if (dtype == HX_C128)
        return launch<double2>(efc_matrix, nact, n_dz, field, dz_index, actuators, g, actuators_out, st);
    return launch<float2>(efc_matrix, nact, n_dz, field, dz_index, actuators, g, actuators_out, st);
}

}  // extern "C"
