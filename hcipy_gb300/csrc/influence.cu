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
#include <cstdlib>

#include "hx_common.cuh"
#include "tc_ptx.cuh"

#include <cmath>

namespace {

constexpr int VC = 8;  // command vectors per thread (forward) / per CTA (transpose)

// Surface: one thread per pixel, VCF command vectors per CTA.  A CTA's 256 consecutive pixels are covered by a
// narrow range of actuator indices (the pokes within 3 pitches of a pupil row), so the CTA first copies that
// range of its VCF command vectors into shared memory, vector-minor (the VCF values of one actuator contiguous),
// and each nonzero then costs VCF/4 16-byte shared loads instead of VCF strided gathers.  The range comes from
// the first and last actuator of each row (CSR columns sorted); a nonzero outside it (unsorted input) or a
// range larger than the staging buffer reads the commands from global memory instead.
template <typename T> struct Stage;
template <> struct Stage<float> {
    static constexpr int VCF = 16;
    static constexpr int ELEMS = 8192;  // 32 KB: 512 actuators x 16 vectors
};
template <> struct Stage<double> {
    static constexpr int VCF = 8;
    static constexpr int ELEMS = 4096;  // 32 KB: 512 actuators x 8 vectors
};

template <typename T>
__global__ void __launch_bounds__(256) influence_apply_kernel(int npix, int nact, const int* __restrict__ row_ptr,
                                                              const int* __restrict__ col_idx,
                                                              const T* __restrict__ vals, int nvec,
                                                              const T* __restrict__ act, T* __restrict__ surf) {
    constexpr int VCF = Stage<T>::VCF;
    __shared__ __align__(16) T s_act[Stage<T>::ELEMS];
    __shared__ int s_lo[8], s_hi[8];
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int v0 = blockIdx.y * VCF;
    const int nv = min(VCF, nvec - v0);
    const int j0 = p < npix ? row_ptr[p] : 0;
    const int j1 = p < npix ? row_ptr[p + 1] : 0;
    int lo = j1 > j0 ? col_idx[j0] : 0x7fffffff;
    int hi = j1 > j0 ? col_idx[j1 - 1] : -1;
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        s_lo[warp] = lo;
        s_hi[warp] = hi;
    }
    __syncthreads();
    lo = s_lo[0];
    hi = s_hi[0];
    for (int w = 1; w < 8; ++w) {
        lo = min(lo, s_lo[w]);
        hi = max(hi, s_hi[w]);
    }
    const int na = hi - lo + 1;
    const bool staged = hi >= lo && lo >= 0 && hi < nact && (long long)na * VCF <= Stage<T>::ELEMS;
    if (staged) {
        // one 16-byte chunk (CH vectors of one actuator) per thread and step: consecutive threads read
        // consecutive actuators of a command vector (coalesced) and write chunks 16 x VCF / CH bytes apart
        constexpr int CH = 16 / sizeof(T);
        for (int k = threadIdx.x; k < na * (VCF / CH); k += blockDim.x) {
            const int q = k / na, a = k - q * na;
            T y[CH];
#pragma unroll
            for (int i = 0; i < CH; ++i) {
                const int v = q * CH + i;
                y[i] = v < nv ? act[(long long)(v0 + v) * nact + lo + a] : T(0);
            }
            if constexpr (sizeof(T) == 4)
                reinterpret_cast<float4*>(s_act)[a * (VCF / CH) + q] = make_float4(y[0], y[1], y[2], y[3]);
            else
                reinterpret_cast<double2*>(s_act)[a * (VCF / CH) + q] = make_double2(y[0], y[1]);
        }
    }
    __syncthreads();
    if (p >= npix) return;
    T acc[VCF];
#pragma unroll
    for (int v = 0; v < VCF; ++v) acc[v] = T(0);
    for (int j = j0; j < j1; ++j) {
        const int a = __ldg(&col_idx[j]);
        const T w = __ldg(&vals[j]);
        const unsigned al = (unsigned)(a - lo);
        if (staged && al < (unsigned)na) {
            const T* x = s_act + al * VCF;
            if constexpr (sizeof(T) == 4) {
#pragma unroll
                for (int q = 0; q < VCF / 4; ++q) {
                    const float4 y = reinterpret_cast<const float4*>(x)[q];
                    acc[4 * q] += w * y.x;
                    acc[4 * q + 1] += w * y.y;
                    acc[4 * q + 2] += w * y.z;
                    acc[4 * q + 3] += w * y.w;
                }
            } else {
#pragma unroll
                for (int q = 0; q < VCF / 2; ++q) {
                    const double2 y = reinterpret_cast<const double2*>(x)[q];
                    acc[2 * q] += w * y.x;
                    acc[2 * q + 1] += w * y.y;
                }
            }
        } else {
#pragma unroll
            for (int v = 0; v < VCF; ++v)
                if (v < nv) acc[v] += w * __ldg(&act[(long long)(v0 + v) * nact + a]);
        }
    }
#pragma unroll
    for (int v = 0; v < VCF; ++v)
        if (v < nv) surf[(long long)(v0 + v) * npix + p] = acc[v];
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

// Blocked transpose: kBA consecutive actuators (neighbours on the actuator grid for the reference's row-major
// actuator order) share one list, the union of their pixel supports, with kBA weights per listed pixel (zeros
// where an actuator does not reach), built at plan time from the CSC form.  Each gradient value gathered from
// L2 then serves the kBA actuators that overlap there instead of being gathered once per actuator (each pixel
// lies under ~23 Gaussian pokes).  A cluster of kTS CTAs takes one actuator block, each CTA one slice of its list
// and up to 8 * VW command vectors (warp w owns vectors w*VW ...): chunks of the list (pixel indices and
// weights) are staged in shared memory and every warp streams its vectors' gradient values over the chunk,
// lanes over consecutive list entries (coalesced).  The slices' partial sums meet in the first CTA's shared
// memory (distributed shared memory) and are added in rank order, so the result is deterministic.
constexpr int kBA = 4;
constexpr int kTS = 8;      // CTAs per cluster (list slices)
constexpr int kTChunk = 512;

template <typename T> struct BlockW;
template <> struct BlockW<float> {
    static constexpr int VW = 8;  // vectors per warp
    __device__ static void load(const float* w, float* out) {
        const float4 v = *reinterpret_cast<const float4*>(w);
        out[0] = v.x;
        out[1] = v.y;
        out[2] = v.z;
        out[3] = v.w;
    }
};
template <> struct BlockW<double> {
    static constexpr int VW = 4;
    __device__ static void load(const double* w, double* out) {
        const double2 a = reinterpret_cast<const double2*>(w)[0];
        const double2 b = reinterpret_cast<const double2*>(w)[1];
        out[0] = a.x;
        out[1] = a.y;
        out[2] = b.x;
        out[3] = b.y;
    }
};

template <typename T, int SPLIT>
__global__ void __launch_bounds__(256, 4) influence_transpose_blocked_kernel(
    int npix, int nact, const int* __restrict__ blk_ptr, const int* __restrict__ blk_pix,
    const T* __restrict__ blk_vals, int nvec, const T* __restrict__ g, T* __restrict__ g_act) {
    constexpr int VW = BlockW<T>::VW;
    constexpr int VPC = 8 * VW;  // vectors per CTA
    __shared__ int s_pix[kTChunk];
    __shared__ __align__(16) T s_w[kTChunk * kBA];
    __shared__ __align__(16) T part[SPLIT][VPC * kBA];
    const int b = (int)blockIdx.x / SPLIT, rank = (int)blockIdx.x % SPLIT;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int v0 = (int)blockIdx.y * VPC + warp * VW;
    const int nv = max(0, min(VW, nvec - v0));
    const int u0 = blk_ptr[b], u1 = blk_ptr[b + 1];
    const int e0 = u0 + (int)((long long)(u1 - u0) * rank / SPLIT);
    const int e1 = u0 + (int)((long long)(u1 - u0) * (rank + 1) / SPLIT);
    // first phase of the cluster barrier: arrive now, wait before the first remote store (every CTA has started)
    if constexpr (SPLIT > 1) hx::ptx::cluster_arrive_relaxed();
    T acc[VW][kBA];
#pragma unroll
    for (int v = 0; v < VW; ++v)
#pragma unroll
        for (int q = 0; q < kBA; ++q) acc[v][q] = T(0);
    for (int c0 = e0; c0 < e1; c0 += kTChunk) {
        const int clen = min(kTChunk, e1 - c0);
        if (c0 > e0) __syncthreads();  // the previous chunk is consumed
        for (int e = threadIdx.x; e < clen; e += blockDim.x) {
            s_pix[e] = __ldg(&blk_pix[c0 + e]);
#pragma unroll
            for (int q = 0; q < kBA; ++q) s_w[e * kBA + q] = __ldg(&blk_vals[(long long)(c0 + e) * kBA + q]);
        }
        __syncthreads();
        if (nv > 0) {
#pragma unroll 2
            for (int e = lane; e < clen; e += 32) {
                const int p = s_pix[e];
                T w[kBA];
                BlockW<T>::load(s_w + e * kBA, w);
                T x[VW];
#pragma unroll
                for (int v = 0; v < VW; ++v) x[v] = v < nv ? __ldg(&g[(long long)(v0 + v) * npix + p]) : T(0);
#pragma unroll
                for (int v = 0; v < VW; ++v)
#pragma unroll
                    for (int q = 0; q < kBA; ++q) acc[v][q] += w[q] * x[v];
            }
        }
    }
#pragma unroll
    for (int v = 0; v < VW; ++v)
#pragma unroll
        for (int q = 0; q < kBA; ++q)
            for (int o = 16; o > 0; o >>= 1) acc[v][q] += __shfl_xor_sync(0xffffffffu, acc[v][q], o);
    // partial sums of this warp's vectors: part[rank][(warp * VW + v) * kBA + q]
    if constexpr (SPLIT > 1) {
        hx::ptx::cluster_wait();  // every CTA of the cluster has started before the first remote store
        if (lane == 0) {
            const uint32_t dst = hx::ptx::map_shared_rank(hx::ptx::smem_addr(&part[rank][warp * VW * kBA]), 0);
#pragma unroll
            for (int v = 0; v < VW; ++v) {
#pragma unroll
                for (int c = 0; c < (int)(kBA * sizeof(T) / 16); ++c) {
                    const uint4 u = *reinterpret_cast<const uint4*>(&acc[v][c * (16 / sizeof(T))]);
                    asm volatile("st.shared::cluster.v4.u32 [%0], {%1, %2, %3, %4};" ::"r"(
                                     dst + (uint32_t)(v * kBA * sizeof(T) + 16 * c)),
                                 "r"(u.x), "r"(u.y), "r"(u.z), "r"(u.w)
                                 : "memory");
                }
            }
        }
        hx::ptx::cluster_sync();
        if (rank != 0) return;
    } else {
        if (lane == 0) {
#pragma unroll
            for (int v = 0; v < VW; ++v)
#pragma unroll
                for (int q = 0; q < kBA; ++q) part[0][(warp * VW + v) * kBA + q] = acc[v][q];
        }
        __syncthreads();
    }
    for (int t = threadIdx.x; t < VPC * kBA; t += blockDim.x) {
        const int vl = t / kBA, q = t % kBA;
        const int v = (int)blockIdx.y * VPC + vl, a = b * kBA + q;
        if (v < nvec && a < nact) {
            T y = part[0][t];
#pragma unroll
            for (int r = 1; r < SPLIT; ++r) y += part[r][t];
            g_act[(long long)v * nact + a] = y;
        }
    }
}

template <typename T>
bool transpose_clusters_ok() {
    static int ok[64];  // per device: 0 unknown, 1 yes, 2 no
    static const bool off = [] {  // HX_NO_CLUSTERS=1: the one-CTA form (tests of that path)
        const char* e = getenv("HX_NO_CLUSTERS");
        return e && e[0] == '1';
    }();
    int dev = 0;
    if (off || cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
    if (!ok[dev]) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(kTS, 1, 1);
        cfg.blockDim = dim3(256);
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = kTS;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int n = 0;
        const bool good =
            cudaOccupancyMaxActiveClusters(&n, influence_transpose_blocked_kernel<T, kTS>, &cfg) == cudaSuccess &&
            n > 0;
        cudaGetLastError();
        ok[dev] = good ? 1 : 2;
    }
    return ok[dev] == 1;
}

template <typename T>
int launch_transpose_blocked(int npix, int nact, const int* blk_ptr, const int* blk_pix, const void* blk_vals,
                             int nvec, const void* g, void* g_act, cudaStream_t st) {
    constexpr int VPC = 8 * BlockW<T>::VW;
    const int nblk = hx::ceil_div(nact, kBA);
    const unsigned gy = (unsigned)hx::ceil_div(nvec, VPC);
    if (transpose_clusters_ok<T>()) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)nblk * kTS, gy, 1);
        cfg.blockDim = dim3(256);
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = kTS;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        HX_TRY(hx::cuda_status(cudaLaunchKernelEx(&cfg, influence_transpose_blocked_kernel<T, kTS>, npix, nact,
                                                  blk_ptr, blk_pix, (const T*)blk_vals, nvec, (const T*)g,
                                                  (T*)g_act),
                               "influence_transpose_blocked_kernel"));
    } else {
        influence_transpose_blocked_kernel<T, 1><<<dim3((unsigned)nblk, gy), 256, 0, st>>>(
            npix, nact, blk_ptr, blk_pix, (const T*)blk_vals, nvec, (const T*)g, (T*)g_act);
    }
    return hx::launch_status("influence_transpose_blocked_kernel");
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
    const auto x = e[(long long)(b % batch_e) * n + i];
    if constexpr (sizeof(T) == 4) {
        out[(long long)b * n + i] = hx::phase_rotate(x, __fmul_rn(scale, s[(long long)(b % batch_s) * n + i]));
    } else {
        T sn, cs;
        sincos_t(scale * s[(long long)(b % batch_s) * n + i], &sn, &cs);
        out[(long long)b * n + i] = hx::make_c<T>(x.x * cs - x.y * sn, x.x * sn + x.y * cs);
    }
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
    const int vcf = dtype == HX_F32 ? Stage<float>::VCF : Stage<double>::VCF;
    HX_CHECK_ARG(hx::ceil_div(nvec, vcf) <= 65535, "hx_influence_apply: too many command vectors (%d)", nvec);
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    dim3 grid(hx::ceil_div(npix, 256), hx::ceil_div(nvec, vcf));
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

int hx_influence_apply_transpose_blocked(int npix, int nact, const int* blk_ptr, const int* blk_pix,
                                         const void* blk_vals, int dtype, int nvec, const void* g_surface,
                                         void* g_actuators, void* stream) {
    HX_CHECK_ARG(npix > 0 && nact > 0 && nvec > 0, "hx_influence_apply_transpose_blocked: sizes must be positive");
    HX_CHECK_ARG(blk_ptr && blk_pix && blk_vals && g_surface && g_actuators,
                 "hx_influence_apply_transpose_blocked: NULL pointer");
    HX_CHECK_ARG(dtype == HX_F32 || dtype == HX_F64,
                 "hx_influence_apply_transpose_blocked: dtype must be HX_F32 or HX_F64");
    HX_CHECK_ARG(((size_t)blk_vals & 15) == 0, "hx_influence_apply_transpose_blocked: blk_vals must be 16-byte aligned");
    const int vpc = dtype == HX_F32 ? 8 * BlockW<float>::VW : 8 * BlockW<double>::VW;
    HX_CHECK_ARG(hx::ceil_div(nvec, vpc) <= 65535, "hx_influence_apply_transpose_blocked: too many vectors (%d)", nvec);
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    const int nblk = hx::ceil_div(nact, kBA);
    cudaStream_t st = (cudaStream_t)stream;
    const double esz = dtype == HX_F32 ? 4.0 : 8.0;
    hx::TraceScope trace(HX_TRACE_DM, esz * ((double)nvec * (npix + nact)) + 4.0 * (nblk + 1), st);
    if (dtype == HX_F32)
        return launch_transpose_blocked<float>(npix, nact, blk_ptr, blk_pix, blk_vals, nvec, g_surface, g_actuators,
                                               st);
    return launch_transpose_blocked<double>(npix, nact, blk_ptr, blk_pix, blk_vals, nvec, g_surface, g_actuators,
                                            st);
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
