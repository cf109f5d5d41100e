// Infinite atmospheric layer on the device (hcipy/atmosphere/infinite_atmospheric_layer.py:216-364).
//
// The achromatic screen (ny x nx) lives in a ring buffer of (ny + 1) x (nx + 1) values: logical pixel (i, j) is
// stored at ((i + row0) mod (ny + 1), (j + col0) mod (nx + 1)).  The ring's spare row and spare column lie outside
// the logical screen; an extrusion (:216-259) moves an offset by one so that the spare slice becomes the new
// edge row or column and the slice that falls off becomes the spare.  The new slice is the autoregressive step
// A . stencil + B . noise; since it is written only into the spare slice, no stencil pixel of the same step is
// overwritten and the stencil is gathered by the same launch that writes (the reference copies the whole
// screen instead).  The extrusions of several layers (one step of each) run as one launch.  The quintic
// sub-pixel shift (hcipy/_math/subpixel_shift.py:7-343: 7-tap B-spline, clamp to edge, rows then columns) reads
// the rings and writes the layers' logical screens and their sum in one tiled pass.
#include <cstdlib>
#include <type_traits>

#include "hx_common.cuh"
#include "tc_ptx.cuh"

namespace {

// ---- extrusion ---------------------------------------------------------------------------------------------
// The new slice (nslice values) is A (nslice x nst) . stencil + B (nslice x nb) . noise.  A cluster of XS CTAs
// computes XRC (or 16) new pixels; CTA `rank` takes the rank-th eighth of the stencil columns and of the noise columns
// (split-K): it gathers only its part of the stencil through the ring mapping into shared memory and streams its
// column slice of the XRC rows of A and B (each warp XRC / 8 rows at once, 16-byte loads where the rows allow
// them).  The XS partial sums of each pixel meet in the first CTA's shared memory (distributed shared memory) and
// are added in rank order there, so the result is deterministic.  A and B stream from HBM once per step; the
// stencil is gathered once per cluster.
constexpr int XL_MAX = 8;       // extrusions per launch
constexpr int XS = 8;           // CTAs per cluster (column slices)
constexpr int XRC = 32;         // new pixels per cluster (16 when one wave of 32-pixel clusters would leave SMs idle)
constexpr int XTHREADS = 256;
constexpr int XCHUNK = 2048;    // stencil values staged per pass

template <typename T>
struct Extrusion {
    T* ring;
    const long long* idx;
    const T* A;
    const T* B;
    const T* noise;
    int ny, nx, row0, col0, where, nst, nb, nslice, block0;
};

template <typename T>
struct ExtrusionSet {
    Extrusion<T> l[XL_MAX];
    int count;
};

// Logical flat index k of the (possibly flipped) 1-D view -> physical index in the ring.
__device__ __forceinline__ long long ring_index(long long k, int ny, int nx, int row0, int col0, bool flip) {
    const long long n = (long long)ny * nx;
    if (flip) k = n - 1 - k;
    const int i = (int)(k / nx), j = (int)(k - (long long)(k / nx) * nx);
    int pi = i + row0, pj = j + col0;  // offsets are in [0, ny] / [0, nx]: one subtraction wraps them
    if (pi > ny) pi -= ny + 1;
    if (pj > nx) pj -= nx + 1;
    return (long long)pi * (nx + 1) + pj;
}

template <typename T> struct Vec16;
template <> struct Vec16<float> {
    using V = float4;
    static constexpr int N = 4;
    __device__ static float dot(const float4& a, const float4& b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
};
template <> struct Vec16<double> {
    using V = double2;
    static constexpr int N = 2;
    __device__ static double dot(const double2& a, const double2& b) { return a.x * b.x + a.y * b.y; }
};

// acc[q] += sum_k w_q[k] x[k] over k in [0, len) for the XRW rows w_q = w + q * ld (rows q >= nr are skipped),
// lanes strided; 16-byte loads when every row and x are aligned.
template <int XRW, typename T>
__device__ __forceinline__ void dot_rows(T* acc, const T* __restrict__ w, long long ld, int nr,
                                         const T* __restrict__ x, int len, int lane) {
    using VT = Vec16<T>;
    using V = typename VT::V;
    const bool vec = ((reinterpret_cast<size_t>(w) | reinterpret_cast<size_t>(x) |
                       (size_t)(ld * (long long)sizeof(T))) & 15) == 0;
    int k0 = 0;
    if (vec) {
        const int nv = len / VT::N;
        const V* xv = reinterpret_cast<const V*>(x);
#pragma unroll 2
        for (int q = lane; q < nv; q += 32) {
            const V xx = xv[q];
            V ww[XRW];
#pragma unroll
            for (int r = 0; r < XRW; ++r)
                if (r < nr) ww[r] = __ldg(reinterpret_cast<const V*>(w + r * ld) + q);
#pragma unroll
            for (int r = 0; r < XRW; ++r)
                if (r < nr) acc[r] += VT::dot(ww[r], xx);
        }
        k0 = VT::N * nv;
    }
    for (int k = k0 + lane; k < len; k += 32) {
        const T xx = x[k];
#pragma unroll
        for (int r = 0; r < XRW; ++r)
            if (r < nr) acc[r] += __ldg(&w[r * ld + k]) * xx;
    }
}

// Bounds of column slice s (of n) of [0, len): multiples of 4 elements, so that every slice keeps the alignment
// of the row it starts from.
__device__ __forceinline__ int slice_bound(int len, int s, int n) {
    return s >= n ? len : (int)(((long long)len * s / n) & ~3LL);
}

// 16-byte remote store of any 16 bytes (the bits travel unchanged).
template <typename T>
__device__ __forceinline__ void st_remote16(uint32_t addr, const T* v) {
    const uint4 u = *reinterpret_cast<const uint4*>(v);
    asm volatile("st.shared::cluster.v4.u32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(u.x), "r"(u.y), "r"(u.z),
                 "r"(u.w)
                 : "memory");
}

// SPLIT: CTAs per cluster (XS, or 1 where clusters cannot be launched); RC: new pixels per cluster (32 or 16).
// Six CTAs per SM for the float clusters (40 registers): the three 1024^2 layers' 768 CTAs fit in one wave.
template <typename T, int SPLIT, int RC>
__global__ void __launch_bounds__(XTHREADS, (sizeof(T) == 4 && SPLIT > 1) ? 6 : 1)
    extrude_layers_kernel(const __grid_constant__ ExtrusionSet<T> set) {
    constexpr int XRW = RC / (XTHREADS / 32);  // rows per warp
    __shared__ __align__(16) T st[XCHUNK];
    __shared__ __align__(16) T part[SPLIT][RC];
    int li = 0;
    for (int q = 1; q < set.count; ++q)
        if ((int)blockIdx.x >= set.l[q].block0) li = q;
    const Extrusion<T>& L = set.l[li];
    const int rank = SPLIT > 1 ? (int)((blockIdx.x - L.block0) % SPLIT) : 0;
    const int r0 = (int)((blockIdx.x - L.block0) / SPLIT) * RC;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rw = r0 + warp * XRW;                     // first row of this warp
    const int nr = max(0, min(XRW, L.nslice - rw));     // rows of this warp inside the slice
    const bool flip = L.where == 1 || L.where == 3;
    // first phase of the cluster barrier: arrive now, wait before the first remote store (every CTA has started)
    if constexpr (SPLIT > 1) hx::ptx::cluster_arrive_relaxed();
    T acc[XRW];
#pragma unroll
    for (int r = 0; r < XRW; ++r) acc[r] = T(0);
    const int s0 = slice_bound(L.nst, rank, SPLIT), s1 = slice_bound(L.nst, rank + 1, SPLIT);
    const int b0 = slice_bound(L.nb, rank, SPLIT), b1 = slice_bound(L.nb, rank + 1, SPLIT);
    // B . noise over this CTA's noise columns (independent of the stencil)
    if (nr > 0 && b1 > b0) dot_rows<XRW>(acc, L.B + (long long)rw * L.nb + b0, L.nb, nr, L.noise + b0, b1 - b0, lane);
    // A . stencil over this CTA's stencil columns, gathered through the ring in chunks
    for (int c0 = s0; c0 < s1; c0 += XCHUNK) {
        const int clen = min(XCHUNK, s1 - c0);
        if (c0 > s0) __syncthreads();  // the previous chunk is consumed
        for (int k = threadIdx.x; k < clen; k += XTHREADS)
            st[k] = L.ring[ring_index(__ldg(&L.idx[c0 + k]), L.ny, L.nx, L.row0, L.col0, flip)];
        __syncthreads();
        if (nr > 0) dot_rows<XRW>(acc, L.A + (long long)rw * L.nst + c0, L.nst, nr, st, clen, lane);
    }
#pragma unroll
    for (int r = 0; r < XRW; ++r)
        for (int o = 16; o > 0; o >>= 1) acc[r] += __shfl_xor_sync(0xffffffffu, acc[r], o);
    if constexpr (SPLIT > 1) {
        // every CTA of the cluster has started before the first remote store; the partial sums of this warp's
        // XRW rows go to the first CTA as 16-byte stores (one 8-byte store for two float rows)
        hx::ptx::cluster_wait();
        static_assert((XRW * sizeof(T)) % 8 == 0, "whole 8-byte stores");
        if (lane == 0) {
            const uint32_t dst = hx::ptx::map_shared_rank(hx::ptx::smem_addr(&part[rank][warp * XRW]), 0);
            if constexpr (XRW * sizeof(T) >= 16) {
#pragma unroll
                for (int c = 0; c < (int)(XRW * sizeof(T) / 16); ++c)
                    st_remote16(dst + 16 * c, acc + c * (16 / sizeof(T)));
            } else {
                const uint2 u = *reinterpret_cast<const uint2*>(acc);
                asm volatile("st.shared::cluster.v2.u32 [%0], {%1, %2};" ::"r"(dst), "r"(u.x), "r"(u.y) : "memory");
            }
        }
        hx::ptx::cluster_sync();
        if (rank != 0) return;
    } else {
        if (lane == 0) {
#pragma unroll
            for (int r = 0; r < XRW; ++r) part[0][warp * XRW + r] = acc[r];
        }
        __syncthreads();
    }
    const int rl = threadIdx.x;
    const int r = r0 + rl;
    if (rl >= RC || r >= L.nslice) return;
    T v = part[0][rl];
#pragma unroll
    for (int q = 1; q < SPLIT; ++q) v += part[q][rl];
    // Destination in logical coordinates after the shift: bottom -> row 0, top -> row ny-1 reversed,
    // left -> column 0, right -> column nx-1 reversed; with the offsets after the shift it lands in the slice
    // that was the spare one.
    const int ny = L.ny, nx = L.nx, w = L.where;
    int i, j;
    if (w == 0) { i = 0; j = r; }
    else if (w == 1) { i = ny - 1; j = nx - 1 - r; }
    else if (w == 2) { i = r; j = 0; }
    else { i = ny - 1 - r; j = nx - 1; }
    int nrow0 = L.row0, ncol0 = L.col0;
    if (w == 0) nrow0 = nrow0 == 0 ? ny : nrow0 - 1;
    else if (w == 1) nrow0 = nrow0 == ny ? 0 : nrow0 + 1;
    else if (w == 2) ncol0 = ncol0 == 0 ? nx : ncol0 - 1;
    else ncol0 = ncol0 == nx ? 0 : ncol0 + 1;
    int pi = i + nrow0, pj = j + ncol0;
    if (pi > ny) pi -= ny + 1;
    if (pj > nx) pj -= nx + 1;
    L.ring[(long long)pi * (nx + 1) + pj] = v;
}

template <typename T>
bool extrude_clusters_ok() {
    static int ok[64];  // per device: 0 unknown, 1 yes, 2 no
    static const bool off = [] {  // HX_NO_CLUSTERS=1: the one-CTA form (tests of that path)
        const char* e = getenv("HX_NO_CLUSTERS");
        return e && e[0] == '1';
    }();
    int dev = 0;
    if (off || cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
    if (!ok[dev]) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(XS, 1, 1);
        cfg.blockDim = dim3(XTHREADS);
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = XS;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int n = 0;
        const bool good =
            cudaOccupancyMaxActiveClusters(&n, extrude_layers_kernel<T, XS, XRC>, &cfg) == cudaSuccess && n > 0;
        cudaGetLastError();
        ok[dev] = good ? 1 : 2;
    }
    return ok[dev] == 1;
}

// ---- sub-pixel shift and the sum of the layers' screens ------------------------------------------------------
// A 32 x 32 output tile per CTA of 32 x 8 threads: the 38 x 38 input tile (clamped to the logical screen,
// wrapped through the ring) in shared memory, the row filter into a 38 x 32 tile, the column filter to the
// output; thread (tx, ty) owns column tx of rows ty + 8 m.  Layers one after the other, their filtered tiles
// summed in registers in layer order.
constexpr int SL_MAX = 8;
constexpr int TS = 32;
constexpr int HALO = 3;
constexpr int TIN = TS + 2 * HALO;

template <typename T>
struct ShiftSet {
    const T* ring[SL_MAX];
    T* out[SL_MAX];
    int row0[SL_MAX], col0[SL_MAX];
    T taps_row[SL_MAX][7];  // along x (within a row), rounded to T on the host
    T taps_col[SL_MAX][7];  // along y (within a column)
    T* sum;
    int count, ring_ny, ring_nx, ny, nx;
};

template <typename T>
__global__ void __launch_bounds__(256) shift_layers_kernel(const __grid_constant__ ShiftSet<T> set) {
    __shared__ T in[TIN][TIN];
    __shared__ T mid[TIN][TS];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x0 = blockIdx.x * TS, y0 = blockIdx.y * TS;
    const int ny = set.ny, nx = set.nx;
    T total[4] = {T(0), T(0), T(0), T(0)};
    for (int l = 0; l < set.count; ++l) {
        const T* ring = set.ring[l];
        const int row0 = set.row0[l], col0 = set.col0[l];
        // columns of the input tile this thread loads: tx and tx + 32 (< TIN)
        int px[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int gx = min(max(x0 + tx + 32 * h - HALO, 0), nx - 1);
            int p = gx + col0;
            if (p >= set.ring_nx) p -= set.ring_nx;
            px[h] = p;
        }
        for (int ly = ty; ly < TIN; ly += 8) {
            const int gy = min(max(y0 + ly - HALO, 0), ny - 1);
            int py = gy + row0;
            if (py >= set.ring_ny) py -= set.ring_ny;
            const T* rrow = ring + (long long)py * set.ring_nx;
            in[ly][tx] = rrow[px[0]];
            if (tx + 32 < TIN) in[ly][tx + 32] = rrow[px[1]];
        }
        T wr[7], wc[7];
#pragma unroll
        for (int k = 0; k < 7; ++k) {
            wr[k] = set.taps_row[l][k];
            wc[k] = set.taps_col[l][k];
        }
        __syncthreads();
        for (int ly = ty; ly < TIN; ly += 8) {
            T s = T(0);
#pragma unroll
            for (int k = 0; k < 7; ++k) s += in[ly][tx + k] * wr[k];
            mid[ly][tx] = s;
        }
        __syncthreads();
        T* out = set.out[l];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            const int y = ty + 8 * m;
            T s = T(0);
#pragma unroll
            for (int k = 0; k < 7; ++k) s += mid[y + k][tx] * wc[k];
            total[m] = l == 0 ? s : total[m] + s;
            if (out && y0 + y < ny && x0 + tx < nx) out[(long long)(y0 + y) * nx + x0 + tx] = s;
        }
    }
    if (set.sum) {
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            const int y = ty + 8 * m;
            if (y0 + y < ny && x0 + tx < nx) set.sum[(long long)(y0 + y) * nx + x0 + tx] = total[m];
        }
    }
}

// out = sum of up to HX_MAX_SCREENS screens (the combined phase of layers applied without propagation between
// them); 4 elements per thread where the pointers allow 16-byte access.
constexpr int MAX_SCREENS = 8;
template <typename T>
struct ScreenSet {
    const T* s[MAX_SCREENS];
};

template <typename T>
__global__ void combine_screens_kernel(const __grid_constant__ ScreenSet<T> set, int count, long long n, T* out) {
    const long long i = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * 4;
    if (i >= n) return;
    if (i + 4 <= n) {
        T a0 = set.s[0][i], a1 = set.s[0][i + 1], a2 = set.s[0][i + 2], a3 = set.s[0][i + 3];
        for (int l = 1; l < count; ++l) {
            const T* p = set.s[l] + i;
            a0 += p[0];
            a1 += p[1];
            a2 += p[2];
            a3 += p[3];
        }
        out[i] = a0;
        out[i + 1] = a1;
        out[i + 2] = a2;
        out[i + 3] = a3;
    } else {
        for (long long k = i; k < n; ++k) {
            T a = set.s[0][k];
            for (int l = 1; l < count; ++l) a += set.s[l][k];
            out[k] = a;
        }
    }
}

}  // namespace

extern "C" {

int hx_atmosphere_extrude_layers(const hx_extrusion* steps, int count, int dtype, void* stream) {
    HX_CHECK_ARG(steps || count == 0, "hx_atmosphere_extrude_layers: NULL steps");
    HX_CHECK_ARG(count >= 0 && count <= XL_MAX, "hx_atmosphere_extrude_layers: count must be 0..%d (got %d)", XL_MAX,
                 count);
    HX_CHECK_ARG(dtype == HX_F32 || dtype == HX_F64, "hx_atmosphere_extrude_layers: dtype must be HX_F32 or HX_F64");
    for (int l = 0; l < count; ++l) {
        const hx_extrusion& e = steps[l];
        HX_CHECK_ARG(e.ring && e.stencil_idx && e.A && e.B && e.noise, "hx_atmosphere_extrude: NULL pointer (step %d)",
                     l);
        HX_CHECK_ARG(e.ny > 0 && e.nx > 0 && e.nst > 0 && e.nb > 0, "hx_atmosphere_extrude: sizes must be positive");
        HX_CHECK_ARG(e.where >= 0 && e.where <= 3,
                     "hx_atmosphere_extrude: where must be 0..3 (bottom, top, left, right)");
        HX_CHECK_ARG(e.row0 >= 0 && e.row0 <= e.ny && e.col0 >= 0 && e.col0 <= e.nx,
                     "hx_atmosphere_extrude: ring offsets out of range (row0 in [0, ny], col0 in [0, nx])");
        for (int q = 0; q < l; ++q)
            HX_CHECK_ARG(steps[q].ring != e.ring, "hx_atmosphere_extrude_layers: ring %d appears twice in one launch",
                         l);
    }
    if (count == 0) return HX_OK;
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t esz = dtype == HX_F32 ? 4 : 8;
    auto run = [&](auto* tag) -> int {
        using T = std::remove_pointer_t<decltype(tag)>;
        const bool cl = extrude_clusters_ok<T>();
        const int split = cl ? XS : 1;
        // float: 16-pixel clusters when they still fit in one wave (six CTAs per SM), so a single 1024-pixel
        // extrusion runs 512 CTAs instead of 256
        int rc = XRC;
        if (cl && sizeof(T) == 4) {
            int dev = 0, sms = 0;
            long long c16 = 0;
            for (int l = 0; l < count; ++l) c16 += hx::ceil_div(steps[l].where <= 1 ? steps[l].nx : steps[l].ny, 16);
            if (cudaGetDevice(&dev) == cudaSuccess &&
                cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
                c16 * XS <= 6LL * sms)
                rc = 16;
        }
        ExtrusionSet<T> set{};
        double bytes = 0.0;
        int b0 = 0;
        for (int l = 0; l < count; ++l) {
            const hx_extrusion& e = steps[l];
            auto& d = set.l[l];
            d.ring = (T*)e.ring;
            d.idx = e.stencil_idx;
            d.A = (const T*)e.A;
            d.B = (const T*)e.B;
            d.noise = (const T*)e.noise;
            d.ny = e.ny;
            d.nx = e.nx;
            d.row0 = e.row0;
            d.col0 = e.col0;
            d.where = e.where;
            d.nst = e.nst;
            d.nb = e.nb;
            d.nslice = e.where <= 1 ? e.nx : e.ny;
            d.block0 = b0;
            b0 += hx::ceil_div(d.nslice, rc) * split;
            bytes += (double)esz * ((double)d.nslice * (e.nst + e.nb) + d.nslice) + (esz + 8.0) * e.nst + esz * e.nb;
        }
        set.count = count;
        hx::TraceScope trace(HX_TRACE_ATMOSPHERE, bytes, st);
        if (cl) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3((unsigned)b0, 1, 1);
            cfg.blockDim = dim3(XTHREADS);
            cfg.stream = st;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = XS;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            if (rc == 16)
                HX_TRY(hx::cuda_status(cudaLaunchKernelEx(&cfg, extrude_layers_kernel<T, XS, 16>, set),
                                       "extrude_layers_kernel"));
            else
                HX_TRY(hx::cuda_status(cudaLaunchKernelEx(&cfg, extrude_layers_kernel<T, XS, XRC>, set),
                                       "extrude_layers_kernel"));
        } else {
            extrude_layers_kernel<T, 1, XRC><<<(unsigned)b0, XTHREADS, 0, st>>>(set);
        }
        return hx::launch_status("extrude_layers_kernel");
    };
    return dtype == HX_F32 ? run((float*)nullptr) : run((double*)nullptr);
}

int hx_atmosphere_extrude(void* ring, int ny, int nx, int row0, int col0, int where, const long long* stencil_idx,
                          int nst, const void* A, const void* B, int nb, const void* noise, int dtype, void* stream) {
    hx_extrusion e{ring, stencil_idx, A, B, noise, ny, nx, row0, col0, where, nst, nb};
    return hx_atmosphere_extrude_layers(&e, 1, dtype, stream);
}

int hx_atmosphere_shift_layers(const void* const* rings, int count, int ring_ny, int ring_nx, int ny, int nx,
                               const int* row0, const int* col0, const double* taps_row, const double* taps_col,
                               void* const* outs, void* sum, int dtype, void* stream) {
    HX_CHECK_ARG(rings && row0 && col0 && taps_row && taps_col, "hx_atmosphere_shift: NULL pointer");
    HX_CHECK_ARG(count >= 1 && count <= SL_MAX, "hx_atmosphere_shift_layers: count must be 1..%d (got %d)", SL_MAX,
                 count);
    HX_CHECK_ARG(ny > 0 && nx > 0 && ring_ny >= ny && ring_nx >= nx,
                 "hx_atmosphere_shift: sizes must be positive and the ring at least ny x nx");
    HX_CHECK_ARG(dtype == HX_F32 || dtype == HX_F64, "hx_atmosphere_shift: dtype must be HX_F32 or HX_F64");
    bool any_out = sum != nullptr;
    for (int l = 0; l < count; ++l) {
        HX_CHECK_ARG(rings[l], "hx_atmosphere_shift: NULL ring %d", l);
        HX_CHECK_ARG(row0[l] >= 0 && row0[l] < ring_ny && col0[l] >= 0 && col0[l] < ring_nx,
                     "hx_atmosphere_shift: ring offsets out of range");
        any_out = any_out || (outs && outs[l]);
    }
    HX_CHECK_ARG(any_out, "hx_atmosphere_shift_layers: no output");
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    dim3 grid(hx::ceil_div(nx, TS), hx::ceil_div(ny, TS));
    dim3 block(32, 8);
    cudaStream_t st = (cudaStream_t)stream;
    int nout = sum != nullptr;
    for (int l = 0; l < count; ++l) nout += outs && outs[l];
    hx::TraceScope trace(HX_TRACE_ATMOSPHERE, (double)(count + nout) * (dtype == HX_F32 ? 4 : 8) * nx * ny, st);
    auto fill = [&](auto& set) {
        using T = std::remove_pointer_t<decltype(set.sum)>;
        for (int l = 0; l < count; ++l) {
            set.ring[l] = (const T*)rings[l];
            set.out[l] = outs ? (T*)outs[l] : nullptr;
            set.row0[l] = row0[l];
            set.col0[l] = col0[l];
            for (int k = 0; k < 7; ++k) {  // float taps round to nearest, as a device conversion would
                set.taps_row[l][k] = (T)taps_row[7 * l + k];
                set.taps_col[l][k] = (T)taps_col[7 * l + k];
            }
        }
        set.sum = (T*)sum;
        set.count = count;
        set.ring_ny = ring_ny;
        set.ring_nx = ring_nx;
        set.ny = ny;
        set.nx = nx;
    };
    if (dtype == HX_F32) {
        ShiftSet<float> set{};
        fill(set);
        shift_layers_kernel<float><<<grid, block, 0, st>>>(set);
    } else {
        ShiftSet<double> set{};
        fill(set);
        shift_layers_kernel<double><<<grid, block, 0, st>>>(set);
    }
    return hx::launch_status("shift_layers_kernel");
}

int hx_atmosphere_shift(const void* ring, int ring_ny, int ring_nx, int ny, int nx, int row0, int col0,
                        const double* taps_row, const double* taps_col, void* out, int dtype, void* stream) {
    HX_CHECK_ARG(ring && out, "hx_atmosphere_shift: NULL pointer");
    void* outs[1] = {out};
    return hx_atmosphere_shift_layers(&ring, 1, ring_ny, ring_nx, ny, nx, &row0, &col0, taps_row, taps_col, outs,
                                      nullptr, dtype, stream);
}

int hx_atmosphere_combine(const void* const* screens, int count, long long n, void* out, int dtype, void* stream) {
    HX_CHECK_ARG(screens && out, "hx_atmosphere_combine: NULL pointer");
    HX_CHECK_ARG(count >= 1 && count <= MAX_SCREENS, "hx_atmosphere_combine: count must be 1..8");
    HX_CHECK_ARG(n > 0, "hx_atmosphere_combine: n must be positive");
    HX_CHECK_ARG(dtype == HX_F32 || dtype == HX_F64, "hx_atmosphere_combine: dtype must be HX_F32 or HX_F64");
    for (int l = 0; l < count; ++l) HX_CHECK_ARG(screens[l], "hx_atmosphere_combine: NULL screen");
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned blocks = (unsigned)hx::ceil_div((n + 3) / 4, 256);
    hx::TraceScope trace(HX_TRACE_ATMOSPHERE, (double)(count + 1) * (dtype == HX_F32 ? 4 : 8) * (double)n, st);
    if (dtype == HX_F32) {
        ScreenSet<float> set{};
        for (int l = 0; l < count; ++l) set.s[l] = (const float*)screens[l];
        combine_screens_kernel<float><<<blocks, 256, 0, st>>>(set, count, n, (float*)out);
    } else {
        ScreenSet<double> set{};
        for (int l = 0; l < count; ++l) set.s[l] = (const double*)screens[l];
        combine_screens_kernel<double><<<blocks, 256, 0, st>>>(set, count, n, (double*)out);
    }
    return hx::launch_status("combine_screens_kernel");
}

}  // extern "C"
