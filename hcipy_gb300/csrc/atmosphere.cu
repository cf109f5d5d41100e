// Infinite atmospheric layer on the device (hcipy/atmosphere/infinite_atmospheric_layer.py:216-364).
//
// The achromatic screen (ny x nx) lives in a ring buffer: logical pixel (i, j) is stored at
// ((i + row0) mod ny, (j + col0) mod nx).  An extrusion (:216-259) moves an offset by one and writes the new
// row or column into the slot that the shift frees, instead of copying the whole screen as the reference
// does.  The new slice is the autoregressive step  A . stencil + B . noise  (one warp per new pixel), with the
// stencil gathered through the ring mapping and the flat reversal the reference applies for 'top'/'right'.
// The quintic sub-pixel shift (hcipy/_math/subpixel_shift.py:7-343: 7-tap B-spline, clamp to edge, rows then
// columns) reads the ring and writes the logical screen in one tiled pass.
#include "hx_common.cuh"

namespace {

// Logical flat index of the (possibly flipped) 1-D view -> physical flat index of the ring.
__device__ __forceinline__ long long ring_index(long long k, int ny, int nx, int row0, int col0, bool flip) {
    const long long n = (long long)ny * nx;
    if (flip) k = n - 1 - k;
    const int i = (int)(k / nx), j = (int)(k % nx);
    const int pi = (i + row0) % ny, pj = (j + col0) % nx;
    return (long long)pi * nx + pj;
}

// Stencil values of the screen before the step (the logical 1-D view, flipped for 'top'/'right').  A separate
// launch from the update below: the new slice overwrites a ring slot that a far stencil pixel may occupy.
template <typename T>
__global__ void gather_stencil_kernel(const T* ring, int ny, int nx, int row0, int col0, bool flip,
                                      const long long* stencil_idx, int nst, T* stencil) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nst) stencil[k] = ring[ring_index(stencil_idx[k], ny, nx, row0, col0, flip)];
}

// new_slice[r] = sum_k A[r, k] stencil[k] + sum_k B[r, k] noise[k], written into the ring slot that the shift
// frees.  where: 0 bottom, 1 top, 2 left, 3 right; row0/col0 are the offsets before the step.  A CTA of 256
// threads computes 2 rows with 4 warps per row, each warp a quarter of the stencil and of the noise, with
// 16-byte loads when the rows allow them: A and B stream from HBM once per step, so the kernel is sized for
// many requests in flight (512 CTAs for a 1024-pixel slice) and starts loading at once (no staging).
constexpr int EXT_ROWS = 2;      // rows per CTA
constexpr int EXT_WARPS_ROW = 4; // warps per row

template <typename T>
__device__ __forceinline__ T dot_part(const T* __restrict__ w, const T* __restrict__ x, int n, int part, int lane) {
    // Elements [part * n / 4, (part + 1) * n / 4) of w . x, lanes strided; x (the stencil or the noise, a few
    // KB shared by every CTA) is read through L1/L2 like w.
    const int k0 = (int)((long long)n * part / EXT_WARPS_ROW);
    const int k1 = (int)((long long)n * (part + 1) / EXT_WARPS_ROW);
    T acc = T(0);
    if (sizeof(T) == 4 && ((k0 & 3) == 0) && ((reinterpret_cast<size_t>(w + k0) & 15) == 0) &&
        ((reinterpret_cast<size_t>(x + k0) & 15) == 0)) {
        const int n4 = (k1 - k0) >> 2;
        const float4* w4 = reinterpret_cast<const float4*>(w + k0);
        const float4* x4 = reinterpret_cast<const float4*>(x + k0);
#pragma unroll 4
        for (int q = lane; q < n4; q += 32) {
            const float4 a = __ldg(&w4[q]);
            const float4 b = __ldg(&x4[q]);
            acc += (T)(a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w);
        }
        for (int k = k0 + 4 * n4 + lane; k < k1; k += 32) acc += w[k] * x[k];
    } else {
#pragma unroll 4
        for (int k = k0 + lane; k < k1; k += 32) acc += __ldg(&w[k]) * __ldg(&x[k]);
    }
    return acc;
}

template <typename T>
__global__ void extrude_kernel(T* ring, int ny, int nx, int row0, int col0, int where, const T* stencil, int nst,
                               const T* A, const T* B, int nb, const T* noise, int nslice) {
    __shared__ T part_sum[EXT_ROWS][EXT_WARPS_ROW];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rl = warp / EXT_WARPS_ROW, part = warp % EXT_WARPS_ROW;
    const int r = blockIdx.x * EXT_ROWS + rl;
    T acc = T(0);
    if (r < nslice) {
        acc = dot_part(A + (long long)r * nst, stencil, nst, part, lane) +
              dot_part(B + (long long)r * nb, noise, nb, part, lane);
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    }
    if (lane == 0) part_sum[rl][part] = acc;
    __syncthreads();
    if (part != 0 || lane != 0 || r >= nslice) return;
    acc = part_sum[rl][0] + part_sum[rl][1] + part_sum[rl][2] + part_sum[rl][3];
    // Destination in logical coordinates after the shift: bottom -> row 0, top -> row ny-1 reversed,
    // left -> column 0, right -> column nx-1 reversed.
    int i, j;
    if (where == 0) { i = 0; j = r; }
    else if (where == 1) { i = ny - 1; j = nx - 1 - r; }
    else if (where == 2) { i = r; j = 0; }
    else { i = ny - 1 - r; j = nx - 1; }
    // Offsets after the shift.
    int nr = row0, nc = col0;
    if (where == 0) nr = (row0 + ny - 1) % ny;
    else if (where == 1) nr = (row0 + 1) % ny;
    else if (where == 2) nc = (col0 + nx - 1) % nx;
    else nc = (col0 + 1) % nx;
    ring[(long long)((i + nr) % ny) * nx + (j + nc) % nx] = acc;
}

struct Taps {
    double row[7];  // applied along x (within a row)
    double col[7];  // applied along y (within a column)
};

constexpr int TS = 32;       // output tile
constexpr int HALO = 3;      // 7-tap kernel
constexpr int TIN = TS + 2 * HALO;

// Separable 7-tap filter with clamp-to-edge of the logical screen read from the ring; out is logical.
template <typename T>
__global__ void ring_shift_kernel(const T* ring, int ny, int nx, int row0, int col0, Taps taps, T* out) {
    __shared__ T in[TIN][TIN + 1];
    __shared__ T mid[TIN][TS + 1];
    __shared__ T wr[7], wc[7];  // taps in the working type, converted once
    const int x0 = blockIdx.x * TS, y0 = blockIdx.y * TS;
    if (threadIdx.y == 0 && threadIdx.x < 7) {
        wr[threadIdx.x] = (T)taps.row[threadIdx.x];
        wc[threadIdx.x] = (T)taps.col[threadIdx.x];
    }
    for (int t = threadIdx.y * blockDim.x + threadIdx.x; t < TIN * TIN; t += blockDim.x * blockDim.y) {
        const int ly = t / TIN, lx = t % TIN;
        const int gy = min(max(y0 + ly - HALO, 0), ny - 1);
        const int gx = min(max(x0 + lx - HALO, 0), nx - 1);
        int py = gy + row0, px = gx + col0;  // offsets are in [0, n): one subtraction wraps them
        if (py >= ny) py -= ny;
        if (px >= nx) px -= nx;
        in[ly][lx] = ring[(long long)py * nx + px];
    }
    __syncthreads();
    // rows: mid[ly][x] = sum_k in[ly][x + k] * row[k]
    for (int t = threadIdx.y * blockDim.x + threadIdx.x; t < TIN * TS; t += blockDim.x * blockDim.y) {
        const int ly = t / TS, x = t % TS;
        T s = T(0);
#pragma unroll
        for (int k = 0; k < 7; ++k) s += in[ly][x + k] * wr[k];
        mid[ly][x] = s;
    }
    __syncthreads();
    for (int t = threadIdx.y * blockDim.x + threadIdx.x; t < TS * TS; t += blockDim.x * blockDim.y) {
        const int y = t / TS, x = t % TS;
        if (y0 + y >= ny || x0 + x >= nx) continue;
        T s = T(0);
#pragma unroll
        for (int k = 0; k < 7; ++k) s += mid[y + k][x] * wc[k];
        out[(long long)(y0 + y) * nx + x0 + x] = s;
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
__global__ void combine_screens_kernel(ScreenSet<T> set, int count, long long n, T* out) {
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

int hx_atmosphere_extrude(void* ring, int ny, int nx, int row0, int col0, int where, const long long* stencil_idx,
                          int nst, const void* A, const void* B, int nb, const void* noise, int dtype, void* work,
                          void* stream) {
    HX_CHECK_ARG(ring && stencil_idx && A && B && noise && work, "hx_atmosphere_extrude: NULL pointer");
    HX_CHECK_ARG(ny > 0 && nx > 0 && nst > 0 && nb > 0, "hx_atmosphere_extrude: sizes must be positive");
    HX_CHECK_ARG(where >= 0 && where <= 3, "hx_atmosphere_extrude: where must be 0..3 (bottom, top, left, right)");
    HX_CHECK_ARG(row0 >= 0 && row0 < ny && col0 >= 0 && col0 < nx, "hx_atmosphere_extrude: ring offsets out of range");
    HX_CHECK_ARG(dtype == HX_F32 || dtype == HX_F64, "hx_atmosphere_extrude: dtype must be HX_F32 or HX_F64");
    const int nslice = (where <= 1) ? nx : ny;
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    cudaStream_t st = (cudaStream_t)stream;
    const bool flip = where == 1 || where == 3;
    const int threads = 32 * EXT_ROWS * EXT_WARPS_ROW;
    dim3 grid(hx::ceil_div(nslice, EXT_ROWS));
    if (dtype == HX_F32) {
        gather_stencil_kernel<float><<<hx::ceil_div(nst, 256), 256, 0, st>>>((const float*)ring, ny, nx, row0, col0,
                                                                             flip, stencil_idx, nst, (float*)work);
        HX_TRY(hx::launch_status("gather_stencil_kernel"));
        hx::TraceScope trace(HX_TRACE_ATMOSPHERE, 4.0 * ((double)nslice * (nst + nb) + nst + nb), st);
        extrude_kernel<float><<<grid, threads, 0, st>>>((float*)ring, ny, nx, row0, col0, where,
                                                          (const float*)work, nst, (const float*)A, (const float*)B,
                                                          nb, (const float*)noise, nslice);
    } else {
        gather_stencil_kernel<double><<<hx::ceil_div(nst, 256), 256, 0, st>>>((const double*)ring, ny, nx, row0,
                                                                              col0, flip, stencil_idx, nst,
                                                                              (double*)work);
        HX_TRY(hx::launch_status("gather_stencil_kernel"));
        hx::TraceScope trace(HX_TRACE_ATMOSPHERE, 8.0 * ((double)nslice * (nst + nb) + nst + nb), st);
        extrude_kernel<double><<<grid, threads, 0, st>>>((double*)ring, ny, nx, row0, col0, where,
                                                           (const double*)work, nst, (const double*)A,
                                                           (const double*)B, nb, (const double*)noise, nslice);
    }
    return hx::launch_status("extrude_kernel");
}

int hx_atmosphere_shift(const void* ring, int ny, int nx, int row0, int col0, const double* taps_row,
                        const double* taps_col, void* out, int dtype, void* stream) {
    HX_CHECK_ARG(ring && taps_row && taps_col && out, "hx_atmosphere_shift: NULL pointer");
    HX_CHECK_ARG(ny > 0 && nx > 0, "hx_atmosphere_shift: sizes must be positive");
    HX_CHECK_ARG(row0 >= 0 && row0 < ny && col0 >= 0 && col0 < nx, "hx_atmosphere_shift: ring offsets out of range");
    HX_CHECK_ARG(dtype == HX_F32 || dtype == HX_F64, "hx_atmosphere_shift: dtype must be HX_F32 or HX_F64");
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    Taps t;
    for (int k = 0; k < 7; ++k) {
        t.row[k] = taps_row[k];
        t.col[k] = taps_col[k];
    }
    dim3 grid(hx::ceil_div(nx, TS), hx::ceil_div(ny, TS));
    dim3 block(32, 8);
    cudaStream_t st = (cudaStream_t)stream;
    hx::TraceScope trace(HX_TRACE_ATMOSPHERE, 2.0 * (dtype == HX_F32 ? 4 : 8) * (double)nx * ny, st);
    if (dtype == HX_F32)
        ring_shift_kernel<float><<<grid, block, 0, st>>>((const float*)ring, ny, nx, row0, col0, t, (float*)out);
    else
        ring_shift_kernel<double><<<grid, block, 0, st>>>((const double*)ring, ny, nx, row0, col0, t, (double*)out);
    return hx::launch_status("ring_shift_kernel");
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
