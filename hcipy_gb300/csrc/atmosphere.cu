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

// new_slice[r] = sum_k A[r, k] stencil[k] + sum_k B[r, k] noise[k], one warp per r, written into the ring slot
// that the shift frees.  where: 0 bottom, 1 top, 2 left, 3 right; row0/col0 are the offsets before the step.
template <typename T>
__global__ void extrude_kernel(T* ring, int ny, int nx, int row0, int col0, int where, const T* stencil, int nst,
                               const T* A, const T* B, int nb, const T* noise, int nslice) {
    extern __shared__ unsigned char smem_raw[];
    T* st = reinterpret_cast<T*>(smem_raw);  // nst stencil values, then nb noise values
    T* nz = st + nst;
    for (int k = threadIdx.x; k < nst; k += blockDim.x) st[k] = stencil[k];
    for (int k = threadIdx.x; k < nb; k += blockDim.x) nz[k] = noise[k];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = blockIdx.x * (blockDim.x >> 5) + warp;
    if (r >= nslice) return;
    T acc = T(0);
    const T* a = A + (long long)r * nst;
    for (int k = lane; k < nst; k += 32) acc += a[k] * st[k];
    const T* b = B + (long long)r * nb;
    for (int k = lane; k < nb; k += 32) acc += b[k] * nz[k];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane != 0) return;
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
    const int x0 = blockIdx.x * TS, y0 = blockIdx.y * TS;
    for (int t = threadIdx.y * blockDim.x + threadIdx.x; t < TIN * TIN; t += blockDim.x * blockDim.y) {
        const int ly = t / TIN, lx = t % TIN;
        const int gy = min(max(y0 + ly - HALO, 0), ny - 1);
        const int gx = min(max(x0 + lx - HALO, 0), nx - 1);
        in[ly][lx] = ring[(long long)((gy + row0) % ny) * nx + (gx + col0) % nx];
    }
    __syncthreads();
    // rows: mid[ly][x] = sum_k in[ly][x + k] * row[k]
    for (int t = threadIdx.y * blockDim.x + threadIdx.x; t < TIN * TS; t += blockDim.x * blockDim.y) {
        const int ly = t / TS, x = t % TS;
        T s = T(0);
#pragma unroll
        for (int k = 0; k < 7; ++k) s += in[ly][x + k] * (T)taps.row[k];
        mid[ly][x] = s;
    }
    __syncthreads();
    for (int t = threadIdx.y * blockDim.x + threadIdx.x; t < TS * TS; t += blockDim.x * blockDim.y) {
        const int y = t / TS, x = t % TS;
        if (y0 + y >= ny || x0 + x >= nx) continue;
        T s = T(0);
#pragma unroll
        for (int k = 0; k < 7; ++k) s += mid[y + k][x] * (T)taps.col[k];
        out[(long long)(y0 + y) * nx + x0 + x] = s;
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
    const size_t esz = dtype == HX_F32 ? 4 : 8;
    const size_t smem = esz * ((size_t)nst + nb);
    HX_CHECK_ARG(smem <= 200 * 1024, "hx_atmosphere_extrude: stencil of %d plus %d noise values exceeds shared memory",
                 nst, nb);
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    cudaStream_t st = (cudaStream_t)stream;
    const bool flip = where == 1 || where == 3;
    const int threads = 256, rows_per_cta = threads / 32;
    dim3 grid(hx::ceil_div(nslice, rows_per_cta));
    if (dtype == HX_F32) {
        gather_stencil_kernel<float><<<hx::ceil_div(nst, 256), 256, 0, st>>>((const float*)ring, ny, nx, row0, col0,
                                                                             flip, stencil_idx, nst, (float*)work);
        HX_TRY(hx::launch_status("gather_stencil_kernel"));
        if (smem > 48 * 1024)
            cudaFuncSetAttribute(extrude_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        extrude_kernel<float><<<grid, threads, smem, st>>>((float*)ring, ny, nx, row0, col0, where,
                                                          (const float*)work, nst, (const float*)A, (const float*)B,
                                                          nb, (const float*)noise, nslice);
    } else {
        gather_stencil_kernel<double><<<hx::ceil_div(nst, 256), 256, 0, st>>>((const double*)ring, ny, nx, row0,
                                                                              col0, flip, stencil_idx, nst,
                                                                              (double*)work);
        HX_TRY(hx::launch_status("gather_stencil_kernel"));
        if (smem > 48 * 1024)
            cudaFuncSetAttribute(extrude_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        extrude_kernel<double><<<grid, threads, smem, st>>>((double*)ring, ny, nx, row0, col0, where,
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
    if (dtype == HX_F32)
        ring_shift_kernel<float><<<grid, block, 0, st>>>((const float*)ring, ny, nx, row0, col0, t, (float*)out);
    else
        ring_shift_kernel<double><<<grid, block, 0, st>>>((const double*)ring, ny, nx, row0, col0, t, (double*)out);
    return hx::launch_status("ring_shift_kernel");
}

}  // extern "C"
