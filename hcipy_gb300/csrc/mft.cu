// Matrix Fourier transform plans (hcipy/fourier/matrix_fourier_transform.py).
//
// A plan holds the phase matrices of the three directions, generated once on
// the device in float64 (sincos of the float64 product a[r]*b[c], exactly the
// numpy outer product the reference exponentiates at :95-102) and stored in the
// plan's element type.  Separable non-uniform weights are folded into the
// matrices, so every execute is two plain GEMMs:
//   forward : T = in . M2f (stacked over the batch), out[b] = alpha * M1f . T[b]
//   backward: T[b] = M1b . in[b],                   out = alpha * T . M2b (stacked)
// The adjoint uses the backward matrices when the grids have uniform weights.
#include "hx_common.cuh"
#include "gemm_simt.cuh"
#include "mft_tc.cuh"

#include <algorithm>
#include <vector>

struct hx_mft_plan {
    int nx, ny, nu, nv;
    int dtype;
    int precision;
    size_t esize;
    void* m1f = nullptr;  // nv x ny : exp(-i v y) wy[y]
    void* m2f = nullptr;  // nx x nu : wx[x] exp(-i x u)
    void* m1b = nullptr;  // ny x nv : exp(+i y v) wv[v]
    void* m2b = nullptr;  // nu x nx : wu[u] exp(+i u x)
    void* m1a = nullptr;  // ny x nv : wy[y] exp(+i y v)
    void* m2a = nullptr;  // nu x nx : exp(+i u x) wx[x]
    bool own_adjoint = false;
    hx::SplitMftPlan* split = nullptr;  // tensor-core operands (HX_PREC_SPLIT)
    int schedule = HX_SCHEDULE_LATENCY;
};

namespace {

// M[r, c] = wr[r] * wc[c] * exp(sign * i * a[r] * b[c]), computed in float64.
template <typename T>
__global__ void phase_matrix_kernel(int rows, int cols, const double* __restrict__ a, const double* __restrict__ b,
                                    double sign, const double* __restrict__ wr, const double* __restrict__ wc,
                                    typename hx::cplx<T>::type* __restrict__ out) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long total = (long long)rows * cols;
    if (idx >= total) return;
    const int r = (int)(idx / cols);
    const int c = (int)(idx % cols);
    const double phase = a[r] * b[c];
    double s, co;
    sincos(phase, &s, &co);
    double w = 1.0;
    if (wr) w *= wr[r];
    if (wc) w *= wc[c];
    out[idx] = hx::make_c<T>((T)(w * co), (T)(w * sign * s));
}

int upload(const double* host, int n, double** dev, cudaStream_t stream) {
    *dev = nullptr;
    if (host == nullptr) return HX_OK;
    HX_TRY(hx::cuda_status(cudaMalloc(dev, sizeof(double) * n), "cudaMalloc(coords)"));
    return hx::cuda_status(cudaMemcpyAsync(*dev, host, sizeof(double) * n, cudaMemcpyHostToDevice, stream), "upload coords");
}

int gen_matrix(int dtype, int rows, int cols, const double* a, const double* b, double sign,
               const double* wr, const double* wc, void** out, cudaStream_t stream) {
    const size_t es = dtype == HX_C64 ? sizeof(float2) : sizeof(double2);
    HX_TRY(hx::cuda_status(cudaMalloc(out, es * (size_t)rows * cols), "cudaMalloc(phase matrix)"));
    const long long total = (long long)rows * cols;
    const unsigned blocks = hx::ceil_div(total, 256);
    if (dtype == HX_C64)
        phase_matrix_kernel<float><<<blocks, 256, 0, stream>>>(rows, cols, a, b, sign, wr, wc, (float2*)*out);
    else
        phase_matrix_kernel<double><<<blocks, 256, 0, stream>>>(rows, cols, a, b, sign, wr, wc, (double2*)*out);
    return hx::launch_status("phase_matrix_kernel");
}

void free_plan(hx_mft_plan* p) {
    if (!p) return;
    cudaFree(p->m1f);
    cudaFree(p->m2f);
    cudaFree(p->m1b);
    cudaFree(p->m2b);
    if (p->own_adjoint) {
        cudaFree(p->m1a);
        cudaFree(p->m2a);
    }
    hx::split_mft_destroy(p->split);
    delete p;
}

// ---- small transforms in one launch ------------------------------------------------------------------
//
// out[r, :] = alpha sum_q (A[r, :] . X[:, S_q]) . B[S_q, :] for a block of RPC output rows: A is R x K1, X one field
// (K1 x K2), B K2 x C, out R x C, with the GEMM path's epilogues; forward A = M1f, X = E, B = M2f, backward A = M1b,
// X = F, B = M2b.  The columns of X are cut into CS slices S_q and the CS CTAs of a thread-block cluster take one
// slice each: CTA q forms w = A[rows] . X[:, S_q] and the partial image w . B[S_q, :], then the cluster adds the CS
// partials of every output column in slice order through distributed shared memory, each CTA finishing C / CS of
// the columns.  A CTA reads K1 x K2 / CS of the field and K2 / CS rows of B, so a transform whose two GEMMs would
// occupy a few dozen SMs runs as one launch over ceil(R / RPC) x CS CTAs, and no intermediate leaves the cluster.
// The products are associated by output rows (the same complex MACs as the two GEMMs); sums run in blocks of kBlk
// terms added into the total, so FP32 rounding grows with sqrt(kBlk) + sqrt(K / kBlk) rather than sqrt(K).
constexpr int kSmThreads = 256;
constexpr int kSmRows = 4;     // output rows per cluster (RPC)
constexpr int kSmSlices = 8;   // CTAs per cluster (CS)
constexpr int kBlk = 16;       // terms per partial sum
constexpr int kSmMaxBytes = 200 * 1024;

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}

__device__ __forceinline__ unsigned cluster_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Shared-memory layout of the small-transform kernel (in elements of the complex type).
struct SmLayout {
    int xw, cw;                      // columns of X per slice, output columns per CTA
    int a, x, b, w, part, total;     // offsets and total size
    __host__ __device__ SmLayout(int K1, int K2, int C, int esize) {
        xw = (K2 + kSmSlices - 1) / kSmSlices;
        xw += xw & 1;  // even: 16-byte chunks of complex64
        cw = (C + kSmSlices - 1) / kSmSlices;
        a = 0;
        x = a + kSmRows * K1;
        b = x + K1 * xw;
        w = b + xw * C;
        part = w + 2 * kSmRows * xw;  // w holds two partial sums per element before they are added
        total = part + kSmSlices * kSmRows * cw;
        (void)esize;
    }
};

template <typename T>
__global__ void __launch_bounds__(kSmThreads) mft_small_kernel(int R, int K1, int K2, int C,
                                                              typename hx::cplx<T>::type alpha,
                                                              const typename hx::cplx<T>::type* __restrict__ A,
                                                              const typename hx::cplx<T>::type* __restrict__ X,
                                                              long long sX,
                                                              const typename hx::cplx<T>::type* __restrict__ B,
                                                              typename hx::cplx<T>::type* __restrict__ out,
                                                              long long sO, hx::Epilogue<typename hx::cplx<T>::type> epi) {
    using Cx = typename hx::cplx<T>::type;
    extern __shared__ __align__(16) unsigned char sm_raw[];
    Cx* sm = reinterpret_cast<Cx*>(sm_raw);
    const SmLayout L(K1, K2, C, (int)sizeof(Cx));
    const int q = (int)cluster_rank();
    const int r0 = (blockIdx.x / kSmSlices) * kSmRows;
    const int z = blockIdx.y;
    const int x0 = q * L.xw;
    const int xn = max(0, min(L.xw, K2 - x0));  // columns of this slice
    const Cx zero = hx::make_c<T>(T(0), T(0));
    // first phase of the cluster barrier: arrive now, wait before the first remote store
    asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory");
    Cx* a_s = sm + L.a;
    Cx* x_s = sm + L.x;
    Cx* b_s = sm + L.b;
    Cx* w_s = sm + L.w;
    Cx* part = sm + L.part;
    // rows of A, the slice of X and the rows of B, by 16-byte asynchronous copies
    constexpr int PER = 16 / (int)sizeof(Cx);  // complex elements per 16-byte chunk
    const Cx* xf = X + sX * z;
    {
        // rows of A (rows past R read as zeros), 16-byte chunks: K1 * sizeof(Cx) is a multiple of 16
        const int cpa = K1 / PER;
        for (int c = threadIdx.x; c < kSmRows * cpa; c += kSmThreads) {
            const int rr = c / cpa, j = c - rr * cpa;
            if (r0 + rr < R) cp_async16(a_s + rr * K1 + j * PER, A + (long long)(r0 + rr) * K1 + j * PER);
            else *reinterpret_cast<float4*>(a_s + rr * K1 + j * PER) = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        const int cpr = xn / PER;  // chunks per row of the X slice
        for (int c = threadIdx.x; c < K1 * cpr; c += kSmThreads) {
            const int y = c / cpr, j = c - y * cpr;
            cp_async16(x_s + y * L.xw + j * PER, xf + (long long)y * K2 + x0 + j * PER);
        }
        const int bchunks = xn * C / PER;
        for (int c = threadIdx.x; c < bchunks; c += kSmThreads) cp_async16(b_s + c * PER, B + (long long)x0 * C + c * PER);
        asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
    }
    __syncthreads();
    // w[rr][xl] = sum_y A[r0 + rr][y] X[y][x0 + xl], two threads per element (the halves of y), added in order
    const int nw = kSmRows * xn;
    const int yh = (K1 / 2 + kBlk - 1) / kBlk * kBlk;  // first y of the second half
    for (int i = threadIdx.x; i < 2 * nw; i += kSmThreads) {
        const int h = i / nw, o = i - h * nw;
        const int rr = o / xn, xl = o - rr * xn;
        Cx acc = zero;
        for (int y0 = h ? yh : 0; y0 < (h ? K1 : min(K1, yh)); y0 += kBlk) {
            Cx blk = zero;
            const int y1 = min(K1, y0 + kBlk);
#pragma unroll 4
            for (int y = y0; y < y1; ++y) {
                const Cx av = a_s[rr * K1 + y], xv = x_s[y * L.xw + xl];
                blk.x = fma(av.x, xv.x, blk.x);
                blk.x = fma(-av.y, xv.y, blk.x);
                blk.y = fma(av.x, xv.y, blk.y);
                blk.y = fma(av.y, xv.x, blk.y);
            }
            acc.x += blk.x;
            acc.y += blk.y;
        }
        w_s[h * kSmRows * L.xw + rr * L.xw + xl] = acc;
    }
    __syncthreads();
    for (int o = threadIdx.x; o < nw; o += kSmThreads) {
        const int rr = o / xn, xl = o - rr * xn;
        const Cx p1 = w_s[kSmRows * L.xw + rr * L.xw + xl];
        w_s[rr * L.xw + xl].x += p1.x;
        w_s[rr * L.xw + xl].y += p1.y;
    }
    __syncthreads();
    // partial image p[rr][u] = sum_xl w[rr][xl] B[x0 + xl][u], sent to the CTA that finishes column u
    asm volatile("barrier.cluster.wait.aligned;" ::: "memory");  // every CTA of the cluster has started
    for (int i = threadIdx.x; i < kSmRows * C; i += kSmThreads) {
        const int rr = i / C, u = i - rr * C;
        Cx acc = zero;
        for (int j0 = 0; j0 < xn; j0 += kBlk) {
            Cx blk = zero;
            const int j1 = min(xn, j0 + kBlk);
#pragma unroll 4
            for (int j = j0; j < j1; ++j) {
                const Cx wv = w_s[rr * L.xw + j], bv = b_s[j * C + u];
                blk.x = fma(wv.x, bv.x, blk.x);
                blk.x = fma(-wv.y, bv.y, blk.x);
                blk.y = fma(wv.x, bv.y, blk.y);
                blk.y = fma(wv.y, bv.x, blk.y);
            }
            acc.x += blk.x;
            acc.y += blk.y;
        }
        const int owner = u / L.cw, ul = u - owner * L.cw;
        Cx* dst = part + (q * kSmRows + rr) * L.cw + ul;
        if (owner == q) {
            *dst = acc;
        } else {
            unsigned raddr;
            asm volatile("mapa.shared::cluster.u32 %0, %1, %2;"
                         : "=r"(raddr)
                         : "r"((unsigned)__cvta_generic_to_shared(dst)), "r"((unsigned)owner));
            if constexpr (sizeof(T) == 4)
                asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" ::"r"(raddr), "f"(acc.x), "f"(acc.y) : "memory");
            else
                asm volatile("st.shared::cluster.v2.f64 [%0], {%1, %2};" ::"r"(raddr), "d"(acc.x), "d"(acc.y) : "memory");
        }
    }
    cluster_barrier();  // every partial is in place
    const long long obase = sO * z;
    const int cn = max(0, min(L.cw, C - q * L.cw));
    for (int i = threadIdx.x; i < kSmRows * cn; i += kSmThreads) {
        const int rr = i / cn, ul = i - rr * cn;
        const long long r = r0 + rr;
        if (r >= R) continue;
        Cx acc = zero;
#pragma unroll
        for (int sp = 0; sp < kSmSlices; ++sp) {
            const Cx p = part[(sp * kSmRows + rr) * L.cw + ul];
            acc.x += p.x;
            acc.y += p.y;
        }
        const int u = q * L.cw + ul;
        Cx v = hx::cmul(alpha, acc);
        const long long frow = (r % epi.rows_per_field) * C;
        if (epi.kind == hx::EPI_MUL) {
            v = hx::cmul(v, epi.mask[frow + u]);
        } else if (epi.kind == hx::EPI_BABINET) {
            const Cx e = epi.src[obase + r * C + u];
            v.x = e.x - v.x;
            v.y = e.y - v.y;
            if (epi.mask) v = hx::cmul(v, epi.mask[frow + u]);
        }
        out[obase + r * C + u] = v;
    }
}

// Whether a transform takes the one-launch form: small enough that its two GEMMs would leave most SMs idle (at
// most 512 points per axis, a few fields), with its slices of X and rows of B in shared memory, rows of whole
// 16-byte chunks, and a cluster of kSmSlices such CTAs resident on this device.
template <typename T>
bool small_form_ok(int R, int K1, int K2, int C, int batch, const void* X, long long sX) {
    using Cx = typename hx::cplx<T>::type;
    static const bool allowed = [] {  // HX_MFT_SMALL=0 keeps every transform on the two GEMMs (comparisons)
        const char* e = getenv("HX_MFT_SMALL");
        return !(e && e[0] == '0');
    }();
    if (!allowed) return false;
    if (R > 512 || C > 512 || K1 > 512 || K2 > 512 || batch > 8 || C < kSmSlices || K2 < 2 * kSmSlices) return false;
    if (sizeof(Cx) == 8 && ((K1 | K2 | C) & 1)) return false;
    if ((reinterpret_cast<uintptr_t>(X) & 15) != 0 || (sX * (long long)sizeof(Cx)) % 16 != 0) return false;
    const SmLayout L(K1, K2, C, (int)sizeof(Cx));
    if (sizeof(Cx) * (size_t)L.total > kSmMaxBytes) return false;
    if (L.xw * (kSmSlices - 1) >= K2) return false;  // every slice holds columns
    static int ok[64];  // per device: 0 unknown, 1 yes, 2 no
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
    if (!ok[dev]) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(kSmSlices, 1, 1);
        cfg.blockDim = dim3(kSmThreads);
        cfg.dynamicSmemBytes = kSmMaxBytes;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = kSmSlices;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int n = 0;
        const bool good = cudaFuncSetAttribute(mft_small_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               kSmMaxBytes) == cudaSuccess &&
                          cudaOccupancyMaxActiveClusters(&n, mft_small_kernel<T>, &cfg) == cudaSuccess && n > 0;
        cudaGetLastError();
        ok[dev] = good ? 1 : 2;
    }
    return ok[dev] == 1;
}

template <typename T>
int run_small(int R, int K1, int K2, int C, typename hx::cplx<T>::type alpha, const void* A, const void* X,
              long long sX, const void* B, void* out, long long sO, int batch,
              hx::Epilogue<typename hx::cplx<T>::type> epi, cudaStream_t stream) {
    using Cx = typename hx::cplx<T>::type;
    const SmLayout L(K1, K2, C, (int)sizeof(Cx));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(hx::ceil_div(R, kSmRows) * kSmSlices, batch, 1);
    cfg.blockDim = dim3(kSmThreads);
    cfg.dynamicSmemBytes = sizeof(Cx) * (size_t)L.total;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kSmSlices;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    hx::TraceScope trace(HX_TRACE_SIMT_GEMM, (double)batch * ((double)R * K1 * K2 + (double)R * K2 * C), stream);
    HX_TRY(hx::cuda_status(cudaLaunchKernelEx(&cfg, mft_small_kernel<T>, R, K1, K2, C, alpha, (const Cx*)A,
                                              (const Cx*)X, sX, (const Cx*)B, (Cx*)out, sO, epi),
                           "mft_small_kernel"));
    return hx::launch_status(sizeof(T) == 4 ? "mft_small_kernel<float>" : "mft_small_kernel<double>");
}

template <typename T>
int execute_t(const hx_mft_plan* p, int direction, int batch, const void* in_, void* out_, double are, double aim,
              int epilogue, const void* mask, const void* src, void* ws_, cudaStream_t stream) {
    using Cx = typename hx::cplx<T>::type;
    const Cx* in = (const Cx*)in_;
    Cx* out = (Cx*)out_;
    Cx* T1 = (Cx*)ws_;
    const Cx one = hx::make_c<T>(T(1), T(0));
    const Cx alpha = hx::make_c<T>((T)are, (T)aim);
    const int nx = p->nx, ny = p->ny, nu = p->nu, nv = p->nv;
    const bool tp = p->schedule == HX_SCHEDULE_THROUGHPUT;
    hx::Epilogue<Cx> epi;
    epi.kind = epilogue;
    epi.mask = (const Cx*)mask;
    epi.src = (const Cx*)src;
    if (!tp) {
        // small transforms: one launch (see mft_small_kernel)
        const bool fwd = direction == HX_FORWARD;
        const int R = fwd ? nv : ny, K1 = fwd ? ny : nv, K2 = fwd ? nx : nu, C = fwd ? nu : nx;
        if (small_form_ok<T>(R, K1, K2, C, batch, in, (long long)K1 * K2)) {
            const void* A = fwd ? p->m1f : direction == HX_BACKWARD ? p->m1b : p->m1a;
            const void* B = fwd ? p->m2f : direction == HX_BACKWARD ? p->m2b : p->m2a;
            epi.rows_per_field = R;
            return run_small<T>(R, K1, K2, C, alpha, A, in, (long long)K1 * K2, B, out, (long long)R * C, batch, epi,
                                stream);
        }
    }
    if (direction == HX_FORWARD) {
        // T (batch*ny x nu) = in (batch*ny x nx) . M2f (nx x nu)
        HX_TRY(hx::cgemm_nn<T>(batch * ny, nu, nx, one, in, nx, 0, (const Cx*)p->m2f, nu, 0, T1, nu, 0, 1, stream, {},
                               tp));
        // out[b] (nv x nu) = alpha * M1f (nv x ny) . T[b] (ny x nu)
        epi.rows_per_field = nv;
        return hx::cgemm_nn<T>(nv, nu, ny, alpha, (const Cx*)p->m1f, ny, 0, T1, nu, (long long)ny * nu, out, nu,
                               (long long)nv * nu, batch, stream, epi, tp);
    }
    const Cx* m1 = (const Cx*)(direction == HX_BACKWARD ? p->m1b : p->m1a);
    const Cx* m2 = (const Cx*)(direction == HX_BACKWARD ? p->m2b : p->m2a);
    // T[b] (ny x nu) = M1 (ny x nv) . in[b] (nv x nu)
    HX_TRY(hx::cgemm_nn<T>(ny, nu, nv, one, m1, nv, 0, in, nu, (long long)nv * nu, T1, nu, (long long)ny * nu, batch,
                           stream, {}, tp));
    // out (batch*ny x nx) = alpha * T (batch*ny x nu) . M2 (nu x nx)
    epi.rows_per_field = ny;
    return hx::cgemm_nn<T>(batch * ny, nx, nu, alpha, T1, nu, 0, m2, nx, 0, out, nx, 0, 1, stream, epi, tp);
}

}  // namespace

extern "C" {

int hx_mft_plan_create(int nx, int ny, int nu, int nv, const double* x, const double* y, const double* u,
                       const double* v, const double* w_in_x, const double* w_in_y, const double* w_out_u,
                       const double* w_out_v, int dtype, int precision, void* stream_, hx_mft_plan** plan) {
    HX_CHECK_ARG(plan != nullptr, "hx_mft_plan_create: plan pointer is NULL");
    *plan = nullptr;
    HX_CHECK_ARG(nx > 0 && ny > 0 && nu > 0 && nv > 0, "hx_mft_plan_create: dimensions must be positive (%d %d %d %d)",
                 nx, ny, nu, nv);
    HX_CHECK_ARG(x && y && u && v, "hx_mft_plan_create: coordinate arrays must not be NULL");
    HX_CHECK_ARG(dtype == HX_C64 || dtype == HX_C128, "hx_mft_plan_create: unknown dtype %d", dtype);
    HX_CHECK_ARG(precision == HX_PREC_FP32 || precision == HX_PREC_SPLIT, "hx_mft_plan_create: unknown precision %d",
                 precision);
    HX_CHECK_ARG(!(precision == HX_PREC_SPLIT && dtype != HX_C64),
                 "hx_mft_plan_create: the split tensor-core form takes complex64 fields");
    if (hx::fault_injected("plan")) return HX_ERR_INJECTED;
    if (hx::fault_injected("alloc")) return HX_ERR_INJECTED;
    cudaStream_t stream = (cudaStream_t)stream_;

    hx_mft_plan* p = new hx_mft_plan();
    p->nx = nx; p->ny = ny; p->nu = nu; p->nv = nv;
    p->dtype = dtype;
    p->precision = precision;
    p->esize = dtype == HX_C64 ? sizeof(float2) : sizeof(double2);

    double *dx, *dy, *du, *dv, *dwx, *dwy, *dwu, *dwv;
    dx = dy = du = dv = dwx = dwy = dwu = dwv = nullptr;
    int rc = HX_OK;
    auto cleanup = [&]() {
        cudaStreamSynchronize(stream);
        for (double* q : {dx, dy, du, dv, dwx, dwy, dwu, dwv}) cudaFree(q);
    };
    do {
        if ((rc = upload(x, nx, &dx, stream))) break;
        if ((rc = upload(y, ny, &dy, stream))) break;
        if ((rc = upload(u, nu, &du, stream))) break;
        if ((rc = upload(v, nv, &dv, stream))) break;
        if ((rc = upload(w_in_x, nx, &dwx, stream))) break;
        if ((rc = upload(w_in_y, ny, &dwy, stream))) break;
        if ((rc = upload(w_out_u, nu, &dwu, stream))) break;
        if ((rc = upload(w_out_v, nv, &dwv, stream))) break;
        if (precision == HX_PREC_SPLIT) {
            // The split form keeps only its sliced operands.
            if ((rc = hx::split_mft_create(nx, ny, nu, nv, dx, dy, du, dv, dwx, dwy, dwu, dwv, stream, &p->split)))
                break;
            break;
        }
        if ((rc = gen_matrix(dtype, nv, ny, dv, dy, -1.0, nullptr, dwy, &p->m1f, stream))) break;
        if ((rc = gen_matrix(dtype, nx, nu, dx, du, -1.0, dwx, nullptr, &p->m2f, stream))) break;
        if ((rc = gen_matrix(dtype, ny, nv, dy, dv, +1.0, nullptr, dwv, &p->m1b, stream))) break;
        if ((rc = gen_matrix(dtype, nu, nx, du, dx, +1.0, dwu, nullptr, &p->m2b, stream))) break;
        const bool weighted_in = (w_in_x != nullptr) || (w_in_y != nullptr);
        const bool weighted_out = (w_out_u != nullptr) || (w_out_v != nullptr);
        if (!weighted_in && !weighted_out) {
            p->m1a = p->m1b;
            p->m2a = p->m2b;
        } else {
            p->own_adjoint = true;
            if ((rc = gen_matrix(dtype, ny, nv, dy, dv, +1.0, dwy, nullptr, &p->m1a, stream))) break;
            if ((rc = gen_matrix(dtype, nu, nx, du, dx, +1.0, nullptr, dwx, &p->m2a, stream))) break;
        }
    } while (false);
    cleanup();
    if (rc != HX_OK) {
        free_plan(p);
        return rc;
    }
    *plan = p;
    return HX_OK;
}

size_t hx_mft_workspace_bytes(const hx_mft_plan* p, int direction, int batch) {
    if (!p || batch <= 0) return 0;
    size_t base = p->esize * (size_t)batch * p->ny * p->nu;
    if (p->precision == HX_PREC_SPLIT) return hx::split_mft_workspace_bytes(p->split, direction, batch);
    return base;
}

int hx_mft_execute(const hx_mft_plan* p, int direction, int batch, const void* in, void* out, double are, double aim,
                   void* ws, size_t ws_bytes, void* stream_) {
    return hx_mft_execute_ex(p, direction, batch, in, out, are, aim, HX_EPI_NONE, nullptr, nullptr, ws, ws_bytes,
                             stream_);
}

int hx_mft_execute_ex(const hx_mft_plan* p, int direction, int batch, const void* in, void* out, double are,
                      double aim, int epilogue, const void* mask, const void* src, void* ws, size_t ws_bytes,
                      void* stream_) {
    HX_CHECK_ARG(p != nullptr, "hx_mft_execute: plan is NULL");
    HX_CHECK_ARG(direction == HX_FORWARD || direction == HX_BACKWARD || direction == HX_ADJOINT,
                 "hx_mft_execute: unknown direction %d", direction);
    HX_CHECK_ARG(batch >= 1, "hx_mft_execute: batch must be >= 1 (got %d)", batch);
    HX_CHECK_ARG(in != nullptr && out != nullptr, "hx_mft_execute: NULL field pointer");
    const size_t need = hx_mft_workspace_bytes(p, direction, batch);
    HX_CHECK_ARG(ws != nullptr && ws_bytes >= need, "hx_mft_execute: workspace of %zu bytes needed, %zu given", need,
                 ws_bytes);
    HX_CHECK_ARG(epilogue == HX_EPI_NONE || epilogue == HX_EPI_MUL || epilogue == HX_EPI_BABINET,
                 "hx_mft_execute_ex: unknown epilogue %d", epilogue);
    HX_CHECK_ARG(epilogue != HX_EPI_MUL || mask != nullptr, "hx_mft_execute_ex: HX_EPI_MUL needs a mask");
    HX_CHECK_ARG(epilogue != HX_EPI_BABINET || src != nullptr, "hx_mft_execute_ex: HX_EPI_BABINET needs src");
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    cudaStream_t stream = (cudaStream_t)stream_;
    if (p->precision == HX_PREC_SPLIT)
        return hx::split_mft_execute(p->split, direction, batch, in, HX_C64, out, HX_C64, are, aim, epilogue,
                                     (const float2*)mask, src, HX_C64, ws, ws_bytes, stream);
    if (p->dtype == HX_C64)
        return execute_t<float>(p, direction, batch, in, out, are, aim, epilogue, mask, src, ws, stream);
    return execute_t<double>(p, direction, batch, in, out, are, aim, epilogue, mask, src, ws, stream);
}

int hx_mft_execute_io(const hx_mft_plan* p, int direction, int batch, const void* in, int in_dtype, void* out,
                      int out_dtype, double are, double aim, int epilogue, const void* mask, const void* src,
                      int src_dtype, void* ws, size_t ws_bytes, void* stream) {
    HX_CHECK_ARG(p != nullptr, "hx_mft_execute_io: plan is NULL");
    const bool ok_t = (in_dtype == HX_C64 || in_dtype == HX_C128) && (out_dtype == HX_C64 || out_dtype == HX_C128) &&
                      (src_dtype == HX_C64 || src_dtype == HX_C128);
    HX_CHECK_ARG(ok_t, "hx_mft_execute_io: dtypes must be HX_C64 or HX_C128");
    if (p->precision != HX_PREC_SPLIT) {
        HX_CHECK_ARG(in_dtype == p->dtype && out_dtype == p->dtype && src_dtype == p->dtype,
                     "hx_mft_execute_io: a plain plan reads and writes its own dtype");
        return hx_mft_execute_ex(p, direction, batch, in, out, are, aim, epilogue, mask, src, ws, ws_bytes, stream);
    }
    HX_CHECK_ARG(direction == HX_FORWARD || direction == HX_BACKWARD || direction == HX_ADJOINT,
                 "hx_mft_execute_io: unknown direction %d", direction);
    HX_CHECK_ARG(batch >= 1 && in && out, "hx_mft_execute_io: bad batch or NULL field");
    HX_CHECK_ARG(epilogue != HX_EPI_MUL || mask != nullptr, "hx_mft_execute_io: HX_EPI_MUL needs a mask");
    HX_CHECK_ARG(epilogue != HX_EPI_BABINET || src != nullptr, "hx_mft_execute_io: HX_EPI_BABINET needs src");
    const size_t need = hx_mft_workspace_bytes(p, direction, batch);
    HX_CHECK_ARG(ws != nullptr && ws_bytes >= need, "hx_mft_execute_io: workspace of %zu bytes needed", need);
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    return hx::split_mft_execute(p->split, direction, batch, in, in_dtype, out, out_dtype, are, aim, epilogue,
                                 (const float2*)mask, src, src_dtype, ws, ws_bytes, (cudaStream_t)stream);
}

int hx_mft_execute_phase(const hx_mft_plan* p, int batch, const void* in, const float* screen, double scale,
                         void* out, int out_dtype, double are, double aim, void* ws, size_t ws_bytes, void* stream) {
    HX_CHECK_ARG(p != nullptr, "hx_mft_execute_phase: plan is NULL");
    HX_CHECK_ARG(p->precision == HX_PREC_SPLIT, "hx_mft_execute_phase: a split-precision plan is needed");
    HX_CHECK_ARG(out_dtype == HX_C64 || out_dtype == HX_C128, "hx_mft_execute_phase: out dtype must be HX_C64 or HX_C128");
    HX_CHECK_ARG(batch >= 1 && in && screen && out, "hx_mft_execute_phase: bad batch or NULL pointer");
    const size_t need = hx_mft_workspace_bytes(p, HX_FORWARD, batch);
    HX_CHECK_ARG(ws != nullptr && ws_bytes >= need, "hx_mft_execute_phase: workspace of %zu bytes needed", need);
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    return hx::split_mft_execute_phase(p->split, batch, in, screen, scale, out, out_dtype, are, aim, ws,
                                       (cudaStream_t)stream);
}

size_t hx_lyot_workspace_bytes(const hx_mft_plan* fpm, const hx_mft_plan* img, int batch) {
    if (!fpm || batch <= 0) return 0;
    if (fpm->precision == HX_PREC_SPLIT)
        return hx::split_lyot_workspace_bytes(fpm->split, img ? img->split : nullptr, batch);
    const size_t es = fpm->esize;
    size_t mft = std::max(hx_mft_workspace_bytes(fpm, HX_FORWARD, batch), hx_mft_workspace_bytes(fpm, HX_BACKWARD, batch));
    if (img) mft = std::max(mft, hx_mft_workspace_bytes(img, HX_FORWARD, batch));
    const size_t focal = es * (size_t)batch * fpm->nu * fpm->nv;
    const size_t pupil = es * (size_t)batch * fpm->nx * fpm->ny;
    auto up = [](size_t x) { return (x + 255) / 256 * 256; };
    return up(focal) + up(pupil) + up(mft);
}

int hx_lyot_execute(const hx_mft_plan* fpm, const hx_mft_plan* img, int batch, const void* e, int e_dtype,
                    const void* one_minus_fpm, const void* stop, double af_re, double af_im, double ab_re,
                    double ab_im, double ai_re, double ai_im, void* lyot_out, int lyot_dtype, void* image_out,
                    int image_dtype, void* ws, size_t ws_bytes, void* stream_) {
    HX_CHECK_ARG(fpm != nullptr && e != nullptr && one_minus_fpm != nullptr, "hx_lyot_execute: NULL argument");
    HX_CHECK_ARG(batch >= 1, "hx_lyot_execute: batch must be >= 1");
    HX_CHECK_ARG(lyot_out != nullptr || (img != nullptr && image_out != nullptr),
                 "hx_lyot_execute: nothing to write (no Lyot-plane output and no image)");
    HX_CHECK_ARG(!img || (img->nx == fpm->nx && img->ny == fpm->ny && img->precision == fpm->precision),
                 "hx_lyot_execute: the image plan must share the pupil grid and the precision of the mask plan");
    HX_CHECK_ARG(!img || image_out != nullptr, "hx_lyot_execute: image plan given without an image output");
    const size_t need = hx_lyot_workspace_bytes(fpm, img, batch);
    HX_CHECK_ARG(ws != nullptr && ws_bytes >= need, "hx_lyot_execute: workspace of %zu bytes needed", need);
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    cudaStream_t stream = (cudaStream_t)stream_;
    if (fpm->precision == HX_PREC_SPLIT)
        return hx::split_lyot_execute(fpm->split, img ? img->split : nullptr, batch, e, e_dtype,
                                      (const float2*)one_minus_fpm, (const float2*)stop, af_re, af_im, ab_re, ab_im,
                                      ai_re, ai_im, lyot_out, lyot_dtype, image_out, image_dtype, ws, stream);
    HX_CHECK_ARG(e_dtype == fpm->dtype && (!lyot_out || lyot_dtype == fpm->dtype) &&
                     (!img || image_dtype == fpm->dtype),
                 "hx_lyot_execute: a plain plan reads and writes its own dtype");
    auto up = [](size_t x) { return (x + 255) / 256 * 256; };
    uint8_t* w = (uint8_t*)ws;
    const size_t es = fpm->esize;
    void* ef = w;
    w += up(es * (size_t)batch * fpm->nu * fpm->nv);
    void* lp = lyot_out ? lyot_out : (void*)w;
    w += up(es * (size_t)batch * fpm->nx * fpm->ny);
    void* mws = w;
    const size_t mws_bytes = ws_bytes - (size_t)(w - (uint8_t*)ws);
    HX_TRY(hx_mft_execute_ex(fpm, HX_FORWARD, batch, e, ef, af_re, af_im, HX_EPI_MUL, one_minus_fpm, nullptr, mws,
                             mws_bytes, stream));
    HX_TRY(hx_mft_execute_ex(fpm, HX_BACKWARD, batch, ef, lp, ab_re, ab_im, HX_EPI_BABINET, stop, e, mws, mws_bytes,
                             stream));
    if (img)
        return hx_mft_execute_ex(img, HX_FORWARD, batch, lp, image_out, ai_re, ai_im, HX_EPI_NONE, nullptr, nullptr,
                                 mws, mws_bytes, stream);
    return HX_OK;
}

int hx_mft_plan_status(const hx_mft_plan* p, int reset) {
    HX_CHECK_ARG(p != nullptr, "hx_mft_plan_status: plan is NULL");
    if (p->precision != HX_PREC_SPLIT) return HX_OK;
    return hx::split_mft_status(p->split, reset);
}

int hx_mft_plan_destroy(hx_mft_plan* p) {
    free_plan(p);
    return HX_OK;
}

int hx_mft_plan_set_schedule(hx_mft_plan* p, int schedule) {
    HX_CHECK_ARG(p != nullptr, "hx_mft_plan_set_schedule: plan is NULL");
    HX_CHECK_ARG(schedule == HX_SCHEDULE_LATENCY || schedule == HX_SCHEDULE_THROUGHPUT,
                 "hx_mft_plan_set_schedule: unknown schedule %d", schedule);
    p->schedule = schedule;
    if (p->split) hx::split_mft_set_schedule(p->split, schedule);
    return HX_OK;
}

int hx_autotune(int on) {
    hx::split_autotune(on);
    return HX_OK;
}

int hx_autotune_entries(void) { return hx::split_autotune_entries(); }

int hx_autotune_entry(int i, long long* shape, int* n, int* bn, int* ksplit, float* ms) {
    HX_CHECK_ARG(shape && n && bn && ksplit && ms, "hx_autotune_entry: NULL pointer");
    const int rc = hx::split_autotune_entry(i, shape, n, bn, ksplit, ms);
    if (rc != HX_OK) hx::set_error("hx_autotune_entry: no entry %d", i);
    return rc;
}

int hx_autotune_clear(void) {
    hx::split_autotune_clear();
    return HX_OK;
}

size_t hx_intensity_sums_workspace_bytes(long long n, int batch) { return hx::intensity_sums_workspace_bytes(n, batch); }

int hx_intensity_sums(const void* field, int dtype, long long n, int batch, const float* weights, double* sums,
                      void* workspace, size_t workspace_bytes, void* stream) {
    HX_CHECK_ARG(n > 0 && batch > 0, "hx_intensity_sums: sizes must be positive");
    HX_CHECK_ARG(field && sums, "hx_intensity_sums: NULL pointer");
    HX_CHECK_ARG(dtype == HX_C64 || dtype == HX_C128, "hx_intensity_sums: dtype must be HX_C64 or HX_C128");
    const size_t need = hx::intensity_sums_workspace_bytes(n, batch);
    HX_CHECK_ARG(workspace != nullptr && workspace_bytes >= need, "hx_intensity_sums: workspace of %zu bytes needed",
                 need);
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    return hx::intensity_sums(field, dtype, n, batch, weights, sums, workspace, (cudaStream_t)stream);
}

int hx_intensity_sums_grad(const void* field, int dtype, long long n, int batch, const float* weights,
                           const double* grad, void* out, void* stream) {
    HX_CHECK_ARG(n > 0 && batch > 0, "hx_intensity_sums_grad: sizes must be positive");
    HX_CHECK_ARG(field && grad && out, "hx_intensity_sums_grad: NULL pointer");
    HX_CHECK_ARG(dtype == HX_C64 || dtype == HX_C128, "hx_intensity_sums_grad: dtype must be HX_C64 or HX_C128");
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    return hx::intensity_sums_grad(field, dtype, n, batch, weights, grad, out, (cudaStream_t)stream);
}

}  // extern "C"
