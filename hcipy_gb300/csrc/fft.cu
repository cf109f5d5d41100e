// FFT-family plans: the zero-padded FastFourierTransform, the Fourier filter
// (FourierFilter / angular-spectrum and Fresnel propagation), the chirp-Z transform, and the
// angular-spectrum and Fresnel transfer functions.  All transforms run fft_line_kernel.
//
// Reference behaviour restated here:
//   FastFourierTransform  hcipy/fourier/fast_fourier_transform.py:223-406
//   FourierFilter         hcipy/fourier/fourier_operations.py:28-151
//   ChirpZTransform       hcipy/fourier/chirp_z_transform.py:39-105
//   ASP transfer function hcipy/propagation/angular_spectrum.py:159-166 with
//                         evaluate_supersampled (hcipy/field/util.py:655-692)
#include "hx_common.cuh"
#include "fft_line.cuh"
#include "fft_pow2.cuh"

#include <algorithm>
#include <complex>
#include <vector>

namespace hx {
namespace {

using cd = std::complex<double>;

// Radices of a length-n transform, largest first.  allow16: radix 16 for power-of-two factors (float lines, whose
// threads hold 16 points: one 16-point butterfly per thread and stage).
std::vector<int> factor_radices(int n, bool allow16 = false) {
    std::vector<int> r;
    if (allow16 && (n & (n - 1)) == 0)
        while (n % 16 == 0 && n > 1) { r.push_back(16); n /= 16; }
    while (n % 8 == 0 && n > 1) { r.push_back(8); n /= 8; }
    while (n % 4 == 0) { r.push_back(4); n /= 4; }
    while (n % 2 == 0) { r.push_back(2); n /= 2; }
    for (int p : {3, 5, 7}) while (n % p == 0) { r.push_back(p); n /= p; }
    if (n != 1) r.clear();
    return r;
}

int next_pow2(int n) {
    int m = 1;
    while (m < n) m <<= 1;
    return m;
}

bool is_mixed(const std::vector<int>& radices) {
    for (int r : radices)
        if (r == 3 || r == 5 || r == 7) return true;
    return false;
}

template <typename T>
int max_points(bool mixed) { return kFftThreads * (mixed ? Ppt<T, true>::value : Ppt<T, false>::value); }

// Launch shape of a line transform: lines per CTA, threads, dynamic shared memory.
template <typename T>
int launch_shape(int M, const std::vector<int>& radices, int nlines, int batch, int min_lines, LineArgs<T>& a,
                 int* threads, size_t* smem) {
    const bool mixed = is_mixed(radices);
    const int cap = max_points<T>(mixed);
    if (M > cap) {
        set_error("FFT length %d exceeds the %d points one CTA holds", M, cap);
        return HX_ERR_UNSUPPORTED;
    }
    int lpc = std::max(1, cap / M);
    // Enough CTAs to fill the GPU (about two per SM), but keep min_lines for coalescing.
    const long long want_ctas = 304;
    const long long ctas_at_lpc = (long long)((nlines + lpc - 1) / lpc) * batch;
    if (ctas_at_lpc < want_ctas) {
        long long lines_needed = ((long long)nlines * batch + want_ctas - 1) / want_ctas;
        lpc = (int)std::max<long long>(std::min<long long>(lpc, std::max<long long>(lines_needed, min_lines)), 1);
    }
    lpc = std::min(lpc, nlines);
    int thr = 32;
    const int ppt = mixed ? Ppt<T, true>::value : Ppt<T, false>::value;
    for (int R : radices) {
        const int bpt = std::max(1, ppt / R);
        const int need = (lpc * (M / R) + bpt - 1) / bpt;
        thr = std::max(thr, need);
    }
    thr = ((thr + 31) / 32) * 32;
    if (thr > kFftThreads) {
        set_error("internal: FFT launch needs %d threads", thr);
        return HX_ERR_UNSUPPORTED;
    }
    a.lines_per_cta = lpc;
    a.pitch = lpc > 1 ? M + 1 : M;
    a.M = M;
    a.nstages = (int)radices.size();
    if (a.nstages > 12) {
        set_error("internal: %d FFT stages", a.nstages);
        return HX_ERR_UNSUPPORTED;
    }
    a.radix_code = 0;
    for (size_t i = 0; i < radices.size(); ++i) a.radix_code |= (unsigned long long)radices[i] << (5 * i);
    *threads = thr;
    *smem = (size_t)smem_elems(lpc * a.pitch) * sizeof(typename cplx<T>::type);
    return HX_OK;
}

template <typename T, int SIGN, bool CONV, bool MIXED>
int launch_line(const LineArgs<T>& a, int threads, size_t smem, int batch, cudaStream_t stream) {
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(fft_line_kernel<T, SIGN, CONV, MIXED>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             227 * 1024);
        configured = true;
    }
    dim3 grid((a.nlines + a.lines_per_cta - 1) / a.lines_per_cta, batch);
    if (grid.y > 65535u) {
        set_error("FFT batch too large (%d)", batch);
        return HX_ERR_UNSUPPORTED;
    }
    TraceScope trace(HX_TRACE_FFT,
                     (double)a.nlines * (a.in_count + a.out_count) * batch * sizeof(typename cplx<T>::type), stream);
    fft_line_kernel<T, SIGN, CONV, MIXED><<<grid, threads, smem, stream>>>(a);
    return launch_status("fft_line_kernel");
}

template <typename T, bool MIXED>
int run_line_m(const LineArgs<T>& a, int threads, size_t smem, int sign, bool conv, int batch, cudaStream_t s) {
    if (conv) return sign < 0 ? launch_line<T, -1, true, MIXED>(a, threads, smem, batch, s)
                              : launch_line<T, 1, true, MIXED>(a, threads, smem, batch, s);
    return sign < 0 ? launch_line<T, -1, false, MIXED>(a, threads, smem, batch, s)
                    : launch_line<T, 1, false, MIXED>(a, threads, smem, batch, s);
}

// Threads per CTA of the register-resident power-of-two kernel: 512.  HX_FFT_P2_THREADS (256 or 512) and
// HX_FFT_P2_THREADS_LF (256, 512 or 1024, strided lines) override it (tuning).
int p2_threads(bool lf) {
    static int v[2] = {0, 0};
    if (!v[lf]) {
        const char* e = getenv(lf ? "HX_FFT_P2_THREADS_LF" : "HX_FFT_P2_THREADS");
        const int x = e ? atoi(e) : 0;
        v[lf] = (x == 256 || x == 512 || (x == 1024 && lf)) ? x : 512;
    }
    return v[lf];
}

template <int N, int SIGN, bool LF>
int launch_p2(const LineArgs<float>& a0, int batch, cudaStream_t stream) {
    using P = Pow2Shape<N>;
    LineArgs<float> a = a0;
    const int lpc = std::max(1, std::min(p2_threads(LF) / P::T, a.nlines));
    a.lines_per_cta = lpc;
    const size_t smem = sizeof(float2) * (size_t)lpc * P::PITCH;
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(fft_pow2_kernel<N, SIGN, LF>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        configured = true;
    }
    dim3 grid((a.nlines + lpc - 1) / lpc, batch);
    if (grid.y > 65535u) {
        set_error("FFT batch too large (%d)", batch);
        return HX_ERR_UNSUPPORTED;
    }
    TraceScope trace(HX_TRACE_FFT, (double)a.nlines * (a.in_count + a.out_count) * batch * sizeof(float2), stream);
    fft_pow2_kernel<N, SIGN, LF><<<grid, lpc * P::T, smem, stream>>>(a);
    return launch_status("fft_pow2_kernel");
}

template <int N>
int run_p2_n(const LineArgs<float>& a, int sign, int batch, cudaStream_t s) {
    const bool lf = a.in_es != 1;
    if (sign < 0) return lf ? launch_p2<N, -1, true>(a, batch, s) : launch_p2<N, -1, false>(a, batch, s);
    return lf ? launch_p2<N, 1, true>(a, batch, s) : launch_p2<N, 1, false>(a, batch, s);
}

// The register-resident kernel takes complex64 power-of-two lines of 256 to 4096 points without Bluestein chirps
// or a spectrum multiply, whose input and output lines are both contiguous or both strided; -1 otherwise.
int run_p2(const LineArgs<float>& a, int sign, bool conv, int batch, cudaStream_t s) {
    if (conv || !a.tws || a.chirp_in || a.chirp_out || a.n_log != a.M || (a.in_es != 1) != (a.out_es != 1))
        return -1;
    switch (a.M) {
        case 256: return run_p2_n<256>(a, sign, batch, s);
        case 512: return run_p2_n<512>(a, sign, batch, s);
        case 1024: return run_p2_n<1024>(a, sign, batch, s);
        case 2048: return run_p2_n<2048>(a, sign, batch, s);
        case 4096: return run_p2_n<4096>(a, sign, batch, s);
        default: return -1;
    }
}

template <typename T>
int run_line(const LineArgs<T>& a, int threads, size_t smem, int sign, bool conv, int batch, cudaStream_t s) {
    if constexpr (sizeof(T) == 4) {
        const int rc = run_p2(a, sign, conv, batch, s);
        if (rc != -1) return rc;
    }
    bool mixed = false;
    unsigned long long code = a.radix_code;
    for (int i = 0; i < a.nstages; ++i, code >>= 5) {
        const int r = (int)(code & 31ull);
        if (r == 3 || r == 5 || r == 7) mixed = true;
    }
    return mixed ? run_line_m<T, true>(a, threads, smem, sign, conv, batch, s)
                 : run_line_m<T, false>(a, threads, smem, sign, conv, batch, s);
}

// ---- device tables ------------------------------------------------------------------------------

template <typename T>
__global__ void twiddle_kernel(int M, typename cplx<T>::type* tw) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= M) return;
    double s, c;
    sincospi(-2.0 * (double)t / (double)M, &s, &c);
    tw[t] = make_c<T>((T)c, (T)s);
}

template <typename T>
__global__ void narrow_kernel(const double2* in, typename cplx<T>::type* out, long long n, double scale) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = make_c<T>((T)(in[i].x * scale), (T)(in[i].y * scale));
}

template <typename T>
__global__ void conj_kernel(const typename cplx<T>::type* in, typename cplx<T>::type* out, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        typename cplx<T>::type v = in[i];
        v.y = -v.y;
        out[i] = v;
    }
}

struct DevBuf {
    void* p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
};

int dev_alloc(DevBuf& b, size_t bytes) {
    if (fault_injected("alloc")) return HX_ERR_INJECTED;
    return cuda_status(cudaMalloc(&b.p, std::max<size_t>(bytes, 16)), "cudaMalloc(fft table)");
}

// Upload complex<double> host values as the plan's element type.
template <typename T>
int upload_c(DevBuf& dst, const std::vector<cd>& v, cudaStream_t s) {
    using Cx = typename cplx<T>::type;
    std::vector<Cx> h(v.size());
    for (size_t i = 0; i < v.size(); ++i) h[i] = make_c<T>((T)v[i].real(), (T)v[i].imag());
    HX_TRY(dev_alloc(dst, sizeof(Cx) * h.size()));
    HX_TRY(cuda_status(cudaMemcpyAsync(dst.p, h.data(), sizeof(Cx) * h.size(), cudaMemcpyHostToDevice, s),
                       "upload table"));
    return cuda_status(cudaStreamSynchronize(s), "upload table sync");
}

template <typename T>
int make_twiddles(DevBuf& dst, int M, cudaStream_t s) {
    HX_TRY(dev_alloc(dst, sizeof(typename cplx<T>::type) * M));
    twiddle_kernel<T><<<ceil_div(M, 256), 256, 0, s>>>(M, (typename cplx<T>::type*)dst.p);
    return launch_status("twiddle_kernel");
}

// Spectrum of a length-M sequence given on the host, computed on the device in float64 and
// stored in T (times `scale`).
template <typename T>
int device_spectrum(DevBuf& dst, const std::vector<cd>& seq, int M, double scale, cudaStream_t s) {
    std::vector<int> rad = factor_radices(M);
    if (rad.empty()) {
        set_error("internal: spectrum length %d is not smooth", M);
        return HX_ERR_UNSUPPORTED;
    }
    DevBuf tw64, in64, out64;
    HX_TRY(make_twiddles<double>(tw64, M, s));
    HX_TRY(upload_c<double>(in64, seq, s));
    HX_TRY(dev_alloc(out64, sizeof(double2) * M));
    LineArgs<double> a = {};
    int thr;
    size_t smem;
    HX_TRY(launch_shape<double>(M, rad, 1, 1, 1, a, &thr, &smem));
    a.n_log = M;
    a.nlines = 1;
    a.tw = (const double2*)tw64.p;
    a.in = (const double2*)in64.p;
    a.in_ls = M; a.in_es = 1; a.in_bs = 0;
    a.in_count = M; a.in_offset = 0; a.load_add = 0;
    a.out = (double2*)out64.p;
    a.out_ls = M; a.out_es = 1; a.out_bs = 0;
    a.out_count = M; a.out_offset = 0; a.store_add = 0; a.out_mod = M;
    a.scale = make_double2(1.0, 0.0);
    HX_TRY(run_line<double>(a, thr, smem, -1, false, 1, s));
    HX_TRY(dev_alloc(dst, sizeof(typename cplx<T>::type) * M));
    narrow_kernel<T><<<ceil_div(M, 256), 256, 0, s>>>((const double2*)out64.p, (typename cplx<T>::type*)dst.p, M,
                                                       scale);
    HX_TRY(launch_status("narrow_kernel"));
    return cuda_status(cudaStreamSynchronize(s), "spectrum sync");
}

// ---- one axis of a zero-padded FFT ----------------------------------------------------------------

// Tables of one axis of length N, for the element type T.  When N is not 2,3,5,7-smooth the axis
// runs Bluestein: a circular convolution of length M >= 2N-1 with the chirp b_n = exp(i pi n^2/N).
struct AxisTables {
    int N = 0, M = 0;
    bool bluestein = false;
    std::vector<int> radices;
    DevBuf tw;
    DevBuf tws;  // stage twiddle tables of the register-resident kernel (complex64 power-of-two axes)
    DevBuf chirp_f, chirp_i;  // conj(b) for forward, b for inverse (length N)
    DevBuf spec_f, spec_i;    // FFT_M of the wrapped kernel / M
};

// Stage twiddle tables of an N-point power-of-two line for fft_pow2_kernel: exp(-2 pi i p k / (16 NS)) for
// NS = 16, 256 and p = 1, 2, 4, 8, each row NS entries long (float64 arguments, rounded once).
template <typename T>
int make_stage_tables(DevBuf& dst, int N, cudaStream_t s) {
    if (sizeof(T) != 4 || N < 256 || N > 4096 || (N & (N - 1)) != 0) return HX_OK;
    std::vector<cd> v(kP2TwEntries, cd(1, 0));
    for (int NS : {16, 256}) {
        const int off = NS == 16 ? p2_tw_offset<16>() : p2_tw_offset<256>();
        if (NS == 256 && N < 4096) continue;
        const int pw[4] = {1, 2, 4, 8};
        for (int row = 0; row < 4; ++row)
            for (int k = 0; k < NS; ++k) {
                const double ang = -2.0 * M_PI * (double)(pw[row] * k) / (16.0 * NS);
                v[off + row * NS + k] = cd(std::cos(ang), std::sin(ang));
            }
    }
    return upload_c<T>(dst, v, s);
}

template <typename T>
int make_axis(AxisTables& ax, int N, cudaStream_t s) {
    constexpr bool r16 = sizeof(T) == 4;
    ax.N = N;
    ax.radices = factor_radices(N, r16);
    if (!ax.radices.empty()) {
        ax.M = N;
        HX_TRY(make_stage_tables<T>(ax.tws, N, s));
        return make_twiddles<T>(ax.tw, N, s);
    }
    ax.bluestein = true;
    ax.M = next_pow2(2 * N - 1);
    ax.radices = factor_radices(ax.M, r16);
    HX_TRY(make_twiddles<T>(ax.tw, ax.M, s));
    std::vector<cd> b(N);
    for (int n = 0; n < N; ++n) {
        // exp(i pi n^2 / N) with n^2 reduced modulo 2N so the argument stays small.
        const long long q = ((long long)n * n) % (2LL * N);
        const double ang = M_PI * (double)q / (double)N;
        b[n] = cd(std::cos(ang), std::sin(ang));
    }
    std::vector<cd> cf(N), ci(N), kf(ax.M, cd(0, 0)), ki(ax.M, cd(0, 0));
    for (int n = 0; n < N; ++n) {
        cf[n] = std::conj(b[n]);
        ci[n] = b[n];
    }
    // forward: X_k = conj(b_k) sum_n x_n conj(b_n) b_(k-n); inverse uses conj of every chirp.
    for (int n = 0; n < N; ++n) {
        kf[n] = b[n];
        ki[n] = std::conj(b[n]);
        if (n > 0) {
            kf[ax.M - n] = b[n];
            ki[ax.M - n] = std::conj(b[n]);
        }
    }
    HX_TRY(upload_c<T>(ax.chirp_f, cf, s));
    HX_TRY(upload_c<T>(ax.chirp_i, ci, s));
    HX_TRY(device_spectrum<T>(ax.spec_f, kf, ax.M, 1.0 / ax.M, s));
    HX_TRY(device_spectrum<T>(ax.spec_i, ki, ax.M, 1.0 / ax.M, s));
    return HX_OK;
}

// Fill the transform part of LineArgs for one axis (plain or Bluestein), direction sign.
template <typename T>
void axis_args(const AxisTables& ax, int sign, LineArgs<T>& a, bool* conv, int* launch_sign) {
    using Cx = typename cplx<T>::type;
    a.tw = (const Cx*)ax.tw.p;
    a.tws = (const Cx*)ax.tws.p;
    a.n_log = ax.N;
    a.out_mod = ax.N;
    if (ax.bluestein) {
        *conv = true;
        *launch_sign = -1;
        a.chirp_in = (const Cx*)(sign < 0 ? ax.chirp_f.p : ax.chirp_i.p);
        a.chirp_out = a.chirp_in;
        a.mid = (const Cx*)(sign < 0 ? ax.spec_f.p : ax.spec_i.p);
        a.mid_ls = 0;
        a.mid_es = 1;
        a.mid_conj = 0;
    } else {
        *conv = false;
        *launch_sign = sign;
        a.chirp_in = nullptr;
        a.chirp_out = nullptr;
        a.mid = nullptr;
    }
}

// One pass of 1-D transforms along an axis: lines of the source (count, offset in the padded
// array, load index shift) to lines of the destination (count, crop offset, store index shift).
// post_es = 0 selects a factor per output position shared by all lines (post[kk]); a 2-D
// factor such as a transfer function uses post[l*post_ls + kk*post_es].
struct PassIO {
    const void* in;
    long long in_ls, in_es, in_bs;
    int in_count, in_off, load_add;
    const void* pre;
    void* out;
    long long out_ls, out_es, out_bs;
    int out_count, out_off, store_add;
    const void* post;
    long long post_ls, post_es;
};

template <typename T>
int axis_pass(const AxisTables& ax, int sign, int batch, int nlines, const PassIO& io, std::complex<double> scale,
              int min_lines, cudaStream_t s) {
    using Cx = typename cplx<T>::type;
    LineArgs<T> a = {};
    int thr;
    size_t smem;
    HX_TRY(launch_shape<T>(ax.M, ax.radices, nlines, batch, min_lines, a, &thr, &smem));
    bool conv;
    int lsign;
    axis_args<T>(ax, sign, a, &conv, &lsign);
    a.nlines = nlines;
    a.in = (const Cx*)io.in;
    a.in_ls = io.in_ls; a.in_es = io.in_es; a.in_bs = io.in_bs;
    a.in_count = io.in_count; a.in_offset = io.in_off; a.load_add = io.load_add;
    a.pre = (const Cx*)io.pre; a.pre_ls = 0;
    a.out = (Cx*)io.out;
    a.out_ls = io.out_ls; a.out_es = io.out_es; a.out_bs = io.out_bs;
    a.out_count = io.out_count; a.out_offset = io.out_off; a.store_add = io.store_add;
    a.post = (const Cx*)io.post; a.post_ls = io.post_ls; a.post_es = io.post_es ? io.post_es : 1;
    a.scale = make_c<T>((T)scale.real(), (T)scale.imag());
    return run_line<T>(a, thr, smem, lsign, conv, batch, s);
}

}  // namespace
}  // namespace hx

// =================================================================================================
// Zero-padded FFT plan
// =================================================================================================

struct hx_fft_plan {
    int ndim;
    int dtype;
    int n_in[2], N[2], n_out[2], c_in[2], c_out[2];
    hx::AxisTables ax[2];
    hx::DevBuf pre[2], post[2], pre_inv[2], post_inv[2];
    bool has_pre[2], has_post[2];
    std::complex<double> scale;
    size_t esize;
};

namespace {

template <typename T>
int fft_plan_tables(hx_fft_plan* p, const double* const* pre, const double* const* post, cudaStream_t s) {
    for (int d = 0; d < p->ndim; ++d) {
        HX_TRY(hx::make_axis<T>(p->ax[d], p->N[d], s));
        p->has_pre[d] = pre && pre[d];
        p->has_post[d] = post && post[d];
        if (p->has_pre[d]) {
            std::vector<hx::cd> v(p->n_in[d]), vi(p->n_in[d]);
            for (int i = 0; i < p->n_in[d]; ++i) {
                v[i] = hx::cd(pre[d][2 * i], pre[d][2 * i + 1]);
                vi[i] = 1.0 / v[i];
            }
            HX_TRY(hx::upload_c<T>(p->pre[d], v, s));
            HX_TRY(hx::upload_c<T>(p->pre_inv[d], vi, s));
        }
        if (p->has_post[d]) {
            std::vector<hx::cd> v(p->n_out[d]), vi(p->n_out[d]);
            for (int i = 0; i < p->n_out[d]; ++i) {
                v[i] = hx::cd(post[d][2 * i], post[d][2 * i + 1]);
                vi[i] = 1.0 / v[i];
            }
            HX_TRY(hx::upload_c<T>(p->post[d], v, s));
            HX_TRY(hx::upload_c<T>(p->post_inv[d], vi, s));
        }
    }
    return HX_OK;
}

// One axis pass of the padded FFT: index shifts N/2 on both sides (ifftshift / fftshift).
template <typename T>
int fft_pass(const hx_fft_plan* p, int d, int sign, int batch, int nlines,
             const void* in, long long in_ls, long long in_es, long long in_bs, int in_count, int in_off,
             const void* pre, void* out, long long out_ls, long long out_es, long long out_bs, int out_count,
             int out_off, const void* post, std::complex<double> scale, int min_lines, cudaStream_t s) {
    const int N = p->ax[d].N;
    hx::PassIO io = {in, in_ls, in_es, in_bs, in_count, in_off, N / 2, pre,
                     out, out_ls, out_es, out_bs, out_count, out_off, -(N / 2), post, 0, 0};
    return hx::axis_pass<T>(p->ax[d], sign, batch, nlines, io, scale, min_lines, s);
}

template <typename T>
int fft_execute_t(const hx_fft_plan* p, int direction, int batch, const void* in, void* out, void* ws,
                  cudaStream_t s) {
    const bool fwd = direction == HX_FORWARD;
    const int sign = fwd ? -1 : 1;
    // Source and destination planes of this direction.
    const int* n_src = fwd ? p->n_in : p->n_out;
    const int* c_src = fwd ? p->c_in : p->c_out;
    const int* n_dst = fwd ? p->n_out : p->n_in;
    const int* c_dst = fwd ? p->c_out : p->c_in;
    auto src_fac = [&](int d) -> const void* {
        return fwd ? (p->has_pre[d] ? p->pre[d].p : nullptr) : (p->has_post[d] ? p->post_inv[d].p : nullptr);
    };
    auto dst_fac = [&](int d) -> const void* {
        return fwd ? (p->has_post[d] ? p->post[d].p : nullptr) : (p->has_pre[d] ? p->pre_inv[d].p : nullptr);
    };
    std::complex<double> scale = fwd ? p->scale : 1.0 / p->scale;
    if (!fwd) {
        double ntot = 1;
        for (int d = 0; d < p->ndim; ++d) ntot *= p->N[d];
        scale /= ntot;
    }
    if (p->ndim == 1) {
        return fft_pass<T>(p, 0, sign, 1, batch, in, n_src[0], 1, 0, n_src[0], c_src[0], src_fac(0), out, n_dst[0], 1,
                           0, n_dst[0], c_dst[0], dst_fac(0), scale, 1, s);
    }
    // pass x: rows of the source (n_src[1] lines) -> intermediate (n_src[1] x n_dst[0])
    const long long src_sz = (long long)n_src[0] * n_src[1];
    const long long mid_sz = (long long)n_src[1] * n_dst[0];
    const long long dst_sz = (long long)n_dst[0] * n_dst[1];
    HX_TRY(fft_pass<T>(p, 0, sign, batch, n_src[1], in, n_src[0], 1, src_sz, n_src[0], c_src[0], src_fac(0), ws,
                       n_dst[0], 1, mid_sz, n_dst[0], c_dst[0], dst_fac(0), 1.0, 1, s));
    // pass y: columns of the intermediate (n_dst[0] lines, stride n_dst[0]) -> destination
    return fft_pass<T>(p, 1, sign, batch, n_dst[0], ws, 1, n_dst[0], mid_sz, n_src[1], c_src[1], src_fac(1), out, 1,
                       n_dst[0], dst_sz, n_dst[1], c_dst[1], dst_fac(1), scale, 8, s);
}

}  // namespace

extern "C" {

int hx_fft_plan_create(int ndim, const int* in_dims, const int* internal_dims, const int* out_dims,
                       const int* in_offsets, const int* out_offsets, const double* const* pre,
                       const double* const* post, double scale_re, double scale_im, int dtype, void* stream,
                       hx_fft_plan** plan) {
    HX_CHECK_ARG(plan != nullptr, "hx_fft_plan_create: plan pointer is NULL");
    *plan = nullptr;
    HX_CHECK_ARG(ndim == 1 || ndim == 2, "hx_fft_plan_create: ndim must be 1 or 2 (got %d)", ndim);
    HX_CHECK_ARG(dtype == HX_C64 || dtype == HX_C128, "hx_fft_plan_create: unknown dtype %d", dtype);
    HX_CHECK_ARG(in_dims && internal_dims && out_dims && in_offsets && out_offsets, "hx_fft_plan_create: NULL dims");
    for (int d = 0; d < ndim; ++d) {
        HX_CHECK_ARG(in_dims[d] > 0 && out_dims[d] > 0 && internal_dims[d] >= in_dims[d] &&
                         internal_dims[d] >= out_dims[d],
                     "hx_fft_plan_create: inconsistent dims on axis %d", d);
        HX_CHECK_ARG(in_offsets[d] >= 0 && in_offsets[d] + in_dims[d] <= internal_dims[d] && out_offsets[d] >= 0 &&
                         out_offsets[d] + out_dims[d] <= internal_dims[d],
                     "hx_fft_plan_create: cutout outside the padded array on axis %d", d);
    }
    if (hx::fault_injected("plan")) return HX_ERR_INJECTED;
    cudaStream_t s = (cudaStream_t)stream;
    hx_fft_plan* p = new hx_fft_plan();
    p->ndim = ndim;
    p->dtype = dtype;
    p->esize = dtype == HX_C64 ? sizeof(float2) : sizeof(double2);
    for (int d = 0; d < ndim; ++d) {
        p->n_in[d] = in_dims[d];
        p->N[d] = internal_dims[d];
        p->n_out[d] = out_dims[d];
        p->c_in[d] = in_offsets[d];
        p->c_out[d] = out_offsets[d];
    }
    p->scale = std::complex<double>(scale_re, scale_im);
    const int rc = dtype == HX_C64 ? fft_plan_tables<float>(p, pre, post, s) : fft_plan_tables<double>(p, pre, post, s);
    if (rc != HX_OK) {
        delete p;
        return rc;
    }
    *plan = p;
    return HX_OK;
}

size_t hx_fft_workspace_bytes(const hx_fft_plan* p, int direction, int batch) {
    if (!p || p->ndim == 1 || batch <= 0) return 0;
    const bool fwd = direction == HX_FORWARD;
    const int* n_src = fwd ? p->n_in : p->n_out;
    const int* n_dst = fwd ? p->n_out : p->n_in;
    return p->esize * (size_t)batch * n_src[1] * n_dst[0];
}

int hx_fft_execute(const hx_fft_plan* p, int direction, int batch, const void* in, void* out, void* ws,
                   size_t ws_bytes, void* stream) {
    HX_CHECK_ARG(p != nullptr, "hx_fft_execute: plan is NULL");
    HX_CHECK_ARG(direction == HX_FORWARD || direction == HX_BACKWARD, "hx_fft_execute: unknown direction %d",
                 direction);
    HX_CHECK_ARG(batch >= 1 && in && out, "hx_fft_execute: bad batch or NULL field");
    const size_t need = hx_fft_workspace_bytes(p, direction, batch);
    HX_CHECK_ARG(ws_bytes >= need && (need == 0 || ws != nullptr), "hx_fft_execute: workspace of %zu bytes needed",
                 need);
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    cudaStream_t s = (cudaStream_t)stream;
    if (p->dtype == HX_C64) return fft_execute_t<float>(p, direction, batch, in, out, ws, s);
    return fft_execute_t<double>(p, direction, batch, in, out, ws, s);
}

int hx_fft_plan_destroy(hx_fft_plan* p) {
    delete p;
    return HX_OK;
}

}  // extern "C"

// =================================================================================================
// Fourier filter: pad -> FFT -> x transfer function -> inverse FFT -> crop
// =================================================================================================

struct hx_filter_plan {
    int ndim, dtype;
    int n[2], N[2], c[2];
    hx::AxisTables ax[2];
    hx::DevBuf tf, tf_conj;  // tf_conj only for the general (Bluestein) route
    bool fused;              // every padded length 2,3,5,7-smooth: TF multiply inside the column pass
    size_t esize;
};

namespace {

// General route: forward transforms along x and y, TF multiply in the y store, inverse transforms.
template <typename T>
int filter_general_t(const hx_filter_plan* p, int adjoint, int batch, const void* in, void* out, void* ws,
                     cudaStream_t s) {
    using Cx = typename hx::cplx<T>::type;
    const void* tf = adjoint ? p->tf_conj.p : p->tf.p;
    if (p->ndim == 1) {
        const int n = p->n[0], N = p->N[0], c = p->c[0];
        Cx* W = (Cx*)ws;
        hx::PassIO f = {in, n, 1, 0, n, c, 0, nullptr, W, N, 1, 0, N, 0, 0, tf, 0, 1};
        HX_TRY(hx::axis_pass<T>(p->ax[0], -1, 1, batch, f, 1.0, 1, s));
        hx::PassIO b = {W, N, 1, 0, N, 0, 0, nullptr, out, n, 1, 0, n, c, 0, nullptr, 0, 0};
        return hx::axis_pass<T>(p->ax[0], 1, 1, batch, b, 1.0 / N, 1, s);
    }
    const int nx = p->n[0], ny = p->n[1], Nx = p->N[0], Ny = p->N[1];
    const long long in_sz = (long long)nx * ny, w_sz = (long long)ny * Nx, w2_sz = (long long)Ny * Nx;
    Cx* W = (Cx*)ws;
    Cx* W2 = W + (long long)batch * w_sz;
    // x forward: ny rows -> W (ny x Nx)
    hx::PassIO p1 = {in, nx, 1, in_sz, nx, p->c[0], 0, nullptr, W, Nx, 1, w_sz, Nx, 0, 0, nullptr, 0, 0};
    HX_TRY(hx::axis_pass<T>(p->ax[0], -1, batch, ny, p1, 1.0, 1, s));
    // y forward with the TF multiply: Nx columns -> W2 (Ny x Nx); TF[k][l] at l + k*Nx
    hx::PassIO p2 = {W, 1, Nx, w_sz, ny, p->c[1], 0, nullptr, W2, 1, Nx, w2_sz, Ny, 0, 0, tf, 1, Nx};
    HX_TRY(hx::axis_pass<T>(p->ax[1], -1, batch, Nx, p2, 1.0, 8, s));
    // y inverse, keep the cutout rows: -> W (ny x Nx)
    hx::PassIO p3 = {W2, 1, Nx, w2_sz, Ny, 0, 0, nullptr, W, 1, Nx, w_sz, ny, p->c[1], 0, nullptr, 0, 0};
    HX_TRY(hx::axis_pass<T>(p->ax[1], 1, batch, Nx, p3, 1.0 / Ny, 8, s));
    // x inverse, keep the cutout columns
    hx::PassIO p4 = {W, Nx, 1, w_sz, Nx, 0, 0, nullptr, out, nx, 1, in_sz, nx, p->c[0], 0, nullptr, 0, 0};
    return hx::axis_pass<T>(p->ax[0], 1, batch, ny, p4, 1.0 / Nx, 1, s);
}

template <typename T>
int filter_execute_t(const hx_filter_plan* p, int adjoint, int batch, const void* in, void* out, void* ws,
                     cudaStream_t s) {
    using Cx = typename hx::cplx<T>::type;
    const Cx one = hx::make_c<T>(T(1), T(0));
    if (!p->fused) return filter_general_t<T>(p, adjoint, batch, in, out, ws, s);
    if (p->ndim == 1) {
        const hx::AxisTables& ax = p->ax[0];
        hx::LineArgs<T> a = {};
        int thr;
        size_t smem;
        HX_TRY(hx::launch_shape<T>(ax.M, ax.radices, batch, 1, 1, a, &thr, &smem));
        a.tw = (const Cx*)ax.tw.p;
        a.n_log = ax.N; a.nlines = batch;
        a.in = (const Cx*)in; a.in_ls = p->n[0]; a.in_es = 1; a.in_bs = 0;
        a.in_count = p->n[0]; a.in_offset = p->c[0]; a.load_add = 0;
        a.mid = (const Cx*)p->tf.p; a.mid_ls = 0; a.mid_es = 1; a.mid_conj = adjoint;
        a.out = (Cx*)out; a.out_ls = p->n[0]; a.out_es = 1; a.out_bs = 0;
        a.out_count = p->n[0]; a.out_offset = p->c[0]; a.store_add = 0; a.out_mod = ax.N;
        a.scale = hx::make_c<T>(T(1.0 / ax.N), T(0));
        return hx::run_line<T>(a, thr, smem, -1, true, 1, s);
    }
    const int nx = p->n[0], ny = p->n[1], Nx = p->N[0], Ny = p->N[1];
    const long long in_sz = (long long)nx * ny, w_sz = (long long)ny * Nx;
    // pass 1: rows, forward FFT along x of the zero-padded rows -> W (ny x Nx)
    {
        const hx::AxisTables& ax = p->ax[0];
        hx::LineArgs<T> a = {};
        int thr;
        size_t smem;
        HX_TRY(hx::launch_shape<T>(ax.M, ax.radices, ny, batch, 1, a, &thr, &smem));
        a.tw = (const Cx*)ax.tw.p;
        a.tws = (const Cx*)ax.tws.p;
        a.n_log = Nx; a.nlines = ny;
        a.in = (const Cx*)in; a.in_ls = nx; a.in_es = 1; a.in_bs = in_sz;
        a.in_count = nx; a.in_offset = p->c[0]; a.load_add = 0;
        a.out = (Cx*)ws; a.out_ls = Nx; a.out_es = 1; a.out_bs = w_sz;
        a.out_count = Nx; a.out_offset = 0; a.store_add = 0; a.out_mod = Nx;
        a.scale = one;
        HX_TRY(hx::run_line<T>(a, thr, smem, -1, false, batch, s));
    }
    // pass 2: columns, FFT along y, x TF column, inverse FFT along y, keep the cutout rows (in place)
    {
        const hx::AxisTables& ax = p->ax[1];
        hx::LineArgs<T> a = {};
        int thr;
        size_t smem;
        HX_TRY(hx::launch_shape<T>(ax.M, ax.radices, Nx, batch, 8, a, &thr, &smem));
        a.tw = (const Cx*)ax.tw.p;
        a.n_log = Ny; a.nlines = Nx;
        a.in = (const Cx*)ws; a.in_ls = 1; a.in_es = Nx; a.in_bs = w_sz;
        a.in_count = ny; a.in_offset = p->c[1]; a.load_add = 0;
        a.mid = (const Cx*)p->tf.p; a.mid_ls = 1; a.mid_es = Nx; a.mid_conj = adjoint;
        a.out = (Cx*)ws; a.out_ls = 1; a.out_es = Nx; a.out_bs = w_sz;
        a.out_count = ny; a.out_offset = p->c[1]; a.store_add = 0; a.out_mod = Ny;
        a.scale = hx::make_c<T>(T(1.0 / Ny), T(0));
        HX_TRY(hx::run_line<T>(a, thr, smem, -1, true, batch, s));
    }
    // pass 3: rows, inverse FFT along x, keep the cutout columns
    {
        const hx::AxisTables& ax = p->ax[0];
        hx::LineArgs<T> a = {};
        int thr;
        size_t smem;
        HX_TRY(hx::launch_shape<T>(ax.M, ax.radices, ny, batch, 1, a, &thr, &smem));
        a.tw = (const Cx*)ax.tw.p;
        a.tws = (const Cx*)ax.tws.p;
        a.n_log = Nx; a.nlines = ny;
        a.in = (const Cx*)ws; a.in_ls = Nx; a.in_es = 1; a.in_bs = w_sz;
        a.in_count = Nx; a.in_offset = 0; a.load_add = 0;
        a.out = (Cx*)out; a.out_ls = nx; a.out_es = 1; a.out_bs = in_sz;
        a.out_count = nx; a.out_offset = p->c[0]; a.store_add = 0; a.out_mod = Nx;
        a.scale = hx::make_c<T>(T(1.0 / Nx), T(0));
        return hx::run_line<T>(a, thr, smem, 1, false, batch, s);
    }
}

}  // namespace

extern "C" {

int hx_filter_plan_create(int ndim, const int* in_dims, const int* internal_dims, const int* in_offsets,
                          const void* transfer_function, int dtype, void* stream, hx_filter_plan** plan) {
    HX_CHECK_ARG(plan != nullptr, "hx_filter_plan_create: plan pointer is NULL");
    *plan = nullptr;
    HX_CHECK_ARG(ndim == 1 || ndim == 2, "hx_filter_plan_create: ndim must be 1 or 2");
    HX_CHECK_ARG(dtype == HX_C64 || dtype == HX_C128, "hx_filter_plan_create: unknown dtype %d", dtype);
    HX_CHECK_ARG(transfer_function != nullptr, "hx_filter_plan_create: transfer function is NULL");
    for (int d = 0; d < ndim; ++d) {
        HX_CHECK_ARG(in_dims[d] > 0 && internal_dims[d] >= in_dims[d] && in_offsets[d] >= 0 &&
                         in_offsets[d] + in_dims[d] <= internal_dims[d],
                     "hx_filter_plan_create: inconsistent dims on axis %d", d);
    }
    if (hx::fault_injected("plan")) return HX_ERR_INJECTED;
    cudaStream_t s = (cudaStream_t)stream;
    hx_filter_plan* p = new hx_filter_plan();
    p->ndim = ndim;
    p->dtype = dtype;
    p->esize = dtype == HX_C64 ? sizeof(float2) : sizeof(double2);
    long long total = 1;
    for (int d = 0; d < ndim; ++d) {
        p->n[d] = in_dims[d];
        p->N[d] = internal_dims[d];
        p->c[d] = in_offsets[d];
        total *= internal_dims[d];
    }
    int rc = HX_OK;
    p->fused = true;
    for (int d = 0; d < ndim && rc == HX_OK; ++d) {
        rc = dtype == HX_C64 ? hx::make_axis<float>(p->ax[d], p->N[d], s) : hx::make_axis<double>(p->ax[d], p->N[d], s);
        if (p->ax[d].bluestein) p->fused = false;
    }
    if (rc == HX_OK) rc = hx::dev_alloc(p->tf, p->esize * total);
    if (rc == HX_OK)
        rc = hx::cuda_status(cudaMemcpyAsync(p->tf.p, transfer_function, p->esize * total, cudaMemcpyDeviceToDevice, s),
                             "copy transfer function");
    if (rc == HX_OK && !p->fused) {
        rc = hx::dev_alloc(p->tf_conj, p->esize * total);
        if (rc == HX_OK) {
            if (dtype == HX_C64)
                hx::conj_kernel<float><<<hx::ceil_div(total, 256), 256, 0, s>>>(
                    (const float2*)p->tf.p, (float2*)p->tf_conj.p, total);
            else
                hx::conj_kernel<double><<<hx::ceil_div(total, 256), 256, 0, s>>>(
                    (const double2*)p->tf.p, (double2*)p->tf_conj.p, total);
            rc = hx::launch_status("conj_kernel");
        }
    }
    if (rc == HX_OK) rc = hx::cuda_status(cudaStreamSynchronize(s), "filter plan sync");
    if (rc != HX_OK) {
        delete p;
        return rc;
    }
    *plan = p;
    return HX_OK;
}

size_t hx_filter_workspace_bytes(const hx_filter_plan* p, int batch) {
    if (!p || batch <= 0) return 0;
    if (!p->fused) {
        if (p->ndim == 1) return p->esize * (size_t)batch * p->N[0];
        return p->esize * (size_t)batch * ((size_t)p->n[1] * p->N[0] + (size_t)p->N[1] * p->N[0]);
    }
    if (p->ndim == 1) return 0;
    return p->esize * (size_t)batch * p->n[1] * p->N[0];
}

int hx_filter_execute(const hx_filter_plan* p, int adjoint, int batch, const void* in, void* out, void* ws,
                      size_t ws_bytes, void* stream) {
    HX_CHECK_ARG(p != nullptr, "hx_filter_execute: plan is NULL");
    HX_CHECK_ARG(batch >= 1 && in && out, "hx_filter_execute: bad batch or NULL field");
    const size_t need = hx_filter_workspace_bytes(p, batch);
    HX_CHECK_ARG(ws_bytes >= need && (need == 0 || ws != nullptr), "hx_filter_execute: workspace of %zu bytes needed",
                 need);
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    cudaStream_t s = (cudaStream_t)stream;
    if (p->dtype == HX_C64) return filter_execute_t<float>(p, adjoint ? 1 : 0, batch, in, out, ws, s);
    return filter_execute_t<double>(p, adjoint ? 1 : 0, batch, in, out, ws, s);
}

int hx_filter_plan_destroy(hx_filter_plan* p) {
    delete p;
    return HX_OK;
}

}  // extern "C"

// =================================================================================================
// Chirp-Z transform along the lines of a strided array (Bluestein, chirp_z_transform.py:51-105)
// =================================================================================================

struct hx_czt_plan {
    int n, m, M, dtype;
    std::vector<int> radices;
    hx::DevBuf tw, awk2, wk2, spec;
    size_t esize;
};

namespace {

template <typename T>
int czt_tables(hx_czt_plan* p, std::complex<double> w, std::complex<double> a, const double* pre, const double* post,
               cudaStream_t s) {
    const int n = p->n, m = p->m, M = p->M;
    const int kmax = std::max(m, n);
    const std::complex<double> lw = std::log(w), la = std::log(a);
    std::vector<hx::cd> wk2(kmax);
    for (int k = 0; k < kmax; ++k) wk2[k] = std::exp(lw * (0.5 * (double)k * (double)k));
    std::vector<hx::cd> awk2(n), post_v(m), kern(M, hx::cd(0, 0));
    for (int k = 0; k < n; ++k) {
        awk2[k] = std::exp(-la * (double)k) * wk2[k];
        if (pre) awk2[k] *= hx::cd(pre[2 * k], pre[2 * k + 1]);
    }
    for (int k = 0; k < m; ++k) {
        post_v[k] = wk2[k];
        if (post) post_v[k] *= hx::cd(post[2 * k], post[2 * k + 1]);
    }
    // 1 / hstack(wk2[n-1:0:-1], wk2[:m]) zero-padded to M
    for (int j = 0; j < n - 1; ++j) kern[j] = 1.0 / wk2[n - 1 - j];
    for (int k = 0; k < m; ++k) kern[n - 1 + k] = 1.0 / wk2[k];
    HX_TRY(hx::make_twiddles<T>(p->tw, M, s));
    HX_TRY(hx::upload_c<T>(p->awk2, awk2, s));
    HX_TRY(hx::upload_c<T>(p->wk2, post_v, s));
    return hx::device_spectrum<T>(p->spec, kern, M, 1.0 / M, s);
}

template <typename T>
int czt_execute_t(const hx_czt_plan* p, int nlines, int batch, const void* in, long long in_ls, long long in_es,
                  long long in_bs, void* out, long long out_ls, long long out_es, long long out_bs, cudaStream_t s) {
    using Cx = typename hx::cplx<T>::type;
    hx::LineArgs<T> a = {};
    int thr;
    size_t smem;
    HX_TRY(hx::launch_shape<T>(p->M, p->radices, nlines, batch, in_es != 1 ? 8 : 1, a, &thr, &smem));
    a.tw = (const Cx*)p->tw.p;
    a.n_log = p->n; a.nlines = nlines;
    a.in = (const Cx*)in; a.in_ls = in_ls; a.in_es = in_es; a.in_bs = in_bs;
    a.in_count = p->n; a.in_offset = 0; a.load_add = 0;
    a.pre = (const Cx*)p->awk2.p; a.pre_ls = 0;
    a.mid = (const Cx*)p->spec.p; a.mid_ls = 0; a.mid_es = 1; a.mid_conj = 0;
    a.out = (Cx*)out; a.out_ls = out_ls; a.out_es = out_es; a.out_bs = out_bs;
    a.out_count = p->m; a.out_offset = 0; a.store_add = p->n - 1; a.out_mod = p->M;
    a.post = (const Cx*)p->wk2.p; a.post_ls = 0; a.post_es = 1;
    a.scale = hx::make_c<T>(T(1), T(0));
    return hx::run_line<T>(a, thr, smem, -1, true, batch, s);
}

}  // namespace

extern "C" {

int hx_czt_plan_create(int n, int m, double w_re, double w_im, double a_re, double a_im, const double* pre,
                       const double* post, int dtype, void* stream, hx_czt_plan** plan) {
    HX_CHECK_ARG(plan != nullptr, "hx_czt_plan_create: plan pointer is NULL");
    *plan = nullptr;
    HX_CHECK_ARG(n > 0 && m > 0, "hx_czt_plan_create: n and m must be positive (%d, %d)", n, m);
    HX_CHECK_ARG(dtype == HX_C64 || dtype == HX_C128, "hx_czt_plan_create: unknown dtype %d", dtype);
    HX_CHECK_ARG(!(w_re == 0 && w_im == 0) && !(a_re == 0 && a_im == 0), "hx_czt_plan_create: w and a must be nonzero");
    if (hx::fault_injected("plan")) return HX_ERR_INJECTED;
    hx_czt_plan* p = new hx_czt_plan();
    p->n = n;
    p->m = m;
    p->dtype = dtype;
    p->M = hx::next_pow2(n + m - 1);
    p->radices = hx::factor_radices(p->M, dtype == HX_C64);
    p->esize = dtype == HX_C64 ? sizeof(float2) : sizeof(double2);
    if (p->M > hx::max_points<double>(false)) {
        delete p;
        hx::set_error("hx_czt_plan_create: n + m - 1 = %d exceeds the supported length %d", n + m - 1,
                      hx::max_points<double>(false));
        return HX_ERR_UNSUPPORTED;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const std::complex<double> w(w_re, w_im), a(a_re, a_im);
    const int rc = dtype == HX_C64 ? czt_tables<float>(p, w, a, pre, post, s) : czt_tables<double>(p, w, a, pre, post, s);
    if (rc != HX_OK) {
        delete p;
        return rc;
    }
    *plan = p;
    return HX_OK;
}

int hx_czt_execute(const hx_czt_plan* p, int nlines, int batch, const void* in, long long in_line_stride,
                   long long in_elem_stride, long long in_batch_stride, void* out, long long out_line_stride,
                   long long out_elem_stride, long long out_batch_stride, void* stream) {
    HX_CHECK_ARG(p != nullptr, "hx_czt_execute: plan is NULL");
    HX_CHECK_ARG(nlines >= 1 && batch >= 1 && in && out, "hx_czt_execute: bad sizes or NULL pointers");
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    cudaStream_t s = (cudaStream_t)stream;
    if (p->dtype == HX_C64)
        return czt_execute_t<float>(p, nlines, batch, in, in_line_stride, in_elem_stride, in_batch_stride, out,
                                    out_line_stride, out_elem_stride, out_batch_stride, s);
    return czt_execute_t<double>(p, nlines, batch, in, in_line_stride, in_elem_stride, in_batch_stride, out,
                                 out_line_stride, out_elem_stride, out_batch_stride, s);
}

int hx_czt_plan_destroy(hx_czt_plan* p) {
    delete p;
    return HX_OK;
}

}  // extern "C"

// =================================================================================================
// Angular-spectrum transfer function on the padded FFT grid, in FFT order
// =================================================================================================

namespace {

// tf[iy, ix] (FFT order) = mean over the os x os dithers of exp(i sqrt(k^2 - kx^2 - ky^2 + 0j) d),
// with kx = zx + (cx + o) dx at the centred index cx = (ix + Nx/2) mod Nx.
template <typename T>
__global__ void asp_tf_kernel(int Nx, int Ny, double zx, double zy, double dx, double dy, double k, double dist,
                              int os, typename hx::cplx<T>::type* tf) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)Nx * Ny) return;
    const int ix = (int)(idx % Nx), iy = (int)(idx / Nx);
    const int cx = (ix + Nx / 2) % Nx, cy = (iy + Ny / 2) % Ny;
    double re = 0, im = 0;
    const double dz = 1.0 / os;
    for (int oy = 0; oy < os; ++oy) {
        const double ky = zy + cy * dy + (-0.5 + dz / 2 + dz * oy) * dy;
        for (int ox = 0; ox < os; ++ox) {
            const double kx = zx + cx * dx + (-0.5 + dz / 2 + dz * ox) * dx;
            const double r = sqrt(kx * kx + ky * ky);
            const double arg = k * k - r * r;
            double s, c;
            if (arg >= 0) {
                sincos(sqrt(arg) * dist, &s, &c);
                re += c;
                im += s;
            } else {
                re += exp(-sqrt(-arg) * dist);
            }
        }
    }
    const double n = (double)os * os;
    tf[idx] = hx::make_c<T>((T)(re / n), (T)(im / n));
}

// Impulse response of the angular-spectrum propagator (angular_spectrum.py:148-153) on a centred
// regular grid (zero, delta), supersampled like the transfer function, written in grid order.
template <typename T>
__global__ void asp_ir_kernel(int Nx, int Ny, double zx, double zy, double dx, double dy, double k, double dist,
                              int os, typename hx::cplx<T>::type* out) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)Nx * Ny) return;
    const int ix = (int)(idx % Nx), iy = (int)(idx / Nx);
    double re = 0, im = 0;
    const double dz = 1.0 / os;
    for (int oy = 0; oy < os; ++oy) {
        const double y = zy + iy * dy + (-0.5 + dz / 2 + dz * oy) * dy;
        for (int ox = 0; ox < os; ++ox) {
            const double x = zx + ix * dx + (-0.5 + dz / 2 + dz * ox) * dx;
            const double r2 = x * x + y * y + dist * dist;
            const double r = sqrt(r2);
            const double cth = dist / r;
            double s, c;
            sincos(k * r, &s, &c);
            // cos_theta/(2 pi) * exp(i k r) * (1/r^2 - i k/r)
            const double ar = 1.0 / r2, ai = -k / r;
            const double f = cth / (2 * M_PI);
            re += f * (c * ar - s * ai);
            im += f * (c * ai + s * ar);
        }
    }
    const double n = (double)os * os;
    out[idx] = hx::make_c<T>((T)(re / n), (T)(im / n));
}

// Fresnel transfer function (hcipy/propagation/fresnel.py:69-80) in FFT order: the mean over os x os dithers of
// exp(i k d) exp(-i d/(2k) (kx^2 + ky^2)), the constant factor evaluated once.
template <typename T>
__global__ void fresnel_tf_kernel(int Nx, int Ny, double zx, double zy, double dx, double dy, double k, double dist,
                                  int os, typename hx::cplx<T>::type* tf) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)Nx * Ny) return;
    const int ix = (int)(idx % Nx), iy = (int)(idx / Nx);
    const int cx = (ix + Nx / 2) % Nx, cy = (iy + Ny / 2) % Ny;
    const double alpha = -0.5 * dist / k;
    double re = 0, im = 0;
    const double dz = 1.0 / os;
    for (int oy = 0; oy < os; ++oy) {
        const double ky = zy + cy * dy + (-0.5 + dz / 2 + dz * oy) * dy;
        for (int ox = 0; ox < os; ++ox) {
            const double kx = zx + cx * dx + (-0.5 + dz / 2 + dz * ox) * dx;
            double s, c;
            sincos(alpha * (kx * kx + ky * ky), &s, &c);
            re += c;
            im += s;
        }
    }
    double ps, pc;
    sincos(k * dist, &ps, &pc);
    const double n = (double)os * os;
    re /= n;
    im /= n;
    tf[idx] = hx::make_c<T>((T)(pc * re - ps * im), (T)(pc * im + ps * re));
}

// Fresnel impulse response (fresnel.py:55-67) on a centred regular grid (zero, delta), grid order: the mean over
// os x os dithers of exp(i k d) / (i lambda d) exp(i k/(2d) (x^2 + y^2)).
template <typename T>
__global__ void fresnel_ir_kernel(int Nx, int Ny, double zx, double zy, double dx, double dy, double k, double lambda,
                                  double dist, int os, typename hx::cplx<T>::type* out) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)Nx * Ny) return;
    const int ix = (int)(idx % Nx), iy = (int)(idx / Nx);
    const double alpha = 0.5 * k / dist;
    double re = 0, im = 0;
    const double dz = 1.0 / os;
    for (int oy = 0; oy < os; ++oy) {
        const double y = zy + iy * dy + (-0.5 + dz / 2 + dz * oy) * dy;
        for (int ox = 0; ox < os; ++ox) {
            const double x = zx + ix * dx + (-0.5 + dz / 2 + dz * ox) * dx;
            double s, c;
            sincos(alpha * (x * x + y * y), &s, &c);
            re += c;
            im += s;
        }
    }
    // exp(i k d) / (i lambda d) = (sin(k d) - i cos(k d)) / (lambda d)
    double ps, pc;
    sincos(k * dist, &ps, &pc);
    const double fr = ps / (lambda * dist), fi = -pc / (lambda * dist);
    const double n = (double)os * os;
    re /= n;
    im /= n;
    out[idx] = hx::make_c<T>((T)(fr * re - fi * im), (T)(fr * im + fi * re));
}

}  // namespace

extern "C" {

int hx_fresnel_transfer_function(int nx, int ny, double zero_x, double zero_y, double delta_x, double delta_y,
                                 double wavenumber, double distance, int oversampling, int dtype, void* out,
                                 void* stream) {
    HX_CHECK_ARG(nx > 0 && ny > 0 && out != nullptr, "hx_fresnel_transfer_function: bad sizes or NULL output");
    HX_CHECK_ARG(oversampling >= 1, "hx_fresnel_transfer_function: oversampling must be >= 1");
    HX_CHECK_ARG(dtype == HX_C64 || dtype == HX_C128, "hx_fresnel_transfer_function: unknown dtype %d", dtype);
    HX_CHECK_ARG(wavenumber > 0, "hx_fresnel_transfer_function: the wavenumber must be positive");
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    cudaStream_t s = (cudaStream_t)stream;
    const long long n = (long long)nx * ny;
    if (dtype == HX_C64)
        fresnel_tf_kernel<float><<<hx::ceil_div(n, 256), 256, 0, s>>>(nx, ny, zero_x, zero_y, delta_x, delta_y,
                                                                      wavenumber, distance, oversampling, (float2*)out);
    else
        fresnel_tf_kernel<double><<<hx::ceil_div(n, 256), 256, 0, s>>>(nx, ny, zero_x, zero_y, delta_x, delta_y,
                                                                       wavenumber, distance, oversampling,
                                                                       (double2*)out);
    return hx::launch_status("fresnel_tf_kernel");
}

int hx_fresnel_impulse_response(int nx, int ny, double zero_x, double zero_y, double delta_x, double delta_y,
                                double wavenumber, double wavelength, double distance, int oversampling, int dtype,
                                void* out, void* stream) {
    HX_CHECK_ARG(nx > 0 && ny > 0 && out != nullptr, "hx_fresnel_impulse_response: bad sizes or NULL output");
    HX_CHECK_ARG(oversampling >= 1, "hx_fresnel_impulse_response: oversampling must be >= 1");
    HX_CHECK_ARG(dtype == HX_C64 || dtype == HX_C128, "hx_fresnel_impulse_response: unknown dtype %d", dtype);
    HX_CHECK_ARG(distance != 0 && wavelength > 0, "hx_fresnel_impulse_response: distance and wavelength must be nonzero");
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    cudaStream_t s = (cudaStream_t)stream;
    const long long n = (long long)nx * ny;
    if (dtype == HX_C64)
        fresnel_ir_kernel<float><<<hx::ceil_div(n, 256), 256, 0, s>>>(nx, ny, zero_x, zero_y, delta_x, delta_y,
                                                                      wavenumber, wavelength, distance, oversampling,
                                                                      (float2*)out);
    else
        fresnel_ir_kernel<double><<<hx::ceil_div(n, 256), 256, 0, s>>>(nx, ny, zero_x, zero_y, delta_x, delta_y,
                                                                       wavenumber, wavelength, distance, oversampling,
                                                                       (double2*)out);
    return hx::launch_status("fresnel_ir_kernel");
}

int hx_asp_impulse_response(int nx, int ny, double zero_x, double zero_y, double delta_x, double delta_y,
                            double wavenumber, double distance, int oversampling, int dtype, void* out, void* stream) {
    HX_CHECK_ARG(nx > 0 && ny > 0 && out != nullptr, "hx_asp_impulse_response: bad sizes or NULL output");
    HX_CHECK_ARG(oversampling >= 1, "hx_asp_impulse_response: oversampling must be >= 1");
    HX_CHECK_ARG(dtype == HX_C64 || dtype == HX_C128, "hx_asp_impulse_response: unknown dtype %d", dtype);
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    cudaStream_t s = (cudaStream_t)stream;
    const long long n = (long long)nx * ny;
    if (dtype == HX_C64)
        asp_ir_kernel<float><<<hx::ceil_div(n, 256), 256, 0, s>>>(nx, ny, zero_x, zero_y, delta_x, delta_y, wavenumber,
                                                                  distance, oversampling, (float2*)out);
    else
        asp_ir_kernel<double><<<hx::ceil_div(n, 256), 256, 0, s>>>(nx, ny, zero_x, zero_y, delta_x, delta_y,
                                                                   wavenumber, distance, oversampling, (double2*)out);
    return hx::launch_status("asp_ir_kernel");
}

int hx_asp_transfer_function(int nx, int ny, double zero_x, double zero_y, double delta_x, double delta_y,
                             double wavenumber, double distance, int oversampling, int dtype, void* out, void* stream) {
    HX_CHECK_ARG(nx > 0 && ny > 0 && out != nullptr, "hx_asp_transfer_function: bad sizes or NULL output");
    HX_CHECK_ARG(oversampling >= 1, "hx_asp_transfer_function: oversampling must be >= 1");
    HX_CHECK_ARG(dtype == HX_C64 || dtype == HX_C128, "hx_asp_transfer_function: unknown dtype %d", dtype);
    if (hx::fault_injected("launch")) return HX_ERR_INJECTED;
    cudaStream_t s = (cudaStream_t)stream;
    const long long n = (long long)nx * ny;
    if (dtype == HX_C64)
        asp_tf_kernel<float><<<hx::ceil_div(n, 256), 256, 0, s>>>(nx, ny, zero_x, zero_y, delta_x, delta_y, wavenumber,
                                                                  distance, oversampling, (float2*)out);
    else
        asp_tf_kernel<double><<<hx::ceil_div(n, 256), 256, 0, s>>>(nx, ny, zero_x, zero_y, delta_x, delta_y,
                                                                   wavenumber, distance, oversampling, (double2*)out);
    return hx::launch_status("asp_tf_kernel");
}

}  // extern "C"
