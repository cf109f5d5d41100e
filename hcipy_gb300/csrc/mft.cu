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
