/*
 * hcipy_gb300 -- C ABI of the GB300 (sm_103a) diffraction kernels.
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, and
 * returns an int status (HX_OK = 0, negative on failure; hx_last_error()
 * gives the message of the last failure on the calling thread).  Device
 * buffers are owned by the caller; a plan owns only its constant tables
 * (phase matrices, twiddles, chirps, transfer functions).  `stream` is a
 * cudaStream_t passed as void* (NULL = the legacy default stream).  All
 * execute calls are asynchronous on that stream.
 *
 * Complex data are interleaved (re, im) pairs: HX_C64 = 2 x float32,
 * HX_C128 = 2 x float64, the layouts of numpy complex64 / complex128.
 * Two-dimensional fields are y-major: element (iy, ix) at iy * nx + ix,
 * the order of HCIPy's flat Field on a 2-D CartesianGrid
 * (hcipy/field/field.py:52-65, Field.shaped).
 *
 * Each declaration names the reference interface it replaces
 * (paths relative to the HCIPy source tree).
 */
#ifndef HCIPY_GB300_H
#define HCIPY_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define HX_API __attribute__((visibility("default")))
#else
#define HX_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define HX_OK 0
#define HX_ERR_INVALID (-1)     /* bad argument; the reference raises ValueError */
#define HX_ERR_CUDA (-2)        /* a CUDA runtime call or launch failed */
#define HX_ERR_UNSUPPORTED (-3) /* valid request that this build does not implement */
#define HX_ERR_TIMEOUT (-4)     /* a bounded device-side wait gave up */
#define HX_ERR_ALLOC (-5)       /* device allocation failed */
#define HX_ERR_INJECTED (-6)    /* host-side fault injection (HX_FAULT=alloc|plan|launch) */

/* Element types. */
#define HX_C64 0
#define HX_C128 1
#define HX_F32 2 /* real arrays: DM surfaces, influence functions, phase screens */
#define HX_F64 3

/* Directions of a Fourier operator. */
#define HX_FORWARD 0  /* FourierTransform.forward */
#define HX_BACKWARD 1 /* FourierTransform.backward (the inverse transform, with output weights) */
#define HX_ADJOINT 2  /* the conjugate transpose of forward (input weights); used by gradients */

/* Arithmetic of the MFT GEMMs. */
#define HX_PREC_FP32 0  /* FP32 CUDA-core complex GEMM (HX_C64) or FP64 (HX_C128) */
#define HX_PREC_SPLIT 1 /* split-operand tensor-core GEMM on tcgen05 (grids up to 8192 points per axis) */

/* Tile policy of a plan's GEMMs (no counterpart in the reference). */
#define HX_SCHEDULE_LATENCY 0    /* fill the GPU with this transform alone (splits K for small shapes) */
#define HX_SCHEDULE_THROUGHPUT 1 /* other transforms run beside it: least SM time, K split only past K' = 4096 */

/* Message of the last failure on this thread ("" if none). */
HX_API const char* hx_last_error(void);
/* Library version as major*10000 + minor*100 + patch. */
HX_API int hx_version(void);
/* Number of kernels this library has launched in this process. */
HX_API long long hx_launch_count(void);

/* Kernel timing (no counterpart in the reference, which has no device kernels).  While enabled, every GEMM
 * and FFT pass the library launches is bracketed by a CUDA event pair recorded on the launching stream and
 * tagged with its algorithmic work (complex multiply-adds for a GEMM, bytes moved for an FFT pass).
 * hx_trace_read waits for the recorded events of one kernel family and returns launches, summed device time
 * and summed work since the last reset. */
#define HX_TRACE_SPLIT_GEMM 0 /* split-operand tcgen05 GEMM of the MFT */
#define HX_TRACE_SIMT_GEMM 1  /* CUDA-core complex GEMM of the MFT (FP32 or FP64) */
#define HX_TRACE_FFT 2        /* line-FFT passes (FFT, filter, chirp-Z) */
#define HX_TRACE_ATMOSPHERE 3 /* screen extrusion and sub-pixel shift (work = bytes) */
#define HX_TRACE_DM 4         /* influence-function products and phase screens (work = bytes) */
HX_API int hx_trace_enable(int on);
HX_API int hx_trace_read(int kind, long long* launches, double* total_ms, double* total_work, int reset);

/* ------------------------------------------------------------------------
 * Matrix Fourier transform.
 * Replaces MatrixFourierTransform (hcipy/fourier/matrix_fourier_transform.py:42-224):
 *   forward : out = alpha * M1 . diag(wy) . in . diag(wx) . M2          (:133-176)
 *   backward: in  = alpha * M1^H . diag(wv) . out . diag(wu) . M2^H     (:179-224)
 *   adjoint : in  = alpha * M1^H . out . M2^H  (weights applied by alpha)
 * with M1[v,y] = exp(-i v y) (nv x ny) and M2[x,u] = exp(-i x u) (nx x nu)
 * built in float64 on the device (:67-111).  x,y,u,v are the separated
 * coordinates of the input and output grids (host arrays of float64).
 * w_in_x/w_in_y/w_out_u/w_out_v are the separable weights of non-uniform
 * separated grids, or NULL for uniform grids, whose scalar weight the caller
 * folds into alpha as the reference folds it into the GEMM alpha (:161-172).
 * A 1-D transform is the case ny = nv = 1, y = v = {0}.
 * ------------------------------------------------------------------------ */
typedef struct hx_mft_plan hx_mft_plan;

HX_API int hx_mft_plan_create(int nx, int ny, int nu, int nv,
                       const double* x, const double* y, const double* u, const double* v,
                       const double* w_in_x, const double* w_in_y,
                       const double* w_out_u, const double* w_out_v,
                       int dtype, int precision, void* stream, hx_mft_plan** plan);

/* Bytes of caller-provided scratch that hx_mft_execute needs for `batch` fields. */
HX_API size_t hx_mft_workspace_bytes(const hx_mft_plan* plan, int direction, int batch);

/* `in` holds `batch` contiguous fields of the source plane, `out` receives
 * `batch` fields of the destination plane (both device pointers of the plan's dtype). */
HX_API int hx_mft_execute(const hx_mft_plan* plan, int direction, int batch,
                   const void* in, void* out, double alpha_re, double alpha_im,
                   void* workspace, size_t workspace_bytes, void* stream);

/* Epilogues fused into the last GEMM of hx_mft_execute_ex (replacing the
 * element-wise steps of the Lyot chain, hcipy/coronagraphy/lyot.py:79-90):
 *   HX_EPI_MUL     : out = (alpha * T) * mask            -- Apodizer.forward on the destination plane
 *                                                           (hcipy/optics/apodization.py:25-29)
 *   HX_EPI_BABINET : out = mask * (src - alpha * T)      -- Babinet subtraction E - P^-1[...] followed
 *                                                           by the Lyot stop; mask may be NULL (no stop)
 * mask has one field of the destination plane (broadcast over the batch);
 * src has `batch` fields of the destination plane. */
#define HX_EPI_NONE 0
#define HX_EPI_MUL 1
#define HX_EPI_BABINET 2

HX_API int hx_mft_execute_ex(const hx_mft_plan* plan, int direction, int batch,
                      const void* in, void* out, double alpha_re, double alpha_im,
                      int epilogue, const void* mask, const void* src,
                      void* workspace, size_t workspace_bytes, void* stream);

HX_API int hx_mft_plan_destroy(hx_mft_plan* plan);

/* hx_mft_execute_ex with independent element types (HX_C64 / HX_C128) for the
 * input, the output and the Babinet source.  Plain plans (HX_PREC_FP32) accept
 * only their own dtype.  Split plans take complex64 or complex128 fields; their
 * results carry ~29-bit operands through exact sums, so writing complex128
 * keeps what a complex64 store would round away.  The mask is complex64 for
 * split plans and the plan's dtype otherwise. */
HX_API int hx_mft_execute_io(const hx_mft_plan* plan, int direction, int batch,
                      const void* in, int in_dtype, void* out, int out_dtype,
                      double alpha_re, double alpha_im, int epilogue, const void* mask,
                      const void* src, int src_dtype, void* workspace, size_t workspace_bytes, void* stream);
/* Forward transform of complex64 fields (batch stacked fields of the plan's input grid) times exp(i scale screen)
 * with screen (ny x nx float32, device, shared by the batch) a phase screen in radians at unit scale: a phase
 * element (the atmosphere's AtmosphericLayer/MultiLayerAtmosphere forward with scale = 1 / wavelength,
 * hcipy/atmosphere/atmospheric_model.py:143-151) followed by the transform, with the phase applied while the
 * first GEMM's operand is sliced.  Split-precision plans only (HX_ERR_INVALID otherwise); the workspace is that
 * of a forward execute.  The phase screen is applied to complex64 values exactly as hx_phase_apply does. */
HX_API int hx_mft_execute_phase(const hx_mft_plan* plan, int batch, const void* in, const float* screen,
                                double scale, void* out, int out_dtype, double alpha_re, double alpha_im, void* ws,
                                size_t ws_bytes, void* stream);

/* ------------------------------------------------------------------------
 * Lyot coronagraph and its final image in one call.
 * Replaces LyotCoronagraph.forward (hcipy/coronagraphy/lyot.py:66-92) followed by
 * FraunhoferPropagator.forward (hcipy/propagation/fraunhofer.py:56-71):
 *   E_f   = alpha_fwd * MFT_fpm(E) * (1 - M)
 *   lyot  = stop * (E - alpha_bwd * MFT_fpm^-1(E_f))
 *   image = alpha_img * MFT_img(lyot)
 * fpm_plan maps the pupil to the focal-plane-mask grid, img_plan (or NULL) the
 * pupil to the image grid; both share the pupil and the precision.  lyot_out
 * and/or image_out receive the results (either may be NULL, not both).  With
 * split plans E_f and lyot stay in float-float between the transforms.
 * one_minus_fpm and stop are complex64 for split plans and the plan dtype
 * otherwise; stop may be NULL (no Lyot stop).
 * ------------------------------------------------------------------------ */
HX_API size_t hx_lyot_workspace_bytes(const hx_mft_plan* fpm_plan, const hx_mft_plan* img_plan, int batch);
HX_API int hx_lyot_execute(const hx_mft_plan* fpm_plan, const hx_mft_plan* img_plan, int batch,
                    const void* e, int e_dtype, const void* one_minus_fpm, const void* stop,
                    double alpha_fwd_re, double alpha_fwd_im, double alpha_bwd_re, double alpha_bwd_im,
                    double alpha_img_re, double alpha_img_im,
                    void* lyot_out, int lyot_dtype, void* image_out, int image_dtype,
                    void* workspace, size_t workspace_bytes, void* stream);

/* Dark-hole contrast sums (no single counterpart in the reference, which forms intensities with numexpr,
 * wavefront.py:113-143, and sums them in numpy): sums[b] = sum_p w[p] |E_b[p]|^2 for batch fields of n
 * points (complex64 or complex128), w a float32 weight or region mask per point (NULL: all ones), in
 * compensated float-float arithmetic with a fixed reduction order (deterministic); the workspace holds the
 * per-chunk partials. */
HX_API size_t hx_intensity_sums_workspace_bytes(long long n, int batch);
HX_API int hx_intensity_sums(const void* field, int dtype, long long n, int batch, const float* weights,
                             double* sums, void* workspace, size_t workspace_bytes, void* stream);
/* Its gradient in torch's convention for a real loss of complex fields: out_b = 2 grad[b] w E_b (field dtype). */
HX_API int hx_intensity_sums_grad(const void* field, int dtype, long long n, int batch, const float* weights,
                                  const double* grad, void* out, void* stream);

/* Status of the plan's bounded device-side waits since the last reset: HX_OK, or
 * HX_ERR_TIMEOUT when a wait of the tensor-core GEMM gave up (its CTA then
 * returned without writing).  Synchronizes with the device; reset != 0 clears it. */
HX_API int hx_mft_plan_status(const hx_mft_plan* plan, int reset);

/* Tile policy of the plan's GEMMs, HX_SCHEDULE_LATENCY (default) or HX_SCHEDULE_THROUGHPUT, for plans whose
 * transforms run concurrently with others (several streams, or parallel branches of a CUDA graph): small
 * transforms then take the tile with the least SM time instead of splitting K to fill the GPU alone (a split
 * tensor-core GEMM still splits a contraction longer than 4096 real terms, to keep its sums exact), and the
 * autotuner's measurements are ranked by duration x occupied SMs; FP32/FP64 plans keep their widest CUDA-core
 * tile instead of narrowing it to occupy the GPU. */
HX_API int hx_mft_plan_set_schedule(hx_mft_plan* plan, int schedule);

/* Tile autotuner of the split tensor-core GEMMs (process-wide; no counterpart in the reference).  When on,
 * the first execution of each GEMM shape times every candidate tile (64 or 128 output columns, with and
 * without a split of K) with CUDA events on the caller's stream, synchronizes, and keeps the fastest for
 * later executions of that shape; executions inside CUDA-graph capture use the kept or default tiles and
 * never measure.  Workspace sizes do not depend on it. */
HX_API int hx_autotune(int on);
HX_API int hx_autotune_entries(void);
/* Entry i of the autotuner's table: shape[4] = {A row tiles, output columns, grid z, K steps}, and for each of the
 * n (<= 8) candidates its tile width, K split and measured milliseconds (arrays of 8). */
HX_API int hx_autotune_entry(int i, long long* shape, int* n, int* bn, int* ksplit, float* ms);
HX_API int hx_autotune_clear(void);

/* No counterpart in the reference.  The same transform as hx_mft_execute for
 * callers that cannot allocate device memory while they run (a real-time loop
 * that must not stall on an allocator, a host framework or plugin ABI that hands
 * over only input and output buffers): the intermediate of the two GEMMs lives in
 * a static device array of HX_MFT_NOALLOC_SCRATCH_BYTES compiled into the library
 * (one per GPU that loads it, held until exit) instead of a caller workspace.
 * The call allocates nothing.  Its first call on a device looks up the array's
 * device address, so make that first call before any stream capture; the address
 * is looked up again when the device's context changes (after cudaDeviceReset,
 * the first call again does the lookup).  Split tensor-core plans run through it
 * too while their scratch fits.  A batch
 * whose scratch need (hx_mft_workspace_bytes) exceeds the array is rejected with
 * HX_ERR_INVALID.  All calls share the array: calls that overlap on the GPU race. */
#define HX_MFT_NOALLOC_SCRATCH_BYTES (16 * 1024 * 1024)
HX_API int hx_mft_execute_noalloc(const hx_mft_plan* plan, int direction, int batch,
                           const void* in, void* out, double alpha_re, double alpha_im, void* stream);

/* ------------------------------------------------------------------------
 * Zero-padded FFT with index fftshifts, crop and separable phase factors.
 * Replaces FastFourierTransform (hcipy/fourier/fast_fourier_transform.py:223-406):
 *   forward : out = crop_out( fftshift( FFT_N( ifftshift( pad_in(in * pre) ) ) ) ) * post * scale
 *   backward: in  = crop_in( fftshift( IFFT_N( ifftshift( pad_out(out / post) ) ) ) ) / pre / scale
 * per axis d (axis 0 = x, contiguous): the source is placed at offset in_offsets[d]
 * of the padded length internal_dims[d] and the result is read from out_offsets[d]
 * (the reference's cutouts, :261-275).  pre[d] (length in_dims[d]) and post[d]
 * (length out_dims[d]) are host arrays of interleaved complex float64 or NULL:
 * the per-axis factors of shift_output and shift_input (:277-321), whose product
 * over the axes is the reference's phase array.  Lengths that are not products
 * of 2, 3, 5 and 7 run Bluestein's algorithm.  ndim is 1 or 2.
 * ------------------------------------------------------------------------ */
typedef struct hx_fft_plan hx_fft_plan;

HX_API int hx_fft_plan_create(int ndim, const int* in_dims, const int* internal_dims, const int* out_dims,
                       const int* in_offsets, const int* out_offsets,
                       const double* const* pre, const double* const* post,
                       double scale_re, double scale_im, int dtype, void* stream, hx_fft_plan** plan);
HX_API size_t hx_fft_workspace_bytes(const hx_fft_plan* plan, int direction, int batch);
/* direction HX_FORWARD (input plane -> output plane) or HX_BACKWARD. */
HX_API int hx_fft_execute(const hx_fft_plan* plan, int direction, int batch, const void* in, void* out,
                   void* workspace, size_t workspace_bytes, void* stream);
HX_API int hx_fft_plan_destroy(hx_fft_plan* plan);

/* ------------------------------------------------------------------------
 * Fourier filter: zero-pad to internal_dims, FFT, multiply by the transfer
 * function (conjugated when adjoint != 0), inverse FFT, crop.
 * Replaces FourierFilter.forward/backward (hcipy/fourier/fourier_operations.py:59-151).
 * transfer_function is a DEVICE array of the plan's dtype in FFT order (the
 * reference's ifftshifted transfer function, :47-48), copied into the plan.
 * The 2-D form is three launches: row FFTs, column FFT x TF x inverse FFT,
 * inverse row FFTs of the kept rows.
 * ------------------------------------------------------------------------ */
typedef struct hx_filter_plan hx_filter_plan;

HX_API int hx_filter_plan_create(int ndim, const int* in_dims, const int* internal_dims, const int* in_offsets,
                          const void* transfer_function, int dtype, void* stream, hx_filter_plan** plan);
HX_API size_t hx_filter_workspace_bytes(const hx_filter_plan* plan, int batch);
HX_API int hx_filter_execute(const hx_filter_plan* plan, int adjoint, int batch, const void* in, void* out,
                      void* workspace, size_t workspace_bytes, void* stream);
HX_API int hx_filter_plan_destroy(hx_filter_plan* plan);

/* ------------------------------------------------------------------------
 * Chirp-Z transform X_k = sum_n x_n (a w^-k)^-n, k < m, along lines of a
 * strided array, by Bluestein's algorithm in one launch.
 * Replaces ChirpZTransform (hcipy/fourier/chirp_z_transform.py:39-105); the
 * optional host arrays pre (length n) and post (length m, interleaved complex
 * float64) multiply the input and output, which is how ZoomFastFourierTransform
 * (hcipy/fourier/zoom_fast_fourier_transform.py:69-119) folds its weights and shifts in.
 * ------------------------------------------------------------------------ */
typedef struct hx_czt_plan hx_czt_plan;

HX_API int hx_czt_plan_create(int n, int m, double w_re, double w_im, double a_re, double a_im,
                       const double* pre, const double* post, int dtype, void* stream, hx_czt_plan** plan);
HX_API int hx_czt_execute(const hx_czt_plan* plan, int nlines, int batch,
                   const void* in, long long in_line_stride, long long in_elem_stride, long long in_batch_stride,
                   void* out, long long out_line_stride, long long out_elem_stride, long long out_batch_stride,
                   void* stream);
HX_API int hx_czt_plan_destroy(hx_czt_plan* plan);

/* ------------------------------------------------------------------------
 * Angular-spectrum transfer function exp(i sqrt(k^2 - kx^2 - ky^2 + 0j) d),
 * averaged over oversampling^2 dithered sub-samples, evaluated in float64 on
 * the padded FFT grid (zero, delta per axis) and written in FFT order.
 * Replaces transfer_function_native with evaluate_supersampled
 * (hcipy/propagation/angular_spectrum.py:159-166, hcipy/field/util.py:655-692).
 * ------------------------------------------------------------------------ */
HX_API int hx_asp_transfer_function(int nx, int ny, double zero_x, double zero_y, double delta_x, double delta_y,
                             double wavenumber, double distance, int oversampling, int dtype, void* out,
                             void* stream);

/* Impulse response cos(theta)/(2 pi) exp(i k r) (1/r^2 - i k/r), r^2 = x^2 + y^2 + d^2,
 * averaged over oversampling^2 dithers, on a regular grid (zero, delta), grid order;
 * the transfer function of the other branch is its FFT
 * (hcipy/propagation/angular_spectrum.py:143-157). */
HX_API int hx_asp_impulse_response(int nx, int ny, double zero_x, double zero_y, double delta_x, double delta_y,
                            double wavenumber, double distance, int oversampling, int dtype, void* out,
                            void* stream);

/* ------------------------------------------------------------------------
 * Fresnel transfer function exp(i k d) exp(-i d/(2k) (kx^2 + ky^2)), averaged over oversampling^2 dithered
 * sub-samples, in float64 on the padded FFT grid (zero, delta per axis), FFT order
 * (hcipy/propagation/fresnel.py:69-80 with evaluate_supersampled).
 * ------------------------------------------------------------------------ */
HX_API int hx_fresnel_transfer_function(int nx, int ny, double zero_x, double zero_y, double delta_x, double delta_y,
                                        double wavenumber, double distance, int oversampling, int dtype, void* out,
                                        void* stream);
/* Fresnel impulse response exp(i k d)/(i lambda d) exp(i k/(2d) (x^2 + y^2)), averaged over oversampling^2 dithers,
 * on a regular grid (zero, delta), grid order; the other branch's transfer function is its FFT
 * (hcipy/propagation/fresnel.py:51-67).  wavenumber k includes the refractive index, wavelength is the vacuum
 * wavelength of the 1/(i lambda d) factor. */
HX_API int hx_fresnel_impulse_response(int nx, int ny, double zero_x, double zero_y, double delta_x, double delta_y,
                                       double wavenumber, double wavelength, double distance, int oversampling,
                                       int dtype, void* out, void* stream);

/* ------------------------------------------------------------------------
 * Deformable mirror.
 * Surface of nvec command vectors at once: surface[v, p] = sum_a Phi[p, a] actuators[v, a]
 * (DeformableMirror.surface / ModeBasis.linear_combination, hcipy/optics/deformable_mirror.py:251-262,
 * hcipy/mode_basis/mode_basis.py:239-258).  Phi (npix x nact) is CSR over pupil pixels; vals, actuators
 * and surface are HX_F32 or HX_F64 device arrays, row-major (vector-major).
 * ------------------------------------------------------------------------ */
HX_API int hx_influence_apply(int npix, int nact, const int* row_ptr, const int* col_idx, const void* vals,
                              int dtype, int nvec, const void* actuators, void* surface, void* stream);
/* The transpose, g_actuators[v, a] = sum_p Phi[p, a] g_surface[v, p], from the CSC form of Phi
 * (col_ptr[nact + 1], row_idx[nnz]): the gradient of a loss with respect to the actuators.  No counterpart
 * in the reference, which has no gradients. */
HX_API int hx_influence_apply_transpose(int npix, int nact, const int* col_ptr, const int* row_idx,
                                        const void* vals, int dtype, int nvec, const void* g_surface,
                                        void* g_actuators, void* stream);
/* The same transpose from blocks of 4 consecutive actuators: block b (actuators 4b .. 4b+3) lists the union of
 * their pixels, blk_pix[blk_ptr[b] .. blk_ptr[b + 1]), with 4 weights per listed pixel in blk_vals (row-major,
 * 16-byte aligned, zero where an actuator of the block does not reach the pixel), so a gradient value gathered
 * once serves the block's actuators that overlap there. */
HX_API int hx_influence_apply_transpose_blocked(int npix, int nact, const int* blk_ptr, const int* blk_pix,
                                                const void* blk_vals, int dtype, int nvec, const void* g_surface,
                                                void* g_actuators, void* stream);

/* Phase screen: out[b, p] = e[b % batch_e, p] exp(i scale s[b % batch_s, p]) for b < batch (batch_e and
 * batch_s are 1 or batch).  e/out are HX_C64 or HX_C128 (dtype), s the matching real type.  Replaces the
 * exponentials of DeformableMirror.forward/backward (scale = +-2k, hcipy/optics/deformable_mirror.py:200-238)
 * and AtmosphericLayer.forward/backward (scale = +-1/lambda, hcipy/atmosphere/atmospheric_model.py:143-151). */
HX_API int hx_phase_apply(long long n, int batch, int batch_e, int batch_s, const void* e, int dtype,
                          const void* s, double scale, void* out, void* stream);
/* Its gradient for real s (no counterpart in the reference): g_s = scale Im(conj(out) g_out) (summed over
 * the batch when batch_s == 1), g_e = g_out exp(-i scale s) (summed when batch_e == 1).  Either output may be
 * NULL. */
HX_API int hx_phase_apply_grad(long long n, int batch, int batch_e, int batch_s, const void* e, int dtype,
                               const void* s, double scale, const void* g_out, void* g_s, void* g_e, void* stream);

/* ------------------------------------------------------------------------
 * Infinite atmospheric layer (hcipy/atmosphere/infinite_atmospheric_layer.py:216-364).
 * The ny x nx achromatic screen is a ring buffer of (ny + 1) x (nx + 1) values: logical pixel (i, j) is stored
 * at ((i + row0) % (ny + 1), (j + col0) % (nx + 1)), row0 in [0, ny], col0 in [0, nx]; the spare row and
 * column are outside the logical screen.  One extrusion (InfiniteAtmosphericLayer._extrude, :216-259):
 * where = 0 bottom, 1 top, 2 left, 3 right; stencil_idx (device, nst int64 in [0, ny*nx)) indexes the
 * logical flat screen (flipped for top/right as in the reference); A (nslice x nst), B (nslice x nb) and
 * noise (nb) are HX_F32 or HX_F64 device arrays, nslice = nx for bottom/top and ny for left/right.  The new
 * slice is written into the spare slice; the caller passes the offsets before the step and then moves them:
 * bottom row0 -= 1, top row0 += 1, left col0 -= 1, right col0 += 1 (mod ny + 1 / nx + 1).
 * ------------------------------------------------------------------------ */
typedef struct hx_extrusion {
    void* ring;
    const long long* stencil_idx;
    const void* A;
    const void* B;
    const void* noise;
    int ny, nx, row0, col0, where, nst, nb;
} hx_extrusion;
HX_API int hx_atmosphere_extrude(void* ring, int ny, int nx, int row0, int col0, int where,
                                 const long long* stencil_idx, int nst, const void* A, const void* B, int nb,
                                 const void* noise, int dtype, void* stream);
/* One extrusion of each of count (0..8) layers in one launch (the step k of every layer of a
 * MultiLayerAtmosphere frame that moves k or more pixels, :216-259 per layer); steps is a host array, each ring
 * at most once. */
HX_API int hx_atmosphere_extrude_layers(const hx_extrusion* steps, int count, int dtype, void* stream);
/* Sub-pixel shift of the logical ny x nx screen of a ring_ny x ring_nx ring (a plain image: ring_ny = ny,
 * ring_nx = nx, offsets 0) into out (ny x nx): the separable 7-tap filter taps_row along x then taps_col along
 * y, clamp to edge (quintic weights of subpixel_shift, hcipy/_math/subpixel_shift.py:7-343; taps are host
 * arrays of 7 float64). */
HX_API int hx_atmosphere_shift(const void* ring, int ring_ny, int ring_nx, int ny, int nx, int row0, int col0,
                               const double* taps_row, const double* taps_col, void* out, int dtype, void* stream);
/* The shifts of count (1..8) layers' rings in one pass (host arrays: rings, row0, col0, taps count x 7):
 * layer l's screen into outs[l] (outs or an entry may be NULL) and the sum of the shifted screens, in layer
 * order, into sum (may be NULL): the evolved screens of MultiLayerAtmosphere and the summed screen its
 * forward applies (hcipy/atmosphere/atmospheric_model.py:264-280). */
HX_API int hx_atmosphere_shift_layers(const void* const* rings, int count, int ring_ny, int ring_nx, int ny, int nx,
                                      const int* row0, const int* col0, const double* taps_row,
                                      const double* taps_col, void* const* outs, void* sum, int dtype,
                                      void* stream);
/* out (n) = the sum of count (1..8) screens of n HX_F32 or HX_F64 values; screens is a host array of device
 * pointers.  The phase of layers applied in sequence without propagation between them
 * (MultiLayerAtmosphere.forward with scintillation off, hcipy/atmosphere/atmospheric_model.py:264-280) is the
 * phase of this sum, so one phase application replaces one per layer. */
HX_API int hx_atmosphere_combine(const void* const* screens, int count, long long n, void* out, int dtype,
                                 void* stream);

/* ------------------------------------------------------------------------
 * Electric-field conjugation: one step of the loop of the reference's EFC tutorial
 * (doc/tutorial_notebooks/ElectricFieldConjugation, the update after the Tikhonov inverse of
 * hcipy/util/matrix_inversion.py:71-100): x = [Re E[dz], Im E[dz]], actuators_out = actuators - gain M . x,
 * with M the nact x 2 n_dz float64 EFC matrix (row-major), E the focal-plane field (HX_C64 or HX_C128),
 * dz_index the n_dz dark-zone pixel indices (int32, device).  One launch (gather, product, update), float-float
 * arithmetic with a fixed reduction order.  actuators_out may equal actuators.
 * ------------------------------------------------------------------------ */
HX_API int hx_efc_step(const double* efc_matrix, int nact, int n_dz, const void* field, int dtype,
                       const int* dz_index, const double* actuators, double gain, double* actuators_out,
                       void* stream);

#ifdef __cplusplus
}
#endif

#endif /* HCIPY_GB300_H */
