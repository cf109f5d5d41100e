// Batched 1-D FFTs along one axis of a strided array, in shared memory, with
// zero-padding, index shifts, cropping, phase factors and (optionally) a
// spectrum multiply plus inverse transform fused into the same launch.
//
// Each CTA owns `lines_per_cta` lines of length M (the shared-memory FFT
// length).  The transform is a mixed-radix Stockham autosort over radices
// {2,3,4,5,7,8}: stage s with radix R and accumulated size Ns reads
// v[r] = buf[j + r M/R], multiplies by the twiddles exp(-+2 pi i r (j mod Ns)/(Ns R)),
// does an R-point DFT in registers and writes buf[(j/Ns) Ns R + j mod Ns + r Ns].
// Every thread keeps its butterflies of a stage in registers across one
// __syncthreads, so the stage runs in place in one shared buffer.  Twiddles
// come from a float64-accurate table exp(-2 pi i t/M), t < M.
//
// Load of line l, FFT index j < M:
//   j >= n_log                      -> 0
//   p = (j + load_add) mod n_log - in_offset   (index shift and zero-pad)
//   value = in[l, p] * pre[l, p] * chirp_in[j] if 0 <= p < in_count, else 0
// Optional conv stage (CONV): forward FFT, times mid[l, k], inverse FFT.
// Store of output kk < out_count:
//   src = (out_offset + kk + store_add) mod out_mod
//   out[l, kk] = buf[src] * chirp_out[src] * post[l, kk] * scale
// This one kernel serves the zero-padded FFT with fftshifts and crop, the
// chirp-Z transform (Bluestein), Bluestein for lengths that are not
// 2,3,5,7-smooth, and the column pass of the Fourier filter.
#pragma once

#include "hx_common.cuh"

namespace hx {

template <typename T>
struct LineArgs {
    using Cx = typename cplx<T>::type;
    int M;                // shared-memory FFT length
    int n_log;            // logical input length (load wrap / zero beyond)
    int nlines;           // lines per field
    int lines_per_cta;
    int pitch;            // shared-memory stride between lines (>= M)
    int nstages;
    unsigned long long radix_code;  // radix of stage s in bits [5s, 5s+5)
    const Cx* tw;         // M entries, exp(-2 pi i t / M)
    // load
    const Cx* in;
    long long in_ls, in_es, in_bs;
    int in_count, in_offset, load_add;
    const Cx* pre;        // indexed [l*pre_ls + p], or null
    long long pre_ls;
    const Cx* chirp_in;   // indexed [j], or null
    // spectrum multiply (CONV)
    const Cx* mid;        // indexed [l*mid_ls + k*mid_es]
    long long mid_ls, mid_es;
    int mid_conj;
    // store
    Cx* out;
    long long out_ls, out_es, out_bs;
    int out_count, out_offset, store_add, out_mod;
    const Cx* chirp_out;  // indexed [src], or null
    const Cx* post;       // indexed [l*post_ls + kk*post_es], or null
    long long post_ls, post_es;
    Cx scale;
    const Cx* tws;        // stage twiddle tables of the register-resident power-of-two kernel (fft_pow2.cuh)
};

template <typename Cx>
__device__ __forceinline__ Cx c_add(Cx a, Cx b) { Cx r; r.x = a.x + b.x; r.y = a.y + b.y; return r; }
template <typename Cx>
__device__ __forceinline__ Cx c_sub(Cx a, Cx b) { Cx r; r.x = a.x - b.x; r.y = a.y - b.y; return r; }
template <typename Cx>
__device__ __forceinline__ Cx c_mul(Cx a, Cx b) {
    Cx r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
template <typename Cx>
__device__ __forceinline__ Cx c_conj(Cx a) { a.y = -a.y; return a; }
// Multiply by SIGN * i.
template <int SIGN, typename Cx>
__device__ __forceinline__ Cx c_rot(Cx z) {
    Cx r;
    if (SIGN < 0) { r.x = z.y; r.y = -z.x; } else { r.x = -z.y; r.y = z.x; }
    return r;
}
template <typename Cx, typename T>
__device__ __forceinline__ Cx c_scale(Cx a, T s) { a.x *= s; a.y *= s; return a; }

// R-point DFTs with W = exp(SIGN 2 pi i / R): y_m = sum_r v_r W^(r m).
template <typename T, int R, int SIGN>
struct Dft;

template <typename T, int SIGN>
struct Dft<T, 2, SIGN> {
    template <typename Cx>
    __device__ __forceinline__ static void run(Cx* v) {
        Cx a = v[0], b = v[1];
        v[0] = c_add(a, b);
        v[1] = c_sub(a, b);
    }
};

template <typename T, int SIGN>
struct Dft<T, 4, SIGN> {
    template <typename Cx>
    __device__ __forceinline__ static void run(Cx* v) {
        Cx t0 = c_add(v[0], v[2]), t1 = c_sub(v[0], v[2]);
        Cx t2 = c_add(v[1], v[3]), t3 = c_rot<SIGN>(c_sub(v[1], v[3]));
        v[0] = c_add(t0, t2);
        v[2] = c_sub(t0, t2);
        v[1] = c_add(t1, t3);
        v[3] = c_sub(t1, t3);
    }
};

template <typename T, int SIGN>
struct Dft<T, 8, SIGN> {
    template <typename Cx>
    __device__ __forceinline__ static void run(Cx* v) {
        const T h = T(0.70710678118654752440);
        Cx a[4], b[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            a[k] = c_add(v[k], v[k + 4]);
            b[k] = c_sub(v[k], v[k + 4]);
        }
        // b_k *= W8^k, W8 = h (1 + SIGN i)
        {
            Cx z = b[1];
            Cx r;
            r.x = h * (z.x - SIGN * z.y);
            r.y = h * (z.y + SIGN * z.x);
            b[1] = r;
        }
        b[2] = c_rot<SIGN>(b[2]);
        {
            Cx z = b[3];
            Cx r;  // W8^3 = h (-1 + SIGN i)
            r.x = h * (-z.x - SIGN * z.y);
            r.y = h * (-z.y + SIGN * z.x);
            b[3] = r;
        }
        Dft<T, 4, SIGN>::run(a);
        Dft<T, 4, SIGN>::run(b);
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            v[2 * m] = a[m];
            v[2 * m + 1] = b[m];
        }
    }
};

// z times exp(SIGN 2 pi i m / 16).
template <typename T, int SIGN, int MM>
__device__ __forceinline__ typename cplx<T>::type w16(typename cplx<T>::type z) {
    constexpr int m = MM % 16;
    if constexpr (m == 0) {
        return z;
    } else if constexpr (m == 4) {
        return c_rot<SIGN>(z);
    } else if constexpr (m == 8) {
        return c_scale(z, T(-1));
    } else if constexpr (m == 12) {
        return c_rot<-SIGN>(z);
    } else {
        // cos and sin of 2 pi m / 16 = m pi / 8 from cos(pi/8), sin(pi/8) and cos(pi/4)
        constexpr double c8 = 0.92387953251128675613, s8 = 0.38268343236508977173, h = 0.70710678118654752440;
        constexpr double cs = m == 1 ? c8 : m == 2 ? h : m == 3 ? s8 : m == 5 ? -s8 : m == 6 ? -h : m == 7 ? -c8
                            : m == 9 ? -c8 : m == 10 ? -h : m == 11 ? -s8 : m == 13 ? s8 : m == 14 ? h : c8;
        constexpr double sn = m == 1 ? s8 : m == 2 ? h : m == 3 ? c8 : m == 5 ? c8 : m == 6 ? h : m == 7 ? s8
                            : m == 9 ? -s8 : m == 10 ? -h : m == 11 ? -c8 : m == 13 ? -c8 : m == 14 ? -h : -s8;
        const T c = T(cs), sg = T(SIGN * sn);
        typename cplx<T>::type r;
        r.x = c * z.x - sg * z.y;
        r.y = c * z.y + sg * z.x;
        return r;
    }
}

// 16 points as 4 x 4: n = 4 n1 + n2, k = k1 + 4 k2; four 4-point DFTs over n1 (in place: slot n2 + 4 k1), the
// twiddles W16^(n2 k1), four 4-point DFTs over n2 (slots 4 k1 + k2).  The result is left in slot order:
// X[k1 + 4 k2] in v[4 k1 + k2] (out_index), and the caller stores it by that map.
template <typename T, int SIGN>
struct Dft<T, 16, SIGN> {
    template <typename Cx>
    __device__ __forceinline__ static void dft4_at(Cx* v, int i0, int st) {
        Cx t[4] = {v[i0], v[i0 + st], v[i0 + 2 * st], v[i0 + 3 * st]};
        Dft<T, 4, SIGN>::run(t);
        v[i0] = t[0];
        v[i0 + st] = t[1];
        v[i0 + 2 * st] = t[2];
        v[i0 + 3 * st] = t[3];
    }
    template <typename Cx>
    __device__ __forceinline__ static void run(Cx* v) {
#pragma unroll
        for (int n2 = 0; n2 < 4; ++n2) dft4_at(v, n2, 4);
        v[5] = w16<T, SIGN, 1>(v[5]);
        v[9] = w16<T, SIGN, 2>(v[9]);
        v[13] = w16<T, SIGN, 3>(v[13]);
        v[6] = w16<T, SIGN, 2>(v[6]);
        v[10] = w16<T, SIGN, 4>(v[10]);
        v[14] = w16<T, SIGN, 6>(v[14]);
        v[7] = w16<T, SIGN, 3>(v[7]);
        v[11] = w16<T, SIGN, 6>(v[11]);
        v[15] = w16<T, SIGN, 9>(v[15]);
#pragma unroll
        for (int k1 = 0; k1 < 4; ++k1) dft4_at(v, 4 * k1, 1);
    }
    // After run(), v[r] holds X[out_index(r)]: the outputs stay in the second pass's order (no register copies).
    __host__ __device__ static constexpr int out_index(int r) { return (r >> 2) + 4 * (r & 3); }
};

template <typename T, int SIGN>
struct Dft<T, 3, SIGN> {
    template <typename Cx>
    __device__ __forceinline__ static void run(Cx* v) {
        const T c = T(-0.5);
        const T s = T(0.86602540378443864676);
        Cx sum = c_add(v[1], v[2]);
        Cx dif = c_sub(v[1], v[2]);
        Cx base;
        base.x = v[0].x + c * sum.x;
        base.y = v[0].y + c * sum.y;
        Cx rot = c_scale(c_rot<SIGN>(dif), s);
        v[0] = c_add(v[0], sum);
        v[1] = c_add(base, rot);
        v[2] = c_sub(base, rot);
    }
};

template <typename T, int SIGN>
struct Dft<T, 5, SIGN> {
    template <typename Cx>
    __device__ __forceinline__ static void run(Cx* v) {
        const T c1 = T(0.30901699437494742410), c2 = T(-0.80901699437494742410);
        const T s1 = T(0.95105651629515357212), s2 = T(0.58778525229247312917);
        Cx p1 = c_add(v[1], v[4]), m1 = c_sub(v[1], v[4]);
        Cx p2 = c_add(v[2], v[3]), m2 = c_sub(v[2], v[3]);
        Cx b1, b2, q1, q2;
        b1.x = v[0].x + c1 * p1.x + c2 * p2.x;
        b1.y = v[0].y + c1 * p1.y + c2 * p2.y;
        b2.x = v[0].x + c2 * p1.x + c1 * p2.x;
        b2.y = v[0].y + c2 * p1.y + c1 * p2.y;
        Cx d1, d2;
        d1.x = s1 * m1.x + s2 * m2.x;
        d1.y = s1 * m1.y + s2 * m2.y;
        d2.x = s2 * m1.x - s1 * m2.x;
        d2.y = s2 * m1.y - s1 * m2.y;
        q1 = c_rot<SIGN>(d1);
        q2 = c_rot<SIGN>(d2);
        v[0] = c_add(v[0], c_add(p1, p2));
        v[1] = c_add(b1, q1);
        v[4] = c_sub(b1, q1);
        v[2] = c_add(b2, q2);
        v[3] = c_sub(b2, q2);
    }
};

template <typename T, int SIGN>
struct Dft<T, 7, SIGN> {
    template <typename Cx>
    __device__ __forceinline__ static void run(Cx* v) {
        const T C[3] = {T(0.62348980185873353053), T(-0.22252093395631440429), T(-0.90096886790241912624)};
        const T S[3] = {T(0.78183148246802980871), T(0.97492791218182360702), T(0.43388373911755812048)};
        Cx p[3], m[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            p[j] = c_add(v[j + 1], v[6 - j]);
            m[j] = c_sub(v[j + 1], v[6 - j]);
        }
        Cx y0 = v[0];
#pragma unroll
        for (int j = 0; j < 3; ++j) y0 = c_add(y0, p[j]);
        Cx out[7];
        out[0] = y0;
#pragma unroll
        for (int k = 1; k <= 3; ++k) {
            Cx b = v[0], d;
            d.x = T(0);
            d.y = T(0);
#pragma unroll
            for (int j = 1; j <= 3; ++j) {
                const int idx = (j * k) % 7;  // cos/sin of 2 pi j k / 7
                const int q = idx <= 3 ? idx : 7 - idx;
                const T cs = C[q - 1];
                const T sn = idx <= 3 ? S[q - 1] : -S[q - 1];
                b.x += cs * p[j - 1].x;
                b.y += cs * p[j - 1].y;
                d.x += sn * m[j - 1].x;
                d.y += sn * m[j - 1].y;
            }
            Cx r = c_rot<SIGN>(d);
            out[k] = c_add(b, r);
            out[7 - k] = c_sub(b, r);
        }
#pragma unroll
        for (int k = 0; k < 7; ++k) v[k] = out[k];
    }
};

// Points each thread holds per stage: 16 for power-of-two lengths, 8 when the
// radices 3, 5 and 7 are in use (their register arrays share one allocation);
// half of that in float64.
template <typename T, bool MIXED>
struct Ppt { static constexpr int value = MIXED ? 8 : 16; };
template <bool MIXED>
struct Ppt<double, MIXED> { static constexpr int value = MIXED ? 4 : 8; };

constexpr int kFftThreads = 512;

// Shared-memory index with one pad element per 32: breaks the power-of-two strides of the early Stockham stages
// (16-way bank conflicts at radix 8) down to 2-way.
__device__ __forceinline__ int sidx(int x) { return x + (x >> 5); }
__host__ __device__ constexpr int smem_elems(int n) { return n + (n >> 5) + 1; }

// One Stockham stage of radix R over all lines in shared memory.
template <typename T, int R, int SIGN, bool MIXED>
__device__ __forceinline__ void fft_stage(typename cplx<T>::type* buf, int M, int pitch, int lines, int Ns,
                                          const typename cplx<T>::type* __restrict__ tw) {
    using Cx = typename cplx<T>::type;
    constexpr int BPT = Ppt<T, MIXED>::value / R > 0 ? Ppt<T, MIXED>::value / R : 1;
    const int nb = M / R;
    const int total = lines * nb;
    const int stride = M / (Ns * R);
    // Power-of-two kernels index with shifts and masks (runtime integer division costs ~20 instructions).
    const int lg_nb = MIXED ? 0 : __ffs(nb) - 1;
    const int lg_ns = MIXED ? 0 : __ffs(Ns) - 1;
    Cx v[BPT][R];
    int dst[BPT];
#pragma unroll
    for (int i = 0; i < BPT; ++i) {
        const int b = threadIdx.x + i * blockDim.x;
        dst[i] = -1;
        if (b < total) {
            int line, j, k, jd;
            if (MIXED) {
                line = b / nb;
                j = b - line * nb;
                k = j % Ns;
                jd = j / Ns;
            } else {
                line = b >> lg_nb;
                j = b & (nb - 1);
                k = j & (Ns - 1);
                jd = j >> lg_ns;
            }
            const int base = line * pitch;
#pragma unroll
            for (int r = 0; r < R; ++r) v[i][r] = buf[sidx(base + j + r * nb)];
            if constexpr (R == 16) {
                // W^r for r < 16 from four table entries W, W^2, W^4, W^8 (at most three products deep).
                const int ks = k * stride;
                Cx w1 = tw[ks], w2 = tw[2 * ks], w4 = tw[4 * ks], w8 = tw[8 * ks];
                if (SIGN > 0) {
                    w1.y = -w1.y;
                    w2.y = -w2.y;
                    w4.y = -w4.y;
                    w8.y = -w8.y;
                }
                const Cx w3 = c_mul(w2, w1);
                Cx wl[8];
                wl[1] = w1;
                wl[2] = w2;
                wl[3] = w3;
                wl[4] = w4;
                wl[5] = c_mul(w4, w1);
                wl[6] = c_mul(w4, w2);
                wl[7] = c_mul(w4, w3);
#pragma unroll
                for (int r = 1; r < 8; ++r) v[i][r] = c_mul(v[i][r], wl[r]);
                v[i][8] = c_mul(v[i][8], w8);
#pragma unroll
                for (int r = 1; r < 8; ++r) v[i][8 + r] = c_mul(v[i][8 + r], c_mul(w8, wl[r]));
            } else {
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    Cx w = tw[r * k * stride];
                    if (SIGN > 0) w.y = -w.y;
                    v[i][r] = c_mul(v[i][r], w);
                }
            }
            Dft<T, R, SIGN>::run(v[i]);
            dst[i] = base + jd * Ns * R + k;
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < BPT; ++i) {
        if (dst[i] >= 0) {
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if constexpr (R == 16) buf[sidx(dst[i] + Dft<T, 16, SIGN>::out_index(r) * Ns)] = v[i][r];
                else buf[sidx(dst[i] + r * Ns)] = v[i][r];
            }
        }
    }
    __syncthreads();
}

template <typename T, int SIGN, bool MIXED>
__device__ __forceinline__ void fft_smem(typename cplx<T>::type* buf, const LineArgs<T>& a, int lines) {
    int Ns = 1;
    unsigned long long code = a.radix_code;
#pragma unroll 1
    for (int s = 0; s < a.nstages; ++s) {
        const int R = (int)(code & 31ull);
        code >>= 5;
        if constexpr (!MIXED && sizeof(T) == 4) {
            if (R == 16) {
                fft_stage<T, 16, SIGN, false>(buf, a.M, a.pitch, lines, Ns, a.tw);
                Ns *= R;
                continue;
            }
        }
        if (R == 8) fft_stage<T, 8, SIGN, MIXED>(buf, a.M, a.pitch, lines, Ns, a.tw);
        else if (R == 4) fft_stage<T, 4, SIGN, MIXED>(buf, a.M, a.pitch, lines, Ns, a.tw);
        else if (R == 2) fft_stage<T, 2, SIGN, MIXED>(buf, a.M, a.pitch, lines, Ns, a.tw);
        else if (MIXED) {
            if (R == 3) fft_stage<T, 3, SIGN, MIXED>(buf, a.M, a.pitch, lines, Ns, a.tw);
            else if (R == 5) fft_stage<T, 5, SIGN, MIXED>(buf, a.M, a.pitch, lines, Ns, a.tw);
            else if (R == 7) fft_stage<T, 7, SIGN, MIXED>(buf, a.M, a.pitch, lines, Ns, a.tw);
        }  // radices are validated at plan time
        Ns *= R;
    }
}

// (line, output index) of the i-th stored element: lines fastest when lines are adjacent in memory.
__device__ __forceinline__ void store_coords(int i, int lines, bool line_fast, int count, int& ll, int& kk) {
    if (line_fast) {
        if (lines == 1) { ll = 0; kk = i; }
        else if (lines == 2) { ll = i & 1; kk = i >> 1; }
        else { ll = i % lines; kk = i / lines; }
    } else if ((count & (count - 1)) == 0) {
        const int lg = __ffs(count) - 1;
        ll = i >> lg;
        kk = i & (count - 1);
    } else {
        ll = i / count;
        kk = i - ll * count;
    }
}

// grid: x = line blocks, y = batch.  SIGN = -1 forward, +1 inverse (of the main FFT).
template <typename T, int SIGN, bool CONV, bool MIXED>
__global__ void __launch_bounds__(kFftThreads) fft_line_kernel(const __grid_constant__ LineArgs<T> a) {
    using Cx = typename cplx<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Cx* buf = reinterpret_cast<Cx*>(smem_raw);

    const int l0 = blockIdx.x * a.lines_per_cta;
    const int lines = min(a.lines_per_cta, a.nlines - l0);
    if (lines <= 0) return;
    const Cx* in = a.in + a.in_bs * blockIdx.y;
    Cx* out = a.out + a.out_bs * blockIdx.y;
    const Cx zero = make_c<T>(T(0), T(0));

    // ---- load ----
    // The buffer is zeroed with 16-byte stores, then only the valid inputs are read and scattered: for a
    // zero-padded transform most FFT points are padding, and inverting the index map (input p -> FFT index j)
    // visits the inputs alone.  U inputs per thread per round (8 in float, 4 in double to stay within 128
    // registers): their global loads are all issued before any shared store.
    constexpr int U = sizeof(T) == 4 ? 8 : 4;
    const bool line_fast = (a.in_es != 1);
    // Index shifts reduced once, so each element needs one conditional subtraction instead of a modulo.
    const int ladd = ((a.load_add % a.n_log) + a.n_log) % a.n_log;
    const int soff = ((a.out_offset + a.store_add) % a.out_mod + a.out_mod) % a.out_mod;
    {
        const int nwords = smem_elems(lines * a.pitch) * (int)sizeof(Cx) / 16;
        float4* b4 = reinterpret_cast<float4*>(buf);
        for (int x = threadIdx.x; x < nwords; x += blockDim.x) b4[x] = make_float4(0.f, 0.f, 0.f, 0.f);
        // a tail of fewer than 16 bytes (an odd number of float2 elements)
        const int tail = smem_elems(lines * a.pitch) - nwords * 16 / (int)sizeof(Cx);
        if ((int)threadIdx.x < tail) buf[nwords * 16 / (int)sizeof(Cx) + threadIdx.x] = zero;
    }
    __syncthreads();
    // valid inputs p in [p_lo, p_hi): the FFT index j = (p + in_offset - load_add) mod n_log lies in [0, n_log)
    const int p_lo = max(0, -a.in_offset);
    const int p_hi = min(a.in_count, a.n_log - a.in_offset);
    const int cnt = max(0, p_hi - p_lo);
    const int nload = lines * cnt;
    int jbase = p_lo + a.in_offset - ladd;  // FFT index of p_lo, in (-n_log, n_log)
    if (jbase < 0) jbase += a.n_log;
    const bool pow2_c = cnt > 0 && (cnt & (cnt - 1)) == 0;
    const int lg_c = __ffs(cnt) - 1;
    for (int i0 = threadIdx.x; i0 < nload; i0 += U * blockDim.x) {
        Cx val[U];
        int dst[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int i = i0 + u * blockDim.x;
            dst[u] = -1;
            if (i < nload) {
                int ll, pp;
                if (line_fast) {
                    if (lines == 1) { ll = 0; pp = i; }
                    else if (lines == 2) { ll = i & 1; pp = i >> 1; }
                    else { ll = i % lines; pp = i / lines; }
                } else if (pow2_c) {
                    ll = i >> lg_c;
                    pp = i & (cnt - 1);
                } else {
                    ll = i / cnt;
                    pp = i - ll * cnt;
                }
                int j = jbase + pp;
                if (j >= a.n_log) j -= a.n_log;
                const int p = p_lo + pp;
                const long long l = l0 + ll;
                Cx v = in[l * a.in_ls + (long long)p * a.in_es];
                if (a.pre) v = c_mul(v, a.pre[l * a.pre_ls + p]);
                if (a.chirp_in) v = c_mul(v, a.chirp_in[j]);
                val[u] = v;
                dst[u] = ll * a.pitch + j;
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (dst[u] >= 0) buf[sidx(dst[u])] = val[u];
    }
    __syncthreads();

    fft_smem<T, SIGN, MIXED>(buf, a, lines);

    if (CONV) {
        const int n = lines * a.M;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const int ll = i / a.M;
            const int k = i - ll * a.M;
            Cx m = a.mid[(long long)(l0 + ll) * a.mid_ls + (long long)k * a.mid_es];
            if (a.mid_conj) m.y = -m.y;
            const int q = sidx(ll * a.pitch + k);
            buf[q] = c_mul(buf[q], m);
        }
        __syncthreads();
        fft_smem<T, -SIGN, MIXED>(buf, a, lines);
    }

    // ---- store ----
    const int nstore = lines * a.out_count;
    const bool line_fast_out = (a.out_es != 1);
    for (int i0 = threadIdx.x; i0 < nstore; i0 += U * blockDim.x) {
        Cx post[U];
        int lls[U], kks[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int i = i0 + u * blockDim.x;
            post[u] = make_c<T>(T(1), T(0));
            lls[u] = -1;
            if (i < nstore) {
                store_coords(i, lines, line_fast_out, a.out_count, lls[u], kks[u]);
                if (a.post) post[u] = a.post[(long long)(l0 + lls[u]) * a.post_ls + (long long)kks[u] * a.post_es];
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (lls[u] < 0) continue;
            const int ll = lls[u], kk = kks[u];
            int src = soff + kk;
            if (src >= a.out_mod) src -= a.out_mod;
            Cx val = c_mul(buf[sidx(ll * a.pitch + src)], a.scale);
            if (a.chirp_out) val = c_mul(val, a.chirp_out[src]);
            if (a.post) val = c_mul(val, post[u]);
            out[(long long)(l0 + ll) * a.out_ls + (long long)kk * a.out_es] = val;
        }
    }
}

}  // namespace hx
