// Register-resident FFT of complex64 lines whose length is a power of two from 256 to 4096 points.
//
// The same transform as fft_line_kernel (zero-padding and index shift on load, phase factors, index shift and
// crop on store; see fft_line.cuh for the index maps), specialised at compile time for one length N:
//   N = 4096: three radix-16 stages;  N = 256: two;  N = 512 / 1024 / 2048: two radix-16 stages and a last
//   radix-2 / 4 / 8 stage.
// Each thread owns one 16-point butterfly per stage (N/16 threads per line).  The first stage reads its 16
// inputs straight from global memory (only the valid ones; padding is never loaded), and the last stage writes
// its outputs, which are then in natural order, straight to global memory, so a 4096-point line makes two round
// trips through shared memory and the index arithmetic is shifts and masks of compile-time constants.  Stockham
// stage with radix R after sub-transforms of length Ns: butterfly j (k = j mod Ns) reads x[j + r N/R], multiplies
// by W^(r k) with W = exp(-+2 pi i / (Ns R)), and writes (j / Ns) Ns R + k + r Ns.  Shared memory holds one
// padding element per 16, so the stride-16 writes of the first stage hit distinct banks.
#pragma once

#include "fft_line.cuh"

namespace hx {

constexpr int kP2MaxThreads = 512;    // contiguous lines
constexpr int kP2MaxThreadsLF = 1024; // strided lines

template <int N> struct Pow2Shape {
    static_assert(N == 256 || N == 512 || N == 1024 || N == 2048 || N == 4096, "supported lengths");
    static constexpr int T = N / 16;                  // threads per line
    static constexpr int S16 = N == 4096 ? 3 : 2;     // radix-16 stages
    static constexpr int RL = N == 4096 ? 1 : N / 256;  // radix of the last stage (1: none)
    static constexpr int PITCH = N + N / 16;          // shared-memory elements per line
};

__device__ __forceinline__ int p2idx(int x) { return x + (x >> 4); }

// Stage twiddle tables of an N-point line (built at plan time, see p2_stage_tables): for the radix-16 stages
// NS = 16 and 256, four rows of NS entries, exp(-2 pi i p k / (16 NS)) for p = 1, 2, 4, 8, so that the threads of a
// warp (consecutive k) read consecutive entries.  Offset of the stage's rows in the table:
template <int NS> __host__ __device__ constexpr int p2_tw_offset() { return NS == 16 ? 0 : 4 * 16; }
constexpr int kP2TwEntries = 4 * 16 + 4 * 256;

// v[r] *= W^(r k) for the 16 points of a radix-16 butterfly, W = exp(-+2 pi i / (16 NS)), from the stage's four
// table rows (W^k, W^2k, W^4k, W^8k) and products at most three deep.
template <int N, int SIGN, int NS>
__device__ __forceinline__ void p2_twiddle16(float2* v, int k, const float2* __restrict__ tws) {
    if (k == 0) return;
    const float2* t = tws + p2_tw_offset<NS>();
    float2 w1 = __ldg(&t[k]), w2 = __ldg(&t[NS + k]), w4 = __ldg(&t[2 * NS + k]), w8 = __ldg(&t[3 * NS + k]);
    if (SIGN > 0) {
        w1.y = -w1.y;
        w2.y = -w2.y;
        w4.y = -w4.y;
        w8.y = -w8.y;
    }
    const float2 w3 = c_mul(w2, w1);
    float2 wl[8];
    wl[1] = w1;
    wl[2] = w2;
    wl[3] = w3;
    wl[4] = w4;
    wl[5] = c_mul(w4, w1);
    wl[6] = c_mul(w4, w2);
    wl[7] = c_mul(w4, w3);
#pragma unroll
    for (int r = 1; r < 8; ++r) v[r] = c_mul(v[r], wl[r]);
    v[8] = c_mul(v[8], w8);
#pragma unroll
    for (int r = 1; r < 8; ++r) v[8 + r] = c_mul(v[8 + r], c_mul(w8, wl[r]));
}

// Radix-16 stage NS (>= 16) read from shared memory: loads, twiddles and the butterfly (result in slot order).
template <int N, int SIGN, int NS>
__device__ __forceinline__ void p2_stage16_in(const float2* buf, int t, float2* v, const float2* __restrict__ tws) {
#pragma unroll
    for (int r = 0; r < 16; ++r) v[r] = buf[p2idx(t + r * (N / 16))];
    p2_twiddle16<N, SIGN, NS>(v, t & (NS - 1), tws);
    Dft<float, 16, SIGN>::run(v);
}

// Writes a radix-16 stage's outputs (slot order) back to shared memory for the next stage.
template <int SIGN, int NS>
__device__ __forceinline__ void p2_stage16_out(float2* buf, int t, const float2* v) {
    const int dst = (t / NS) * 16 * NS + (t & (NS - 1));
#pragma unroll
    for (int r = 0; r < 16; ++r) buf[p2idx(dst + Dft<float, 16, SIGN>::out_index(r) * NS)] = v[r];
}

// grid: x = blocks of lines_per_cta lines, y = batch; blockDim = lines_per_cta * N / 16.  LF: lines adjacent in
// memory (a column pass), so consecutive threads take consecutive lines and the global accesses coalesce across
// lines; else consecutive threads take consecutive points of one line.
template <int N, int SIGN, bool LF>
__global__ void __launch_bounds__(LF ? kP2MaxThreadsLF : kP2MaxThreads) fft_pow2_kernel(
    const __grid_constant__ LineArgs<float> a) {
    using P = Pow2Shape<N>;
    constexpr int T = P::T;
    extern __shared__ __align__(16) float2 p2_smem[];
    const int lpc = a.lines_per_cta;
    const int ll = LF ? (int)threadIdx.x % lpc : (int)threadIdx.x / T;
    const int t = LF ? (int)threadIdx.x / lpc : (int)threadIdx.x % T;
    const long long l = (long long)blockIdx.x * lpc + ll;
    const bool lok = l < a.nlines;
    float2* buf = p2_smem + ll * P::PITCH;
    const float2* in = a.in + a.in_bs * blockIdx.y;
    float2* out = a.out + a.out_bs * blockIdx.y;
    const int ladd = ((a.load_add % N) + N) % N;
    const int soff = ((a.out_offset + a.store_add) % N + N) % N;

    auto store = [&](int kf, float2 val) {
        int kk = kf - soff;
        if (kk < 0) kk += N;
        if (lok && kk < a.out_count) {
            val = c_mul(val, a.scale);
            if (a.post) val = c_mul(val, a.post[l * a.post_ls + (long long)kk * a.post_es]);
            out[l * a.out_ls + (long long)kk * a.out_es] = val;
        }
    };

    // ---- stage 0 (radix 16, no twiddles): inputs j = t + r N/16, input p = (j + load_add) mod N - in_offset ----
    float2 v[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) {
        int jj = t + r * T + ladd;
        if (jj >= N) jj -= N;
        const int p = jj - a.in_offset;
        float2 x = make_float2(0.0f, 0.0f);
        if (lok && p >= 0 && p < a.in_count) {
            x = in[l * a.in_ls + (long long)p * a.in_es];
            if (a.pre) x = c_mul(x, a.pre[l * a.pre_ls + p]);
        }
        v[r] = x;
    }
    Dft<float, 16, SIGN>::run(v);
    p2_stage16_out<SIGN, 1>(buf, t, v);
    __syncthreads();

    if constexpr (N == 256) {
        // stage 1 is the last: outputs (t / 16) 256 + t % 16 + m 16 = t + m 16
        p2_stage16_in<N, SIGN, 16>(buf, t, v, a.tws);
#pragma unroll
        for (int r = 0; r < 16; ++r) store(t + Dft<float, 16, SIGN>::out_index(r) * 16, v[r]);
    } else {
        p2_stage16_in<N, SIGN, 16>(buf, t, v, a.tws);
        __syncthreads();
        p2_stage16_out<SIGN, 16>(buf, t, v);
        __syncthreads();
        if constexpr (N == 4096) {
            // stage 2 is the last: outputs t + m 256
            p2_stage16_in<N, SIGN, 256>(buf, t, v, a.tws);
#pragma unroll
            for (int r = 0; r < 16; ++r) store(t + Dft<float, 16, SIGN>::out_index(r) * 256, v[r]);
        } else {
            // last stage, radix RL after 256-point sub-transforms: butterflies b = t + i N/16 (i < 16 / RL), inputs
            // b + r 256, twiddles W_N^(r b), outputs b + r 256 in natural order
            constexpr int RL = P::RL;
#pragma unroll
            for (int i = 0; i < 16 / RL; ++i) {
                const int b = t + i * T;
                float2 u[RL];
#pragma unroll
                for (int r = 0; r < RL; ++r) {
                    u[r] = buf[p2idx(b + r * 256)];
                    if (r > 0) {
                        float2 w = a.tw[r * b];
                        if (SIGN > 0) w.y = -w.y;
                        u[r] = c_mul(u[r], w);
                    }
                }
                Dft<float, RL, SIGN>::run(u);
#pragma unroll
                for (int r = 0; r < RL; ++r) store(b + r * 256, u[r]);
            }
        }
    }
}

}  // namespace hx
