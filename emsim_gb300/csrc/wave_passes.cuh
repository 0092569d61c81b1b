// Fused row / column pass kernels of the multislice engine (power-of-two fast path).
//
// A multislice step psi <- IFFT2(P * FFT2(psi * t_s)) / N is split into two HBM passes:
//   row pass  : [inverse row FFT of the previous step] -> x exp(i sigma V_s) -> forward row FFT
//   col pass  : forward column FFT -> x P(k) * band-limit / N -> inverse column FFT
// so that between steps the wave is kept in "row-inverse pending" form and each step
// reads and writes psi twice (2 x 16 B/px) plus V_s once (4 B/px).  The same two
// kernels, with other op flags, give space_propagate, singleslice_propagate, the lens
// (column pass with the CTF instead of P) and the final |psi|^2.
#pragma once

#include "engine.h"
#include "fft.cuh"

namespace emsim_gb300 {

constexpr double TWO_PI = 6.283185307179586476925286766559;
constexpr double INV_TWO_PI = 0.15915494309189533576888376337251;

template <int N>
struct RowAddr {
    __device__ __forceinline__ int operator()(int b, int p) const { return fft::RowLayout<N>::addr(b, p); }
};

struct ColAddrRt {
    int B;
    __device__ __forceinline__ int operator()(int b, int p) const { return (p + (p >> 3)) * B + b; }
};

// ---------------------------------------------------------------------------------
// row pass: blockDim.x = B * (N/8) threads hold B whole rows of image blockIdx.y
// ---------------------------------------------------------------------------------
template <int N, int OPS>
__global__ void __launch_bounds__(512) row_pass_kernel(RowArgs a) {
    constexpr int T = N / 8;
    constexpr bool WARP_ONLY = (T <= 32);
    extern __shared__ float2 sm[];
    const int b = threadIdx.x / T;
    const int t = threadIdx.x - b * T;
    const int B = blockDim.x / T;
    const int row = blockIdx.x * B + b;
    const long long img = blockIdx.y;
    RowAddr<N> addr;

    float2 v[8];
    if (OPS & ROW_CONST_IN) {
#pragma unroll
        for (int m = 0; m < 8; ++m) v[m] = a.const_val;
    } else {
        const float2* src = a.in + img * a.in_img_stride + (long long)row * N;
#pragma unroll
        for (int m = 0; m < 8; ++m) v[m] = src[t + m * T];
    }

    if (OPS & ROW_IFFT) fft::fft_regs<N, true, WARP_ONLY>(v, sm, b, t, addr, a.tw);

    if (OPS & ROW_GRAD) {
        // dL/dV = 2 sigma Im(mu conj(phi)) with mu = v (the back-propagated wave)
        const float2* ph = a.phi + img * a.phi_img_stride + (long long)row * N;
        float* g = a.grad + img * a.grad_img_stride + (long long)row * N;
        const float s2 = 2.f * a.sigma_grad;
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            const float2 f = ph[t + m * T];
            g[t + m * T] = s2 * (v[m].y * f.x - v[m].x * f.y);
        }
    }

    if (OPS & ROW_TRANSMIT) {
        const float* vs = a.slice + img * a.slice_img_stride + (long long)row * N;
#pragma unroll
        for (int m = 0; m < 8; ++m) v[m] = cmul(v[m], transmit_factor(a.sigma_pi, __ldg(vs + t + m * T)));
    }

    if (OPS & ROW_STORE_PHI) {
        float2* ph = a.phi + img * a.phi_img_stride + (long long)row * N;
#pragma unroll
        for (int m = 0; m < 8; ++m) ph[t + m * T] = v[m];
    }

    if (OPS & ROW_FFT) fft::fft_regs<N, false, WARP_ONLY>(v, sm, b, t, addr, a.tw);

    if (OPS & ROW_OUT_INTENSITY) {
        float* dst = a.out_int + img * a.out_int_img_stride + (long long)row * N;
#pragma unroll
        for (int m = 0; m < 8; ++m) dst[t + m * T] = v[m].x * v[m].x + v[m].y * v[m].y;
    } else {
        float2* dst = a.out + img * a.out_img_stride + (long long)row * N;
#pragma unroll
        for (int m = 0; m < 8; ++m) dst[t + m * T] = v[m];
    }
}

// ---------------------------------------------------------------------------------
// column pass: blockDim.x = B * (N/8) threads hold B whole columns (b fastest)
// ---------------------------------------------------------------------------------
__device__ __forceinline__ float2 lens_factor(int k1, int k2, double fy2, double c2, const ColArgs& a) {
    const float f2 = freq_sq_ref(k1, k2, a.dfx, a.dfy);
    if (!(f2 <= a.aper2)) return make_float2(0.f, 0.f);
    const double fx = (double)k1 * a.dfx64;
    const double q = fma(fx, fx, fy2);
    double chi = q * fma(a.c1, q, -c2);
    chi = fma(-TWO_PI, rint(chi * INV_TWO_PI), chi);  // reduce mod 2 pi in FP64
    float s, c;
    sincosf((float)chi, &s, &c);
    float scale = a.lens_scale;
    if (a.es > 0.0) {
        // quasi-coherent spatial envelope: |grad chi| / (2 pi) = f |Cs lambda^3 f^2 - df lambda|
        // = f |2 c1 f^2 - c2| / pi, damped by exp(-(pi alpha_s / lambda)^2 |grad chi / 2 pi|^2)
        const double g = fma(2.0 * a.c1, q, -c2);
        scale *= (float)exp(-a.es * q * g * g);
    }
    return make_float2(c * scale, -s * scale);
}

// threads per CTA of the column pass: 512 with two CTAs per SM (64 registers), 1024 from
// length 2048 on
template <int N>
struct ColThreads {
    static constexpr int MAX = (N / 8 >= 256) ? 1024 : 512;
    static constexpr int MIN_BLOCKS = (N / 8 >= 256) ? 1 : 2;
};

// x P(k1, k2) / N inside the band-limit disc, 0 outside, for column `col`, rows t + m*T
template <int N>
__device__ __forceinline__ void propagate_col(float2 (&v)[8], int col, int t, const ColArgs& a) {
    constexpr int T = N / 8;
    const int k2a = abs(fftfreq_int(col, a.n_cols));
    const float2 p2 = __ldg(a.p2 + col);
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        const float4 q = __ldg(a.p1 + t + m * T);
        v[m] = (k2a <= __float_as_int(q.z)) ? cmul(v[m], cmul(make_float2(q.x, q.y), p2)) : make_float2(0.f, 0.f);
    }
}

// tiles of B columns: live ones first [0, lo) and last [tiles - hi, tiles), the rest dead
struct LiveTiles {
    int lo, hi;
};
inline LiveTiles live_tiles(const ColArgs& a, int B, int tiles_per_img) {
    if (a.live_lo < 0 || a.live_hi < 0) return {tiles_per_img, 0};
    const int lo = (a.live_lo + B - 1) / B, hi = (a.live_hi + B - 1) / B;
    if (lo + hi >= tiles_per_img) return {tiles_per_img, 0};
    return {lo, hi};
}

template <int N, int MODE>
__global__ void __launch_bounds__(ColThreads<N>::MAX, ColThreads<N>::MIN_BLOCKS)
    col_pass_kernel(ColArgs a, int dead_lo, int dead_hi) {
    constexpr int T = N / 8;
    extern __shared__ float2 sm[];
    const int B = blockDim.x / T;
    const int b = threadIdx.x & (B - 1);
    const int t = threadIdx.x / B;
    const int col = blockIdx.x * B + b;
    const long long img = blockIdx.y;
    ColAddrRt addr{B};

    float2* base = a.data + img * a.img_stride + col;
    const long long ld = a.n_cols;
    if (MODE == COL_PROPAGATE && (int)blockIdx.x >= dead_lo && (int)blockIdx.x < dead_hi) {
        // every column of this tile lies outside the band-limit: the output is zero
#pragma unroll
        for (int m = 0; m < 8; ++m) base[(long long)(t + m * T) * ld] = make_float2(0.f, 0.f);
        return;
    }
    float2 v[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) v[m] = base[(long long)(t + m * T) * ld];

    if (MODE != COL_INV) fft::fft_regs<N, false, false>(v, sm, b, t, addr, a.tw);

    if (MODE == COL_PROPAGATE) propagate_col<N>(v, col, t, a); else if (MODE == COL_LENS) {
        const int k2 = fftfreq_int(col, a.n_cols);
        const double fy = (double)k2 * a.dfy64;
        const double fy2 = fy * fy;
        const double c2 = a.c2v[a.n_c2 > 1 ? img : 0];
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            const int k1 = fftfreq_int(t + m * T, N);
            v[m] = cmul(v[m], lens_factor(k1, k2, fy2, c2, a));
        }
    }

    if (MODE == COL_PROPAGATE || MODE == COL_LENS || MODE == COL_INV) fft::fft_regs<N, true, false>(v, sm, b, t, addr, a.tw);

#pragma unroll
    for (int m = 0; m < 8; ++m) base[(long long)(t + m * T) * ld] = v[m];
}

// ---------------------------------------------------------------------------------
// launchers for one length
// ---------------------------------------------------------------------------------
inline int row_threads(int n) { return n / 8 > 256 ? n / 8 : 256; }

template <int N>
int launch_row_n(int ops, const RowArgs& a, int n_img, cudaStream_t st) {
    constexpr int T = N / 8;
    int threads = row_threads(N);
    int B = tile_with_hint(threads / T, pass_tuning(N).row_rows, 1);
    if (B > a.n_rows) B = a.n_rows;
    threads = B * T;
    const size_t smem = (size_t)fft::RowLayout<N>::words(B) * sizeof(float2);
    dim3 grid(a.n_rows / B, n_img);
    switch (ops) {
#define EMSIM_ROW_CASE(OPS)                                                                                 \
    case OPS: {                                                                                             \
        EMSIM_TRY(ensure_smem_attr((const void*)row_pass_kernel<N, OPS>, smem));                            \
        row_pass_kernel<N, OPS><<<grid, threads, smem, st>>>(a);                                            \
        break;                                                                                              \
    }
        EMSIM_ROW_CASE(ROW_FFT)
        EMSIM_ROW_CASE(ROW_IFFT)
        EMSIM_ROW_CASE(ROW_TRANSMIT | ROW_FFT)
        EMSIM_ROW_CASE(ROW_IFFT | ROW_TRANSMIT | ROW_FFT)
        EMSIM_ROW_CASE(ROW_IFFT | ROW_OUT_INTENSITY)
        EMSIM_ROW_CASE(ROW_CONST_IN | ROW_TRANSMIT | ROW_FFT)
        EMSIM_ROW_CASE(ROW_IFFT | ROW_TRANSMIT | ROW_FFT | ROW_STORE_PHI)
        EMSIM_ROW_CASE(ROW_CONST_IN | ROW_TRANSMIT | ROW_FFT | ROW_STORE_PHI)
        EMSIM_ROW_CASE(ROW_IFFT | ROW_GRAD | ROW_TRANSMIT | ROW_FFT)
        EMSIM_ROW_CASE(ROW_IFFT | ROW_GRAD)
#undef EMSIM_ROW_CASE
        default:
            set_error("row pass: unsupported op combination");
            return EMSIM_GB300_ERR_UNSUPPORTED;
    }
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

inline int col_B_for(int n, int n_cols) {
    const int T = n / 8;
    int B = (T >= 256 ? 1024 : 512) / T;
    if (B > 64) B = 64;
    if (B > n_cols) B = n_cols;
    return B;
}

template <int N>
int launch_col_n(int mode, const ColArgs& a, int n_img, cudaStream_t st) {
    constexpr int T = N / 8;
    const int B = tile_with_hint(col_B_for(N, a.n_cols), pass_tuning(N).col_cols, 1);
    const int threads = B * T;
    const size_t smem = (size_t)(N + N / 8) * B * sizeof(float2);
    const int tiles_per_img = a.n_cols / B;
    dim3 grid(tiles_per_img, n_img);
    const LiveTiles lt = live_tiles(a, B, tiles_per_img);
    const int dead_lo = lt.lo, dead_hi = tiles_per_img - lt.hi;
    switch (mode) {
#define EMSIM_COL_CASE(MODE)                                                                                \
    case MODE: {                                                                                            \
        EMSIM_TRY(ensure_smem_attr((const void*)col_pass_kernel<N, MODE>, smem));                           \
        col_pass_kernel<N, MODE><<<grid, threads, smem, st>>>(a, dead_lo, dead_hi);                         \
        break;                                                                                              \
    }
        EMSIM_COL_CASE(COL_PROPAGATE)
        EMSIM_COL_CASE(COL_LENS)
        EMSIM_COL_CASE(COL_FWD)
        EMSIM_COL_CASE(COL_INV)
#undef EMSIM_COL_CASE
        default:
            set_error("column pass: unsupported mode");
            return EMSIM_GB300_ERR_UNSUPPORTED;
    }
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

}  // namespace emsim_gb300
