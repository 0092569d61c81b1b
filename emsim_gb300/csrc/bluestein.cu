// Line DFTs of lengths that are not powers of two, by Bluestein's chirp-z algorithm
// (L. Bluestein, "A linear filtering approach to the computation of discrete Fourier
// transform", IEEE Trans. Audio Electroacoust. 18 (1970) 451-455) on the power-of-two
// fast path:
//   X_k = sum_j x_j W^{jk},  W = exp(-2 pi i / n),  jk = (j^2 + k^2 - (k - j)^2) / 2
//       = w_k * sum_j (x_j w_j) conj(w)_{k-j},     w_j = exp(-i pi j^2 / n),
// a circular convolution of length M = 2^m >= 2n - 1 evaluated as
// IFFT_M(FFT_M(a) * H) with H = FFT_M(h) / M precomputed per length (h_m = conj(w)_m for
// |m| < n, wrapped).  The inverse transform swaps w and conj(w).  Phases j^2 pi / n are
// formed from j^2 mod 2n in integers and FP64, so the tables are accurate for any n.
//
// Used by generic_dft_rows / generic_dft_cols for every length n >= 3 with 2n - 1 <= 4096
// that is not a power of two (others keep the direct DFT).  One kernel per direction does
// the whole line transform in registers and shared memory: load the line times the
// chirp, zero-padded to M; forward FFT_M (the fast path's register Stockham FFT); times
// H; inverse FFT_M; times the chirp, store the first n outputs.  One read and one write
// of each line, O(M log M) arithmetic instead of O(n^2).
#include <map>
#include <mutex>
#include <string>
#include <utility>

#include "engine.h"
#include "wave_passes.cuh"

namespace emsim_gb300 {
namespace {

struct Chirp {
    int n = 0, M = 0;
    float2* hf = nullptr;  // FFT_M(h) / M of the forward kernel h_m = conj(w)_m
    float2* hi = nullptr;  // same for the inverse (h_m = w_m); follows hf
    float2* w = nullptr;   // w_j = exp(-i pi j^2 / n), j < n
};

std::mutex g_mu;
std::map<std::pair<int, int>, Chirp> g_chirps;  // (device, n)

int next_pow2(int v) {
    int p = 1;
    while (p < v) p <<= 1;
    return p;
}

__global__ void chirp_tables_kernel(int n, int M, float2* w, float2* hf, float2* hi) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M) return;
    const long long two_n = 2LL * n;
    if (m < n) {
        const double ph = M_PI * (double)(((long long)m * m) % two_n) / (double)n;
        double s, c;
        sincos(ph, &s, &c);
        w[m] = make_float2((float)c, (float)-s);
    }
    const int d = m < n ? m : (m > M - n ? M - m : -1);  // |k - j| for this wrapped index
    if (d < 0) {
        hf[m] = make_float2(0.f, 0.f);
        hi[m] = make_float2(0.f, 0.f);
    } else {
        const double ph = M_PI * (double)(((long long)d * d) % two_n) / (double)n;
        double s, c;
        sincos(ph, &s, &c);
        const double inv_m = 1.0 / (double)M;
        hf[m] = make_float2((float)(c * inv_m), (float)(s * inv_m));   // conj(w)_d / M
        hi[m] = make_float2((float)(c * inv_m), (float)(-s * inv_m));  // w_d / M
    }
}

__device__ __forceinline__ float2 chirp(const float2* __restrict__ w, int j, int inverse) {
    float2 c = __ldg(w + j);
    if (inverse) c.y = -c.y;
    return c;
}

// B lines of length n per CTA (T = M / 8 threads each, row layout); lines are contiguous
template <int M>
__global__ void __launch_bounds__(512) blu_rows_kernel(const float2* in, float2* out, long long lines, int n,
                                                       const float2* __restrict__ w, const float2* __restrict__ h,
                                                       int inverse, const float2* __restrict__ tw) {
    constexpr int T = M / 8;
    constexpr bool WARP_ONLY = (T <= 32);
    extern __shared__ float2 sm[];
    const int B = blockDim.x / T;
    const int b = threadIdx.x / T;
    const int t = threadIdx.x - b * T;
    const long long line = (long long)blockIdx.x * B + b;
    const bool live = line < lines;
    float2 v[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        const int j = t + m * T;
        v[m] = (live && j < n) ? cmul(in[line * n + j], chirp(w, j, inverse)) : make_float2(0.f, 0.f);
    }
    fft::fft_regs<M, false, WARP_ONLY>(v, sm, b, t, RowAddr<M>{}, tw);
#pragma unroll
    for (int m = 0; m < 8; ++m) v[m] = cmul(v[m], __ldg(h + t + m * T));
    fft::fft_regs<M, true, WARP_ONLY>(v, sm, b, t, RowAddr<M>{}, tw);
    if (live) {
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            const int k = t + m * T;
            if (k < n) out[line * n + k] = cmul(v[m], chirp(w, k, inverse));
        }
    }
}

// B columns of length n per CTA (column layout, b fastest), in place; the last tile may
// be partial
template <int M>
__global__ void __launch_bounds__(ColThreads<M>::MAX) blu_cols_kernel(float2* data, int n, int n_cols,
                                                                      long long img_stride,
                                                                      const float2* __restrict__ w,
                                                                      const float2* __restrict__ h, int inverse,
                                                                      const float2* __restrict__ tw) {
    constexpr int T = M / 8;
    extern __shared__ float2 sm[];
    const int B = blockDim.x / T;
    const int b = threadIdx.x & (B - 1);
    const int t = threadIdx.x / B;
    const int col = blockIdx.x * B + b;
    const bool live = col < n_cols;
    float2* base = data + blockIdx.y * img_stride + col;
    const long long ld = n_cols;
    ColAddrRt addr{B};
    float2 v[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        const int j = t + m * T;
        v[m] = (live && j < n) ? cmul(base[j * ld], chirp(w, j, inverse)) : make_float2(0.f, 0.f);
    }
    fft::fft_regs<M, false, false>(v, sm, b, t, addr, tw);
#pragma unroll
    for (int m = 0; m < 8; ++m) v[m] = cmul(v[m], __ldg(h + t + m * T));
    fft::fft_regs<M, true, false>(v, sm, b, t, addr, tw);
    if (live) {
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            const int k = t + m * T;
            if (k < n) base[k * ld] = cmul(v[m], chirp(w, k, inverse));
        }
    }
}

template <int M>
int blu_rows_n(const float2* in, float2* out, long long lines, int n, const float2* w, const float2* h, bool inverse,
               cudaStream_t st) {
    constexpr int T = M / 8;
    const int threads = T > 256 ? T : 256;
    const int B = threads / T;
    const size_t smem = (size_t)fft::RowLayout<M>::words(B) * sizeof(float2);
    EMSIM_TRY(ensure_smem_attr((const void*)blu_rows_kernel<M>, smem));
    const long long grid = (lines + B - 1) / B;
    EMSIM_REQUIRE(grid <= 0x7fffffffLL, EMSIM_GB300_ERR_UNSUPPORTED, "bluestein rows: too many lines");
    blu_rows_kernel<M><<<(unsigned)grid, threads, smem, st>>>(in, out, lines, n, w, h, inverse ? 1 : 0,
                                                             twiddle_table());
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

template <int M>
int blu_cols_n(float2* data, int n, int n_cols, int n_img, const float2* w, const float2* h, bool inverse,
               cudaStream_t st) {
    constexpr int T = M / 8;
    int B = ColThreads<M>::MAX / T;
    if (B > 64) B = 64;
    while (B > 1 && B / 2 >= n_cols) B >>= 1;  // a power of two, not far above n_cols
    const size_t smem = (size_t)(M + M / 8) * B * sizeof(float2);
    EMSIM_TRY(ensure_smem_attr((const void*)blu_cols_kernel<M>, smem));
    blu_cols_kernel<M><<<dim3((n_cols + B - 1) / B, n_img), B * T, smem, st>>>(
        data, n, n_cols, (long long)n * n_cols, w, h, inverse ? 1 : 0, twiddle_table());
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

// the chirp tables of length n on the current device, created on first use (nullptr when
// n is a power of two, below 3 or beyond the fast path's 4096 after padding)
const Chirp* chirp_for(int n, int* status) {
    *status = EMSIM_GB300_OK;
    if (n < 3 || (n & (n - 1)) == 0 || 2 * n - 1 > 4096) return nullptr;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_chirps.find({dev, n});
    if (it != g_chirps.end()) return &it->second;
    Chirp c;
    c.n = n;
    c.M = next_pow2(2 * n - 1);
    if (c.M < 8) c.M = 8;
    float2* buf = nullptr;
    if (cudaMalloc((void**)&buf, sizeof(float2) * ((size_t)n + 2 * (size_t)c.M)) != cudaSuccess) {
        set_error("bluestein: cudaMalloc of the chirp tables failed");
        *status = EMSIM_GB300_ERR_CUDA;
        return nullptr;
    }
    c.hf = buf;
    c.hi = buf + c.M;
    c.w = c.hi + c.M;
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
        cudaFree(buf);
        set_error("bluestein: stream creation failed");
        *status = EMSIM_GB300_ERR_CUDA;
        return nullptr;
    }
    chirp_tables_kernel<<<(c.M + 255) / 256, 256, 0, st>>>(n, c.M, c.w, c.hf, c.hi);
    RowArgs r;
    r.in = c.hf;
    r.out = c.hf;
    r.in_img_stride = r.out_img_stride = c.M;
    r.n_rows = 2;  // hf and hi are adjacent rows of length M
    r.tw = twiddle_table();
    r.err = error_word();
    int s = cudaGetLastError() == cudaSuccess ? launch_row(c.M, ROW_FFT, r, 1, st) : EMSIM_GB300_ERR_CUDA;
    if (s == EMSIM_GB300_OK && cudaStreamSynchronize(st) != cudaSuccess) s = EMSIM_GB300_ERR_CUDA;
    cudaStreamDestroy(st);
    if (s != EMSIM_GB300_OK) {
        cudaFree(buf);
        set_error("bluestein: building the chirp tables failed");
        *status = s;
        return nullptr;
    }
    return &(g_chirps[{dev, n}] = c);
}

}  // namespace

int bluestein_prepare(int n) {
    int st;
    chirp_for(n, &st);
    return st;
}

bool bluestein_rows(const float2* in, float2* out, int n_rows, int n, bool inverse, int n_img, cudaStream_t st,
                    int* status) {
    const Chirp* c = chirp_for(n, status);
    if (!c) return *status != EMSIM_GB300_OK;
    const long long lines = (long long)n_rows * n_img;
    const float2* h = inverse ? c->hi : c->hf;
    switch (c->M) {
#define EMSIM_CASE(M) \
    case M: *status = blu_rows_n<M>(in, out, lines, n, c->w, h, inverse, st); return true;
        EMSIM_FAST_SIZES(EMSIM_CASE)
#undef EMSIM_CASE
    }
    set_error("bluestein rows: padded length not on the fast path");
    *status = EMSIM_GB300_ERR_UNSUPPORTED;
    return true;
}

bool bluestein_cols(float2* data, int n_rows, int n_cols, bool inverse, int n_img, cudaStream_t st, int* status) {
    const Chirp* c = chirp_for(n_rows, status);
    if (!c) return *status != EMSIM_GB300_OK;
    const float2* h = inverse ? c->hi : c->hf;
    switch (c->M) {
#define EMSIM_CASE(M) \
    case M: *status = blu_cols_n<M>(data, n_rows, n_cols, n_img, c->w, h, inverse, st); return true;
        EMSIM_FAST_SIZES(EMSIM_CASE)
#undef EMSIM_CASE
    }
    set_error("bluestein cols: padded length not on the fast path");
    *status = EMSIM_GB300_ERR_UNSUPPORTED;
    return true;
}

}  // namespace emsim_gb300
