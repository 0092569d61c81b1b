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
// that is not a power of two (others keep the direct DFT).  Each call pads its lines into
// a stream-ordered scratch buffer (cudaMallocAsync), runs the fast row or column FFT
// kernels on it, and multiplies back: O(M log M) per line instead of O(n^2).
#include <map>
#include <mutex>
#include <string>
#include <utility>

#include "engine.h"

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

// rows: lines of length n, contiguous, into lines_p padded lines of length M
__global__ void pre_rows_kernel(const float2* __restrict__ in, float2* __restrict__ p, long long lines, long long total,
                                int n, int M, const float2* __restrict__ w, int inverse) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const long long line = i / M;
        const int j = (int)(i - line * M);
        float2 v = make_float2(0.f, 0.f);
        if (line < lines && j < n) {
            float2 c = w[j];
            if (inverse) c.y = -c.y;
            v = cmul(in[line * n + j], c);
        }
        p[i] = v;
    }
}

__global__ void post_rows_kernel(const float2* __restrict__ p, float2* __restrict__ out, long long lines, int n, int M,
                                 const float2* __restrict__ w, int inverse) {
    const long long total = lines * n;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const long long line = i / n;
        const int k = (int)(i - line * n);
        float2 c = w[k];
        if (inverse) c.y = -c.y;
        out[i] = cmul(p[line * M + k], c);
    }
}

// multiply element (.., j, ..) of every padded line by H[j]; stride = distance between
// consecutive j (1 for rows, n_cols_p for columns)
__global__ void mul_kernel(float2* __restrict__ p, long long total, int M, long long stride,
                           const float2* __restrict__ h) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const int j = (int)((i / stride) % M);
        p[i] = cmul(p[i], h[j]);
    }
}

// columns: (n_img, n, n_cols) into (n_img, M, n_cols_p)
__global__ void pre_cols_kernel(const float2* __restrict__ in, float2* __restrict__ p, long long total, int n, int M,
                                int n_cols, int n_cols_p, const float2* __restrict__ w, int inverse) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const long long img = i / ((long long)M * n_cols_p);
        const long long rem = i - img * M * n_cols_p;
        const int j = (int)(rem / n_cols_p);
        const int c = (int)(rem - (long long)j * n_cols_p);
        float2 v = make_float2(0.f, 0.f);
        if (j < n && c < n_cols) {
            float2 f = w[j];
            if (inverse) f.y = -f.y;
            v = cmul(in[(img * n + j) * n_cols + c], f);
        }
        p[i] = v;
    }
}

__global__ void post_cols_kernel(const float2* __restrict__ p, float2* __restrict__ out, long long total, int n, int M,
                                 int n_cols, int n_cols_p, const float2* __restrict__ w, int inverse) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
        const long long img = i / ((long long)n * n_cols);
        const long long rem = i - img * n * n_cols;
        const int k = (int)(rem / n_cols);
        const int c = (int)(rem - (long long)k * n_cols);
        float2 f = w[k];
        if (inverse) f.y = -f.y;
        out[i] = cmul(p[(img * M + k) * n_cols_p + c], f);
    }
}

int grid_for_total(long long total) {
    long long b = (total + 255) / 256;
    if (b > 8192) b = 8192;
    return b < 1 ? 1 : (int)b;
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
    const int M = c->M;
    const long long lines = (long long)n_rows * n_img;
    long long g = 4096 / M;  // largest row tile of the fast row kernels at length M
    if (g < 1) g = 1;
    const long long lines_p = (lines + g - 1) / g * g;
    float2* p = nullptr;
    if (cudaMallocAsync((void**)&p, sizeof(float2) * (size_t)(lines_p * M), st) != cudaSuccess) {
        set_error("bluestein rows: cudaMallocAsync of the scratch lines failed");
        *status = EMSIM_GB300_ERR_CUDA;
        return true;
    }
    const long long total = lines_p * M;
    pre_rows_kernel<<<grid_for_total(total), 256, 0, st>>>(in, p, lines, total, n, M, c->w, inverse ? 1 : 0);
    RowArgs r;
    r.in = p;
    r.out = p;
    r.in_img_stride = r.out_img_stride = total;
    r.n_rows = (int)lines_p;
    r.tw = twiddle_table();
    r.err = error_word();
    int s = cudaGetLastError() == cudaSuccess ? launch_row(M, ROW_FFT, r, 1, st) : EMSIM_GB300_ERR_CUDA;
    if (s == EMSIM_GB300_OK) {
        mul_kernel<<<grid_for_total(total), 256, 0, st>>>(p, total, M, 1, inverse ? c->hi : c->hf);
        s = cudaGetLastError() == cudaSuccess ? launch_row(M, ROW_IFFT, r, 1, st) : EMSIM_GB300_ERR_CUDA;
    }
    if (s == EMSIM_GB300_OK) {
        post_rows_kernel<<<grid_for_total(lines * n), 256, 0, st>>>(p, out, lines, n, M, c->w, inverse ? 1 : 0);
        if (cudaGetLastError() != cudaSuccess) s = EMSIM_GB300_ERR_CUDA;
    }
    cudaFreeAsync(p, st);
    if (s != EMSIM_GB300_OK) set_error("bluestein rows: launch failed");
    *status = s;
    return true;
}

bool bluestein_cols(float2* data, int n_rows, int n_cols, bool inverse, int n_img, cudaStream_t st, int* status) {
    const Chirp* c = chirp_for(n_rows, status);
    if (!c) return *status != EMSIM_GB300_OK;
    const int M = c->M, n = n_rows;
    // column tiles of the fast column kernels are powers of two up to 64 columns
    const int n_cols_p = n_cols < 64 ? next_pow2(n_cols) : (n_cols + 63) / 64 * 64;
    const long long total = (long long)n_img * M * n_cols_p;
    float2* p = nullptr;
    if (cudaMallocAsync((void**)&p, sizeof(float2) * (size_t)total, st) != cudaSuccess) {
        set_error("bluestein cols: cudaMallocAsync of the scratch columns failed");
        *status = EMSIM_GB300_ERR_CUDA;
        return true;
    }
    pre_cols_kernel<<<grid_for_total(total), 256, 0, st>>>(data, p, total, n, M, n_cols, n_cols_p, c->w,
                                                           inverse ? 1 : 0);
    ColArgs a;
    a.data = p;
    a.img_stride = (long long)M * n_cols_p;
    a.n_rows = M;
    a.n_cols = n_cols_p;
    a.tw = twiddle_table();
    a.err = error_word();
    int s = cudaGetLastError() == cudaSuccess ? launch_col(M, COL_FWD, a, n_img, st) : EMSIM_GB300_ERR_CUDA;
    if (s == EMSIM_GB300_OK) {
        mul_kernel<<<grid_for_total(total), 256, 0, st>>>(p, total, M, n_cols_p, inverse ? c->hi : c->hf);
        s = cudaGetLastError() == cudaSuccess ? launch_col(M, COL_INV, a, n_img, st) : EMSIM_GB300_ERR_CUDA;
    }
    if (s == EMSIM_GB300_OK) {
        const long long t2 = (long long)n_img * n * n_cols;
        post_cols_kernel<<<grid_for_total(t2), 256, 0, st>>>(p, data, t2, n, M, n_cols, n_cols_p, c->w,
                                                             inverse ? 1 : 0);
        if (cudaGetLastError() != cudaSuccess) s = EMSIM_GB300_ERR_CUDA;
    }
    cudaFreeAsync(p, st);
    if (s != EMSIM_GB300_OK) set_error("bluestein cols: launch failed");
    *status = s;
    return true;
}

}  // namespace emsim_gb300
