// Projected-potential slices on the power-of-two fast path.
//
// The reference (SliceBuilder.cu:108-133 + slice_builder_cuda.py:88-99) runs an R2C per
// (element, slice), a broadcast multiply by the scattering factors, a multi-pass element
// reduction, a C2R, then a second R2C/C2R pair for the band-limit and a clip.  All of
// that is linear and the filters are real and symmetric, so here
//   V_s + i V_{s+1} = IFFT2( sum_e T_e(k) * FFT2(h_{e,s} + i h_{e,s+1}) )
// with T_e = F(k) * SF_e(k) / N (F = band-limit, symmetrised exactly as the C2R of the
// reference sees it).  Two slices share each complex transform and the element sum,
// multiply and band-limit happen in registers between the forward and inverse column
// FFTs.  Three passes over HBM:
//   A  rows   : hist pair (2 x float) -> forward row FFT -> Z[e, pair]       (complex)
//   B  columns: for each e: fwd col FFT of Z[e, pair], accumulate T_e * Zhat;
//               inverse col FFT -> W[pair] (written over Z[0, pair])
//   C  rows   : W[pair] -> inverse row FFT -> clip(re) -> V[2p], clip(im) -> V[2p+1]
#pragma once

#include <cstdlib>
#include <cstring>

#include "fft16.cuh"
#include "slices.h"
#include "wave_passes.cuh"

namespace emsim_gb300 {

template <int N>
__global__ void __launch_bounds__(512) slice_rows_fwd_kernel(SliceArgs a) {
    constexpr int T = N / 8;
    constexpr bool WARP_ONLY = (T <= 32);
    extern __shared__ float2 sm[];
    const int b = threadIdx.x / T;
    const int t = threadIdx.x - b * T;
    const int B = blockDim.x / T;
    const int row = blockIdx.x * B + b;
    const int img = blockIdx.y;  // e * n_pairs + pair
    const int e = img / a.n_pairs;
    const int pair = img - e * a.n_pairs;
    const long long npix = (long long)a.n1 * N;
    const int s0 = 2 * pair, s1 = 2 * pair + 1;
    const float* h0 = a.hist + ((long long)e * a.n_slices + s0) * npix + (long long)row * N;
    const float* h1 = s1 < a.n_slices ? a.hist + ((long long)e * a.n_slices + s1) * npix + (long long)row * N : nullptr;
    float2 v[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) v[m] = make_float2(__ldg(h0 + t + m * T), h1 ? __ldg(h1 + t + m * T) : 0.f);
    fft::fft_regs<N, false, WARP_ONLY>(v, sm, b, t, RowAddr<N>{}, a.tw);
    float2* dst = a.work + (long long)img * npix + (long long)row * N;
#pragma unroll
    for (int m = 0; m < 8; ++m) dst[t + m * T] = v[m];
}

template <int N>
__global__ void __launch_bounds__(ColThreads<N>::MAX, ColThreads<N>::MIN_BLOCKS) slice_cols_kernel(SliceArgs a) {
    constexpr int T = N / 8;
    extern __shared__ float2 sm[];
    const int B = blockDim.x / T;
    const int b = threadIdx.x & (B - 1);
    const int t = threadIdx.x / B;
    const int col = blockIdx.x * B + b;
    const int pair = blockIdx.y;
    const long long npix = (long long)N * a.n2;
    const long long ld = a.n2;
    ColAddrRt addr{B};
    float2 acc[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) acc[m] = make_float2(0.f, 0.f);
    for (int e = 0; e < a.n_elems; ++e) {
        const float2* src = a.work + ((long long)e * a.n_pairs + pair) * npix + col;
        float2 v[8];
#pragma unroll
        for (int m = 0; m < 8; ++m) v[m] = src[(long long)(t + m * T) * ld];
        fft::fft_regs<N, false, false>(v, sm, b, t, addr, a.tw);
        const float* te = a.filt + (long long)e * npix + col;
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            const float w = __ldg(te + (long long)(t + m * T) * ld);
            acc[m].x = fmaf(w, v[m].x, acc[m].x);
            acc[m].y = fmaf(w, v[m].y, acc[m].y);
        }
    }
    fft::fft_regs<N, true, false>(acc, sm, b, t, addr, a.tw);
    float2* dst = a.work + (long long)pair * npix + col;  // element 0's slot of this pair
#pragma unroll
    for (int m = 0; m < 8; ++m) dst[(long long)(t + m * T) * ld] = acc[m];
}

// Pass B straight from bucketed atoms (no histogram).  The row DFT of row r of slice pair
// (img, e, pair) at column frequency k2 is z = sum over the bucket's atoms of
// W^(j k2) (even slice) + i W^(j k2) (odd slice), W = exp(-2 pi i / n2): each term is a
// 2^22-scaled fixed-point table entry and the sum is kept in integers (32-bit for rows
// of up to 511 atoms, 64-bit beyond), so it is exact and independent of the order in
// which the counting sort placed the atoms.  One rounding to float32 follows.  Then, per
// element: forward column FFT, x T_e; over all elements: inverse column FFT -> W[img, pair].
//
// Four columns per table lookup (Q4, tiles of B >= 4 columns): a row's atoms arrive
// bucketed by j mod 4, and W^(j (c + k n2/4)) = W^(j c) (-i)^(j k), so the partial sums
// A_q over the atoms with j = q mod 4 at column c give the columns c + k n2/4, k = 0..3,
// as the DFT4 sum_q (-i)^(q k) A_q, evaluated exactly in integers (the same integers as
// four direct sums, hence the same float32 values).  A tile then holds the columns
// c0 + c + k n2/4 (c < B/4); its lanes each take one c and a row at a time.
constexpr int ITEM_CACHE = 6144;  // items of one (image, element, pair) plane staged in shared memory

// the exact partial sums of one row bucket's sub-range [lo, hi) at column `col`
template <class I>
__device__ __forceinline__ void wq_sum(const unsigned* __restrict__ items, unsigned lo, unsigned hi, int col,
                                       int kmask, int n2, const int2* __restrict__ wq, I& x, I& y) {
    x = 0;
    y = 0;
    for (unsigned k = lo; k < hi; ++k) {
        const unsigned u = items[k];
        // the odd slice of the pair reads the i W half of the table
        const int idx = (((int)(u & 0x7fffffffu) * col) & kmask) + (int)(u >> 31) * n2;
        const int2 w = wq[idx + (idx >> 4)];
        x += w.x;
        y += w.y;
    }
}

// columns col, col + n2/4, col + n2/2, col + 3 n2/4 of row bucket ro[0..4] (offsets of its
// four j mod 4 sub-ranges, relative to items)
template <class I>
__device__ __forceinline__ void wq_sum4(const unsigned* __restrict__ items, const unsigned* ro, unsigned base, int col,
                                        int kmask, int n2, const int2* __restrict__ wq, float2 (&out)[4]) {
    I ax[4], ay[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) wq_sum<I>(items, ro[q] - base, ro[q + 1] - base, col, kmask, n2, wq, ax[q], ay[q]);
    const I px = ax[0] + ax[2], py = ay[0] + ay[2], mx = ax[0] - ax[2], my = ay[0] - ay[2];
    const I qx = ax[1] + ax[3], qy = ay[1] + ay[3], rx = ax[1] - ax[3], ry = ay[1] - ay[3];
    constexpr float S = (float)(1.0 / WQ_SCALE);
    out[0] = make_float2((float)(px + qx) * S, (float)(py + qy) * S);  // sum_q A_q
    out[1] = make_float2((float)(mx + ry) * S, (float)(my - rx) * S);  // A0 - A2 - i (A1 - A3)
    out[2] = make_float2((float)(px - qx) * S, (float)(py - qy) * S);  // A0 - A1 + A2 - A3
    out[3] = make_float2((float)(mx - ry) * S, (float)(my + rx) * S);  // A0 - A2 + i (A1 - A3)
}

template <int N, bool Q4>
__global__ void __launch_bounds__(ColThreads<N>::MAX, ColThreads<N>::MIN_BLOCKS) slice_cols_atoms_kernel(SliceArgs a) {
    constexpr int T = N / 8;
    constexpr int NOFF = Q4 ? ROW_SUB * N : N;  // staged offsets per plane (+1)
    extern __shared__ float2 sm[];
    const int B = blockDim.x / T;
    const int b = threadIdx.x & (B - 1);
    const int t = threadIdx.x / B;
    const int Bq = B / ROW_SUB;  // Q4: column lanes per tile
    // the tile's column b: consecutive columns without Q4; c0 + (b mod B/4) + (b div B/4) n2/4 with it
    const int col = Q4 ? blockIdx.x * Bq + (b & (Bq - 1)) + (b / Bq) * (a.n2 / ROW_SUB) : blockIdx.x * B + b;
    const int y = blockIdx.y;  // img * n_pairs + pair
    const int img = y / a.n_pairs;
    const int pair = y - img * a.n_pairs;
    if (a.img_slices && 2 * pair >= a.img_slices[img]) return;  // past this image's stack
    const long long npix = (long long)N * a.n2;
    const long long ld = a.n2;
    ColAddrRt addr{B};
    // W_n2 table (even slice, then times i for the odd slice), padded by one entry every
    // 16: the lookups (j * col) mod n2 of consecutive columns have stride j, which the
    // padding spreads over the banks
    int2* wq = reinterpret_cast<int2*>(sm + (N + N / 8) * B);
    for (int i = threadIdx.x; i < 2 * a.n2; i += blockDim.x) wq[i + (i >> 4)] = a.wq[i];
    // the plane's bucket offsets and (up to ITEM_CACHE) items, staged in shared memory by
    // coalesced loads: the sums below then wait on shared, not global, memory per atom
    unsigned* s_off = reinterpret_cast<unsigned*>(wq + 2 * a.n2 + a.n2 / 8 + 1);
    unsigned* s_items = s_off + NOFF + 1;
    __syncthreads();
    constexpr float INV_SCALE = (float)(1.0 / WQ_SCALE);
    const int kmask = a.n2 - 1;
    float2 acc[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) acc[m] = make_float2(0.f, 0.f);
    for (int e = 0; e < a.n_elems; ++e) {
        const unsigned* off_g = a.bucket_off + ((long long)(img * a.n_elems + e) * a.n_pairs + pair) * (ROW_SUB * N);
        if (e > 0) __syncthreads();  // every thread is done with the previous plane's items and transform
        if (Q4) {
            for (int i = threadIdx.x; i <= NOFF; i += blockDim.x) s_off[i] = __ldg(off_g + i);
        } else {  // row starts only
            for (int i = threadIdx.x; i <= N; i += blockDim.x) s_off[i] = __ldg(off_g + ROW_SUB * i);
        }
        __syncthreads();
        const unsigned base = s_off[0], count = s_off[NOFF] - base;
        // an element without atoms in this slice pair adds exactly zero: skip its transform
        if (count == 0) continue;
        const bool cached = count <= (unsigned)ITEM_CACHE;
        if (cached)
            for (unsigned i = threadIdx.x; i < count; i += blockDim.x) s_items[i] = __ldg(a.items + base + i);
        __syncthreads();
        const unsigned* items = cached ? s_items : a.items + base;  // indexed from the plane's first item
        float2 v[8];
        if (Q4) {
            // lane (c, g): column lane c, rows g, g + N/2 (blockDim = 4 Bq T, so 4 T = N/2
            // rows per round).  The four columns land in a row-major [N][B] stage, the
            // column index XORed with (r mod 4) Bq so that a warp's stores (Bq lanes x
            // 32/Bq rows, one column block k at a time) spread over the banks.
            const int c = threadIdx.x & (Bq - 1);
            const int cl = blockIdx.x * Bq + c;
            for (int r = threadIdx.x / Bq; r < N; r += N / 2) {
                const unsigned* ro = s_off + ROW_SUB * r;
                float2 o[4];
                if (ro[4] - ro[0] <= (unsigned)WQ_SMALL) wq_sum4<int>(items, ro, base, cl, kmask, a.n2, wq, o);
                else wq_sum4<long long>(items, ro, base, cl, kmask, a.n2, wq, o);
                const int sw = (r & 3) * Bq;
#pragma unroll
                for (int k = 0; k < 4; ++k) sm[r * B + ((k * Bq + c) ^ sw)] = o[k];
            }
            __syncthreads();
#pragma unroll
            for (int m = 0; m < 8; ++m) {
                const int r = t + m * T;
                v[m] = sm[r * B + (b ^ ((r & 3) * Bq))];
            }
            __syncthreads();  // the transform below reuses the stage as its exchange buffer
        } else {
#pragma unroll
            for (int m = 0; m < 8; ++m) {
                const int r = t + m * T;
                const unsigned lo = s_off[r] - base, hi = s_off[r + 1] - base;
                if (hi - lo <= (unsigned)WQ_SMALL) {
                    int re, im;  // exact: at most WQ_SMALL entries below 2^22
                    wq_sum<int>(items, lo, hi, col, kmask, a.n2, wq, re, im);
                    v[m] = make_float2((float)re * INV_SCALE, (float)im * INV_SCALE);
                } else {
                    long long re, im;
                    wq_sum<long long>(items, lo, hi, col, kmask, a.n2, wq, re, im);
                    v[m] = make_float2((float)re * INV_SCALE, (float)im * INV_SCALE);
                }
            }
        }
        fft::fft_regs<N, false, false>(v, sm, b, t, addr, a.tw);
        const float* te = a.filt + (long long)e * npix + col;
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            const float w = __ldg(te + (long long)(t + m * T) * ld);
            acc[m].x = fmaf(w, v[m].x, acc[m].x);
            acc[m].y = fmaf(w, v[m].y, acc[m].y);
        }
    }
    fft::fft_regs<N, true, false>(acc, sm, b, t, addr, a.tw);
    float2* dst = a.work + (long long)y * npix + col;
#pragma unroll
    for (int m = 0; m < 8; ++m) dst[(long long)(t + m * T) * ld] = acc[m];
}

inline size_t slice_cols_atoms_smem(int n, int B, int n2, bool q4) {
    const int noff = q4 ? ROW_SUB * n : n;
    return (size_t)(n + n / 8) * B * sizeof(float2) + (size_t)(2 * n2 + n2 / 8 + 1) * sizeof(int2) +
           (size_t)(noff + 1 + ITEM_CACHE) * sizeof(unsigned);
}

template <int N, bool Q4>
int slice_cols_atoms_launch(const SliceArgs& a, int B, cudaStream_t st) {
    constexpr int T = N / 8;
    const size_t smem = slice_cols_atoms_smem(N, B, a.n2, Q4);
    EMSIM_TRY(ensure_smem_attr((const void*)slice_cols_atoms_kernel<N, Q4>, smem));
    slice_cols_atoms_kernel<N, Q4><<<dim3(a.n2 / B, a.n_img * a.n_pairs), B * T, smem, st>>>(a);
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

// EMSIM_GB300_SLICE_SUMS=direct: one lookup per atom and column everywhere (A/B; the
// results are bitwise the same)
inline bool slice_sums4_enabled() {
    static const bool on = [] {
        const char* v = std::getenv("EMSIM_GB300_SLICE_SUMS");
        return !(v && std::strcmp(v, "direct") == 0);
    }();
    return on;
}

template <int N>
int slice_cols_atoms_n(const SliceArgs& a, cudaStream_t st) {
    const int B = col_B_for(N, a.n2);
    // four columns per lookup where the tile holds at least four columns (N <= 2048) and
    // the four offsets per row fit beside the table (not for 2048 x 4096)
    if (slice_sums4_enabled() && B >= ROW_SUB && slice_cols_atoms_smem(N, B, a.n2, true) <= SMEM_ATTR_MAX)
        return slice_cols_atoms_launch<N, true>(a, B, st);
    return slice_cols_atoms_launch<N, false>(a, B, st);
}

__device__ __forceinline__ float clip_low(float v) { return v < 1e-13f ? 1e-13f : v; }

template <int N>
__global__ void __launch_bounds__(512) slice_rows_inv_kernel(SliceArgs a) {
    constexpr int T = N / 8;
    constexpr bool WARP_ONLY = (T <= 32);
    extern __shared__ float2 sm[];
    const int b = threadIdx.x / T;
    const int t = threadIdx.x - b * T;
    const int B = blockDim.x / T;
    const int row = blockIdx.x * B + b;
    const int y = blockIdx.y;  // img * n_pairs + pair
    const int img = y / a.n_pairs;
    const int pair = y - img * a.n_pairs;
    if (a.img_slices && 2 * pair >= a.img_slices[img]) return;  // past this image's stack
    const long long npix = (long long)a.n1 * N;
    const float2* src = a.work + (long long)y * npix + (long long)row * N;
    float2 v[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) v[m] = src[t + m * T];
    fft::fft_regs<N, true, WARP_ONLY>(v, sm, b, t, RowAddr<N>{}, a.tw);
    const int s0 = 2 * pair, s1 = 2 * pair + 1;
    float* out = a.out + (long long)img * a.n_slices * npix;
    float* o0 = out + (long long)s0 * npix + (long long)row * N;
#pragma unroll
    for (int m = 0; m < 8; ++m) o0[t + m * T] = clip_low(v[m].x);
    if (s1 < a.n_slices) {
        float* o1 = out + (long long)s1 * npix + (long long)row * N;
#pragma unroll
        for (int m = 0; m < 8; ++m) o1[t + m * T] = clip_low(v[m].y);
    }
}

template <int N>
int rows_launch(void (*k)(SliceArgs), const SliceArgs& a, int n_rows, int n_img, cudaStream_t st) {
    constexpr int T = N / 8;
    int threads = row_threads(N);
    int B = threads / T;
    if (B > n_rows) B = n_rows;
    threads = B * T;
    const size_t smem = (size_t)fft::RowLayout<N>::words(B) * sizeof(float2);
    EMSIM_TRY(ensure_smem_attr((const void*)k, smem));
    k<<<dim3(n_rows / B, n_img), threads, smem, st>>>(a);
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

// Pass A on rows of length n2 (= N here)
template <int N>
int slice_rows_fwd_n(const SliceArgs& a, cudaStream_t st) {
    return rows_launch<N>(slice_rows_fwd_kernel<N>, a, a.n1, a.n_elems * a.n_pairs, st);
}
// length 256: the same pass with the radix-16 FFT (16 threads and values per row)
__global__ void __launch_bounds__(256) slice_rows_inv16_kernel(SliceArgs a) {
    constexpr int N = 256, T = fft16::T;
    extern __shared__ float2 sm[];
    const int b = threadIdx.x / T;
    const int t = threadIdx.x - b * T;
    const int B = blockDim.x / T;
    const int row = blockIdx.x * B + b;
    const int y = blockIdx.y;  // img * n_pairs + pair
    const int img = y / a.n_pairs;
    const int pair = y - img * a.n_pairs;
    if (a.img_slices && 2 * pair >= a.img_slices[img]) return;  // past this image's stack
    const long long npix = (long long)a.n1 * N;
    const float2* src = a.work + (long long)y * npix + (long long)row * N;
    float2 v[16];
#pragma unroll
    for (int m = 0; m < 16; ++m) v[m] = src[t + m * T];
    fft16::fft256<true, true>(v, sm, b, t, fft16::RowSlot{}, a.tw);
    const int s0 = 2 * pair, s1 = 2 * pair + 1;
    float* out = a.out + (long long)img * a.n_slices * npix;
    float* o0 = out + (long long)s0 * npix + (long long)row * N;
#pragma unroll
    for (int m = 0; m < 16; ++m) o0[t + m * T] = clip_low(v[m].x);
    if (s1 < a.n_slices) {
        float* o1 = out + (long long)s1 * npix + (long long)row * N;
#pragma unroll
        for (int m = 0; m < 16; ++m) o1[t + m * T] = clip_low(v[m].y);
    }
}

template <int N>
int slice_rows_inv_n(const SliceArgs& a, cudaStream_t st) {
    if (N == 256 && a.n1 % 16 == 0) {
        const int B = 16;  // rows per CTA, 256 threads
        const size_t smem = (size_t)B * N * sizeof(float2);
        EMSIM_TRY(ensure_smem_attr((const void*)slice_rows_inv16_kernel, smem));
        slice_rows_inv16_kernel<<<dim3(a.n1 / B, a.n_img * a.n_pairs), B * fft16::T, smem, st>>>(a);
        EMSIM_CHECK_LAUNCH();
        return EMSIM_GB300_OK;
    }
    return rows_launch<N>(slice_rows_inv_kernel<N>, a, a.n1, a.n_img * a.n_pairs, st);
}
// Pass B on columns of length n1 (= N here)
template <int N>
int slice_cols_n(const SliceArgs& a, cudaStream_t st) {
    constexpr int T = N / 8;
    const int B = col_B_for(N, a.n2);
    const size_t smem = (size_t)(N + N / 8) * B * sizeof(float2);
    EMSIM_TRY(ensure_smem_attr((const void*)slice_cols_kernel<N>, smem));
    slice_cols_kernel<N><<<dim3(a.n2 / B, a.n_pairs), B * T, smem, st>>>(a);
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}


}  // namespace emsim_gb300
