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

#include "fft16.cuh"
#include "slices.h"
#include "wave_passes.cuh"
#include "wave_r16.cuh"

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
// 2^22-scaled fixed-point table entry and the sum is kept in integers (32-bit for buckets
// of up to 511 atoms, 64-bit beyond), so it is exact and independent of the order in
// which the counting sort placed the atoms.  One rounding to float32 follows.  Then, per element: forward column FFT, x T_e; over all
// elements: inverse column FFT -> W[img, pair].
constexpr int ITEM_CACHE = 6144;  // items of one (image, element, pair) plane staged in shared memory

template <int N>
__global__ void __launch_bounds__(ColThreads<N>::MAX, ColThreads<N>::MIN_BLOCKS) slice_cols_atoms_kernel(SliceArgs a) {
    constexpr int T = N / 8;
    extern __shared__ float2 sm[];
    const int B = blockDim.x / T;
    const int b = threadIdx.x & (B - 1);
    const int t = threadIdx.x / B;
    const int col = blockIdx.x * B + b;
    const int y = blockIdx.y;  // img * pairs_here + pair - pair0
    const int img = y / a.pairs_here();
    const int pair = a.pair0 + (y - img * a.pairs_here());
    if (a.img_slices && 2 * pair >= a.img_slices[img]) return;  // past this image's stack
    const long long npix = (long long)N * a.n2;
    const long long ld = a.n2;
    if (blockIdx.x * B >= a.live_lo && (blockIdx.x + 1) * B <= a.n2 - a.live_hi) {
        // every column of the tile lies outside the filters' support: the spectrum is zero
        float2* dst = a.work + (long long)y * npix + col;
#pragma unroll
        for (int m = 0; m < 8; ++m) dst[(long long)(t + m * T) * ld] = make_float2(0.f, 0.f);
        return;
    }
    ColAddrRt addr{B};
    // W_n2 table, padded by one entry every 16: the lookups (j * col) mod n2 of the B
    // consecutive columns of a row have stride j, which the padding spreads over the banks.
    // The odd slice of a pair takes i W^m = (-sin, cos), exactly the integers of W^m.
    int2* wq = reinterpret_cast<int2*>(sm + (N + N / 8) * B);
    for (int i = threadIdx.x; i < a.n2; i += blockDim.x) wq[i + (i >> 4)] = a.wq[i];
    // the plane's bucket offsets and (up to ITEM_CACHE) items, staged in shared memory by
    // coalesced loads: the sums below then wait on shared, not global, memory per atom
    unsigned* s_off = reinterpret_cast<unsigned*>(wq + a.n2 + a.n2 / 16 + 1);
    unsigned* s_items = s_off + N + 1;
    __syncthreads();
    constexpr float INV_SCALE = (float)(1.0 / WQ_SCALE);
    const int kmask = a.n2 - 1;
    float2 acc[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) acc[m] = make_float2(0.f, 0.f);
    for (int e = 0; e < a.n_elems; ++e) {
        const unsigned* off_g = a.bucket_off + ((long long)(img * a.n_elems + e) * a.n_pairs + pair) * N;
        if (e > 0) __syncthreads();  // every thread is done with the previous plane's items
        for (int i = threadIdx.x; i <= N; i += blockDim.x) s_off[i] = __ldg(off_g + i);
        __syncthreads();
        const unsigned base = s_off[0], count = s_off[N] - base;
        // an element without atoms in this slice pair adds exactly zero: skip its transform
        if (count == 0) continue;
        const bool cached = count <= (unsigned)ITEM_CACHE;
        if (cached)
            for (unsigned i = threadIdx.x; i < count; i += blockDim.x) s_items[i] = __ldg(a.items + base + i);
        __syncthreads();
        const unsigned* items = cached ? s_items : a.items + base;  // indexed from the plane's first item
        float2 v[8];
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            const int r = t + m * T;
            const unsigned lo = s_off[r] - base, hi = s_off[r + 1] - base;
            if (hi - lo <= (unsigned)WQ_SMALL) {
                int re = 0, im = 0;  // exact: at most WQ_SMALL entries below 2^22
                for (unsigned k = lo; k < hi; ++k) {
                    const unsigned u = items[k];
                    const int idx = ((int)(u & 0xfffu) * col) & kmask;
                    const int2 w = wq[idx + (idx >> 4)];
                    const bool odd = (u >> 31) != 0;  // the odd slice of the pair: i W^m
                    re += odd ? -w.y : w.x;
                    im += odd ? w.x : w.y;
                }
                v[m] = make_float2((float)re * INV_SCALE, (float)im * INV_SCALE);
            } else {
                long long re = 0, im = 0;
                for (unsigned k = lo; k < hi; ++k) {
                    const unsigned u = items[k];
                    const int idx = ((int)(u & 0xfffu) * col) & kmask;
                    const int2 w = wq[idx + (idx >> 4)];
                    const bool odd = (u >> 31) != 0;
                    re += odd ? -w.y : w.x;
                    im += odd ? w.x : w.y;
                }
                v[m] = make_float2((float)re * INV_SCALE, (float)im * INV_SCALE);
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

constexpr int OFF_CACHE_BYTES = 40 * 1024;  // bucket offsets of every element of one pair

int persistent_grid(const void* func, int threads, size_t smem, int n_tiles);

// The same pass as persistent CTAs that take runs of `run` consecutive live column tiles,
// in (image, slice pair, tile) order, from a work queue (an atomic counter), so that
// planes of uneven atom counts and stacks of uneven slice counts balance over the SMs.
// The W_n2 table is staged once per CTA, and a slice pair's bucket offsets (every
// element) and items once per run instead of once per tile: the tiles of a pair read the
// same atoms, so a 4-column tile no longer starts with a round trip to L2 for them; each
// element's filter column is loaded before its sums and transform, which hide the load.
// Dead tiles (outside the filters' support) are written as zeros after the live ones.
// Results are bitwise those of the per-tile form.
template <int N>
__global__ void __launch_bounds__(ColThreads<N>::MAX, ColThreads<N>::MIN_BLOCKS)
    slice_cols_atoms_persist_kernel(SliceArgs a, int lt_lo, int lt_hi, int run) {
    constexpr int T = N / 8;
    constexpr float INV_SCALE = (float)(1.0 / WQ_SCALE);
    extern __shared__ float2 sm[];
    const int B = blockDim.x / T;
    const int b = threadIdx.x & (B - 1);
    const int t = threadIdx.x / B;
    const int E = a.n_elems;
    const int P = a.pairs_here();
    const int tiles = a.n2 / B;
    const int live = lt_lo + lt_hi;
    const long long npix = (long long)N * a.n2;
    const long long ld = a.n2;
    ColAddrRt addr{B};
    int2* wq = reinterpret_cast<int2*>(sm + (N + N / 8) * B);
    unsigned* s_off = reinterpret_cast<unsigned*>(wq + a.n2 + a.n2 / 16 + 1);  // E x (N + 1)
    unsigned* s_items = s_off + E * (N + 1);
    for (int i = threadIdx.x; i < a.n2; i += blockDim.x) wq[i + (i >> 4)] = a.wq[i];
    const int kmask = a.n2 - 1;
    __shared__ unsigned s_run;
    const long long n_live = (long long)a.n_img * P * live;
    const long long n_runs = (n_live + run - 1) / run;
    long long cur_y = -1;
    bool cached = false;
    for (;;) {
        if (threadIdx.x == 0) s_run = atomicAdd(a.tile_counter, 1u);
        __syncthreads();
        const long long r0 = s_run;
        __syncthreads();  // every thread has its run before the next one is taken
        if (r0 >= n_runs) break;
        const long long g_end = (r0 + 1) * run < n_live ? (r0 + 1) * run : n_live;
        for (long long g = r0 * run; g < g_end; ++g) {
            const long long y = g / live;  // img * pairs_here + pair - pair0
            const int j = (int)(g - y * live);
            const int ct = j < lt_lo ? j : tiles - lt_hi + (j - lt_lo);
            const int img = (int)(y / P);
            const int pair = a.pair0 + (int)(y - (long long)img * P);
            if (a.img_slices && 2 * pair >= a.img_slices[img]) continue;  // past this image's stack
            if (y != cur_y) {
                // stage the pair's offsets for every element, then (if they fit) its items,
                // element after element
                __syncthreads();  // every thread is done with the previous pair's offsets and items
                for (int e = 0; e < E; ++e) {
                    const unsigned* off_g = a.bucket_off + ((long long)(img * E + e) * a.n_pairs + pair) * N;
                    for (int i = threadIdx.x; i <= N; i += blockDim.x) s_off[e * (N + 1) + i] = __ldg(off_g + i);
                }
                __syncthreads();
                unsigned total = 0;
                for (int e = 0; e < E; ++e) total += s_off[e * (N + 1) + N] - s_off[e * (N + 1)];
                cached = total <= (unsigned)ITEM_CACHE;
                if (cached) {
                    unsigned at = 0;
                    for (int e = 0; e < E; ++e) {
                        const unsigned base = s_off[e * (N + 1)], count = s_off[e * (N + 1) + N] - base;
                        for (unsigned i = threadIdx.x; i < count; i += blockDim.x) s_items[at + i] = __ldg(a.items + base + i);
                        at += count;
                    }
                }
                __syncthreads();
                cur_y = y;
            }
            const int col = ct * B + b;
            float2 acc[8];
    #pragma unroll
            for (int m = 0; m < 8; ++m) acc[m] = make_float2(0.f, 0.f);
            unsigned at = 0;  // this element's first item in the staged items
            for (int e = 0; e < E; ++e) {
                const unsigned* off = s_off + e * (N + 1);
                const unsigned base = off[0], count = off[N] - base;
                const unsigned* items = cached ? s_items + at : a.items + base;  // indexed from the plane's first item
                at += count;
                if (count == 0) continue;  // an element without atoms in this slice pair adds exactly zero
                // the filter column, loaded before the sums and the transform hide its latency
                const float* te = a.filt + (long long)e * npix + col;
                float f[8];
    #pragma unroll
                for (int m = 0; m < 8; ++m) f[m] = __ldg(te + (long long)(t + m * T) * ld);
                float2 v[8];
    #pragma unroll
                for (int m = 0; m < 8; ++m) {
                    const int r = t + m * T;
                    const unsigned lo = off[r] - base, hi = off[r + 1] - base;
                    if (hi - lo <= (unsigned)WQ_SMALL) {
                        int re = 0, im = 0;  // exact: at most WQ_SMALL entries below 2^22
                        for (unsigned k = lo; k < hi; ++k) {
                            const unsigned u = items[k];
                            const int idx = ((int)(u & 0xfffu) * col) & kmask;
                            const int2 w = wq[idx + (idx >> 4)];
                            const bool odd = (u >> 31) != 0;  // the odd slice of the pair: i W^m
                            re += odd ? -w.y : w.x;
                            im += odd ? w.x : w.y;
                        }
                        v[m] = make_float2((float)re * INV_SCALE, (float)im * INV_SCALE);
                    } else {
                        long long re = 0, im = 0;
                        for (unsigned k = lo; k < hi; ++k) {
                            const unsigned u = items[k];
                            const int idx = ((int)(u & 0xfffu) * col) & kmask;
                            const int2 w = wq[idx + (idx >> 4)];
                            const bool odd = (u >> 31) != 0;
                            re += odd ? -w.y : w.x;
                            im += odd ? w.x : w.y;
                        }
                        v[m] = make_float2((float)re * INV_SCALE, (float)im * INV_SCALE);
                    }
                }
                fft::fft_regs<N, false, false>(v, sm, b, t, addr, a.tw);
    #pragma unroll
                for (int m = 0; m < 8; ++m) {
                    acc[m].x = fmaf(f[m], v[m].x, acc[m].x);
                    acc[m].y = fmaf(f[m], v[m].y, acc[m].y);
                }
            }
            fft::fft_regs<N, true, false>(acc, sm, b, t, addr, a.tw);
            float2* dst = a.work + y * npix + col;
    #pragma unroll
            for (int m = 0; m < 8; ++m) dst[(long long)(t + m * T) * ld] = acc[m];
        }
    }
    // the tiles outside the filters' support: zero spectra
    const int dead = tiles - live;
    const long long n_dead = (long long)a.n_img * P * dead;
    for (long long d = blockIdx.x; d < n_dead; d += gridDim.x) {
        const long long y = d / dead;
        const int img = (int)(y / P);
        const int pair = a.pair0 + (int)(y - (long long)img * P);
        if (a.img_slices && 2 * pair >= a.img_slices[img]) continue;
        const int col = (lt_lo + (int)(d - y * dead)) * B + b;
        float2* dst = a.work + y * npix + col;
#pragma unroll
        for (int m = 0; m < 8; ++m) dst[(long long)(t + m * T) * ld] = make_float2(0.f, 0.f);
    }
}

// From length 512 the same pass runs as persistent CTAs of 512 threads with 16 values per
// thread (the radix-16 column transforms of the wave passes, twiddles staged in shared
// memory up to 2048).  They take runs of `run` consecutive live column tiles, in (image,
// slice pair, tile) order, from a work queue (an atomic counter), so that planes of
// uneven atom counts and stacks of uneven slice counts balance over the SMs.  The W_n2
// table is staged once per CTA, and a pair's bucket offsets (every element) and items
// once per pair and CTA instead of once per tile.  The row transforms of the atoms are
// summed per atom: each thread takes atoms of the plane, looks up W^(j k2) for the tile's
// B columns and adds the fixed-point entries into (column, row) slots with integer
// shared-memory atomics, so the work is uniform over the atoms and no warp waits for the
// longest of its rows' buckets; the sums are the same integers as the per-row ones.  A
// plane with a row bucket above WQ_SMALL atoms takes 64-bit per-row sums instead.  Dead
// tiles (outside the filters' support) are written as zeros after the live ones.
template <int N>
struct ColAtoms16 {
    static constexpr int T = N / 16;
    static constexpr int B = 512 / T;        // columns per tile
    static constexpr int PAD = 32 / B;       // sum slots: column b at b (N + PAD), conflict-free reads
    static constexpr int STRIDE = N + PAD;
    static constexpr int TW = r16::col_tw_entries<N>();
};

template <int N>
__global__ void __launch_bounds__(512, 1) slice_cols_atoms16_kernel(SliceArgs a, int lt_lo, int lt_hi, int run) {
    using C = ColAtoms16<N>;
    constexpr int T = C::T;
    constexpr int B = C::B;
    constexpr float INV_SCALE = (float)(1.0 / WQ_SCALE);
    extern __shared__ __align__(16) float2 sm[];
    const int b = threadIdx.x & (B - 1);
    const int t = threadIdx.x / B;
    const int E = a.n_elems;
    const int P = a.pairs_here();
    const int tiles = a.n2 / B;
    const int live = lt_lo + lt_hi;
    const long long npix = (long long)N * a.n2;
    const long long ld = a.n2;
    // shared memory: exchange slots / integer sums, twiddles, the padded W_n2 table, the
    // pair's bucket offsets for every element, one flag per element (a row bucket above
    // WQ_SMALL), the staged items
    float2* xbuf = sm;
    float2* s_tw = xbuf + B * C::STRIDE;
    int2* wq = reinterpret_cast<int2*>(s_tw + C::TW);
    unsigned* s_off = reinterpret_cast<unsigned*>(wq + a.n2 + a.n2 / 16 + 1);  // E x (N + 1)
    int* s_big = reinterpret_cast<int*>(s_off + E * (N + 1));
    unsigned* s_items = reinterpret_cast<unsigned*>(s_big + E);
    int* acc_re = reinterpret_cast<int*>(xbuf);
    int* acc_im = acc_re + B * C::STRIDE;
    for (int i = threadIdx.x; i < C::TW; i += blockDim.x) s_tw[i] = __ldg(a.tw + i * (fft::TW_SIZE / N));
    for (int i = threadIdx.x; i < a.n2; i += blockDim.x) wq[i + (i >> 4)] = a.wq[i];
    const fft16::ColSlot addr{B, B >= 16 ? 0 : (16 / B) - 1};
    const int kmask = a.n2 - 1;
    __shared__ unsigned s_run;
    const long long n_live = (long long)a.n_img * P * live;
    const long long n_runs = (n_live + run - 1) / run;
    long long cur_y = -1;
    bool cached = false;
    for (;;) {
        if (threadIdx.x == 0) s_run = atomicAdd(a.tile_counter, 1u);
        __syncthreads();
        const long long r0 = s_run;
        __syncthreads();  // every thread has its run before the next one is taken
        if (r0 >= n_runs) break;
        const long long g_end = (r0 + 1) * run < n_live ? (r0 + 1) * run : n_live;
        for (long long g = r0 * run; g < g_end; ++g) {
            const long long y = g / live;  // img * pairs_here + pair - pair0
            const int j = (int)(g - y * live);
            const int ct = j < lt_lo ? j : tiles - lt_hi + (j - lt_lo);
            const int img = (int)(y / P);
            const int pair = a.pair0 + (int)(y - (long long)img * P);
            if (a.img_slices && 2 * pair >= a.img_slices[img]) continue;  // past this image's stack
            if (y != cur_y) {
                __syncthreads();  // every thread is done with the previous pair's offsets and items
                for (int e = 0; e < E; ++e) {
                    const unsigned* off_g = a.bucket_off + ((long long)(img * E + e) * a.n_pairs + pair) * N;
                    for (int i = threadIdx.x; i <= N; i += blockDim.x) s_off[e * (N + 1) + i] = __ldg(off_g + i);
                }
                __syncthreads();
                unsigned total = 0;
                for (int e = 0; e < E; ++e) total += s_off[e * (N + 1) + N] - s_off[e * (N + 1)];
                cached = total <= (unsigned)ITEM_CACHE;
                if (cached) {
                    unsigned at = 0;
                    for (int e = 0; e < E; ++e) {
                        const unsigned base = s_off[e * (N + 1)], count = s_off[e * (N + 1) + N] - base;
                        for (unsigned i = threadIdx.x; i < count; i += blockDim.x)
                            s_items[at + i] = __ldg(a.items + base + i);
                        at += count;
                    }
                }
                for (int e = 0; e < E; ++e) {
                    bool big = false;
                    const unsigned* off = s_off + e * (N + 1);
                    for (int r = threadIdx.x; r < N; r += blockDim.x) big |= (off[r + 1] - off[r]) > (unsigned)WQ_SMALL;
                    const int any = __syncthreads_or(big);
                    if (threadIdx.x == 0) s_big[e] = any;
                }
                __syncthreads();
                cur_y = y;
            }
            const int col = ct * B + b;
            const int c0 = ct * B;
            float2 acc[16];
#pragma unroll
            for (int m = 0; m < 16; ++m) acc[m] = make_float2(0.f, 0.f);
            unsigned at = 0;  // this element's first item in the staged items
            for (int e = 0; e < E; ++e) {
                const unsigned* off = s_off + e * (N + 1);
                const unsigned base = off[0], count = off[N] - base;
                const unsigned* items = cached ? s_items + at : a.items + base;  // from the plane's first item
                at += count;
                if (count == 0) continue;  // an element without atoms in this slice pair adds exactly zero
                float2 v[16];
                if (!s_big[e]) {
                    int4* z4 = reinterpret_cast<int4*>(acc_re);
                    for (int i = threadIdx.x; i < B * C::STRIDE / 2; i += blockDim.x) z4[i] = make_int4(0, 0, 0, 0);
                    __syncthreads();
                    // exact: every (column, row) slot sums at most WQ_SMALL entries below 2^22
                    for (unsigned k = threadIdx.x; k < count; k += blockDim.x) {
                        const unsigned u = items[k];
                        const int r = (int)((u >> 12) & 0xfffu), jj = (int)(u & 0xfffu);
                        const bool odd = (u >> 31) != 0;  // the odd slice of the pair: i W^m
                        int idx = (jj * c0) & kmask;
#pragma unroll 4
                        for (int bb = 0; bb < B; ++bb) {
                            const int2 w = wq[idx + (idx >> 4)];
                            atomicAdd(acc_re + bb * C::STRIDE + r, odd ? -w.y : w.x);
                            atomicAdd(acc_im + bb * C::STRIDE + r, odd ? w.x : w.y);
                            idx = (idx + jj) & kmask;
                        }
                    }
                    __syncthreads();
#pragma unroll
                    for (int m = 0; m < 16; ++m) {
                        const int o = b * C::STRIDE + t + m * T;
                        v[m] = make_float2((float)acc_re[o] * INV_SCALE, (float)acc_im[o] * INV_SCALE);
                    }
                    __syncthreads();  // the sums are read: the slots become the exchange buffer
                } else {
#pragma unroll
                    for (int m = 0; m < 16; ++m) {
                        const int r = t + m * T;
                        long long re = 0, im = 0;
                        for (unsigned k = off[r] - base; k < off[r + 1] - base; ++k) {
                            const unsigned u = items[k];
                            const int idx = ((int)(u & 0xfffu) * col) & kmask;
                            const int2 w = wq[idx + (idx >> 4)];
                            const bool odd = (u >> 31) != 0;
                            re += odd ? -w.y : w.x;
                            im += odd ? w.x : w.y;
                        }
                        v[m] = make_float2((float)re * INV_SCALE, (float)im * INV_SCALE);
                    }
                }
                r16::fft_col<N, false>(v, xbuf, b, t, addr, a.tw, s_tw);
                const float* te = a.filt + (long long)e * npix + col;
#pragma unroll
                for (int m = 0; m < 16; ++m) {
                    const float f = __ldg(te + (long long)(t + m * T) * ld);
                    acc[m].x = fmaf(f, v[m].x, acc[m].x);
                    acc[m].y = fmaf(f, v[m].y, acc[m].y);
                }
            }
            r16::fft_col<N, true>(acc, xbuf, b, t, addr, a.tw, s_tw);
            float2* dst = a.work + y * npix + col;
#pragma unroll
            for (int m = 0; m < 16; ++m) dst[(long long)(t + m * T) * ld] = acc[m];
        }
    }
    // the tiles outside the filters' support: zero spectra
    const int dead = tiles - live;
    const long long n_dead = (long long)a.n_img * P * dead;
    for (long long d = blockIdx.x; d < n_dead; d += gridDim.x) {
        const long long y = d / dead;
        const int img = (int)(y / P);
        const int pair = a.pair0 + (int)(y - (long long)img * P);
        if (a.img_slices && 2 * pair >= a.img_slices[img]) continue;
        const int col = (lt_lo + (int)(d - y * dead)) * B + b;
        float2* dst = a.work + y * npix + col;
#pragma unroll
        for (int m = 0; m < 16; ++m) dst[(long long)(t + m * T) * ld] = make_float2(0.f, 0.f);
    }
}

// Tiles per work-queue run: up to 16 of one pair (a handful of queue operations per
// pair), fewer when that would leave fewer than 8 runs per CTA (the tail).
inline int queue_run(int live, long long planes, int grid) {
    long long run = live < 16 ? (live > 0 ? live : 1) : 16;
    const long long n_live = planes * live;
    while (run > 1 && n_live < run * 8LL * grid) run >>= 1;
    return (int)run;
}

template <int N>
int slice_cols_atoms_n(const SliceArgs& a, cudaStream_t st) {
    constexpr int T = N / 8;
    const int B = col_B_for(N, a.n2);
    const size_t off_bytes = (size_t)a.n_elems * (N + 1) * sizeof(unsigned);
    // Persistent from length 512, on the work queue.  From 2048 (tiles of at most 4
    // columns) with 16 values per thread and per-atom sums: 1.15x the per-tile form on the
    // 2048^2 slab (about 4,200 atoms per slice pair).  Per-atom sums cost each atom B table
    // lookups and 2B shared-memory atomics, and they lose to the per-row sums in registers
    // on wide tiles and on dense planes (a 512^2 group of iced blobs, 16 columns per tile
    // and ~26k atoms per slice pair, ran 3.5x slower that way): there, and at 512 and 1024,
    // the 8-value form with per-row sums runs (1.11x the per-tile form on 512^2 blobs).
    // Below 512 the per-tile form, whose many small CTAs already overlap their staging.
    if (off_bytes <= (size_t)OFF_CACHE_BYTES && a.tile_counter != nullptr) {
        const long long planes = (long long)a.n_img * a.n_pairs;
        const long long per_plane = planes > 0 ? (long long)a.n_atoms / planes : 0;
        if constexpr (N >= 2048) {
            using C = ColAtoms16<N>;
            if (a.n2 >= C::B && per_plane <= ITEM_CACHE) {
                const int tiles = a.n2 / C::B;
                int lt_lo = (a.live_lo + C::B - 1) / C::B, lt_hi = (a.live_hi + C::B - 1) / C::B;
                if (a.live_lo < 0 || a.live_hi < 0) lt_lo = lt_hi = 0;
                if (lt_lo + lt_hi >= tiles) {
                    lt_lo = tiles;
                    lt_hi = 0;
                }
                const size_t smem = ((size_t)C::B * C::STRIDE + C::TW) * sizeof(float2) +
                                    (size_t)(a.n2 + a.n2 / 16 + 1) * sizeof(int2) + off_bytes +
                                    a.n_elems * sizeof(int) + (size_t)ITEM_CACHE * sizeof(unsigned);
                const void* k = (const void*)slice_cols_atoms16_kernel<N>;
                EMSIM_TRY(ensure_smem_attr(k, smem));
                const long long n_tiles = (long long)a.n_img * a.pairs_here() * tiles;
                const int grid = persistent_grid(k, 512, smem, (int)(n_tiles < (1 << 30) ? n_tiles : (1 << 30)));
                const int run = queue_run(lt_lo + lt_hi, (long long)a.n_img * a.pairs_here(), grid);
                EMSIM_CHECK_CUDA(cudaMemsetAsync(a.tile_counter, 0, sizeof(unsigned), st));
                slice_cols_atoms16_kernel<N><<<grid, 512, smem, st>>>(a, lt_lo, lt_hi, run);
                EMSIM_CHECK_LAUNCH();
                return EMSIM_GB300_OK;
            }
        }
        if constexpr (N >= 512) {
            const int tiles = a.n2 / B;
            int lt_lo = (a.live_lo + B - 1) / B, lt_hi = (a.live_hi + B - 1) / B;
            if (a.live_lo < 0 || a.live_hi < 0) lt_lo = lt_hi = 0;
            if (lt_lo + lt_hi >= tiles) {
                lt_lo = tiles;
                lt_hi = 0;
            }
            const size_t smem = (size_t)(N + N / 8) * B * sizeof(float2) +
                                (size_t)(a.n2 + a.n2 / 16 + 1) * sizeof(int2) + off_bytes +
                                (size_t)ITEM_CACHE * sizeof(unsigned);
            const void* k = (const void*)slice_cols_atoms_persist_kernel<N>;
            EMSIM_TRY(ensure_smem_attr(k, smem));
            const long long n_tiles = (long long)a.n_img * a.pairs_here() * tiles;
            const int grid = persistent_grid(k, B * T, smem, (int)(n_tiles < (1 << 30) ? n_tiles : (1 << 30)));
            const int run = queue_run(lt_lo + lt_hi, (long long)a.n_img * a.pairs_here(), grid);
            EMSIM_CHECK_CUDA(cudaMemsetAsync(a.tile_counter, 0, sizeof(unsigned), st));
            slice_cols_atoms_persist_kernel<N><<<grid, B * T, smem, st>>>(a, lt_lo, lt_hi, run);
            EMSIM_CHECK_LAUNCH();
            return EMSIM_GB300_OK;
        }
    }
    const size_t smem = (size_t)(N + N / 8) * B * sizeof(float2) + (size_t)(a.n2 + a.n2 / 16 + 1) * sizeof(int2) +
                        (size_t)(N + 1 + ITEM_CACHE) * sizeof(unsigned);
    EMSIM_TRY(ensure_smem_attr((const void*)slice_cols_atoms_kernel<N>, smem));
    slice_cols_atoms_kernel<N><<<dim3(a.n2 / B, a.n_img * a.pairs_here()), B * T, smem, st>>>(a);
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
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
    const int y = blockIdx.y;  // img * pairs_here + pair - pair0
    const int img = y / a.pairs_here();
    const int local = y - img * a.pairs_here();
    const int pair = a.pair0 + local;
    if (a.img_slices && 2 * pair >= a.img_slices[img]) return;  // past this image's stack
    const long long npix = (long long)a.n1 * N;
    const float2* src = a.work + (long long)y * npix + (long long)row * N;
    float2 v[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) v[m] = src[t + m * T];
    fft::fft_regs<N, true, WARP_ONLY>(v, sm, b, t, RowAddr<N>{}, a.tw);
    float* out = a.out + (long long)img * a.out_stride_slices() * npix;
    float* o0 = out + (long long)(2 * local) * npix + (long long)row * N;
#pragma unroll
    for (int m = 0; m < 8; ++m) o0[t + m * T] = clip_low(v[m].x);
    if (2 * pair + 1 < a.n_slices) {
        float* o1 = out + (long long)(2 * local + 1) * npix + (long long)row * N;
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
    const int y = blockIdx.y;  // img * pairs_here + pair - pair0
    const int img = y / a.pairs_here();
    const int local = y - img * a.pairs_here();
    const int pair = a.pair0 + local;
    if (a.img_slices && 2 * pair >= a.img_slices[img]) return;  // past this image's stack
    const long long npix = (long long)a.n1 * N;
    const float2* src = a.work + (long long)y * npix + (long long)row * N;
    float2 v[16];
#pragma unroll
    for (int m = 0; m < 16; ++m) v[m] = src[t + m * T];
    fft16::fft256<true, true>(v, sm, b, t, fft16::RowSlot{}, a.tw);
    float* out = a.out + (long long)img * a.out_stride_slices() * npix;
    float* o0 = out + (long long)(2 * local) * npix + (long long)row * N;
#pragma unroll
    for (int m = 0; m < 16; ++m) o0[t + m * T] = clip_low(v[m].x);
    if (2 * pair + 1 < a.n_slices) {
        float* o1 = out + (long long)(2 * local + 1) * npix + (long long)row * N;
#pragma unroll
        for (int m = 0; m < 16; ++m) o1[t + m * T] = clip_low(v[m].y);
    }
}

// lengths 1024..4096: the same pass with 16 values per thread (fft16n: radix-16 passes,
// then one radix-2/4/8 pass), L / 16 threads per row, 256 threads per CTA, each row's
// threads synchronising with a named barrier of their own
template <int L>
__global__ void __launch_bounds__(256) slice_rows_inv16n_kernel(SliceArgs a) {
    constexpr int T = L / 16;
    constexpr int SYNC = T <= 32 ? fft16::SYNC_WARP : fft16::SYNC_SEQ;
    extern __shared__ float2 sm[];
    const int b = threadIdx.x / T;
    const int t = threadIdx.x - b * T;
    const int B = blockDim.x / T;
    const int row = blockIdx.x * B + b;
    const int y = blockIdx.y;  // img * pairs_here + pair - pair0
    const int img = y / a.pairs_here();
    const int local = y - img * a.pairs_here();
    const int pair = a.pair0 + local;
    if (a.img_slices && 2 * pair >= a.img_slices[img]) return;  // past this image's stack
    const long long npix = (long long)a.n1 * L;
    const float2* src = a.work + (long long)y * npix + (long long)row * L;
    float2 v[16];
#pragma unroll
    for (int m = 0; m < 16; ++m) v[m] = src[t + m * T];
    fft16::fft16n<L, true, SYNC>(v, sm, b, t, fft16::RowSlotN<L>{}, a.tw);
    float* out = a.out + (long long)img * a.out_stride_slices() * npix;
    float* o0 = out + (long long)(2 * local) * npix + (long long)row * L;
#pragma unroll
    for (int m = 0; m < 16; ++m) o0[t + m * T] = clip_low(v[m].x);
    if (2 * pair + 1 < a.n_slices) {
        float* o1 = out + (long long)(2 * local + 1) * npix + (long long)row * L;
#pragma unroll
        for (int m = 0; m < 16; ++m) o1[t + m * T] = clip_low(v[m].y);
    }
}

template <int N>
int slice_rows_inv_n(const SliceArgs& a, cudaStream_t st) {
    // 16 values per thread from length 1024 (the 2048^2 slab's build 1.045x; 0.99x at 512)
    if constexpr (N >= 1024) {
        constexpr int B = 256 / (N / 16);  // rows per CTA
        if (a.n1 % B == 0) {
            const size_t smem = (size_t)B * N * sizeof(float2);
            EMSIM_TRY(ensure_smem_attr((const void*)slice_rows_inv16n_kernel<N>, smem));
            slice_rows_inv16n_kernel<N><<<dim3(a.n1 / B, a.n_img * a.pairs_here()), 256, smem, st>>>(a);
            EMSIM_CHECK_LAUNCH();
            return EMSIM_GB300_OK;
        }
    }
    if (N == 256 && a.n1 % 16 == 0) {
        const int B = 16;  // rows per CTA, 256 threads
        const size_t smem = (size_t)B * N * sizeof(float2);
        EMSIM_TRY(ensure_smem_attr((const void*)slice_rows_inv16_kernel, smem));
        slice_rows_inv16_kernel<<<dim3(a.n1 / B, a.n_img * a.pairs_here()), B * fft16::T, smem, st>>>(a);
        EMSIM_CHECK_LAUNCH();
        return EMSIM_GB300_OK;
    }
    return rows_launch<N>(slice_rows_inv_kernel<N>, a, a.n1, a.n_img * a.pairs_here(), st);
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
