// Persistent, TMA-staged versions of the fused row and column passes.
//
// Each CTA loops over tiles (B rows, or B columns of n1 rows) of all images.  Tiles are
// brought into shared memory by the TMA engine (1-D bulk copies for row tiles, which
// are contiguous; 2-D tensor copies for column tiles) on a two-stage mbarrier pipeline:
// while tile i is transformed in registers + shared memory, tile i+1 is already in
// flight, so HBM stays busy through the FFT phases.  The stage being computed doubles
// as the FFT exchange buffer (the data is in registers once it has been read), so a
// CTA needs just two tiles of shared memory.  Row results go straight from registers to
// global memory with coalesced stores; column results, whose rows are B columns wide, go
// back into the stage and out with tensor copies, and the stage is refilled with the
// tile after next once those have read it, during the next tile's first transform
// (1.06x the 1024^2 and 1.09x the 2048^2 step against strided stores from registers).
//
// Every barrier wait is bounded (the wait_ns of the kernel's arguments); on timeout the
// row kernel records tma::DEV_MBAR_TIMEOUT in the device error word, waits (bounded, at
// least the default limit) for its own copy still in flight, and returns; the column
// kernel, which has no other load in flight then, waits for its own stores to finish.
#pragma once

#include "tma.cuh"
#include "wave_passes.cuh"

namespace emsim_gb300 {

// ---------------------------------------------------------------------------------
// rows
// ---------------------------------------------------------------------------------
template <int N>
struct RowTma {
    static constexpr int T = N / 8;
    static constexpr int THREADS = T > 256 ? T : 256;  // B = THREADS / T rows per tile
    static constexpr int MIN_BLOCKS = T > 256 ? 1 : 3;
};

template <int N, int OPS>
__global__ void __launch_bounds__(RowTma<N>::THREADS, RowTma<N>::MIN_BLOCKS)
    row_tma_kernel(RowArgs a, int B, int tiles_per_img, int n_tiles) {
    constexpr int T = N / 8;
    constexpr bool WARP_ONLY = (T <= 32);
    constexpr bool LOAD_PSI = !(OPS & ROW_CONST_IN);
    constexpr bool LOAD_V = (OPS & ROW_TRANSMIT) != 0;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int tid = threadIdx.x;
    const int b = tid / T;
    const int t = tid - b * T;
    const int te = B * N;  // elements per tile
    float2* stage0 = reinterpret_cast<float2*>(smem_raw);
    float2* stage1 = stage0 + te;
    float* vst0 = reinterpret_cast<float*>(stage1 + te);
    float* vst1 = vst0 + (LOAD_V ? te : 0);
    uint64_t* bar = reinterpret_cast<uint64_t*>(vst1 + (LOAD_V ? te : 0));
    const uint32_t tx = (LOAD_PSI ? te * 8u : 0u) + (LOAD_V ? te * 4u : 0u);

    auto issue = [&](int tile, int buf) {
        const int img = tile / tiles_per_img;
        const long long r0 = (long long)(tile - img * tiles_per_img) * B;
        tma::mbar_arrive_expect_tx(&bar[buf], tx);
        if (LOAD_PSI)
            tma::bulk_g2s(buf ? stage1 : stage0, a.in + img * a.in_img_stride + r0 * N, te * 8u, &bar[buf]);
        if (LOAD_V)
            tma::bulk_g2s(buf ? vst1 : vst0, a.slice + img * a.slice_img_stride + r0 * N, te * 4u, &bar[buf]);
    };

    if (tid == 0) {
        tma::mbar_init(&bar[0], 1);
        tma::mbar_init(&bar[1], 1);
        tma::fence_mbar_init();
    }
    __syncthreads();
    // programmatic dependent launch: the chain's data is only touched after this point
    tma::pdl_wait();
    tma::pdl_launch_dependents();
    const bool pipelined = tx > 0;
    if (pipelined && tid == 0) {
        if ((int)blockIdx.x < n_tiles) issue(blockIdx.x, 0);
        if ((int)(blockIdx.x + gridDim.x) < n_tiles) issue(blockIdx.x + gridDim.x, 1);
    }

    int it = 0;
    for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x, ++it) {
        const int buf = it & 1;
        float2* stage = buf ? stage1 : stage0;
        if (pipelined && !tma::mbar_wait(&bar[buf], (it >> 1) & 1, a.wait_ns)) {
            if (tid == 0) tma::record_error(a.err, tma::DEV_MBAR_TIMEOUT);
            tma::mbar_drain(&bar[buf ^ 1], ((it + 1) >> 1) & 1, a.wait_ns);
            return;
        }
        float2 v[8];
        float vs[8];
        if (LOAD_PSI) {
#pragma unroll
            for (int m = 0; m < 8; ++m) v[m] = stage[b * N + t + m * T];
        } else {
#pragma unroll
            for (int m = 0; m < 8; ++m) v[m] = a.const_val;
        }
        if (LOAD_V) {
            const float* vsrc = buf ? vst1 : vst0;
#pragma unroll
            for (int m = 0; m < 8; ++m) vs[m] = vsrc[b * N + t + m * T];
        }
        // the stage is reused as the (swizzled) exchange buffer below
        fft::tile_sync<WARP_ONLY>();

        const int img = tile / tiles_per_img;
        const long long row = (long long)(tile - img * tiles_per_img) * B + b;
        if (OPS & ROW_IFFT) fft::fft_regs<N, true, WARP_ONLY>(v, stage, b, t, RowAddr<N>{}, a.tw);
        if (OPS & ROW_GRAD) {
            // dL/dV = 2 sigma Im(mu conj(phi)) with mu = v (the back-propagated wave)
            const float2* ph = a.phi + img * a.phi_img_stride + row * N;
            float* g = a.grad + img * a.grad_img_stride + row * N;
            const float s2 = 2.f * a.sigma_grad;
#pragma unroll
            for (int m = 0; m < 8; ++m) {
                const float2 f = ph[t + m * T];
                g[t + m * T] = s2 * (v[m].y * f.x - v[m].x * f.y);
            }
        }
        if (OPS & ROW_TRANSMIT) {
#pragma unroll
            for (int m = 0; m < 8; ++m) v[m] = cmul(v[m], transmit_factor(a.sigma_pi, vs[m]));
        }
        if (OPS & ROW_STORE_PHI) {
            float2* ph = a.phi + img * a.phi_img_stride + row * N;
#pragma unroll
            for (int m = 0; m < 8; ++m) ph[t + m * T] = v[m];
        }
        if (OPS & ROW_FFT) fft::fft_regs<N, false, WARP_ONLY>(v, stage, b, t, RowAddr<N>{}, a.tw);

        if (OPS & ROW_OUT_INTENSITY) {
            float* dst = a.out_int + img * a.out_int_img_stride + row * N;
#pragma unroll
            for (int m = 0; m < 8; ++m) dst[t + m * T] = v[m].x * v[m].x + v[m].y * v[m].y;
        } else {
            float2* dst = a.out + img * a.out_img_stride + row * N;
#pragma unroll
            for (int m = 0; m < 8; ++m) dst[t + m * T] = v[m];
        }
        // refill this stage with the tile two steps ahead once every thread is done with it
        tma::fence_proxy_async();
        __syncthreads();
        if (pipelined && tid == 0 && tile + 2 * (int)gridDim.x < n_tiles) issue(tile + 2 * gridDim.x, buf);
    }
}

// ---------------------------------------------------------------------------------
// columns
// ---------------------------------------------------------------------------------
// Exchange layout of a B-column tile: element (p, b) at swz(p) * B + b.  With B >= 16 a
// half-warp touches one position; below that the XOR of p's low bits with (p >> 3)
// spreads the positions a half-warp touches over distinct banks for the contiguous
// gathers and the stride-1/8/64 Stockham scatters.
struct ColSwz {
    int B, mask;
    __device__ __forceinline__ int operator()(int b, int p) const { return (p ^ ((p >> 3) & mask)) * B + b; }
};

template <int N>
struct ColTma {
    static constexpr int T = N / 8;
    static constexpr int THREADS = 512;
    static constexpr int BOXR = N < 256 ? N : 256;  // rows per tensor copy
};

// Tiles of B columns.  The pipeline walks the live tiles only: per image the first lt_lo
// and the last lt_hi of the tiles_per_img tiles (all of them when nothing is dead); the
// dead tiles between them (propagate: outside the band-limit in every row) are then
// written as zeros without being loaded.
template <int N, int MODE>
__global__ void __launch_bounds__(512, 2)
    col_tma_kernel(const __grid_constant__ CUtensorMap map, ColArgs a, int B, int tiles_per_img, int lt_lo,
                   int lt_hi, int n_img) {
    constexpr int T = N / 8;
    constexpr int BOXR = ColTma<N>::BOXR;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int tid = threadIdx.x;
    const int b = tid & (B - 1);
    const int t = tid / B;
    const int te = N * B;
    float2* stage0 = reinterpret_cast<float2*>(smem_raw);
    float2* stage1 = stage0 + te;
    uint64_t* bar = reinterpret_cast<uint64_t*>(stage1 + te);
    const ColSwz addr{B, B >= 16 ? 0 : (16 / B) - 1};
    const int live_per_img = lt_lo + lt_hi;
    const int n_tiles = live_per_img * n_img;
    // live tile index -> (image, column tile)
    auto locate = [&](int tile, int& img, int& ct) {
        img = tile / live_per_img;
        const int j = tile - img * live_per_img;
        ct = j < lt_lo ? j : tiles_per_img - lt_hi + (j - lt_lo);
    };

    auto issue = [&](int tile, int buf) {
        int img, ct;
        locate(tile, img, ct);
        const int c0 = ct * B;
        float2* dst = buf ? stage1 : stage0;
        tma::mbar_arrive_expect_tx(&bar[buf], te * 8u);
#pragma unroll 1
        for (int j = 0; j < N / BOXR; ++j)
            tma::tensor_g2s_2d(dst + j * BOXR * B, &map, 2 * c0, img * N + j * BOXR, &bar[buf]);
    };

    if (tid == 0) {
        tma::mbar_init(&bar[0], 1);
        tma::mbar_init(&bar[1], 1);
        tma::fence_mbar_init();
    }
    __syncthreads();
    // programmatic dependent launch: the chain's data is only touched after this point
    tma::pdl_wait();
    tma::pdl_launch_dependents();
    if (tid == 0) {
        if ((int)blockIdx.x < n_tiles) issue(blockIdx.x, 0);
        if ((int)(blockIdx.x + gridDim.x) < n_tiles) issue(blockIdx.x + gridDim.x, 1);
    }

    int it = 0;
    for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x, ++it) {
        const int buf = it & 1;
        float2* stage = buf ? stage1 : stage0;
        if (!tma::mbar_wait(&bar[buf], (it >> 1) & 1, a.wait_ns)) {
            // no load is in flight into the other stage yet; the previous tile's store is
            if (tid == 0) {
                tma::record_error(a.err, tma::DEV_MBAR_TIMEOUT);
                tma::bulk_wait<0>();
            }
            return;
        }
        float2 v[8];
#pragma unroll
        for (int m = 0; m < 8; ++m) v[m] = stage[(t + m * T) * B + b];
        __syncthreads();

        int img, ct;
        locate(tile, img, ct);
        const int col = ct * B + b;
        if (MODE != COL_INV) fft::fft_regs<N, false, false>(v, stage, b, t, addr, a.tw);
        if (tid == 0 && it > 0) {
            // the previous tile's store has had this tile's first transform to read the
            // other stage: refill it with the tile after this one
            tma::bulk_wait_read<0>();
            if (tile + (int)gridDim.x < n_tiles) issue(tile + gridDim.x, buf ^ 1);
        }
        if (MODE == COL_PROPAGATE) {
            propagate_col<N>(v, col, t, a);
        } else if (MODE == COL_LENS) {
            const int k2 = fftfreq_int(col, a.n_cols);
            const double fy = (double)k2 * a.dfy64;
            const double c2 = a.c2v[a.n_c2 > 1 ? img : 0];
#pragma unroll
            for (int m = 0; m < 8; ++m) v[m] = cmul(v[m], lens_factor(fftfreq_int(t + m * T, N), k2, fy * fy, c2, a));
        }
        if (MODE == COL_PROPAGATE || MODE == COL_LENS || MODE == COL_INV)
            fft::fft_regs<N, true, false>(v, stage, b, t, addr, a.tw);

        // the results into the stage in the tile's layout, then tensor stores of it (the
        // stage is refilled once they have read it, during the next tile's first transform)
#pragma unroll
        for (int m = 0; m < 8; ++m) stage[(t + m * T) * B + b] = v[m];
        tma::fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
#pragma unroll 1
            for (int j = 0; j < N / BOXR; ++j)
                tma::tensor_s2g_2d(&map, 2 * ct * B, img * N + j * BOXR, stage + j * BOXR * B);
            tma::bulk_commit();
        }
    }
    if (tid == 0) tma::bulk_wait<0>();  // every store complete before the CTA ends
    const int dead_per_img = tiles_per_img - live_per_img;
    for (int d = blockIdx.x; d < dead_per_img * n_img; d += gridDim.x) {
        const int img = d / dead_per_img;
        const int col = (lt_lo + d - img * dead_per_img) * B + b;
        float2* base = a.data + (long long)img * a.img_stride + col;
#pragma unroll
        for (int m = 0; m < 8; ++m) base[(long long)(t + m * T) * a.n_cols] = make_float2(0.f, 0.f);
    }
}

// ---------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------
// persistent grid: resident CTAs per SM x SMs, capped at the tile count
int persistent_grid(const void* func, int threads, size_t smem, int n_tiles);
// 2-D tensor map over n_rows_total rows of n_cols complex64 (as 2 * n_cols floats), box of
// (2 * box_cols) floats x box_rows rows
int make_col_tensor_map(CUtensorMap* map, const float2* data, long long n_rows_total, int n_cols, int box_cols,
                        int box_rows);
bool tma_enabled();

template <int N>
int launch_row_tma_n(int ops, const RowArgs& a, int n_img, cudaStream_t st) {
    constexpr int T = N / 8;
    int B = tile_with_hint(RowTma<N>::THREADS / T, pass_tuning(N).row_rows, 1);
    if (B > a.n_rows) B = a.n_rows;
    const int threads = B * T;
    const int tiles_per_img = a.n_rows / B;
    const int n_tiles = tiles_per_img * n_img;
    const size_t te = (size_t)B * N;
    const bool load_v = (ops & ROW_TRANSMIT) != 0;
    const size_t smem = 2 * te * sizeof(float2) + (load_v ? 2 * te * sizeof(float) : 0) + 2 * sizeof(uint64_t);
    switch (ops) {
#define EMSIM_ROW_TMA_CASE(OPS)                                                                  \
    case OPS: {                                                                                  \
        const void* k = (const void*)row_tma_kernel<N, OPS>;                                     \
        EMSIM_TRY(ensure_smem_attr(k, smem));                                                    \
        const int grid = persistent_grid(k, threads, smem, n_tiles);                             \
        launch_pdl(row_tma_kernel<N, OPS>, grid, threads, smem, st, a, B, tiles_per_img, n_tiles); \
        break;                                                                                   \
    }
        EMSIM_ROW_TMA_CASE(ROW_FFT)
        EMSIM_ROW_TMA_CASE(ROW_IFFT)
        EMSIM_ROW_TMA_CASE(ROW_TRANSMIT | ROW_FFT)
        EMSIM_ROW_TMA_CASE(ROW_IFFT | ROW_TRANSMIT | ROW_FFT)
        EMSIM_ROW_TMA_CASE(ROW_IFFT | ROW_OUT_INTENSITY)
        EMSIM_ROW_TMA_CASE(ROW_CONST_IN | ROW_TRANSMIT | ROW_FFT)
        EMSIM_ROW_TMA_CASE(ROW_IFFT | ROW_TRANSMIT | ROW_FFT | ROW_STORE_PHI)
        EMSIM_ROW_TMA_CASE(ROW_CONST_IN | ROW_TRANSMIT | ROW_FFT | ROW_STORE_PHI)
        EMSIM_ROW_TMA_CASE(ROW_IFFT | ROW_GRAD | ROW_TRANSMIT | ROW_FFT)
        EMSIM_ROW_TMA_CASE(ROW_IFFT | ROW_GRAD)
#undef EMSIM_ROW_TMA_CASE
        default:
            set_error("row pass: unsupported op combination");
            return EMSIM_GB300_ERR_UNSUPPORTED;
    }
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

inline int col_tma_B(int n, int n_cols) {
    int B = 512 / (n / 8);
    if (B > 64) B = 64;
    if (B > n_cols) B = n_cols;
    return B;
}

template <int N>
int launch_col_tma_n(int mode, const ColArgs& a, int n_img, cudaStream_t st) {
    constexpr int T = N / 8;
    const int B = tile_with_hint(col_tma_B(N, a.n_cols), pass_tuning(N).col_cols, 2);
    const int threads = B * T;
    const int tiles_per_img = a.n_cols / B;
    const LiveTiles lt = mode == COL_PROPAGATE ? live_tiles(a, B, tiles_per_img) : LiveTiles{tiles_per_img, 0};
    const size_t smem = 2 * (size_t)N * B * sizeof(float2) + 2 * sizeof(uint64_t);
    CUtensorMap map;
    EMSIM_TRY(make_col_tensor_map(&map, a.data, (long long)n_img * N, a.n_cols, B, ColTma<N>::BOXR));
    switch (mode) {
#define EMSIM_COL_TMA_CASE(MODE)                                                                 \
    case MODE: {                                                                                 \
        const void* k = (const void*)col_tma_kernel<N, MODE>;                                    \
        EMSIM_TRY(ensure_smem_attr(k, smem));                                                    \
        const int grid = persistent_grid(k, threads, smem, tiles_per_img * n_img);               \
        launch_pdl(col_tma_kernel<N, MODE>, grid, threads, smem, st, map, a, B, tiles_per_img, lt.lo, lt.hi, n_img); \
        break;                                                                                   \
    }
        EMSIM_COL_TMA_CASE(COL_PROPAGATE)
        EMSIM_COL_TMA_CASE(COL_LENS)
        EMSIM_COL_TMA_CASE(COL_FWD)
        EMSIM_COL_TMA_CASE(COL_INV)
#undef EMSIM_COL_TMA_CASE
        default:
            set_error("column pass: unsupported mode");
            return EMSIM_GB300_ERR_UNSUPPORTED;
    }
    EMSIM_CHECK_LAUNCH();
    return EMSIM_GB300_OK;
}

}  // namespace emsim_gb300
