// Row and column passes with 16 values per thread (fft16.cuh): the persistent, TMA-staged
// structure of row_tma_kernel / col_tma_kernel (two-stage mbarrier pipeline of bulk or
// tensor copies, the stage being computed doubling as the exchange buffer, bounded waits,
// dead column tiles written as zeros) with L / 16 threads per line.  The column pass
// also writes its tiles back with tensor copies from the stage (1.03x the 2048^2 step
// against strided stores from registers, 1.09x at 4096^2, bitwise the same waves).  Length 256 runs the
// two-pass fft256; lengths 512..4096 run fft16n (radix-16 passes, then radix 2/4/8).
// Selected per length by the pass tuning (row_tma = 2, col_tma = 2), which the autotuner
// sets when it measures faster than the radix-8 kernels.
//
// Rows: 256 threads per CTA, B = 256 / (L / 16) rows per tile; a row's threads share a
// warp up to L = 512 and synchronise with a named barrier of their own beyond, so the rows
// of a CTA exchange independently.  Columns: 512 threads, B = 512 / (L / 16) columns per
// tile interleaved b-fastest (a warp spans the tile's columns, so the CTA synchronises);
// the propagator's row factors are staged once per CTA in shared memory.
#pragma once

#include <string>

#include "fft16.cuh"
#include "wave_tma.cuh"

namespace emsim_gb300 {
namespace r16 {

template <int L>
struct RowCfg {
    static constexpr int T = L / 16;
    static constexpr int THREADS = 256;
    static constexpr int SYNC = T <= 32 ? fft16::SYNC_WARP : fft16::SYNC_SEQ;
};

template <int L>
struct ColCfg {
    static constexpr int T = L / 16;
    static constexpr int THREADS = 512;
    static constexpr int BOXR = L < 256 ? L : 256;  // rows per tensor copy
};

template <int L, bool INV, int SYNC, class AddrF>
__device__ __forceinline__ void fft_line(float2 (&v)[16], float2* __restrict__ sm, int b, int t, AddrF addr,
                                         const float2* __restrict__ tw) {
    if constexpr (L == 256) fft16::fft256<INV, SYNC == fft16::SYNC_WARP>(v, sm, b, t, addr, tw);
    else fft16::fft16n<L, INV, SYNC>(v, sm, b, t, addr, tw);
}

// The column pass's transforms read the twiddles of their length from a copy in shared
// memory (every (4096 / L)-th entry of the device table, staged once per CTA), which
// spares the persistent CTA a global load at the start of every butterfly group.
template <int L, bool INV>
__device__ __forceinline__ void fft_col(float2 (&v)[16], float2* __restrict__ sm, int b, int t,
                                        const fft16::ColSlot& addr, const float2* __restrict__ tw,
                                        const float2* __restrict__ s_tw) {
    if constexpr (L == 256) fft16::fft256<INV, false>(v, sm, b, t, addr, tw);
    else if constexpr (L > 2048) fft16::fft16n<L, INV, fft16::SYNC_CTA>(v, sm, b, t, addr, tw);
    else fft16::fft16n<L, INV, fft16::SYNC_CTA, true, L>(v, sm, b, t, addr, s_tw);
}

// (lengths 512..2048: at 4096 the two stages and the row factors already take 192 KB)
template <int L>
constexpr int col_tw_entries() { return L == 256 || L > 2048 ? 0 : L; }

template <int L, int OPS>
__global__ void __launch_bounds__(256, 2) row16_kernel(RowArgs a, int B, int tiles_per_img, int n_tiles) {
    constexpr int T = RowCfg<L>::T;
    constexpr int SYNC = RowCfg<L>::SYNC;
    constexpr bool LOAD_PSI = !(OPS & ROW_CONST_IN);
    constexpr bool LOAD_V = (OPS & ROW_TRANSMIT) != 0;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int tid = threadIdx.x;
    const int b = tid / T;
    const int t = tid - b * T;
    const int te = B * L;
    float2* stage0 = reinterpret_cast<float2*>(smem_raw);
    float2* stage1 = stage0 + te;
    float* vst0 = reinterpret_cast<float*>(stage1 + te);
    float* vst1 = vst0 + (LOAD_V ? te : 0);
    uint64_t* bar = reinterpret_cast<uint64_t*>(vst1 + (LOAD_V ? te : 0));
    const uint32_t tx = (LOAD_PSI ? te * 8u : 0u) + (LOAD_V ? te * 4u : 0u);
    const fft16::RowSlotN<L> addr{};

    auto issue = [&](int tile, int buf) {
        const int img = tile / tiles_per_img;
        const long long r0 = (long long)(tile - img * tiles_per_img) * B;
        tma::mbar_arrive_expect_tx(&bar[buf], tx);
        if (LOAD_PSI)
            tma::bulk_g2s(buf ? stage1 : stage0, a.in + img * a.in_img_stride + r0 * L, te * 8u, &bar[buf]);
        if (LOAD_V)
            tma::bulk_g2s(buf ? vst1 : vst0, a.slice + img * a.slice_img_stride + r0 * L, te * 4u, &bar[buf]);
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
        float2 v[16];
        float vs[16];
        if (LOAD_PSI) {
#pragma unroll
            for (int m = 0; m < 16; ++m) v[m] = stage[b * L + t + m * T];
        } else {
#pragma unroll
            for (int m = 0; m < 16; ++m) v[m] = a.const_val;
        }
        if (LOAD_V) {
            const float* vsrc = buf ? vst1 : vst0;
#pragma unroll
            for (int m = 0; m < 16; ++m) vs[m] = vsrc[b * L + t + m * T];
        }
        // the stage is reused as the exchange buffer below (each row in its own region)
        fft16::seq_sync<SYNC, T>(b);

        if (OPS & ROW_IFFT) fft_line<L, true, SYNC>(v, stage, b, t, addr, a.tw);
        if (OPS & ROW_TRANSMIT) {
#pragma unroll
            for (int m = 0; m < 16; ++m) v[m] = cmul(v[m], transmit_factor(a.sigma_pi, vs[m]));
        }
        if (OPS & ROW_FFT) fft_line<L, false, SYNC>(v, stage, b, t, addr, a.tw);

        const int img = tile / tiles_per_img;
        const long long row = (long long)(tile - img * tiles_per_img) * B + b;
        if (OPS & ROW_OUT_INTENSITY) {
            float* dst = a.out_int + img * a.out_int_img_stride + row * L;
#pragma unroll
            for (int m = 0; m < 16; ++m) dst[t + m * T] = v[m].x * v[m].x + v[m].y * v[m].y;
        } else {
            float2* dst = a.out + img * a.out_img_stride + row * L;
#pragma unroll
            for (int m = 0; m < 16; ++m) dst[t + m * T] = v[m];
        }
        // refill this stage with the tile two steps ahead once every thread is done with it
        tma::fence_proxy_async();
        __syncthreads();
        if (pipelined && tid == 0 && tile + 2 * (int)gridDim.x < n_tiles) issue(tile + 2 * gridDim.x, buf);
    }
}

template <int L, int MODE>
__global__ void __launch_bounds__(512, 1)
    col16_kernel(const __grid_constant__ CUtensorMap map, ColArgs a, int B, int tiles_per_img, int lt_lo, int lt_hi,
                 int n_img) {
    constexpr int T = ColCfg<L>::T;
    constexpr int BOXR = ColCfg<L>::BOXR;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int tid = threadIdx.x;
    const int b = tid & (B - 1);
    const int t = tid / B;
    const int te = L * B;
    float2* stage0 = reinterpret_cast<float2*>(smem_raw);
    float2* stage1 = stage0 + te;
    uint64_t* bar = reinterpret_cast<uint64_t*>(stage1 + te);
    // propagate: the row factors p1 (the same for every tile) staged once in shared memory
    float4* s_p1 = reinterpret_cast<float4*>(bar + 2);
    if (MODE == COL_PROPAGATE)
        for (int i = threadIdx.x; i < L; i += blockDim.x) s_p1[i] = __ldg(a.p1 + i);
    float2* s_tw = reinterpret_cast<float2*>(s_p1 + L);
    for (int i = threadIdx.x; i < col_tw_entries<L>(); i += blockDim.x) s_tw[i] = __ldg(a.tw + i * (fft::TW_SIZE / L));
    const fft16::ColSlot addr{B, B >= 16 ? 0 : (16 / B) - 1};
    const int live_per_img = lt_lo + lt_hi;
    const int n_tiles = live_per_img * n_img;
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
        for (int j = 0; j < L / BOXR; ++j)
            tma::tensor_g2s_2d(dst + j * BOXR * B, &map, 2 * c0, img * L + j * BOXR, &bar[buf]);
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
        float2 v[16];
#pragma unroll
        for (int m = 0; m < 16; ++m) v[m] = stage[(t + m * T) * B + b];
        __syncthreads();

        int img, ct;
        locate(tile, img, ct);
        const int col = ct * B + b;
        if (MODE != COL_INV) fft_col<L, false>(v, stage, b, t, addr, a.tw, s_tw);
        if (tid == 0 && it > 0) {
            // the previous tile's store has had this tile's first transform to read the
            // other stage: refill it with the tile after this one
            tma::bulk_wait_read<0>();
            if (tile + (int)gridDim.x < n_tiles) issue(tile + gridDim.x, buf ^ 1);
        }
        if (MODE == COL_PROPAGATE) {
            const int k2a = abs(fftfreq_int(col, a.n_cols));
            const float2 p2 = __ldg(a.p2 + col);
#pragma unroll
            for (int m = 0; m < 16; ++m) {
                const float4 q = s_p1[t + m * T];
                v[m] = (k2a <= __float_as_int(q.z)) ? cmul(v[m], cmul(make_float2(q.x, q.y), p2))
                                                    : make_float2(0.f, 0.f);
            }
        } else if (MODE == COL_LENS) {
            const int k2 = fftfreq_int(col, a.n_cols);
            const double fy = (double)k2 * a.dfy64;
            const double c2 = a.c2v[a.n_c2 > 1 ? img : 0];
#pragma unroll
            for (int m = 0; m < 16; ++m) v[m] = cmul(v[m], lens_factor(fftfreq_int(t + m * T, L), k2, fy * fy, c2, a));
        }
        if (MODE == COL_PROPAGATE || MODE == COL_LENS || MODE == COL_INV)
            fft_col<L, true>(v, stage, b, t, addr, a.tw, s_tw);

        // the results into the stage in the tile's layout, then tensor stores of it (the
        // stage is refilled once they have read it, during the next tile's first transform)
#pragma unroll
        for (int m = 0; m < 16; ++m) stage[(t + m * T) * B + b] = v[m];
        tma::fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
#pragma unroll 1
            for (int j = 0; j < L / BOXR; ++j)
                tma::tensor_s2g_2d(&map, 2 * ct * B, img * L + j * BOXR, stage + j * BOXR * B);
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
        for (int m = 0; m < 16; ++m) base[(long long)(t + m * T) * a.n_cols] = make_float2(0.f, 0.f);
    }
}

}  // namespace r16

// false when the call is not for this kernel (op combination, unaligned operands, tile
// shape), else the launch status in *status
template <int L>
bool launch_row16_n(int ops, const RowArgs& a, int n_img, cudaStream_t st, int* status) {
    using C = r16::RowCfg<L>;
    if (pass_tuning(L).row_tma != 2 || !tma_enabled() || (ops & (ROW_STORE_PHI | ROW_GRAD))) return false;
    if (!(ops & ROW_CONST_IN) && !aligned16(a.in)) return false;
    if ((ops & ROW_TRANSMIT) && (!aligned16(a.slice) || (a.slice_img_stride & 3) != 0)) return false;
    int B = tile_with_hint(C::THREADS / C::T, pass_tuning(L).row_rows, 1);
    if (B > a.n_rows) B = a.n_rows;
    if (B < 1 || a.n_rows % B != 0) return false;
    const int threads = B * C::T;
    const int tiles_per_img = a.n_rows / B;
    const int n_tiles = tiles_per_img * n_img;
    const size_t te = (size_t)B * L;
    const bool load_v = (ops & ROW_TRANSMIT) != 0;
    const size_t smem = 2 * te * sizeof(float2) + (load_v ? 2 * te * sizeof(float) : 0) + 2 * sizeof(uint64_t);
    switch (ops) {
#define EMSIM_ROW16_CASE(OPS)                                                                  \
    case OPS: {                                                                                \
        const void* k = (const void*)r16::row16_kernel<L, OPS>;                                \
        *status = ensure_smem_attr(k, smem);                                                   \
        if (*status != EMSIM_GB300_OK) return true;                                            \
        const int grid = persistent_grid(k, threads, smem, n_tiles);                           \
        launch_pdl(r16::row16_kernel<L, OPS>, grid, threads, smem, st, a, B, tiles_per_img, n_tiles); \
        break;                                                                                 \
    }
        EMSIM_ROW16_CASE(ROW_FFT)
        EMSIM_ROW16_CASE(ROW_IFFT)
        EMSIM_ROW16_CASE(ROW_TRANSMIT | ROW_FFT)
        EMSIM_ROW16_CASE(ROW_IFFT | ROW_TRANSMIT | ROW_FFT)
        EMSIM_ROW16_CASE(ROW_IFFT | ROW_OUT_INTENSITY)
        EMSIM_ROW16_CASE(ROW_CONST_IN | ROW_TRANSMIT | ROW_FFT)
#undef EMSIM_ROW16_CASE
        default:
            return false;
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(std::string("radix-16 row pass launch: ") + cudaGetErrorString(e));
        *status = EMSIM_GB300_ERR_CUDA;
    } else {
        *status = EMSIM_GB300_OK;
    }
    return true;
}

template <int L>
bool launch_col16_n(int mode, const ColArgs& a, int n_img, cudaStream_t st, int* status) {
    using C = r16::ColCfg<L>;
    if (pass_tuning(L).col_tma != 2 || !tma_enabled() || !aligned16(a.data)) return false;
    int B = C::THREADS / C::T;
    if (B > a.n_cols) B = a.n_cols;
    B = tile_with_hint(B, pass_tuning(L).col_cols, 2);
    if (B < 2 || (B & (B - 1)) != 0 || a.n_cols % B != 0) return false;
    const int threads = B * C::T;
    const int tiles_per_img = a.n_cols / B;
    const LiveTiles lt = mode == COL_PROPAGATE ? live_tiles(a, B, tiles_per_img) : LiveTiles{tiles_per_img, 0};
    const size_t smem = 2 * (size_t)L * B * sizeof(float2) + 2 * sizeof(uint64_t) + L * sizeof(float4) +
                        r16::col_tw_entries<L>() * sizeof(float2);
    CUtensorMap map;
    *status = make_col_tensor_map(&map, a.data, (long long)n_img * L, a.n_cols, B, C::BOXR);
    if (*status != EMSIM_GB300_OK) return true;
    switch (mode) {
#define EMSIM_COL16_CASE(MODE)                                                                               \
    case MODE: {                                                                                             \
        const void* k = (const void*)r16::col16_kernel<L, MODE>;                                             \
        *status = ensure_smem_attr(k, smem);                                                                 \
        if (*status != EMSIM_GB300_OK) return true;                                                          \
        const int grid = persistent_grid(k, threads, smem, tiles_per_img * n_img);                           \
        launch_pdl(r16::col16_kernel<L, MODE>, grid, threads, smem, st, map, a, B, tiles_per_img, lt.lo, lt.hi,  \
                   n_img);                                                                                   \
        break;                                                                                               \
    }
        EMSIM_COL16_CASE(COL_PROPAGATE)
        EMSIM_COL16_CASE(COL_LENS)
        EMSIM_COL16_CASE(COL_FWD)
        EMSIM_COL16_CASE(COL_INV)
#undef EMSIM_COL16_CASE
        default:
            return false;
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(std::string("radix-16 column pass launch: ") + cudaGetErrorString(e));
        *status = EMSIM_GB300_ERR_CUDA;
    } else {
        *status = EMSIM_GB300_OK;
    }
    return true;
}

}  // namespace emsim_gb300
