// Shared-memory Stockham FFT for power-of-two lengths 8..4096, written for the fused
// multislice kernels.
//
// Algorithm: the Stockham autosort formulation (Govindaraju et al., "High performance
// discrete Fourier transforms on graphics processors", SC08): pass p with stride Ns and
// radix R takes butterfly j from positions j + r*N/R, twiddles input r by
// W_{Ns R}^{r (j mod Ns)}, does a radix-R DFT and writes output r to
// (j / Ns) * Ns * R + (j mod Ns) + r * Ns.  Passes use radix 8 while possible, the last
// pass radix 4 or 2.
//
// Register contract: a sequence of length N is handled by T = N/8 threads; thread t
// holds v[m] = x[t + m*T] (m = 0..7) on entry and v[m] = X[t + m*T] on return.  A
// radix-R pass lets thread t run the 8/R butterflies j = t + q*T, whose inputs are the
// same eight positions, so every pass (first, middle or last) starts from that layout
// and the first gather / last scatter never touch shared memory.  Only the passes in
// between exchange through shared memory, laid out so that the passes' scatters and
// gathers are free of bank conflicts (see RowLayout / ColLayout).
//
// Two shared-memory layouts:
//   RowLayout: each sequence owns a contiguous padded region; threads of a sequence are
//              consecutive (p-fastest).  Used when sequences are contiguous in HBM (rows).
//   ColLayout: B sequences interleaved element-major; thread b-fastest.  Used for
//              column tiles so global loads are B*8-byte contiguous segments.
#pragma once

#include "common.cuh"

namespace emsim_gb300 {
namespace fft {

constexpr int TW_LOG2 = 12;
constexpr int TW_SIZE = 1 << TW_LOG2;  // largest fast-path length
constexpr float SQRT1_2 = 0.70710678118654752440f;


__host__ __device__ constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n >> 1); }

// The device twiddle table holds exp(-2 pi i m / TW_SIZE), m < TW_SIZE (FP64-derived);
// W_L^q of any power-of-two L <= TW_SIZE is entry q * TW_SIZE / L.

// Twiddle tables are read-only and never alias the exchange buffer; TW_SMEM selects a
// shared-memory copy (plain load) or the device table (read-only cache).
template <bool INV, bool TW_SMEM>
__device__ __forceinline__ float2 twiddle(const float2* __restrict__ tw, int m) {
    const float2 w = TW_SMEM ? tw[m] : __ldg(tw + m);
    return INV ? make_float2(w.x, -w.y) : w;
}

template <bool INV>
__device__ __forceinline__ void dft2(float2& a, float2& b) {
    float2 t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

template <bool INV>
__device__ __forceinline__ void dft4(float2& x0, float2& x1, float2& x2, float2& x3) {
    float2 a0 = cadd(x0, x2), a1 = csub(x0, x2);
    float2 b0 = cadd(x1, x3), b1 = cmul_mi<INV>(csub(x1, x3));
    x0 = cadd(a0, b0);
    x2 = csub(a0, b0);
    x1 = cadd(a1, b1);
    x3 = csub(a1, b1);
}

// natural-order radix-8 DFT of y[0..7]
template <bool INV>
__device__ __forceinline__ void dft8(float2& y0, float2& y1, float2& y2, float2& y3,
                                     float2& y4, float2& y5, float2& y6, float2& y7) {
    float2 e0 = y0, e1 = y2, e2 = y4, e3 = y6;
    float2 o0 = y1, o1 = y3, o2 = y5, o3 = y7;
    dft4<INV>(e0, e1, e2, e3);
    dft4<INV>(o0, o1, o2, o3);
    // o_k *= W8^{k} (forward W8 = exp(-i pi/4))
    if (INV) {
        o1 = make_float2((o1.x - o1.y) * SQRT1_2, (o1.x + o1.y) * SQRT1_2);
        o3 = make_float2(-(o3.x + o3.y) * SQRT1_2, (o3.x - o3.y) * SQRT1_2);
    } else {
        o1 = make_float2((o1.x + o1.y) * SQRT1_2, (o1.y - o1.x) * SQRT1_2);
        o3 = make_float2((o3.y - o3.x) * SQRT1_2, -(o3.x + o3.y) * SQRT1_2);
    }
    o2 = cmul_mi<INV>(o2);
    y0 = cadd(e0, o0);
    y4 = csub(e0, o0);
    y1 = cadd(e1, o1);
    y5 = csub(e1, o1);
    y2 = cadd(e2, o2);
    y6 = csub(e2, o2);
    y3 = cadd(e3, o3);
    y7 = csub(e3, o3);
}

// Row layout: sequence b owns N consecutive float2 slots; element p sits at slot
// p ^ G(p >> 4) with G(h) = (h & 7) | ((h & 4) << 1).  The XOR permutes slots inside each
// 16-slot (128-byte) block, so for 16 consecutive threads (T >= 16) every access of the
// passes is conflict-free: contiguous gathers t + m*T (constant XOR), the stride-8
// scatter of the Ns = 1 pass (t/2 spreads the low bits), and the Ns = 8 scatter (bit 2
// of p >> 4 moves the two 8-thread groups into different halves of the block).
template <int N>
struct RowLayout {
    static constexpr int STRIDE = N;
    __device__ __forceinline__ static int addr(int b, int p) {
        const int h = p >> 4;
        return b * STRIDE + (p ^ ((h & 7) | ((h & 4) << 1)));
    }
    static constexpr int words(int B) { return B * STRIDE; }
};

template <int N, int B>
struct ColLayout {
    __device__ __forceinline__ static int addr(int b, int p) { return (p + (p >> 3)) * B + b; }
    static constexpr int words() { return (N + N / 8) * B; }
};

// Barrier among the threads that share a tile.  When a whole sequence lives inside one
// warp (T <= 32, row layout) a warp barrier is enough.
template <bool WARP_ONLY>
__device__ __forceinline__ void tile_sync() {
    if (WARP_ONLY) __syncwarp();
    else __syncthreads();
}

// One radix-R Stockham pass over the register-held values.
// If LAST, the outputs stay in registers (slot m = q + r*(8/R) holds position t + m*T);
// otherwise they are scattered to shared memory.
template <int N, int R, bool INV, bool LAST, bool TW_SMEM, class AddrF>
__device__ __forceinline__ void stockham_pass(float2 (&v)[8], int Ns, float2* __restrict__ sm, int b, int t,
                                              AddrF addr, const float2* __restrict__ ptw) {
    constexpr int T = N / 8;
    constexpr int Q = 8 / R;  // butterflies per thread
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int j = t + q * T;
        const int k = j & (Ns - 1);  // Ns is a power of two
        float2 x[R];
#pragma unroll
        for (int r = 0; r < R; ++r) x[r] = v[q + r * Q];
        if (Ns > 1) {
            // W_{Ns R}^{r k}: one table load of w = W_{Ns R}^k, higher powers by complex
            // products (at most three roundings deep, ~3e-7 relative)
            const float2 w1 = twiddle<INV, TW_SMEM>(ptw, k * (TW_SIZE / (Ns * R)));
            x[1] = cmul(x[1], w1);
            if (R >= 4) {
                const float2 w2 = cmul(w1, w1);
                const float2 w3 = cmul(w2, w1);
                x[2] = cmul(x[2], w2);
                x[3] = cmul(x[3], w3);
                if (R == 8) {
                    const float2 w4 = cmul(w2, w2);
                    x[4] = cmul(x[4], w4);
                    x[5] = cmul(x[5], cmul(w4, w1));
                    x[6] = cmul(x[6], cmul(w4, w2));
                    x[7] = cmul(x[7], cmul(w4, w3));
                }
            }
        }
        if (R == 8) dft8<INV>(x[0], x[1], x[2], x[3], x[4], x[5], x[6], x[7]);
        else if (R == 4) dft4<INV>(x[0], x[1], x[2], x[3]);
        else dft2<INV>(x[0], x[1]);
        if (LAST) {
#pragma unroll
            for (int r = 0; r < R; ++r) v[q + r * Q] = x[r];
        } else {
            const int base = (j / Ns) * Ns * R + k;
#pragma unroll
            for (int r = 0; r < R; ++r) sm[addr(b, base + r * Ns)] = x[r];
        }
    }
}

// Full length-N transform of the register-held sequence (see the register contract).
// All threads of the tile must call this together.  Shared memory is free again on
// return.  Unnormalised in both directions.
// ptw: the twiddle table (shared-memory copy when TW_SMEM, else device memory).
template <int N, bool INV, bool WARP_ONLY, bool TW_SMEM = false, class AddrF>
__device__ __forceinline__ void fft_regs(float2 (&v)[8], float2* __restrict__ sm, int b, int t, AddrF addr,
                                         const float2* __restrict__ ptw) {
    static_assert(N >= 8 && N <= TW_SIZE && (N & (N - 1)) == 0, "power-of-two length 8..4096");
    constexpr int T = N / 8;
    constexpr int LOG = ilog2(N);
    constexpr int N8 = LOG / 3;       // radix-8 passes
    constexpr int REM = LOG - 3 * N8;  // 0: none, 1: radix 2, 2: radix 4
    constexpr int NPASS = N8 + (REM ? 1 : 0);
    int Ns = 1;
#pragma unroll
    for (int p = 0; p < NPASS; ++p) {
        if (p > 0) {
#pragma unroll
            for (int m = 0; m < 8; ++m) v[m] = sm[addr(b, t + m * T)];
            tile_sync<WARP_ONLY>();
        }
        const bool last = (p == NPASS - 1);
        if (p < N8) {
            if (last) stockham_pass<N, 8, INV, true, TW_SMEM>(v, Ns, sm, b, t, addr, ptw);
            else stockham_pass<N, 8, INV, false, TW_SMEM>(v, Ns, sm, b, t, addr, ptw);
            Ns *= 8;
        } else if (REM == 2) {
            stockham_pass<N, 4, INV, true, TW_SMEM>(v, Ns, sm, b, t, addr, ptw);
        } else {
            stockham_pass<N, 2, INV, true, TW_SMEM>(v, Ns, sm, b, t, addr, ptw);
        }
        if (!last) tile_sync<WARP_ONLY>();
    }
}

}  // namespace fft
}  // namespace emsim_gb300
