// FFTs with 16 values per thread.  Length 256: two radix-16 Stockham passes, 16 threads
// per sequence, one shared-memory exchange per transform instead of the two of the
// radix-8 form (8 x 8 x 4), and no third pass.  Lengths 512..4096 (fft16n): radix-16
// passes then one radix-2/4/8 pass (2048 = 16 x 16 x 8: two exchanges instead of the
// three of 8 x 8 x 8 x 4), N / 16 threads per sequence.
//
// Register contract (as fft_regs, with 16 values): thread t of a sequence holds
// v[m] = x[t + 16 m] on entry and v[m] = X[t + 16 m] on return.  Pass 1 (stride 1) runs
// the DFT16 of x[t + 16 r] and scatters output r to position 16 t + r; pass 2 (stride 16)
// gathers positions t + 16 r, applies W256^(r t) and runs the DFT16, whose outputs are
// X[t + 16 r] in registers.  The 16 threads of a sequence sit in one warp, so warp
// barriers order the exchange.
//
// DFT16 = radix-4 x radix-4 (the same four-step split one level down): four DFT4 over
// x[q + 4 n], twiddles W16^(q s), four DFT4 over q.
#pragma once

#include "fft.cuh"

namespace emsim_gb300 {
namespace fft16 {

constexpr int N = 256;
constexpr int T = 16;

// Exchange layouts.  Rows (sequence b contiguous, its 16 threads in one warp): the low
// four bits of p are XORed with the 16-element block index, so the pass-1 scatter
// (16 t + r over t) and the pass-2 gather (t + 16 r over t) each touch 16 different bank
// pairs.  Columns (B sequences interleaved, b fastest, as the tile arrives by TMA): with
// B >= 16 a half-warp touches one position; below that p's low bits are XORed with
// (p >> 4) & (16 / B - 1), which spreads the 16 / B positions a half-warp touches.
struct RowSlot {
    __device__ __forceinline__ int operator()(int b, int p) const { return b * N + (p ^ ((p >> 4) & 15)); }
};
// The same row layout for any length L: the scatters of the radix-16 passes (positions
// 16 j + r, and (j / 16) 256 + j % 16 + 16 r) and the contiguous gathers t + m T touch
// distinct bank pairs within every half-warp.
template <int L>
struct RowSlotN {
    __device__ __forceinline__ int operator()(int b, int p) const { return b * L + (p ^ ((p >> 4) & 15)); }
};
struct ColSlot {
    int B, mask;
    __device__ __forceinline__ int operator()(int b, int p) const { return (p ^ ((p >> 4) & mask)) * B + b; }
};

// x * W16^k for the constant k of the DFT16 inner twiddles (forward W16 = exp(-2 pi i / 16))
template <bool INV, int K>
__device__ __forceinline__ float2 w16(float2 x) {
    constexpr float C1 = 0.92387953251128675613f;  // cos(pi / 8)
    constexpr float S1 = 0.38268343236508977173f;  // sin(pi / 8)
    constexpr float R2 = 0.70710678118654752440f;  // cos(pi / 4)
    const float sg = INV ? -1.f : 1.f;             // the inverse uses conj(W)
    switch (K) {
        case 0: return x;
        case 1: return cmul(x, make_float2(C1, -sg * S1));
        case 2: return make_float2(R2 * (x.x + sg * x.y), R2 * (x.y - sg * x.x));
        case 3: return cmul(x, make_float2(S1, -sg * C1));
        case 4: return cmul_mi<INV>(x);
        case 6: return make_float2(R2 * (sg * x.y - x.x), -R2 * (x.y + sg * x.x));
        case 9: return cmul(x, make_float2(-C1, sg * S1));
        default: return x;
    }
}

// natural-order DFT16 of x[0..15] in place
template <bool INV>
__device__ __forceinline__ void dft16(float2 (&x)[16]) {
    // level 1: DFT4 over n of x[q + 4 n]; output s lands in x[q + 4 s]
#pragma unroll
    for (int q = 0; q < 4; ++q) fft::dft4<INV>(x[q], x[q + 4], x[q + 8], x[q + 12]);
    // inner twiddles W16^(q s) on x[q + 4 s]
    x[1 + 4 * 1] = w16<INV, 1>(x[1 + 4 * 1]);
    x[1 + 4 * 2] = w16<INV, 2>(x[1 + 4 * 2]);
    x[1 + 4 * 3] = w16<INV, 3>(x[1 + 4 * 3]);
    x[2 + 4 * 1] = w16<INV, 2>(x[2 + 4 * 1]);
    x[2 + 4 * 2] = w16<INV, 4>(x[2 + 4 * 2]);
    x[2 + 4 * 3] = w16<INV, 6>(x[2 + 4 * 3]);
    x[3 + 4 * 1] = w16<INV, 3>(x[3 + 4 * 1]);
    x[3 + 4 * 2] = w16<INV, 6>(x[3 + 4 * 2]);
    x[3 + 4 * 3] = w16<INV, 9>(x[3 + 4 * 3]);
    // level 2: DFT4 over q of x[q + 4 s]; output u lands in x[u + 4 s] = X[s + 4 u]
#pragma unroll
    for (int s = 0; s < 4; ++s) fft::dft4<INV>(x[4 * s], x[4 * s + 1], x[4 * s + 2], x[4 * s + 3]);
    // X[s + 4 u] is in x[u + 4 s]: transpose the 4 x 4 index (register renaming)
    float2 y[16];
#pragma unroll
    for (int s = 0; s < 4; ++s)
#pragma unroll
        for (int u = 0; u < 4; ++u) y[s + 4 * u] = x[u + 4 * s];
#pragma unroll
    for (int i = 0; i < 16; ++i) x[i] = y[i];
}

template <bool WARP>
__device__ __forceinline__ void sync() {
    if (WARP) __syncwarp();
    else __syncthreads();
}

// the 256-point transform of the register-held sequence (see the contract above); all
// threads of the CTA call it together.  sm: the exchange buffer (256 float2 per sequence,
// laid out by addr); WARP: a sequence's threads share a warp (rows), else the CTA
// synchronises (columns); tw: the device table exp(-2 pi i m / 4096)
template <bool INV, bool WARP, class AddrF, bool TW_SMEM = false>
__device__ __forceinline__ void fft256(float2 (&v)[16], float2* __restrict__ sm, int b, int t, AddrF addr,
                                       const float2* __restrict__ tw) {
    // pass 1: stride 1
    dft16<INV>(v);
    sync<WARP>();  // the previous use of the exchange slots is over
#pragma unroll
    for (int r = 0; r < 16; ++r) sm[addr(b, 16 * t + r)] = v[r];
    sync<WARP>();
    // pass 2: stride 16, twiddles W256^(r t)
#pragma unroll
    for (int r = 0; r < 16; ++r) v[r] = sm[addr(b, t + 16 * r)];
    // W256^t and W256^(8 t) from the table, the other powers as running products (at most
    // seven roundings deep), so that only four twiddles are live at a time
    const float2 w1 = fft::twiddle<INV, TW_SMEM>(tw, t * (fft::TW_SIZE / N));
    const float2 w8 = fft::twiddle<INV, TW_SMEM>(tw, ((8 * t) & (N - 1)) * (fft::TW_SIZE / N));
    v[8] = cmul(v[8], w8);
    float2 wr = w1;
#pragma unroll
    for (int r = 1; r < 8; ++r) {
        if (r > 1) wr = cmul(wr, w1);
        v[r] = cmul(v[r], wr);
        v[8 + r] = cmul(v[8 + r], cmul(w8, wr));
    }
    dft16<INV>(v);
}

// ---- lengths 512..4096 -------------------------------------------------------------
template <int L>
struct Shape {
    static constexpr int T = L / 16;                  // threads per sequence
    static constexpr int LOG = fft::ilog2(L);
    static constexpr int P16 = LOG / 4;              // radix-16 passes
    static constexpr int REM = LOG - 4 * P16;        // last pass radix 2^REM (0: none)
    static constexpr int NPASS = P16 + (REM ? 1 : 0);
};

// How the threads of one sequence synchronise around an exchange: within a warp, the
// whole CTA, or a named barrier per sequence (id 1 + b, T threads; T a multiple of 32).
enum SyncKind : int { SYNC_WARP = 0, SYNC_CTA = 1, SYNC_SEQ = 2 };

template <int KIND, int TS>
__device__ __forceinline__ void seq_sync(int b) {
    if (KIND == SYNC_WARP) __syncwarp();
    else if (KIND == SYNC_CTA) __syncthreads();
    else asm volatile("bar.sync %0, %1;" ::"r"(1 + b), "r"(TS) : "memory");
}

// One radix-R Stockham pass (stride Ns) over the 16 register-held values: thread t runs
// the 16 / R butterflies j = t + q T, whose inputs are its own positions; outputs go to
// shared memory, or stay in registers (slot q + r 16 / R holds position j + r Ns) when
// LAST.
// tw: a table of TWN entries exp(-2 pi i m / TWN) (the device table, TWN = TW_SIZE, or a
// copy of its every (TW_SIZE / L)-th entry, TWN = L, e.g. staged in shared memory).
template <int L, int R, bool INV, bool LAST, bool TW_SMEM, int TWN, class AddrF>
__device__ __forceinline__ void pass(float2 (&v)[16], int Ns, float2* __restrict__ sm, int b, int t, AddrF addr,
                                     const float2* __restrict__ tw) {
    constexpr int T = L / 16;
    constexpr int Q = 16 / R;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int j = t + q * T;
        const int k = j & (Ns - 1);
        float2 x[16];
#pragma unroll
        for (int r = 0; r < R; ++r) x[r] = v[q + r * Q];
        if (Ns > 1) {
            const int stride = TWN / (Ns * R);
            const float2 w1 = fft::twiddle<INV, TW_SMEM>(tw, k * stride);
            if (R == 16) {
                // W^k and W^(8k) from the table, the other powers as running products
                const float2 w8 = fft::twiddle<INV, TW_SMEM>(tw, 8 * k * stride);
                x[8] = cmul(x[8], w8);
                float2 wr = w1;
#pragma unroll
                for (int r = 1; r < 8; ++r) {
                    if (r > 1) wr = cmul(wr, w1);
                    x[r] = cmul(x[r], wr);
                    x[8 + r] = cmul(x[8 + r], cmul(w8, wr));
                }
            } else {
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
        }
        if (R == 16) dft16<INV>(x);
        else if (R == 8) fft::dft8<INV>(x[0], x[1], x[2], x[3], x[4], x[5], x[6], x[7]);
        else if (R == 4) fft::dft4<INV>(x[0], x[1], x[2], x[3]);
        else fft::dft2<INV>(x[0], x[1]);
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

// Length-L transform (512 <= L <= 4096) of the register-held sequence: thread t holds
// x[t + m L / 16] on entry and X[t + m L / 16] on return.  Every thread of the sequence
// (of the CTA for SYNC_CTA) calls it; the exchange slots are free on entry and on return.
// Unnormalised both ways.
template <int L, bool INV, int SYNC, bool TW_SMEM = false, int TWN = fft::TW_SIZE, class AddrF>
__device__ __forceinline__ void fft16n(float2 (&v)[16], float2* __restrict__ sm, int b, int t, AddrF addr,
                                       const float2* __restrict__ tw) {
    using S = Shape<L>;
    static_assert(L >= 512 && L <= fft::TW_SIZE && (L & (L - 1)) == 0, "power-of-two length 512..4096");
    int Ns = 1;
#pragma unroll
    for (int p = 0; p < S::NPASS; ++p) {
        if (p > 0) {
#pragma unroll
            for (int m = 0; m < 16; ++m) v[m] = sm[addr(b, t + m * S::T)];
            seq_sync<SYNC, S::T>(b);
        }
        const bool last = (p == S::NPASS - 1);
        if (p < S::P16) {
            if (last) pass<L, 16, INV, true, TW_SMEM, TWN>(v, Ns, sm, b, t, addr, tw);
            else pass<L, 16, INV, false, TW_SMEM, TWN>(v, Ns, sm, b, t, addr, tw);
            Ns *= 16;
        } else if (S::REM == 3) {
            pass<L, 8, INV, true, TW_SMEM, TWN>(v, Ns, sm, b, t, addr, tw);
        } else if (S::REM == 2) {
            pass<L, 4, INV, true, TW_SMEM, TWN>(v, Ns, sm, b, t, addr, tw);
        } else {
            pass<L, 2, INV, true, TW_SMEM, TWN>(v, Ns, sm, b, t, addr, tw);
        }
        if (!last) seq_sync<SYNC, S::T>(b);
    }
}

}  // namespace fft16
}  // namespace emsim_gb300
