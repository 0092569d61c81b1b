// Internal interfaces between the kernel translation units and the C-ABI layer.
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <mutex>

#include "common.cuh"

namespace emsim_gb300 {

// Limit of the pipelined kernels' bounded mbarrier waits (ns), process-wide
// (emsim_gb300_set_wait_limit_ns); every RowArgs / ColArgs takes it when constructed.
unsigned long long wait_limit_ns();

// ---------------------------------------------------------------------------
// row passes: one CTA holds B whole rows; each row is transformed in registers/smem
// ---------------------------------------------------------------------------
enum RowOps : int {
    ROW_IFFT = 1,           // inverse (unnormalised) row FFT right after the load
    ROW_TRANSMIT = 2,       // multiply by exp(i sigma V[row, :])
    ROW_FFT = 4,            // forward row FFT before the store
    ROW_OUT_INTENSITY = 8,  // store |psi|^2 as float instead of complex
    ROW_CONST_IN = 16,      // input is the constant plane wave const_val (nothing is loaded)
    ROW_STORE_PHI = 32,     // adjoint recompute: store the transmitted wave phi (after TRANSMIT)
    ROW_GRAD = 64,          // adjoint: grad[row] = 2 sigma_grad Im(v conj(phi)) before TRANSMIT
};

struct RowArgs {
    const float2* in = nullptr;
    long long in_img_stride = 0;  // float2 elements between images
    float2* out = nullptr;
    long long out_img_stride = 0;
    float* out_int = nullptr;
    long long out_int_img_stride = 0;
    const float* slice = nullptr;  // (n1, n2) float32 per image
    long long slice_img_stride = 0;
    float sigma = 0.f;
    float sigma_pi = 0.f;  // sigma / pi (FP64-derived): the transmit's sincospif argument scale
    float2 const_val = {0.f, 0.f};
    float2* phi = nullptr;  // ROW_STORE_PHI output / ROW_GRAD input, (n1, n2) per image
    long long phi_img_stride = 0;
    float* grad = nullptr;  // ROW_GRAD output, (n1, n2) float per image
    long long grad_img_stride = 0;
    float sigma_grad = 0.f;
    int n_rows = 0;
    const float2* tw = nullptr;  // per-pass twiddle tables of the device (twiddle_table())
    int* err = nullptr;          // device error word (error_word())
    unsigned long long wait_ns = wait_limit_ns();  // bounded mbarrier wait limit
};

// ---------------------------------------------------------------------------
// column passes: one CTA holds a tile of B whole columns
// ---------------------------------------------------------------------------
enum ColMode : int {
    COL_PROPAGATE = 0,  // fwd col FFT, x P(k)*band-limit/N, inverse col FFT
    COL_LENS = 1,       // fwd col FFT, x exp(-i chi(k))*aperture*scale, inverse col FFT
    COL_FWD = 2,        // forward col FFT only
    COL_INV = 3,        // inverse col FFT only
};

struct ColArgs {
    const float2* tw = nullptr;  // per-pass twiddle tables of the device (twiddle_table())
    int* err = nullptr;          // device error word (error_word())
    unsigned long long wait_ns = wait_limit_ns();  // bounded mbarrier wait limit
    float2* data = nullptr;
    long long img_stride = 0;
    int n_rows = 0;  // FFT length along columns (n1)
    int n_cols = 0;  // n2
    // propagate: separable FP64-derived factors p1[k1] (1/N folded in; .z holds the
    // band-limit cutoff |k2| <= cut of row k1 as int bits), p2[k2]
    const float4* p1 = nullptr;
    const float2* p2 = nullptr;
    // propagate: columns [live_lo, n_cols - live_hi) are outside the band-limit for every
    // row, so their output is zero; tiles made only of such columns are written as zeros
    // without being loaded or transformed (-1: no such columns)
    int live_lo = -1, live_hi = -1;
    float dfx = 0.f, dfy = 0.f;  // reference float32 frequency steps
    float filter2 = 0.f;         // (0.6667 * fmax)^2 in float32
    // lens: chi = f2 * (c1 * f2 - c2) in FP64; c2 = pi * lambda * defocus, one value for
    // all images (n_c2 == 1) or one per image of the launch (n_c2 == images <= LENS_MAX)
    double c1 = 0.0;
    double dfx64 = 0.0, dfy64 = 0.0;
    float aper2 = 0.f;       // (aperture / lambda)^2 in float32
    float lens_scale = 1.f;  // normalisation folded into the transfer function
    int n_c2 = 1;
    double c2v[64] = {};
    // lens: spatial-coherence envelope exp(-es * f^2 * (2 c1 f^2 - c2)^2), es = (alpha_s /
    // lambda)^2 for an illumination semi-angle alpha_s (rad); 0: fully coherent
    double es = 0.0;
};
constexpr int LENS_MAX = 64;  // images per lens launch with distinct defocus

// true when n is a power of two in [8, 4096] (the fused fast path)
inline bool fast_len(int n) { return n >= 8 && n <= 4096 && (n & (n - 1)) == 0; }

int launch_row(int n2, int ops, const RowArgs& a, int n_img, cudaStream_t st);
int launch_col(int n1, int mode, const ColArgs& a, int n_img, cudaStream_t st);

// Per-length tuning of the two passes (emsim_gb300_set_pass_tuning): use the TMA kernel
// (-1: when it applies, 0: never) and the rows / columns per tile (0: built-in).  Tiles
// only regroup independent rows or columns, so results do not depend on the tuning.
struct PassTuning {
    int row_tma = -1, row_rows = 0, col_tma = -1, col_cols = 0;
};
PassTuning pass_tuning(int n);

inline bool aligned16(const void* p) { return ((uintptr_t)p & 15) == 0; }

// Radix-16 row and column passes of length 256 (wave_r16.cu), used when
// pass_tuning(256).row_tma / col_tma == 2: false when they do not apply, else launch and
// put the status in *status.
bool launch_row16(int n2, int ops, const RowArgs& a, int n_img, cudaStream_t st, int* status);
bool launch_col16(int n1, int mode, const ColArgs& a, int n_img, cudaStream_t st, int* status);

// Split-BF16 tensor-core passes (wave_bf16.cu), used when the precision mode is 1 and the
// call has their shape (length 256; row IFFT|TRANSMIT|FFT, column PROPAGATE).  They
// return false when they do not apply, else launch and put the status in *status.
int precision_mode();
bool launch_row_bf16(int n2, int ops, const RowArgs& a, int n_img, cudaStream_t st, int* status);
bool launch_col_bf16(int n1, int mode, const ColArgs& a, int n_img, cudaStream_t st, int* status);
// the tile a launcher uses: hint when it is a power of two in [min_tile, def), else def
inline int tile_with_hint(int def, int hint, int min_tile) {
    if (hint >= min_tile && hint < def && (hint & (hint - 1)) == 0) return hint;
    return def;
}

// row-pass geometry actually used (rows per CTA) - exposed for tests and the autotuner
int row_tile(int n2);
int col_tile(int n1);

// generic (any n1, n2) path: direct DFT along rows / columns + element-wise kernels
// the power-of-two lengths of the fast path, for switch-case instantiation
#define EMSIM_FAST_SIZES(X) X(8) X(16) X(32) X(64) X(128) X(256) X(512) X(1024) X(2048) X(4096)

// Bluestein line DFTs (bluestein.cu) for lengths n >= 3 that are not powers of two with
// 2n - 1 <= 4096: return false when they do not apply, else run and put the status in
// *status.  bluestein_prepare builds the chirp tables of a length ahead of use.
int bluestein_prepare(int n);
bool bluestein_rows(const float2* in, float2* out, int n_rows, int n, bool inverse, int n_img, cudaStream_t st,
                    int* status);
bool bluestein_cols(float2* data, int n_rows, int n_cols, bool inverse, int n_img, cudaStream_t st, int* status);

int generic_dft_rows(const float2* in, float2* out, int n_rows, int n, bool inverse, const float2* tw_n,
                     int n_img, cudaStream_t st);
int generic_dft_cols(float2* data, int n_rows, int n_cols, bool inverse, const float2* tw_n, int n_img,
                     cudaStream_t st);

int ensure_twiddles(int device);
// device address of the FFT twiddle table on the current device (after ensure_twiddles)
const float2* twiddle_table();
// device address of the error word kernels set when a bounded wait gives up
int* error_word();

// opt a kernel into more than 48 KB of dynamic shared memory (once per device)
int ensure_smem_attr(const void* func, size_t smem_bytes);

// Programmatic dependent launch of the persistent pass kernels (tma::pdl_wait): on for
// eager launches unless the environment sets EMSIM_GB300_PDL=0; inside a stream capture
// only with EMSIM_GB300_PDL=2 (in captured graphs it measured no faster).
bool pdl_enabled(cudaStream_t st);

// Launch k<<<grid, block, smem, st>>>(args...), with programmatic stream serialisation
// when pdl_enabled(st): the kernel may start while its predecessor in the stream finishes
// (it must call tma::pdl_wait() before touching the chain's global data).
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl_enabled(st) ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k, static_cast<KArgs>(args)...);
}

// element-wise kernels (any size)
int ew_transmit(const float2* in, const float* slice, float2* out, long long n, float sigma_pi, int n_img,
                long long in_stride, long long slice_stride, long long out_stride, cudaStream_t st);
int ew_fill(float2* out, long long n, float2 value, cudaStream_t st);
int ew_intensity(const float2* in, float* out, long long n, cudaStream_t st);
// y[i] += a * x[i] (float32, one rounding: fmaf)
int ew_axpy(float* y, const float* x, float a, long long n, cudaStream_t st);
int ew_propagate(float2* data, const ColArgs& a, int n_img, cudaStream_t st);
int ew_lens(float2* data, const ColArgs& a, int n_img, cudaStream_t st);
int prop_tables(float4* p1, float2* p2, const int* cut, int n1, int n2, double dfx64, double dfy64,
                double phase_coef, double inv_n, cudaStream_t st);
// band-limit cutoffs: cut[k1] = largest |k2| with f2(k1, k2) <= filter2 in the reference's
// float32 arithmetic (f2 grows with |k2|), -1 when even k2 = 0 is cut
void bandlimit_cutoffs(int n1, int n2, float dfx, float dfy, float filter2, int* cut);

}  // namespace emsim_gb300
