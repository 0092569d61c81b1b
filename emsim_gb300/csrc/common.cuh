// Shared helpers for the emsim GB300 engine: complex arithmetic on float2, status
// codes, error recording and launch checking.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/emsim_gb300.h"

namespace emsim_gb300 {

// ---------------------------------------------------------------------------
// error recording: every C-ABI call returns a status; the message of the last
// failure on the calling host thread is kept for emsim_gb300_last_error().
// ---------------------------------------------------------------------------
void set_error(const std::string& msg);
const char* get_error();

#define EMSIM_CHECK_CUDA(expr)                                                     \
    do {                                                                           \
        cudaError_t _e = (expr);                                                   \
        if (_e != cudaSuccess) {                                                   \
            ::emsim_gb300::set_error(std::string(#expr) + ": " +                   \
                                     cudaGetErrorString(_e));                      \
            return EMSIM_GB300_ERR_CUDA;                                           \
        }                                                                          \
    } while (0)

#define EMSIM_CHECK_LAUNCH()                                                       \
    do {                                                                           \
        cudaError_t _e = cudaGetLastError();                                       \
        if (_e != cudaSuccess) {                                                   \
            ::emsim_gb300::set_error(std::string("kernel launch: ") +              \
                                     cudaGetErrorString(_e));                      \
            return EMSIM_GB300_ERR_CUDA;                                           \
        }                                                                          \
    } while (0)

#define EMSIM_REQUIRE(cond, code, msg)                                             \
    do {                                                                           \
        if (!(cond)) {                                                             \
            ::emsim_gb300::set_error(msg);                                         \
            return code;                                                           \
        }                                                                          \
    } while (0)

#define EMSIM_TRY(expr)                                                            \
    do {                                                                           \
        int _s = (expr);                                                           \
        if (_s != EMSIM_GB300_OK) return _s;                                       \
    } while (0)

// ---------------------------------------------------------------------------
// complex helpers
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
__host__ __device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__host__ __device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
// multiply by -i (forward) / +i (inverse)
template <bool INV>
__host__ __device__ __forceinline__ float2 cmul_mi(float2 a) {
    return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// fftfreq integer of FFT index i for length n (i for i < ceil(n/2), else i - n);
// the reference reaches the same integer through its ifftshift index arithmetic
// (WavePropagator_kernel.cu:73-78).
__host__ __device__ __forceinline__ int fftfreq_int(int i, int n) { return i < (n + 1) / 2 ? i : i - n; }

// |f|^2 in float32 exactly as the reference's CPU path evaluates it
// (WavePropagator.cpp:63-71): fx = k*dfx, f2 = fx*fx + fy*fy, no fused multiply-add,
// so band-limit and aperture decisions fall on the same pixels as the FP32 reference.
__device__ __forceinline__ float freq_sq_ref(int k1, int k2, float dfx, float dfy) {
    float fx = __fmul_rn((float)k1, dfx);
    float fy = __fmul_rn((float)k2, dfy);
    return __fadd_rn(__fmul_rn(fx, fx), __fmul_rn(fy, fy));
}

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// Transmission factor exp(i sigma V) as (cos, sin)(pi x) with x = (sigma / pi) V: the
// argument is scaled once by the FP64-derived sigma / pi, and sincospif needs no large-
// argument range reduction (CUDA's sincosf carries one), which keeps the fused passes'
// code small.
__device__ __forceinline__ float2 transmit_factor(float sigma_pi, float v) {
    float s, c;
    sincospif(sigma_pi * v, &s, &c);
    return make_float2(c, s);
}

}  // namespace emsim_gb300
