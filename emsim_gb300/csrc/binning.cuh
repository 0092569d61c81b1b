// The reference's CUDA binning rule (SliceBuilder_kernel.cu:9-123), shared by the dense
// histogram kernels and the sorted-atom slice builder so both bin every atom identically.
#pragma once

#include <cmath>

#include "common.cuh"

namespace emsim_gb300 {

struct BinAxis {
    float start, end, d;
    int n;
};

// start = -d * floorf((float)(n + 1) / 2.0f); end = start + (float)n * d, which nvcc
// contracts into one fused multiply-add (SliceBuilder_kernel.cu:30-34, 87-92).
inline BinAxis make_axis(int n, double d) {
    BinAxis a;
    a.d = (float)d;
    const float half = std::floor((float)(n + 1) / 2.0f);
    a.start = -a.d * half;
    a.end = std::fma((float)n, a.d, a.start);
    a.n = n;
    return a;
}

__device__ __forceinline__ bool bin_axis(float x, const BinAxis& ax, int& idx) {
    if (!(ax.start <= x && x <= ax.end)) return false;
    // LEFT_CLOSE: float difference compared against the double literal 1e-12
    if ((double)__fsub_rn(ax.end, x) < 1e-12) {
        idx = ax.n - 1;
    } else {
        int i = (int)floorf(__fdiv_rn(__fsub_rn(x, ax.start), ax.d));
        // x a hair below end can round up to n; the reference then writes past the row
        idx = i < ax.n ? i : ax.n - 1;
    }
    return true;
}

}  // namespace emsim_gb300
