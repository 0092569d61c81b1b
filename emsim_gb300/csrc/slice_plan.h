// The slice-builder plan shared by the translation units that build slices
// (slices.cu: binning and the binned build; smooth.cu: the off-grid build and its
// coordinate adjoint).
#pragma once

#include "engine.h"

struct emsim_gb300_slice_plan {
    int n_elems = 0, n_slices = 0, n1 = 0, n2 = 0;
    double dz = 0, d1 = 0, d2 = 0;
    bool fast = false;
    int device = 0;
    const float2* tw = nullptr;
    float2* tw1 = nullptr;  // generic path twiddles exp(-2 pi i m / n)
    float2* tw2 = nullptr;
    float* filt = nullptr;  // (n_elems, n1, n2): F(k) * SF_e(k) / N
    int2* wq = nullptr;     // fast path: W_n2^m then i W_n2^m, m < n2, 2^22-scaled fixed point (WQ_SCALE)
    // columns k2 with |fftfreq(k2)| <= col_cut carry nonzero filter values (-1: none)
    int col_cut = -1;
};

namespace emsim_gb300 {

// EMSIM_GB300_OK when p is a plan of the current device
int check_slice_device(const emsim_gb300_slice_plan* p);

}  // namespace emsim_gb300
