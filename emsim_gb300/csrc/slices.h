// Internal interface of the slice builder (binning + projected-potential slices).
#pragma once

#include "engine.h"

namespace emsim_gb300 {

struct SliceArgs {
    const float* hist = nullptr;  // (n_elems, n_slices, n1, n2)
    float* out = nullptr;         // (n_slices, n1, n2)
    float2* work = nullptr;       // (n_elems, n_pairs, n1, n2) complex
    const float* filt = nullptr;  // (n_elems, n1, n2) real: band-limit * SF_e / N
    const float2* tw = nullptr;   // FFT twiddle table of the device
    int n_elems = 0, n_slices = 0, n_pairs = 0, n1 = 0, n2 = 0;
    int n_img = 1;  // slice stacks in the call (work / out hold n_img stacks back to back)
    // bucketed atoms (build from atoms)
    const unsigned* bucket_off = nullptr;  // (n_img * n_elems * n_pairs * n1 + 1) start offsets into items
    const unsigned* items = nullptr;       // (slice parity << 31) | (row << 12) | column, grouped by bucket
    const int2* wq = nullptr;              // W_n2^m then i W_n2^m, m < n2, WQ_SCALE fixed point
    const int* img_slices = nullptr;       // per image slice count (<= n_slices); pairs beyond are skipped
    unsigned* tile_counter = nullptr;      // one word of device scratch: the column pass's work queue
    unsigned n_atoms = 0;                  // atoms bucketed (all images and elements): sizes the planes
    // columns [0, live_lo) and [n2 - live_hi, n2) hold the filters' support (T_e nonzero
    // for some element and row); every other column of the slice spectra is zero
    int live_lo = 0, live_hi = 0;
    // chunked builds: this call covers slice pairs [pair0, pair0 + chunk_pairs) of every
    // image (0: all n_pairs); work holds chunk_pairs pairs per image and out holds
    // out_slices slices per image, slice 2 (pair - pair0) first (0: n_slices)
    int pair0 = 0, chunk_pairs = 0, out_slices = 0;
    __host__ __device__ int pairs_here() const { return chunk_pairs ? chunk_pairs : n_pairs; }
    __host__ __device__ int out_stride_slices() const { return out_slices ? out_slices : n_slices; }
};

// fixed-point scale of the row-transform table: 511 entries sum below 2^31
constexpr double WQ_SCALE = 4194304.0;  // 2^22
constexpr int WQ_SMALL = 511;           // buckets up to this size accumulate in 32 bits

// dense histogram -> slices (three passes)
int slice_fast_build(const SliceArgs& a, cudaStream_t st);
// bucketed atoms -> slices (column pass from atoms + inverse row pass)
int slice_atoms_build(const SliceArgs& a, cudaStream_t st);

}  // namespace emsim_gb300
