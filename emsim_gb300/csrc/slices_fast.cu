// Size dispatch of the projected-potential slice passes (kernels in slice_passes.cuh).
#include "slice_passes.cuh"

namespace emsim_gb300 {

#define EMSIM_SLICE_SIZES(X) X(8) X(16) X(32) X(64) X(128) X(256) X(512) X(1024) X(2048) X(4096)

int slice_fast_build(const SliceArgs& a, cudaStream_t st) {
    switch (a.n2) {
#define EMSIM_CASE(N) \
    case N: EMSIM_TRY(slice_rows_fwd_n<N>(a, st)); break;
        EMSIM_SLICE_SIZES(EMSIM_CASE)
#undef EMSIM_CASE
        default: set_error("slice build: row length not on the fast path"); return EMSIM_GB300_ERR_UNSUPPORTED;
    }
    switch (a.n1) {
#define EMSIM_CASE(N) \
    case N: EMSIM_TRY(slice_cols_n<N>(a, st)); break;
        EMSIM_SLICE_SIZES(EMSIM_CASE)
#undef EMSIM_CASE
        default: set_error("slice build: column length not on the fast path"); return EMSIM_GB300_ERR_UNSUPPORTED;
    }
    switch (a.n2) {
#define EMSIM_CASE(N) \
    case N: return slice_rows_inv_n<N>(a, st);
        EMSIM_SLICE_SIZES(EMSIM_CASE)
#undef EMSIM_CASE
    }
    return EMSIM_GB300_ERR_UNSUPPORTED;
}

int slice_atoms_build(const SliceArgs& a, cudaStream_t st) {
    switch (a.n1) {
#define EMSIM_CASE(N) \
    case N: EMSIM_TRY(slice_cols_atoms_n<N>(a, st)); break;
        EMSIM_SLICE_SIZES(EMSIM_CASE)
#undef EMSIM_CASE
        default: set_error("slice build: column length not on the fast path"); return EMSIM_GB300_ERR_UNSUPPORTED;
    }
    switch (a.n2) {
#define EMSIM_CASE(N) \
    case N: return slice_rows_inv_n<N>(a, st);
        EMSIM_SLICE_SIZES(EMSIM_CASE)
#undef EMSIM_CASE
    }
    set_error("slice build: row length not on the fast path");
    return EMSIM_GB300_ERR_UNSUPPORTED;
}

}  // namespace emsim_gb300
