// Dispatch of the passes with 16 values per thread (wave_r16.cuh) and their length-256
// instantiation; the longer lengths are instantiated beside the radix-8 kernels of the
// same length (wave_fast_<n>.cu), so the sizes compile in parallel.
#include "wave_r16.cuh"

namespace emsim_gb300 {

template bool launch_row16_n<256>(int, const RowArgs&, int, cudaStream_t, int*);
template bool launch_col16_n<256>(int, const ColArgs&, int, cudaStream_t, int*);

#define EMSIM_R16_EXTERN(L)                                                                   \
    extern template bool launch_row16_n<L>(int, const RowArgs&, int, cudaStream_t, int*);     \
    extern template bool launch_col16_n<L>(int, const ColArgs&, int, cudaStream_t, int*);
EMSIM_R16_EXTERN(512)
EMSIM_R16_EXTERN(1024)
EMSIM_R16_EXTERN(2048)
EMSIM_R16_EXTERN(4096)
#undef EMSIM_R16_EXTERN

bool launch_row16(int n2, int ops, const RowArgs& a, int n_img, cudaStream_t st, int* status) {
    switch (n2) {
        case 256: return launch_row16_n<256>(ops, a, n_img, st, status);
        case 512: return launch_row16_n<512>(ops, a, n_img, st, status);
        case 1024: return launch_row16_n<1024>(ops, a, n_img, st, status);
        case 2048: return launch_row16_n<2048>(ops, a, n_img, st, status);
        case 4096: return launch_row16_n<4096>(ops, a, n_img, st, status);
        default: return false;
    }
}

bool launch_col16(int n1, int mode, const ColArgs& a, int n_img, cudaStream_t st, int* status) {
    switch (n1) {
        case 256: return launch_col16_n<256>(mode, a, n_img, st, status);
        case 512: return launch_col16_n<512>(mode, a, n_img, st, status);
        case 1024: return launch_col16_n<1024>(mode, a, n_img, st, status);
        case 2048: return launch_col16_n<2048>(mode, a, n_img, st, status);
        case 4096: return launch_col16_n<4096>(mode, a, n_img, st, status);
        default: return false;
    }
}

}  // namespace emsim_gb300
