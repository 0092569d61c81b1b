// Explicit instantiations of the fused row/column passes (radix 8, and 16 values per
// thread) for length(s): 2048.
// One translation unit per size group so the fast path compiles in parallel.
#include "wave_r16.cuh"
#include "wave_tma.cuh"

namespace emsim_gb300 {
template int launch_row_n<2048>(int, const RowArgs&, int, cudaStream_t);
template int launch_col_n<2048>(int, const ColArgs&, int, cudaStream_t);
template int launch_row_tma_n<2048>(int, const RowArgs&, int, cudaStream_t);
template int launch_col_tma_n<2048>(int, const ColArgs&, int, cudaStream_t);
template bool launch_row16_n<2048>(int, const RowArgs&, int, cudaStream_t, int*);
template bool launch_col16_n<2048>(int, const ColArgs&, int, cudaStream_t, int*);
}  // namespace emsim_gb300
