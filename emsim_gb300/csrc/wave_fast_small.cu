// Explicit instantiations of the fused row/column passes for length(s): 8 16 32 64 128.
// One translation unit per size group so the fast path compiles in parallel.
#include "wave_tma.cuh"

namespace emsim_gb300 {
template int launch_row_n<8>(int, const RowArgs&, int, cudaStream_t);
template int launch_col_n<8>(int, const ColArgs&, int, cudaStream_t);
template int launch_row_tma_n<8>(int, const RowArgs&, int, cudaStream_t);
template int launch_col_tma_n<8>(int, const ColArgs&, int, cudaStream_t);
template int launch_row_n<16>(int, const RowArgs&, int, cudaStream_t);
template int launch_col_n<16>(int, const ColArgs&, int, cudaStream_t);
template int launch_row_tma_n<16>(int, const RowArgs&, int, cudaStream_t);
template int launch_col_tma_n<16>(int, const ColArgs&, int, cudaStream_t);
template int launch_row_n<32>(int, const RowArgs&, int, cudaStream_t);
template int launch_col_n<32>(int, const ColArgs&, int, cudaStream_t);
template int launch_row_tma_n<32>(int, const RowArgs&, int, cudaStream_t);
template int launch_col_tma_n<32>(int, const ColArgs&, int, cudaStream_t);
template int launch_row_n<64>(int, const RowArgs&, int, cudaStream_t);
template int launch_col_n<64>(int, const ColArgs&, int, cudaStream_t);
template int launch_row_tma_n<64>(int, const RowArgs&, int, cudaStream_t);
template int launch_col_tma_n<64>(int, const ColArgs&, int, cudaStream_t);
template int launch_row_n<128>(int, const RowArgs&, int, cudaStream_t);
template int launch_col_n<128>(int, const ColArgs&, int, cudaStream_t);
template int launch_row_tma_n<128>(int, const RowArgs&, int, cudaStream_t);
template int launch_col_tma_n<128>(int, const ColArgs&, int, cudaStream_t);
}  // namespace emsim_gb300
