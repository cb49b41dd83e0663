// Field-parallel small-grid step kernels (df64; lengths 32 ... 256 at radix 2, 4 and 8; 512 at 4 and 8).
#include "gf_fpar.cuh"

namespace gf {
template cudaError_t launch_row_fp<df64>(const Geom&, const ModArgs&, const Bufs&, cudaStream_t);
template cudaError_t launch_col_fp<df64>(const Geom&, const ModArgs&, const StepArgs&, const Bufs&, cudaStream_t);
template cudaError_t launch_adj_row_fp<df64>(const Geom&, const AdjArgs&, const Bufs&, cudaStream_t);
template cudaError_t launch_adj_col_fp<df64>(const Geom&, const ModArgs&, const AdjArgs&, const Bufs&, cudaStream_t);
}  // namespace gf
