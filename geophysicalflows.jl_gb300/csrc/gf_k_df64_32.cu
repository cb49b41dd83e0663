// FFT-length-32 kernels for df64 (one translation unit per precision and length).
#include "gf_inst_n.cuh"

namespace gf {
GF_INST_N(df64, 32)
}  // namespace gf
