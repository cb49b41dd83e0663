// FFT-length-128 kernels for df64 (one translation unit per precision and length).
#include "gf_inst_n.cuh"

namespace gf {
GF_INST_N(df64, 128)
}  // namespace gf
