// FFT-length-256 kernels for df64 (one translation unit per precision and length).
#include "gf_inst_n.cuh"

namespace gf {
GF_INST_N(df64, 256)
}  // namespace gf
