// FFT-length-512 kernels for df64 (one translation unit per precision and length).
#include "gf_inst_n.cuh"

namespace gf {
GF_INST_N(df64, 512)
}  // namespace gf
