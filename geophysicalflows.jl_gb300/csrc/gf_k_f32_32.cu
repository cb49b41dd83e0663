// FFT-length-32 kernels for float (one translation unit per precision and length).
#include "gf_inst_n.cuh"

namespace gf {
GF_INST_N(float, 32)
}  // namespace gf
