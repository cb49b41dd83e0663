// FFT-length-512 kernels for float (one translation unit per precision and length).
#include "gf_inst_n.cuh"

namespace gf {
GF_INST_N(float, 512)
}  // namespace gf
