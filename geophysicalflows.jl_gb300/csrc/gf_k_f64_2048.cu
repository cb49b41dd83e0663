// FFT-length-2048 kernels for double (one translation unit per precision and length).
#include "gf_inst_n.cuh"

namespace gf {
GF_INST_N(double, 2048)
}  // namespace gf
