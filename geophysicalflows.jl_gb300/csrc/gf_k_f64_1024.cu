// FFT-length-1024 kernels for double (one translation unit per precision and length).
#include "gf_inst_n.cuh"

namespace gf {
GF_INST_N(double, 1024)
}  // namespace gf
