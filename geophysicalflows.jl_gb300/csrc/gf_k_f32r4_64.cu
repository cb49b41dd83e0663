// FFT-length-64 FP32 step kernels at radix 4 (autotuner candidates).
#include "gf_inst_n.cuh"

namespace gf {
GF_INST_NR(float, 64, 4)
}  // namespace gf
