// FFT-length-128 FP32 step kernels at radix 4 (autotuner candidates).
#include "gf_inst_n.cuh"

namespace gf {
GF_INST_NR(float, 128, 4)
}  // namespace gf
