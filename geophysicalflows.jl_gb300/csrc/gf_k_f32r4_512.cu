// FFT-length-512 FP32 step kernels at radix 4 (autotuner candidates).
#include "gf_inst_n.cuh"

namespace gf {
GF_INST_NR(float, 512, 4)
}  // namespace gf
