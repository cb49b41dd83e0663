// FFT-length-1024 FP32 step kernels at radix 16 (autotuner candidates).
#include "gf_inst_n.cuh"

namespace gf {
GF_INST_NR(float, 1024, 16)
}  // namespace gf
