// Row-pass kernel instantiations for float storage and arithmetic.
#include "gf_inst.cuh"

namespace gf {
GF_INSTANTIATE_ROW(float)
}  // namespace gf
