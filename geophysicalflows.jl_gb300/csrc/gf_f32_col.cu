// Col-pass kernel instantiations for float storage and arithmetic.
#include "gf_inst.cuh"

namespace gf {
GF_INSTANTIATE_COL(float)
}  // namespace gf
