// Col-pass kernel instantiations for double storage and arithmetic.
#include "gf_inst.cuh"

namespace gf {
GF_INSTANTIATE_COL(double)
}  // namespace gf
