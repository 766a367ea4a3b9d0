// 2D fused transform passes, float arithmetic.
#include "rhs2d_impl.cuh"

namespace dd {
DD_RHS2D_INSTANTIATE(, float)
}  // namespace dd
