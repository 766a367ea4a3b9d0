// 2D fused transform passes, double arithmetic.
#include "rhs2d_impl.cuh"

namespace dd {
DD_RHS2D_INSTANTIATE(, double)
}  // namespace dd
