// 3D fused transform passes, double arithmetic.
#include "rhs3d_impl.cuh"

namespace dd {
DD_RHS3D_INSTANTIATE(, double)
}  // namespace dd
