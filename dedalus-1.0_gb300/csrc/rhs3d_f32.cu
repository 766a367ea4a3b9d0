// 3D fused transform passes, float arithmetic.
#include "rhs3d_impl.cuh"

namespace dd {
DD_RHS3D_INSTANTIATE(, float)
}  // namespace dd
