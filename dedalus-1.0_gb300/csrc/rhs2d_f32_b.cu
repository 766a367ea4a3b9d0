// 2D fused transform passes, float arithmetic: Boussinesq forms.
#include "rhs2d_impl.cuh"

namespace dd {
DD_RHS2D_INSTANTIATE_B(, float)
}  // namespace dd
