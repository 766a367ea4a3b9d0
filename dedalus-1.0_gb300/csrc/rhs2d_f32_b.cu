// 2D fused transform passes, float arithmetic: Boussinesq forms.
#include "rhs2d_impl.cuh"

namespace dd {
DD_RHS2D_INSTANTIATE_B(, float)
DD_RHS2D_INSTANTIATE_LO(, PHYS_BOUSS_DIV)
}  // namespace dd
