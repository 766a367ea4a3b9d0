// 2D fused transform passes, double arithmetic: Boussinesq forms.
#include "rhs2d_impl.cuh"

namespace dd {
DD_RHS2D_INSTANTIATE_B(, double)
}  // namespace dd
