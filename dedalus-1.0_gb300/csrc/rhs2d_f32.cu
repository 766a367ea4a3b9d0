// 2D fused transform passes, float arithmetic: hydro forms.
#include "rhs2d_impl.cuh"

namespace dd {
DD_RHS2D_INSTANTIATE_A(, float)
DD_RHS2D_INSTANTIATE_LO(, PHYS_HYDRO_DIV)
}  // namespace dd
