// 3D fused transform passes, float arithmetic: hydro forms.
#include "rhs3d_impl.cuh"

namespace dd {
DD_RHS3D_INSTANTIATE_A(, float)
DD_RHS3D_INSTANTIATE_LO(, P3_HYDRO_DIV)
}  // namespace dd
