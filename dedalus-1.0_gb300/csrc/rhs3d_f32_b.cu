// 3D fused transform passes, float arithmetic: MHD forms.
#include "rhs3d_impl.cuh"

namespace dd {
DD_RHS3D_INSTANTIATE_B(, float)
DD_RHS3D_INSTANTIATE_LO(, P3_MHD_DIV)
}  // namespace dd
