// 3D fused transform passes, double arithmetic: MHD forms.
#include "rhs3d_impl.cuh"

namespace dd {
DD_RHS3D_INSTANTIATE_B(, double)
}  // namespace dd
