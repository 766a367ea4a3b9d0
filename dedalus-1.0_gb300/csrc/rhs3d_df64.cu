// 3D fused transform passes, double-float arithmetic (hydro only).
#include "rhs3d_impl.cuh"

namespace dd {
DD_RHS3D_INSTANTIATE_PH(, df64, P3_HYDRO)
}  // namespace dd
