// 2D fused transform passes, double arithmetic: hydro forms.
#include "rhs2d_impl.cuh"

namespace dd {
DD_RHS2D_INSTANTIATE_A(, double)
}  // namespace dd
