// Float transforms with float grid-point values: the closure's gradient and
// stress fields on the FP32 path (the values a float transform produces, at
// half the bytes of double storage).
#include "fft_impl.cuh"

namespace dd {
DD_FFT_INSTANTIATE_X(, float, float)
}  // namespace dd
