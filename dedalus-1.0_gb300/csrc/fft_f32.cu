// Pruned real transforms, float arithmetic.
#include "fft_impl.cuh"

namespace dd {
DD_FFT_INSTANTIATE(, float)
}  // namespace dd
