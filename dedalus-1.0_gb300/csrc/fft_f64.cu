// Pruned real transforms, double arithmetic.
#include "fft_impl.cuh"

namespace dd {
DD_FFT_INSTANTIATE(, double)
}  // namespace dd
