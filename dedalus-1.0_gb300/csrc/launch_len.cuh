// Runtime-length dispatch for transform passes (lengths 8 .. 512).
#pragma once
#include "fft_passes.cuh"
#include "plan.cuh"

namespace dd {

template <typename T, bool INV, bool LD_E, bool ST_E, class Op>
int launch_pass_len(int L, const Op& op, int npen, int nslow, int nfield, cudaStream_t st) {
    switch (L) {
        case 8:   return launch_pass<T, 8, INV, LD_E, ST_E>(op, npen, nslow, nfield, st);
        case 16:  return launch_pass<T, 16, INV, LD_E, ST_E>(op, npen, nslow, nfield, st);
        case 32:  return launch_pass<T, 32, INV, LD_E, ST_E>(op, npen, nslow, nfield, st);
        case 64:  return launch_pass<T, 64, INV, LD_E, ST_E>(op, npen, nslow, nfield, st);
        case 128: return launch_pass<T, 128, INV, LD_E, ST_E>(op, npen, nslow, nfield, st);
        case 256: return launch_pass<T, 256, INV, LD_E, ST_E>(op, npen, nslow, nfield, st);
        case 512: return launch_pass<T, 512, INV, LD_E, ST_E>(op, npen, nslow, nfield, st);
        default:
            set_error("transform length %d is not supported (powers of two 8..512)", L);
            return DD_ERR_UNSUPPORTED;
    }
}

}  // namespace dd
