// Runtime-length dispatch for transform passes: powers of two 8 .. 512 and
// 24, 48, 96, 192 (3 x a power of two).
#pragma once
#include <type_traits>

#include "fft_passes.cuh"
#include "plan.cuh"

namespace dd {

// Lengths instantiated for an operation: the operation's own range
// (generic transforms 8..512, fused 3D 16..512, fused 2D 32..512), and for
// double-float arithmetic the powers of two 16..256.
template <typename T> struct PrecLen { static constexpr int lmin = 8, lmax = 512; };
template <> struct PrecLen<df64> { static constexpr int lmin = 16, lmax = 256; };
template <typename T, class Op, int L>
constexpr bool len_ok() {
    return L >= Op::lmin && L <= Op::lmax && L >= PrecLen<T>::lmin && L <= PrecLen<T>::lmax &&
           (!std::is_same<T, df64>::value || (L & (L - 1)) == 0);
}

#define DD_LEN_CASE(N, CALL)                              \
    case N:                                               \
        if constexpr (len_ok<T, Op, N>()) { return CALL; } \
        break;

template <typename T, bool INV, bool LD_E, bool ST_E, class Op>
int launch_pass_len(int L, const Op& op, int npen, int nslow, int nfield, cudaStream_t st) {
    switch (L) {
        DD_LEN_CASE(8, (launch_pass<T, 8, INV, LD_E, ST_E>(op, npen, nslow, nfield, st)))
        DD_LEN_CASE(16, (launch_pass<T, 16, INV, LD_E, ST_E>(op, npen, nslow, nfield, st)))
        DD_LEN_CASE(24, (launch_pass<T, 24, INV, LD_E, ST_E>(op, npen, nslow, nfield, st)))
        DD_LEN_CASE(48, (launch_pass<T, 48, INV, LD_E, ST_E>(op, npen, nslow, nfield, st)))
        DD_LEN_CASE(96, (launch_pass<T, 96, INV, LD_E, ST_E>(op, npen, nslow, nfield, st)))
        DD_LEN_CASE(192, (launch_pass<T, 192, INV, LD_E, ST_E>(op, npen, nslow, nfield, st)))
        DD_LEN_CASE(32, (launch_pass<T, 32, INV, LD_E, ST_E>(op, npen, nslow, nfield, st)))
        DD_LEN_CASE(64, (launch_pass<T, 64, INV, LD_E, ST_E>(op, npen, nslow, nfield, st)))
        DD_LEN_CASE(128, (launch_pass<T, 128, INV, LD_E, ST_E>(op, npen, nslow, nfield, st)))
        DD_LEN_CASE(256, (launch_pass<T, 256, INV, LD_E, ST_E>(op, npen, nslow, nfield, st)))
        DD_LEN_CASE(512, (launch_pass<T, 512, INV, LD_E, ST_E>(op, npen, nslow, nfield, st)))
        default: break;
    }
    set_error("transform length %d is not supported for %s%s (lengths %d..%d)", L, Op::name, PrecName<T>::s,
              Op::lmin > PrecLen<T>::lmin ? Op::lmin : PrecLen<T>::lmin,
              Op::lmax < PrecLen<T>::lmax ? Op::lmax : PrecLen<T>::lmax);
    return DD_ERR_UNSUPPORTED;
}

}  // namespace dd
