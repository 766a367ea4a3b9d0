// Exponential-time-differencing phi functions with the reference's exact
// arithmetic (forward_step_cy_3d.pyx:50-59, 80-91, 112-123 for 3D;
// forward_step_cy_2d.pyx:50-59, 78-89, 108-119 and f_taylor 123-148 for 2D).
// Operation order is kept and FMA contraction is prevented with the _rn
// intrinsics, so the only difference from the CPU is the last-bit accuracy of
// exp/pow.
#pragma once
#include <cuda_runtime.h>

namespace dd {

__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double rdiv(double a, double b) { return __ddiv_rn(a, b); }

// f_taylor(k, Z) = sum_{j=k}^{14} Z**(j-k) / j!   (forward_step_cy_2d.pyx:123)
__device__ __forceinline__ double f_taylor(int k, double Z) {
    double factj = 1., sum = 0.;
    if (k > 2)
        for (int j = 1; j < k; j++) factj = rmul(factj, (double)j);
    for (int j = k; j < 15; j++) {
        if (j > 1) factj = rmul(factj, (double)j);
        sum = radd(sum, rdiv(pow(Z, (double)(j - k)), factj));
    }
    return sum;
}

// 3D hand-unrolled polynomials: sum_{j} Z^j / (j + off)!, highest power first.
template <int OFF>
__device__ __forceinline__ double poly3d(double Z) {
    // denominators (j + OFF)! for j = 13 - (OFF - 1) .. 1
    const double den[14] = {2., 6., 24., 120., 720., 5040., 40320., 362880., 3628800.,
                            39916800., 479001600., 6227020800., 87178291200., 1307674368000.};
    // OFF = 1: terms j = 13..1 with (j+1)!  -> den[j-1];  then + 1.
    // OFF = 2: terms j = 12..1 with (j+2)!  -> den[j];    then + 0.5
    constexpr int JMAX = (OFF == 1) ? 13 : 12;
    double pw[14];
    pw[1] = Z;
#pragma unroll
    for (int j = 2; j <= JMAX; j++) pw[j] = rmul(pw[j - 1], Z);
    double s = rdiv(pw[JMAX], den[JMAX + OFF - 2]);
#pragma unroll
    for (int j = JMAX - 1; j >= 1; j--) s = radd(s, rdiv(pw[j], den[j + OFF - 2]));
    return radd(s, OFF == 1 ? 1. : 0.5);
}

// phi functions for Z != 0: f0 = e^Z, f1 = (e^Z - 1)/Z, f2 = (f1 - 1)/Z,
// Taylor series for |Z| < 0.5.
template <int NDIM>
__device__ __forceinline__ void etd_phis(double Z, double& f0, double& f1, double& f2) {
    if ((Z < 0.5) && (Z > -0.5)) {
        if (NDIM == 2) {
            f0 = f_taylor(0, Z);
            f1 = f_taylor(1, Z);
            f2 = f_taylor(2, Z);
        } else {
            f0 = exp(Z);
            f1 = poly3d<1>(Z);
            f2 = poly3d<2>(Z);
        }
    } else {
        f0 = exp(Z);
        f1 = rdiv(rsub(f0, 1.), Z);
        f2 = rdiv(rsub(f1, 1.), Z);
    }
}

// Stage updates on one complex entry (s = start, d, d1, d2 = derivatives).
// etd1: forward_step_cy_3d.pyx:50-60
__device__ __forceinline__ double2 etd1_entry(double2 s, double2 d, double Z, double f0, double f1, double dt) {
    double2 o;
    if (Z == 0.) {
        o.x = radd(s.x, rmul(dt, d.x));
        o.y = radd(s.y, rmul(dt, d.y));
    } else {
        o.x = radd(rmul(s.x, f0), rmul(rmul(d.x, f1), dt));
        o.y = radd(rmul(s.y, f0), rmul(rmul(d.y, f1), dt));
    }
    return o;
}

// etd2rk2: forward_step_cy_3d.pyx:112-124
__device__ __forceinline__ double2 etd2rk2_entry(double2 s, double2 d1, double2 d2, double Z,
                                                 double f0, double f1, double f2, double dt) {
    double2 o;
    if (Z == 0.) {
        o.x = radd(s.x, rmul(dt, d2.x));
        o.y = radd(s.y, rmul(dt, d2.y));
    } else {
        o.x = radd(radd(rmul(s.x, f0), rmul(rmul(rmul(rsub(d2.x, d1.x), 2.), f2), dt)), rmul(rmul(d1.x, f1), dt));
        o.y = radd(radd(rmul(s.y, f0), rmul(rmul(rmul(rsub(d2.y, d1.y), 2.), f2), dt)), rmul(rmul(d1.y, f1), dt));
    }
    return o;
}

// etd2rk1: forward_step_cy_3d.pyx:80-92
__device__ __forceinline__ double2 etd2rk1_entry(double2 s, double2 d1, double2 d2, double Z,
                                                 double f2, double dt) {
    double2 o;
    const double ax = rsub(d2.x, d1.x), ay = rsub(d2.y, d1.y);
    if (Z == 0.) {
        const double h = rdiv(dt, 2.);
        o.x = radd(s.x, rmul(h, ax));
        o.y = radd(s.y, rmul(h, ay));
    } else {
        o.x = radd(s.x, rmul(rmul(ax, f2), dt));
        o.y = radd(s.y, rmul(rmul(ay, f2), dt));
    }
    return o;
}

// The same stage updates with fused multiply-adds and the products by dt
// hoisted (f1h = f1 dt, f2h2 = 2 f2 dt): equal mathematically, rounded
// differently in the last bit.  The fused RK steps use these; the standalone
// stage kernels above keep the reference's operation order.  With Z == 0 the
// phi tables hold f0 = f1 = 1, f2 = 1/2, which reduces these to the Euler forms.
__device__ __forceinline__ double2 etd1_fma(double2 s, double2 d, double f0, double f1h) {
    return make_double2(fma(f1h, d.x, s.x * f0), fma(f1h, d.y, s.y * f0));
}

__device__ __forceinline__ double2 etd2rk2_fma(double2 s, double2 d1, double2 d2, double f0, double f1h,
                                               double f2h2) {
    return make_double2(fma(f1h, d1.x, fma(f2h2, d2.x - d1.x, s.x * f0)),
                        fma(f1h, d1.y, fma(f2h2, d2.y - d1.y, s.y * f0)));
}

}  // namespace dd
