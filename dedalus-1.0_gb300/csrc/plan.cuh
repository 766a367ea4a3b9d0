// Host-side plan: one grid geometry with its wavenumber tables and twiddles.
#pragma once
#include "geometry.cuh"
#include "fft_engine.cuh"

struct dd_plan {
    int ndim;
    int device;
    dd::Geo3 g3;          // valid when ndim == 3
    dd::Geo2 g2;          // valid when ndim == 2
    // wavenumber tables in the reference's k-layout order (device, float64):
    //   3D: kx[Nh], ky[Ny], kz[Nz];  2D: kx[Nh], ky[Ny]
    double* kx;
    double* ky;
    double* kz;
    // the same tables rounded to float (FP32 stage arithmetic)
    float* kxf;
    float* kyf;
    float* kzf;
    // twiddle tables W_L^m, m < L, per axis length (device): fp64 and fp32 as
    // (g, t) with W = g (1 + i t) for the FMA butterflies, double-float as (cos, sin)
    double2* tw64_x; double2* tw64_y; double2* tw64_z;
    float2* tw32_x;  float2* tw32_y;  float2* tw32_z;
    float4* twdf_x;  float4* twdf_y;  float4* twdf_z;   // double-float (hi, lo) pairs
    // rounded-down 1/N_total used by the forward transform
    double inv_n;
    // tile schedule of the fused 2D y passes (dd_plan_set_schedule; 0 = default)
    int sched_y2d;
};

namespace dd {

template <typename T> struct TwSel;
template <> struct TwSel<double> {
    static const double2* x(const dd_plan* p) { return p->tw64_x; }
    static const double2* y(const dd_plan* p) { return p->tw64_y; }
    static const double2* z(const dd_plan* p) { return p->tw64_z; }
};
template <> struct TwSel<float> {
    static const float2* x(const dd_plan* p) { return p->tw32_x; }
    static const float2* y(const dd_plan* p) { return p->tw32_y; }
    static const float2* z(const dd_plan* p) { return p->tw32_z; }
};

template <> struct TwSel<df64> {
    static const float4* x(const dd_plan* p) { return p->twdf_x; }
    static const float4* y(const dd_plan* p) { return p->twdf_y; }
    static const float4* z(const dd_plan* p) { return p->twdf_z; }
};

// Run `body` with T bound to the arithmetic type of precision code `prec`
// (DD_FP64 -> double, DD_FP32 -> float, DD_DF64 -> df64).
#define DD_PREC_DISPATCH(prec, T, ...)                                 \
    do {                                                               \
        if ((prec) == DD_FP64) { using T = double; __VA_ARGS__; }       \
        else if ((prec) == DD_FP32) { using T = float; __VA_ARGS__; }   \
        else { using T = ::dd::df64; __VA_ARGS__; }                     \
    } while (0)

// Same for FP64 / FP32 only.
#define DD_PREC_DISPATCH_2(prec, T, ...)                               \
    do {                                                               \
        if ((prec) == DD_FP64) { using T = double; __VA_ARGS__; }       \
        else { using T = float; __VA_ARGS__; }                          \
    } while (0)

// Dispatch a pass on a runtime length.
template <typename T, bool INV, bool LD_E, bool ST_E, class Op>
int launch_pass_len(int L, const Op& op, int npen, int nslow, int nfield, cudaStream_t st);

}  // namespace dd
