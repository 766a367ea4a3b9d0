// Stage-update kernels with the reference's Cython signatures
// (forward_step_cy_3d.pyx:17-124, forward_step_cy_2d.pyx:21-120) and the
// phi-function table used by the fused timesteppers.
#include "dd_common.cuh"
#include "etd.cuh"

namespace dd {

__global__ void k_euler(const double2* __restrict__ s, double2* o, const double2* __restrict__ d,
                        double dt, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 a = s[i], b = d[i];
        double2 r;
        r.x = radd(a.x, rmul(dt, b.x));
        r.y = radd(a.y, rmul(dt, b.y));
        o[i] = r;
    }
}

template <int NDIM>
__global__ void k_etd1(const double2* s, double2* o, const double2* __restrict__ d,
                       const double* __restrict__ intf, double dt, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double Z = rmul(intf[i], dt);
        double f0 = 1., f1 = 1., f2 = 0.5;
        if (Z != 0.) etd_phis<NDIM>(Z, f0, f1, f2);
        o[i] = etd1_entry(s[i], d[i], Z, f0, f1, dt);
    }
}

template <int NDIM>
__global__ void k_etd2rk1(const double2* s, double2* o, const double2* __restrict__ d1,
                          const double2* __restrict__ d2, const double* __restrict__ intf,
                          double dt, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double Z = rmul(intf[i], dt);
        double f0 = 1., f1 = 1., f2 = 0.5;
        if (Z != 0.) etd_phis<NDIM>(Z, f0, f1, f2);
        o[i] = etd2rk1_entry(s[i], d1[i], d2[i], Z, f2, dt);
    }
}

template <int NDIM>
__global__ void k_etd2rk2(const double2* s, double2* o, const double2* __restrict__ d1,
                          const double2* __restrict__ d2, const double* __restrict__ intf,
                          double dt, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double Z = rmul(intf[i], dt);
        double f0 = 1., f1 = 1., f2 = 0.5;
        if (Z != 0.) etd_phis<NDIM>(Z, f0, f1, f2);
        o[i] = etd2rk2_entry(s[i], d1[i], d2[i], Z, f0, f1, f2, dt);
    }
}

// table[q] = {Z, f0, f1, f2} for integer squared wavenumber q with
// Z = -(nu * q**vo) * h, i.e. the reference's intfactor * dt for k2 == q.
template <int NDIM>
__global__ void k_phi_table(double nu, int vo, double h, int qmax, double4* tab) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q > qmax) return;
    const double k2 = (double)q;
    double k2v = (vo == 1) ? k2 : (vo == 2 ? rmul(k2, k2) : pow(k2, (double)vo));
    const double IF = rmul(nu, k2v);
    const double Z = rmul(-IF, h);
    double f0 = 1., f1 = 1., f2 = 0.5;
    if (Z != 0.) etd_phis<NDIM>(Z, f0, f1, f2);
    tab[q] = make_double4(Z, f0, f1, f2);
}

static unsigned ew_blocks(int64_t n) {
    int64_t b = (n + 255) / 256;
    if (b > 152 * 32) b = 152 * 32;
    if (b < 1) b = 1;
    return (unsigned)b;
}

}  // namespace dd

using namespace dd;

extern "C" {

int dd_euler(const void* start, void* output, const void* deriv, double dt, int64_t n, void* stream) {
    DD_CHECK_ARG(start && output && deriv, "dd_euler: null pointer");
    DD_CHECK_ARG(n >= 0, "dd_euler: negative size");
    if (n == 0) return DD_OK;
    cudaStream_t st = (cudaStream_t)stream;
    DD_KT("euler", st, k_euler<<<ew_blocks(n), 256, 0, st>>>((const double2*)start, (double2*)output,
                                                             (const double2*)deriv, dt, n));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

int dd_etd1(int ndim, const void* start, void* output, const void* deriv, const double* intfactor,
            double dt, int64_t n, void* stream) {
    DD_CHECK_ARG(start && output && deriv && intfactor, "dd_etd1: null pointer");
    DD_CHECK_ARG(ndim == 2 || ndim == 3, "dd_etd1: ndim must be 2 or 3");
    DD_CHECK_ARG(n >= 0, "dd_etd1: negative size");
    if (n == 0) return DD_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (ndim == 2)
        DD_KT("etd12", st, k_etd1<2><<<ew_blocks(n), 256, 0, st>>>((const double2*)start, (double2*)output, (const double2*)deriv, intfactor, dt, n));
    else
        DD_KT("etd13", st, k_etd1<3><<<ew_blocks(n), 256, 0, st>>>((const double2*)start, (double2*)output, (const double2*)deriv, intfactor, dt, n));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

int dd_etd2rk1(int ndim, const void* start, void* output, const void* deriv1, const void* deriv2,
               const double* intfactor, double dt, int64_t n, void* stream) {
    DD_CHECK_ARG(start && output && deriv1 && deriv2 && intfactor, "dd_etd2rk1: null pointer");
    DD_CHECK_ARG(ndim == 2 || ndim == 3, "dd_etd2rk1: ndim must be 2 or 3");
    DD_CHECK_ARG(n >= 0, "dd_etd2rk1: negative size");
    if (n == 0) return DD_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (ndim == 2)
        DD_KT("etd2rk12", st, k_etd2rk1<2><<<ew_blocks(n), 256, 0, st>>>((const double2*)start, (double2*)output, (const double2*)deriv1,
                                                   (const double2*)deriv2, intfactor, dt, n));
    else
        DD_KT("etd2rk13", st, k_etd2rk1<3><<<ew_blocks(n), 256, 0, st>>>((const double2*)start, (double2*)output, (const double2*)deriv1,
                                                   (const double2*)deriv2, intfactor, dt, n));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

int dd_etd2rk2(int ndim, const void* start, void* output, const void* deriv1, const void* deriv2,
               const double* intfactor, double dt, int64_t n, void* stream) {
    DD_CHECK_ARG(start && output && deriv1 && deriv2 && intfactor, "dd_etd2rk2: null pointer");
    DD_CHECK_ARG(ndim == 2 || ndim == 3, "dd_etd2rk2: ndim must be 2 or 3");
    DD_CHECK_ARG(n >= 0, "dd_etd2rk2: negative size");
    if (n == 0) return DD_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (ndim == 2)
        DD_KT("etd2rk22", st, k_etd2rk2<2><<<ew_blocks(n), 256, 0, st>>>((const double2*)start, (double2*)output, (const double2*)deriv1,
                                                   (const double2*)deriv2, intfactor, dt, n));
    else
        DD_KT("etd2rk23", st, k_etd2rk2<3><<<ew_blocks(n), 256, 0, st>>>((const double2*)start, (double2*)output, (const double2*)deriv1,
                                                   (const double2*)deriv2, intfactor, dt, n));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

int dd_phi_table(int ndim, double nu, int viscosity_order, double h, int qmax, void* table, void* stream) {
    DD_CHECK_ARG(table, "dd_phi_table: null pointer");
    DD_CHECK_ARG(ndim == 2 || ndim == 3, "dd_phi_table: ndim must be 2 or 3");
    DD_CHECK_ARG(qmax >= 0, "dd_phi_table: qmax must be >= 0");
    DD_CHECK_ARG(viscosity_order >= 1, "dd_phi_table: viscosity_order must be >= 1");
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned nb = (unsigned)((qmax + 256) / 256);
    if (ndim == 2) DD_KT("phi_table2", st, k_phi_table<2><<<nb, 256, 0, st>>>(nu, viscosity_order, h, qmax, (double4*)table));
    else           DD_KT("phi_table3", st, k_phi_table<3><<<nb, 256, 0, st>>>(nu, viscosity_order, h, qmax, (double4*)table));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

}  // extern "C"
