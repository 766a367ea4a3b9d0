// Small field operations behind the representation's user API: spectral
// derivative (representations.py:419-425), scaled copies, and the largest
// squared grid value of a vector field (fields.py:153-157, for the CFL step).
#include "dd_common.cuh"
#include "geometry.cuh"
#include "plan.cuh"

namespace dd {

// out = in * (1j * k_axis) with numpy's complex product ((-b k), a k).
// axis: 0 = x, 1 = y, 2 = z (component names, not storage order).
__global__ void k_deriv(int ndim, int n0, int n1, int n2, int axis, const double* kx, const double* ky,
                        const double* kz, const double2* in, double2* out) {
    const int64_t n = (int64_t)n0 * n1 * n2;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double k;
        if (ndim == 3) {  // [ky][kz][kx]
            const int ix = (int)(i % n2);
            const int64_t r = i / n2;
            const int iz = (int)(r % n1), iy = (int)(r / n1);
            k = axis == 0 ? kx[ix] : (axis == 1 ? ky[iy] : kz[iz]);
        } else {          // [kx][ky]
            const int iy = (int)(i % n1), ix = (int)(i / n1);
            k = axis == 0 ? kx[ix] : ky[iy];
        }
        const double2 a = in[i];
        out[i] = make_double2(-(a.y * k), a.x * k);
    }
}

// y = x * w (accumulate == 0) or y = y + x * w, complex x, y and real w: the
// numpy forms `comp = kd / 6.` and `comp += kd / 3.` (time_step.py:435, 452),
// numpy dividing by multiplying with the reciprocal.
__global__ void k_scale_add(const double2* x, double2* y, double w, int accumulate, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 a = x[i];
        double2 r = make_double2(__dmul_rn(a.x, w), __dmul_rn(a.y, w));
        if (accumulate) { const double2 b = y[i]; r = make_double2(__dadd_rn(b.x, r.x), __dadd_rn(b.y, r.y)); }
        y[i] = r;
    }
}

// out = max over components c and grid points i of x_c[i]^2.  The squares are
// non-negative, so their IEEE bit patterns order like the values and one
// 64-bit atomicMax per warp merges them; the result is exact and
// independent of the launch shape (a NaN anywhere wins, as with numpy's max).
// *out must hold +0.0 (all-zero bits) on entry.
__global__ void k_max_square(CPtrs x, int ncomp, int64_t n, unsigned long long* out) {
    double m = 0.0;
#pragma unroll
    for (int c = 0; c < DD_MAXF; c++) {   // constant indices keep x in the parameter space
        if (c >= ncomp) break;
        const double* xc = (const double*)x.p[c];
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
            const double v = xc[i];
            const double q = v * v;
            m = (q > m || q != q) ? q : m;
        }
    }
    unsigned long long b = (unsigned long long)__double_as_longlong(m);
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, b, o);
        b = t > b ? t : b;
    }
    if ((threadIdx.x & 31) == 0 && b != 0ull) atomicMax(out, b);
}

static unsigned grid_for(int64_t n) {
    int64_t b = (n + 255) / 256;
    if (b > 152 * 16) b = 152 * 16;
    return (unsigned)(b < 1 ? 1 : b);
}

}  // namespace dd

using namespace dd;

extern "C" {

int dd_deriv(const dd_plan* p, int axis, const void* k_in, void* k_out, void* stream) {
    DD_CHECK_ARG(p && k_in && k_out, "dd_deriv: null pointer");
    DD_CHECK_ARG(axis >= 0 && axis < p->ndim, "dd_deriv: axis %d out of range", axis);
    int n0, n1, n2;
    if (p->ndim == 3) { n0 = p->g3.Ny; n1 = p->g3.Nz; n2 = p->g3.Nh; }
    else { n0 = p->g2.Nh; n1 = p->g2.Ny; n2 = 1; }
    const int64_t n = (int64_t)n0 * n1 * n2;
    DD_KT("deriv", (cudaStream_t)stream,
          k_deriv<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>(p->ndim, n0, n1, n2, axis, p->kx, p->ky, p->kz,
                                                                 (const double2*)k_in, (double2*)k_out));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

int dd_scale_add(const void* x, void* y, double w, int accumulate, int64_t n, void* stream) {
    DD_CHECK_ARG(x && y && n >= 0, "dd_scale_add: bad arguments");
    if (n == 0) return DD_OK;
    DD_KT("scale_add", (cudaStream_t)stream,
          k_scale_add<<<grid_for(n), 256, 0, (cudaStream_t)stream>>>((const double2*)x, (double2*)y, w, accumulate, n));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

int dd_max_square(int ncomp, const double* const* x, int64_t n, double* out, void* stream) {
    DD_CHECK_ARG(x && out && n >= 0, "dd_max_square: bad arguments");
    DD_CHECK_ARG(ncomp >= 1 && ncomp <= DD_MAXF, "dd_max_square: ncomp %d out of range", ncomp);
    CPtrs xs{};
    for (int c = 0; c < ncomp; c++) {
        DD_CHECK_ARG(x[c], "dd_max_square: null component pointer %d", c);
        xs.p[c] = x[c];
    }
    const cudaStream_t st = (cudaStream_t)stream;
    DD_CUDA(cudaMemsetAsync(out, 0, sizeof(double), st));
    if (n == 0) return DD_OK;
    DD_KT("max_square", st,
          k_max_square<<<grid_for(n), 256, 0, st>>>(xs, ncomp, n, (unsigned long long*)out));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

}  // extern "C"
