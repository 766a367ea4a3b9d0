/*
 * CPU oracle -- test infrastructure only (the checker, never the product).
 *
 * Plain-C restatement of the reference's native hot-path kernels:
 *   - dedalus/time_stepping/forward_step_cy_3d.pyx:17-124  (3D euler/etd1/etd2rk1/etd2rk2)
 *   - dedalus/time_stepping/forward_step_cy_2d.pyx:21-148  (2D variants + f_taylor)
 *   - dedalus/data_objects/dealias_cy_3d.pyx:13-37 / dealias_cy_2d.pyx:59-78 (dealias_23)
 *
 * All arrays are contiguous and of identical shape, so each stage kernel is a
 * flat loop over n complex128 entries stored as interleaved (re, im) doubles.
 * The arithmetic follows the reference expression by expression (same
 * operation order, no FMA contraction: build with -ffp-contract=off).  The
 * complex-by-real products of the reference are complex products with a zero
 * imaginary part, which equal the component-wise products written here.
 *
 * The only difference between the 2D and 3D reference kernels is the Taylor
 * branch for |Z| < 0.5: 3D uses exp(Z) for f0 and hand-unrolled 14-term
 * polynomials for f1/f2 (forward_step_cy_3d.pyx:54-59, 84-91, 116-123); 2D
 * uses the f_taylor loop (pow-based, 15 terms) for f0, f1 and f2
 * (forward_step_cy_2d.pyx:54-59, 123-148).
 */
#include <math.h>
#include <stdint.h>

/* forward_step_cy_2d.pyx:123-148: sum_{j=k}^{14} Z**(j-k)/j! */
static double f_taylor(int k, double Z)
{
    int j;
    double factj = 1.;
    double sum = 0.;
    if (k > 2) {
        for (j = 1; j < k; j++) factj *= j;
    }
    for (j = k; j < 15; j++) {
        if (j > 1) factj *= j;
        sum = sum + pow(Z, (double)(j - k)) / factj;
    }
    return sum;
}

/* forward_step_cy_3d.pyx:56 (f1 polynomial, highest power first) */
static double poly_f1_3d(double Z)
{
    return Z*Z*Z*Z*Z*Z*Z*Z*Z*Z*Z*Z*Z/87178291200. + Z*Z*Z*Z*Z*Z*Z*Z*Z*Z*Z*Z/6227020800.
         + Z*Z*Z*Z*Z*Z*Z*Z*Z*Z*Z/479001600. + Z*Z*Z*Z*Z*Z*Z*Z*Z*Z/39916800.
         + Z*Z*Z*Z*Z*Z*Z*Z*Z/3628800. + Z*Z*Z*Z*Z*Z*Z*Z/362880. + Z*Z*Z*Z*Z*Z*Z/40320.
         + Z*Z*Z*Z*Z*Z/5040. + Z*Z*Z*Z*Z/720. + Z*Z*Z*Z/120. + Z*Z*Z/24. + Z*Z/6. + Z/2. + 1.;
}

/* forward_step_cy_3d.pyx:87 (f2 polynomial) */
static double poly_f2_3d(double Z)
{
    return Z*Z*Z*Z*Z*Z*Z*Z*Z*Z*Z*Z/87178291200. + Z*Z*Z*Z*Z*Z*Z*Z*Z*Z*Z/6227020800.
         + Z*Z*Z*Z*Z*Z*Z*Z*Z*Z/479001600. + Z*Z*Z*Z*Z*Z*Z*Z*Z/39916800.
         + Z*Z*Z*Z*Z*Z*Z*Z/3628800. + Z*Z*Z*Z*Z*Z*Z/362880. + Z*Z*Z*Z*Z*Z/40320.
         + Z*Z*Z*Z*Z/5040. + Z*Z*Z*Z/720. + Z*Z*Z/120. + Z*Z/24. + Z/6. + 0.5;
}

/* phi functions for the non-zero-Z branches; ndim selects the reference variant */
static void phis(int ndim, double Z, double *f0, double *f1, double *f2)
{
    if ((Z < 0.5) && (Z > -0.5)) {
        if (ndim == 2) {
            *f0 = f_taylor(0, Z);
            *f1 = f_taylor(1, Z);
            if (f2) *f2 = f_taylor(2, Z);
        } else {
            *f0 = exp(Z);
            *f1 = poly_f1_3d(Z);
            if (f2) *f2 = poly_f2_3d(Z);
        }
    } else {
        *f0 = exp(Z);
        *f1 = (*f0 - 1.) / Z;
        if (f2) *f2 = (*f1 - 1.) / Z;
    }
}

/* forward_step_cy_3d.pyx:17-31: output = start + dt * deriv */
void dd_oracle_euler(const double *start, double *out, const double *deriv,
                     double dt, int64_t n)
{
    for (int64_t i = 0; i < n; i++) {
        double sr = start[2*i], si = start[2*i+1];
        out[2*i]   = sr + dt * deriv[2*i];
        out[2*i+1] = si + dt * deriv[2*i+1];
    }
}

/* forward_step_cy_3d.pyx:34-60 (ndim==3) / forward_step_cy_2d.pyx:36-60 (ndim==2) */
void dd_oracle_etd1(int ndim, const double *start, double *out, const double *deriv,
                    const double *intfactor, double dt, int64_t n)
{
    for (int64_t i = 0; i < n; i++) {
        double Z = intfactor[i] * dt;
        double sr = start[2*i], si = start[2*i+1];
        double dr = deriv[2*i], di = deriv[2*i+1];
        if (Z == 0.) {
            out[2*i]   = sr + dt * dr;
            out[2*i+1] = si + dt * di;
        } else {
            double f0, f1;
            phis(ndim, Z, &f0, &f1, 0);
            out[2*i]   = sr * f0 + dr * f1 * dt;
            out[2*i+1] = si * f0 + di * f1 * dt;
        }
    }
}

/* forward_step_cy_3d.pyx:63-92 / forward_step_cy_2d.pyx:63-90 */
void dd_oracle_etd2rk1(int ndim, const double *start, double *out, const double *deriv1,
                       const double *deriv2, const double *intfactor, double dt, int64_t n)
{
    for (int64_t i = 0; i < n; i++) {
        double Z = intfactor[i] * dt;
        double sr = start[2*i], si = start[2*i+1];
        double ar = deriv2[2*i] - deriv1[2*i], ai = deriv2[2*i+1] - deriv1[2*i+1];
        if (Z == 0.) {
            out[2*i]   = sr + dt / 2. * ar;
            out[2*i+1] = si + dt / 2. * ai;
        } else {
            double f0, f1, f2;
            phis(ndim, Z, &f0, &f1, &f2);
            out[2*i]   = sr + ar * f2 * dt;
            out[2*i+1] = si + ai * f2 * dt;
        }
    }
}

/* forward_step_cy_3d.pyx:95-124 / forward_step_cy_2d.pyx:93-120 */
void dd_oracle_etd2rk2(int ndim, const double *start, double *out, const double *deriv1,
                       const double *deriv2, const double *intfactor, double dt, int64_t n)
{
    for (int64_t i = 0; i < n; i++) {
        double Z = intfactor[i] * dt;
        double sr = start[2*i], si = start[2*i+1];
        double d1r = deriv1[2*i], d1i = deriv1[2*i+1];
        double d2r = deriv2[2*i], d2i = deriv2[2*i+1];
        if (Z == 0.) {
            out[2*i]   = sr + dt * d2r;
            out[2*i+1] = si + dt * d2i;
        } else {
            double f0, f1, f2;
            phis(ndim, Z, &f0, &f1, &f2);
            out[2*i]   = sr * f0 + (d2r - d1r) * 2. * f2 * dt + d1r * f1 * dt;
            out[2*i+1] = si * f0 + (d2i - d1i) * 2. * f2 * dt + d1i * f1 * dt;
        }
    }
}

/* dealias_cy_3d.pyx:25-37 (static-k branch): data[y,z,x] = 0 where any
 * |k_i| >= 2/3 knyquist_i; knyquist is ordered (ky, kz, kx). */
void dd_oracle_dealias_23_3d(double *data, const double *kx, int nx, const double *ky, int ny,
                             const double *kz, int nz, const double *knyquist)
{
    double tx = 2. / 3. * knyquist[2], ty = 2. / 3. * knyquist[0], tz = 2. / 3. * knyquist[1];
    for (int y = 0; y < ny; y++)
        for (int z = 0; z < nz; z++)
            for (int x = 0; x < nx; x++) {
                if (((kx[x] >= tx) || (kx[x] <= -tx)) ||
                    ((ky[y] >= ty) || (ky[y] <= -ty)) ||
                    ((kz[z] >= tz) || (kz[z] <= -tz))) {
                    int64_t i = ((int64_t)y * nz + z) * nx + x;
                    data[2*i] = 0.;
                    data[2*i+1] = 0.;
                }
            }
}

/* dealias_cy_2d.pyx:69-78 (static-k branch): data[x,y]; knyquist is (kx, ky). */
void dd_oracle_dealias_23_2d(double *data, const double *kx, int nx, const double *ky, int ny,
                             const double *knyquist)
{
    double tx = 2. / 3. * knyquist[0], ty = 2. / 3. * knyquist[1];
    for (int x = 0; x < nx; x++)
        for (int y = 0; y < ny; y++) {
            if (((kx[x] >= tx) || (kx[x] <= -tx)) || ((ky[y] >= ty) || (ky[y] <= -ty))) {
                int64_t i = (int64_t)x * ny + y;
                data[2*i] = 0.;
                data[2*i+1] = 0.;
            }
        }
}
