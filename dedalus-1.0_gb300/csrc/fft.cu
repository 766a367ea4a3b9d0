// Plans and the pruned 2D/3D real transforms (r2c forward with 1/N and 2/3
// dealiasing, c2r backward of the kept modes).
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <vector>

#include "fft_impl.cuh"

namespace dd {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}
const char* last_error() { return g_err; }

// Supported axis lengths: powers of two 8..512 and 3 x a power of two 24..192.
static bool is_supported_len(int64_t n) {
    if (n >= 8 && n <= 512 && (n & (n - 1)) == 0) return true;
    return n == 24 || n == 48 || n == 96 || n == 192;
}

// exp(-2 pi i m / L) for m < L, from the first octant by symmetry so that the
// quadrant points are exact.  Long double keeps the rounding to double
// essentially correct.
static void make_twiddles(int L, std::vector<double>& re, std::vector<double>& im) {
    re.resize(L);
    im.resize(L);
    const long double two_pi = 6.283185307179586476925286766559005768L;
    for (int m = 0; m < L; m++) {
        const int q = (4 * m) / L;            // quadrant
        const int r = m - q * (L / 4);        // 0 <= r < L/4
        long double c, s;
        if (8 * r <= L) {
            const long double a = two_pi * r / L;
            c = cosl(a); s = sinl(a);
        } else {
            const long double a = two_pi * (L / 4 - r) / L;
            c = sinl(a); s = cosl(a);
        }
        if (r == 0) { c = 1.0L; s = 0.0L; }
        long double C, S;  // cos, sin of q*pi/2 + angle(r)
        switch (q) {
            case 0: C = c; S = s; break;
            case 1: C = -s; S = c; break;
            case 2: C = -c; S = -s; break;
            default: C = s; S = -c; break;
        }
        re[m] = (double)C;
        im[m] = (double)(-S);
    }
}

// The FP64 and FP32 tables hold W_L^m = g (1 + i t) as (g, t) for the
// fused multiply-add butterflies (fft_engine.cuh): g = Re W, t = Im W / Re W
// (an IEEE division of the rounded parts, so every host gives the same
// table); where Re W = 0 the pair is (2^-60, Im W 2^60), exact powers of two
// whose product is Im W.  The double-float table keeps (cos, sin).
static int upload_twiddles(int L, double2** d64, float2** d32, float4** ddf) {
    std::vector<double> re, im;
    make_twiddles(L, re, im);
    std::vector<double2> h64(L);
    std::vector<float2> h32(L);
    std::vector<float4> hdf(L);
    const double tiny = ldexp(1.0, -60), huge = ldexp(1.0, 60);
    for (int m = 0; m < L; m++) {
        double g, t;
        if (re[m] == 0.0) { g = tiny; t = im[m] * huge; }
        else { g = re[m]; t = im[m] / re[m]; }
        h64[m] = make_double2(g, t);
        const float g32 = (float)g;
        h32[m] = make_float2(g32, re[m] == 0.0 ? (float)t : (float)(im[m] / (double)g32));
        const df64 a(re[m]), b(im[m]);
        hdf[m] = make_float4(a.hi, a.lo, b.hi, b.lo);
    }
    DD_CUDA(cudaMalloc((void**)d64, sizeof(double2) * L));
    DD_CUDA(cudaMalloc((void**)d32, sizeof(float2) * L));
    DD_CUDA(cudaMalloc((void**)ddf, sizeof(float4) * L));
    DD_CUDA(cudaMemcpy(*d64, h64.data(), sizeof(double2) * L, cudaMemcpyHostToDevice));
    DD_CUDA(cudaMemcpy(*d32, h32.data(), sizeof(float2) * L, cudaMemcpyHostToDevice));
    DD_CUDA(cudaMemcpy(*ddf, hdf.data(), sizeof(float4) * L, cudaMemcpyHostToDevice));
    return DD_OK;
}

static int upload_doubles(const double* h, int n, double** d) {
    DD_CUDA(cudaMalloc((void**)d, sizeof(double) * (n > 0 ? n : 1)));
    if (n > 0) DD_CUDA(cudaMemcpy(*d, h, sizeof(double) * n, cudaMemcpyHostToDevice));
    return DD_OK;
}

// a wavenumber table as double and as float (rounded to nearest)
static int upload_k(const double* h, int n, double** d, float** f) {
    DD_TRY(upload_doubles(h, n, d));
    std::vector<float> hf(n > 0 ? n : 1, 0.f);
    for (int i = 0; i < n; i++) hf[i] = (float)h[i];
    DD_CUDA(cudaMalloc((void**)f, sizeof(float) * hf.size()));
    DD_CUDA(cudaMemcpy(*f, hf.data(), sizeof(float) * hf.size(), cudaMemcpyHostToDevice));
    return DD_OK;
}

DD_FFT_INSTANTIATE(extern, double)
DD_FFT_INSTANTIATE(extern, float)

}  // namespace dd

using namespace dd;

extern "C" {

int dd_version(void) { return 100; }
const char* dd_last_error(void) { return dd::last_error(); }

int dd_plan_create(int ndim, const int64_t* xshape, const double* kx, const double* ky, const double* kz,
                   int mx, int my, int mz, dd_plan** out) {
    DD_CHECK_ARG(out && xshape && kx && ky, "dd_plan_create: null pointer");
    DD_CHECK_ARG(ndim == 2 || ndim == 3, "dd_plan_create: ndim must be 2 or 3 (got %d)", ndim);
    DD_CHECK_ARG(ndim == 2 || kz, "dd_plan_create: kz table required in 3D");
    *out = nullptr;
    for (int i = 0; i < ndim; i++)
        DD_CHECK_SUPPORTED(is_supported_len(xshape[i]),
                           "dd_plan_create: axis %d has size %lld; sizes must be powers of two in [8, 512] or 24, 48, 96, 192",
                           i, (long long)xshape[i]);
    dd_plan* p = (dd_plan*)calloc(1, sizeof(dd_plan));
    DD_CHECK_ARG(p, "dd_plan_create: out of host memory");
    p->ndim = ndim;
    cudaGetDevice(&p->device);
    int rc = DD_OK;
    int Nx, Ny, Nz = 1;
    if (ndim == 3) { Nz = (int)xshape[0]; Ny = (int)xshape[1]; Nx = (int)xshape[2]; }
    else { Ny = (int)xshape[0]; Nx = (int)xshape[1]; }
    const int Nh = Nx / 2 + 1;
    auto fail = [&](int code) { dd_plan_destroy(p); return code; };
    if (mx < 0 || mx > Nx / 2 || my < 0 || 2 * my + 1 > Ny || (ndim == 3 && (mz < 0 || 2 * mz + 1 > Nz))) {
        set_error("dd_plan_create: kept-mode bounds out of range (mx=%d my=%d mz=%d)", mx, my, mz);
        return fail(DD_ERR_INVALID);
    }
    if (ndim == 3) {
        Geo3& g = p->g3;
        g.Nz = Nz; g.Ny = Ny; g.Nx = Nx; g.Nh = Nh;
        g.Mx = mx; g.My = my; g.Mz = mz;
        g.Kx = mx + 1; g.Ky = 2 * my + 1; g.Kz = 2 * mz + 1;
        p->inv_n = 1.0 / ((double)Nx * Ny * Nz);
        if ((rc = upload_k(kx, Nh, &p->kx, &p->kxf)) || (rc = upload_k(ky, Ny, &p->ky, &p->kyf)) ||
            (rc = upload_k(kz, Nz, &p->kz, &p->kzf)))
            return fail(rc);
    } else {
        Geo2& g = p->g2;
        g.Ny = Ny; g.Nx = Nx; g.Nh = Nh;
        g.Mx = mx; g.My = my;
        g.Kx = mx + 1; g.Ky = 2 * my + 1;
        p->inv_n = 1.0 / ((double)Nx * Ny);
        if ((rc = upload_k(kx, Nh, &p->kx, &p->kxf)) || (rc = upload_k(ky, Ny, &p->ky, &p->kyf))) return fail(rc);
    }
    if ((rc = upload_twiddles(Nx, &p->tw64_x, &p->tw32_x, &p->twdf_x)) ||
        (rc = upload_twiddles(Ny, &p->tw64_y, &p->tw32_y, &p->twdf_y)))
        return fail(rc);
    if (ndim == 3 && (rc = upload_twiddles(Nz, &p->tw64_z, &p->tw32_z, &p->twdf_z))) return fail(rc);
    *out = p;
    return DD_OK;
}

int dd_plan_destroy(dd_plan* p) {
    if (!p) return DD_OK;
    void* bufs[] = {p->kx, p->ky, p->kz, p->kxf, p->kyf, p->kzf, p->tw64_x, p->tw64_y, p->tw64_z, p->tw32_x, p->tw32_y, p->tw32_z,
                    p->twdf_x, p->twdf_y, p->twdf_z};
    for (void* b : bufs)
        if (b) cudaFree(b);
    free(p);
    return DD_OK;
}

int dd_plan_set_schedule(dd_plan* p, int which, int variant) {
    DD_CHECK_ARG(p, "dd_plan_set_schedule: null plan");
    DD_CHECK_ARG(which == 0, "dd_plan_set_schedule: unknown pass group %d", which);
    DD_CHECK_ARG(variant >= 0 && variant < kYSchedVariants, "dd_plan_set_schedule: variant %d out of range", variant);
    p->sched_y2d = variant;
    return DD_OK;
}

int dd_plan_get_schedule(const dd_plan* p, int which, int* variant, int* count) {
    DD_CHECK_ARG(p && variant && count, "dd_plan_get_schedule: null pointer");
    DD_CHECK_ARG(which == 0, "dd_plan_get_schedule: unknown pass group %d", which);
    *variant = p->sched_y2d;
    const int n = p->ndim == 2 ? p->g2.Ny : 0;
    *count = (n == 64 || n == 128 || n == 256 || n == 512) ? kYSchedVariants : 1;
    return DD_OK;
}

int dd_plan_workspace_size(const dd_plan* p, int nfield, int precision, size_t* bytes) {
    DD_CHECK_ARG(p && bytes, "dd_plan_workspace_size: null pointer");
    DD_CHECK_ARG(nfield >= 1 && nfield <= 8, "nfield must be in [1, 8]");
    DD_CHECK_ARG(precision >= DD_FP64 && precision <= DD_DF64, "precision must be DD_FP64, DD_FP32 or DD_DF64");
    DD_PREC_DISPATCH(precision, T, *bytes = ws_bytes<T>(p, nfield));
    return DD_OK;
}

int dd_fft_r2c(const dd_plan* p, int nfield, const double* const* x, void* const* k, int precision,
               void* work, size_t work_bytes, void* stream) {
    DD_CHECK_ARG(p && x && k && work, "dd_fft_r2c: null pointer");
    DD_CHECK_ARG(nfield >= 1 && nfield <= 8, "nfield must be in [1, 8]");
    for (int f = 0; f < nfield; f++) DD_CHECK_ARG(x[f] && k[f], "dd_fft_r2c: null field pointer %d", f);
    DD_CHECK_ARG(precision >= DD_FP64 && precision <= DD_DF64, "precision must be DD_FP64, DD_FP32 or DD_DF64");
    DD_CHECK_SUPPORTED(precision != DD_DF64, "the standalone transforms run in FP64 or FP32");
    DD_PREC_DISPATCH_2(precision, T, return fft_r2c<T>(p, nfield, x, k, work, work_bytes, (cudaStream_t)stream));
    return DD_OK;
}

int dd_fft_c2r(const dd_plan* p, int nfield, const void* const* k, double* const* x, int precision,
               void* work, size_t work_bytes, void* stream) {
    DD_CHECK_ARG(p && x && k && work, "dd_fft_c2r: null pointer");
    DD_CHECK_ARG(nfield >= 1 && nfield <= 8, "nfield must be in [1, 8]");
    for (int f = 0; f < nfield; f++) DD_CHECK_ARG(x[f] && k[f], "dd_fft_c2r: null field pointer %d", f);
    DD_CHECK_ARG(precision >= DD_FP64 && precision <= DD_DF64, "precision must be DD_FP64, DD_FP32 or DD_DF64");
    DD_CHECK_SUPPORTED(precision != DD_DF64, "the standalone transforms run in FP64 or FP32");
    DD_PREC_DISPATCH_2(precision, T, return fft_c2r<T>(p, nfield, k, x, work, work_bytes, (cudaStream_t)stream));
    return DD_OK;
}

int dd_dealias(const dd_plan* p, void* k, void* stream) {
    DD_CHECK_ARG(p && k, "dd_dealias: null pointer");
    cudaStream_t st = (cudaStream_t)stream;
    if (p->ndim == 3) DD_KT("dealias3", st, k_dealias3<<<ew_grid(p->g3.kcount()), 256, 0, st>>>(p->g3, (double2*)k));
    else DD_KT("dealias2", st, k_dealias2<<<ew_grid(p->g2.kcount()), 256, 0, st>>>(p->g2, (double2*)k));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

}  // extern "C"
