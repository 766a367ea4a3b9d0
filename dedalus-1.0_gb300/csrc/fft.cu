// Plans and the pruned 2D/3D real transforms (r2c forward with 1/N and 2/3
// dealiasing, c2r backward of the kept modes).
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <vector>

#include "launch_len.cuh"

namespace dd {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}
const char* last_error() { return g_err; }

static bool is_pow2(int64_t n) { return n >= 8 && n <= 512 && (n & (n - 1)) == 0; }

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

static int upload_twiddles(int L, double2** d64, float2** d32) {
    std::vector<double> re, im;
    make_twiddles(L, re, im);
    std::vector<double2> h64(L);
    std::vector<float2> h32(L);
    for (int m = 0; m < L; m++) {
        h64[m] = make_double2(re[m], im[m]);
        h32[m] = make_float2((float)re[m], (float)im[m]);
    }
    DD_CUDA(cudaMalloc((void**)d64, sizeof(double2) * L));
    DD_CUDA(cudaMalloc((void**)d32, sizeof(float2) * L));
    DD_CUDA(cudaMemcpy(*d64, h64.data(), sizeof(double2) * L, cudaMemcpyHostToDevice));
    DD_CUDA(cudaMemcpy(*d32, h32.data(), sizeof(float2) * L, cudaMemcpyHostToDevice));
    return DD_OK;
}

static int upload_doubles(const double* h, int n, double** d) {
    DD_CUDA(cudaMalloc((void**)d, sizeof(double) * (n > 0 ? n : 1)));
    if (n > 0) DD_CUDA(cudaMemcpy(*d, h, sizeof(double) * n, cudaMemcpyHostToDevice));
    return DD_OK;
}

// -------------------------------------------------------- zero / dealias
template <typename KT>
__global__ void k_zero_nonkept3(Geo3 g, Ptrs k) {
    using KV = typename Vec2<KT>::type;
    KV* K = (KV*)k.p[blockIdx.y];
    const int64_t n = g.kcount();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int kx = (int)(i % g.Nh);
        const int ky = (int)(i / ((int64_t)g.Nh * g.Nz));
        if (kx >= g.Kx || !kept_full(ky, g.Ny, g.My)) { KV z; z.x = 0; z.y = 0; K[i] = z; }
    }
}

template <typename KT>
__global__ void k_zero_nonkept2(Geo2 g, Ptrs k) {
    using KV = typename Vec2<KT>::type;
    KV* K = (KV*)k.p[blockIdx.y];
    const int64_t n0 = (int64_t)g.Kx * g.Ny, n = g.kcount();
    for (int64_t i = n0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        KV z; z.x = 0; z.y = 0; K[i] = z;
    }
}

__global__ void k_dealias3(Geo3 g, double2* K) {
    const int64_t n = g.kcount();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int kx = (int)(i % g.Nh);
        const int64_t r = i / g.Nh;
        const int kz = (int)(r % g.Nz), ky = (int)(r / g.Nz);
        if (kx > g.Mx || !kept_full(ky, g.Ny, g.My) || !kept_full(kz, g.Nz, g.Mz)) K[i] = make_double2(0., 0.);
    }
}

__global__ void k_dealias2(Geo2 g, double2* K) {
    const int64_t n = g.kcount();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int ky = (int)(i % g.Ny), kx = (int)(i / g.Ny);
        if (kx > g.Mx || !kept_full(ky, g.Ny, g.My)) K[i] = make_double2(0., 0.);
    }
}

static unsigned ew_grid(int64_t n) {
    int64_t b = (n + 255) / 256;
    if (b > 152 * 16) b = 152 * 16;
    return (unsigned)(b < 1 ? 1 : b);
}

// -------------------------------------------------------- transforms
template <typename T>
size_t ws_bytes(const dd_plan* pl, int nf) {
    if (pl->ndim == 3) return (size_t)nf * (pl->g3.w1count() + pl->g3.w2count()) * sizeof(C<T>);
    return (size_t)nf * pl->g2.wcount() * sizeof(C<T>);
}

template <typename T>
int fft_c2r(const dd_plan* pl, int nf, const void* const* k, double* const* x, void* work, size_t wb,
            cudaStream_t st) {
    DD_CHECK_ARG(wb >= ws_bytes<T>(pl, nf), "workspace too small: %zu < %zu bytes", wb, ws_bytes<T>(pl, nf));
    CPtrs kin{}; Ptrs xo{};
    for (int f = 0; f < nf; f++) { kin.p[f] = k[f]; xo.p[f] = x[f]; }
    if (pl->ndim == 3) {
        const Geo3& g = pl->g3;
        C<T>* W1 = (C<T>*)work;
        C<T>* W2 = W1 + (size_t)nf * g.w1count();
        Ptrs w1{}, w2{}; CPtrs w1c{}, w2c{};
        for (int f = 0; f < nf; f++) {
            w1.p[f] = W1 + f * g.w1count(); w1c.p[f] = w1.p[f];
            w2.p[f] = W2 + f * g.w2count(); w2c.p[f] = w2.p[f];
        }
        OpZInv3<T, double> a{g, kin, w1, TwSel<T>::z(pl)};
        DD_TRY((launch_pass_len<T, true, false, false>(g.Nz, a, g.Kx, g.Ky, nf, st)));
        OpYInv3<T> b{g, w1c, w2, TwSel<T>::y(pl)};
        DD_TRY((launch_pass_len<T, true, false, false>(g.Ny, b, g.Kx, g.Nz, nf, st)));
        const int nrows = g.Nz * g.Ny;
        OpXc2r3<T, double> c{nrows, g.Nx, g.Kx, w2c, xo, TwSel<T>::x(pl)};
        DD_TRY((launch_pass_len<T, true, true, true>(g.Nx, c, (nrows + 1) / 2, 1, nf, st)));
    } else {
        const Geo2& g = pl->g2;
        C<T>* W = (C<T>*)work;
        Ptrs w{}; CPtrs wc{};
        for (int f = 0; f < nf; f++) { w.p[f] = W + f * g.wcount(); wc.p[f] = w.p[f]; }
        OpYInv2<T, double> a{g, kin, w, TwSel<T>::y(pl)};
        DD_TRY((launch_pass_len<T, true, true, false>(g.Ny, a, g.Kx, 1, nf, st)));
        OpXc2r3<T, double> c{g.Ny, g.Nx, g.Kx, wc, xo, TwSel<T>::x(pl)};
        DD_TRY((launch_pass_len<T, true, true, true>(g.Nx, c, (g.Ny + 1) / 2, 1, nf, st)));
    }
    return DD_OK;
}

template <typename T>
int fft_r2c(const dd_plan* pl, int nf, const double* const* x, void* const* k, void* work, size_t wb,
            cudaStream_t st) {
    DD_CHECK_ARG(wb >= ws_bytes<T>(pl, nf), "workspace too small: %zu < %zu bytes", wb, ws_bytes<T>(pl, nf));
    CPtrs xin{}; Ptrs ko{};
    for (int f = 0; f < nf; f++) { xin.p[f] = x[f]; ko.p[f] = k[f]; }
    const T s = (T)pl->inv_n;
    if (pl->ndim == 3) {
        const Geo3& g = pl->g3;
        C<T>* W1 = (C<T>*)work;
        C<T>* W2 = W1 + (size_t)nf * g.w1count();
        Ptrs w1{}, w2{}; CPtrs w1c{}, w2c{};
        for (int f = 0; f < nf; f++) {
            w1.p[f] = W1 + f * g.w1count(); w1c.p[f] = w1.p[f];
            w2.p[f] = W2 + f * g.w2count(); w2c.p[f] = w2.p[f];
        }
        const int nrows = g.Nz * g.Ny;
        OpXr2c3<T, double> a{nrows, g.Nx, g.Kx, s, xin, w2, TwSel<T>::x(pl)};
        DD_TRY((launch_pass_len<T, false, true, true>(g.Nx, a, (nrows + 1) / 2, 1, nf, st)));
        OpYFwd3<T> b{g, w2c, w1, TwSel<T>::y(pl)};
        DD_TRY((launch_pass_len<T, false, false, false>(g.Ny, b, g.Kx, g.Nz, nf, st)));
        OpZFwd3<T, double> c{g, w1c, ko, TwSel<T>::z(pl)};
        DD_TRY((launch_pass_len<T, false, false, false>(g.Nz, c, g.Kx, g.Ky, nf, st)));
        DD_KT("zero_nonkept3", st, k_zero_nonkept3<double><<<dim3(ew_grid(g.kcount()), nf), 256, 0, st>>>(g, ko));
        DD_LAUNCH_CHECK();
    } else {
        const Geo2& g = pl->g2;
        C<T>* W = (C<T>*)work;
        Ptrs w{}; CPtrs wc{};
        for (int f = 0; f < nf; f++) { w.p[f] = W + f * g.wcount(); wc.p[f] = w.p[f]; }
        OpXr2c3<T, double> a{g.Ny, g.Nx, g.Kx, s, xin, w, TwSel<T>::x(pl)};
        DD_TRY((launch_pass_len<T, false, true, true>(g.Nx, a, (g.Ny + 1) / 2, 1, nf, st)));
        OpYFwd2<T, double> b{g, wc, ko, TwSel<T>::y(pl)};
        DD_TRY((launch_pass_len<T, false, false, true>(g.Ny, b, g.Kx, 1, nf, st)));
        const int64_t nz = g.kcount() - (int64_t)g.Kx * g.Ny;
        if (nz > 0) {
            DD_KT("zero_nonkept2", st, k_zero_nonkept2<double><<<dim3(ew_grid(nz), nf), 256, 0, st>>>(g, ko));
            DD_LAUNCH_CHECK();
        }
    }
    return DD_OK;
}

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
        DD_CHECK_SUPPORTED(is_pow2(xshape[i]), "dd_plan_create: axis %d has size %lld; sizes must be powers of two in [8, 512]",
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
        if ((rc = upload_doubles(kx, Nh, &p->kx)) || (rc = upload_doubles(ky, Ny, &p->ky)) ||
            (rc = upload_doubles(kz, Nz, &p->kz)))
            return fail(rc);
    } else {
        Geo2& g = p->g2;
        g.Ny = Ny; g.Nx = Nx; g.Nh = Nh;
        g.Mx = mx; g.My = my;
        g.Kx = mx + 1; g.Ky = 2 * my + 1;
        p->inv_n = 1.0 / ((double)Nx * Ny);
        if ((rc = upload_doubles(kx, Nh, &p->kx)) || (rc = upload_doubles(ky, Ny, &p->ky))) return fail(rc);
    }
    if ((rc = upload_twiddles(Nx, &p->tw64_x, &p->tw32_x)) || (rc = upload_twiddles(Ny, &p->tw64_y, &p->tw32_y)))
        return fail(rc);
    if (ndim == 3 && (rc = upload_twiddles(Nz, &p->tw64_z, &p->tw32_z))) return fail(rc);
    *out = p;
    return DD_OK;
}

int dd_plan_destroy(dd_plan* p) {
    if (!p) return DD_OK;
    void* bufs[] = {p->kx, p->ky, p->kz, p->tw64_x, p->tw64_y, p->tw64_z, p->tw32_x, p->tw32_y, p->tw32_z};
    for (void* b : bufs)
        if (b) cudaFree(b);
    free(p);
    return DD_OK;
}

int dd_plan_workspace_size(const dd_plan* p, int nfield, int precision, size_t* bytes) {
    DD_CHECK_ARG(p && bytes, "dd_plan_workspace_size: null pointer");
    DD_CHECK_ARG(nfield >= 1 && nfield <= 8, "nfield must be in [1, 8]");
    DD_CHECK_ARG(precision == DD_FP64 || precision == DD_FP32, "precision must be DD_FP64 or DD_FP32");
    *bytes = precision == DD_FP64 ? ws_bytes<double>(p, nfield) : ws_bytes<float>(p, nfield);
    return DD_OK;
}

int dd_fft_r2c(const dd_plan* p, int nfield, const double* const* x, void* const* k, int precision,
               void* work, size_t work_bytes, void* stream) {
    DD_CHECK_ARG(p && x && k && work, "dd_fft_r2c: null pointer");
    DD_CHECK_ARG(nfield >= 1 && nfield <= 8, "nfield must be in [1, 8]");
    for (int f = 0; f < nfield; f++) DD_CHECK_ARG(x[f] && k[f], "dd_fft_r2c: null field pointer %d", f);
    if (precision == DD_FP64) return fft_r2c<double>(p, nfield, x, k, work, work_bytes, (cudaStream_t)stream);
    if (precision == DD_FP32) return fft_r2c<float>(p, nfield, x, k, work, work_bytes, (cudaStream_t)stream);
    DD_CHECK_ARG(false, "precision must be DD_FP64 or DD_FP32");
}

int dd_fft_c2r(const dd_plan* p, int nfield, const void* const* k, double* const* x, int precision,
               void* work, size_t work_bytes, void* stream) {
    DD_CHECK_ARG(p && x && k && work, "dd_fft_c2r: null pointer");
    DD_CHECK_ARG(nfield >= 1 && nfield <= 8, "nfield must be in [1, 8]");
    for (int f = 0; f < nfield; f++) DD_CHECK_ARG(x[f] && k[f], "dd_fft_c2r: null field pointer %d", f);
    if (precision == DD_FP64) return fft_c2r<double>(p, nfield, k, x, work, work_bytes, (cudaStream_t)stream);
    if (precision == DD_FP32) return fft_c2r<float>(p, nfield, k, x, work, work_bytes, (cudaStream_t)stream);
    DD_CHECK_ARG(false, "precision must be DD_FP64 or DD_FP32");
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
