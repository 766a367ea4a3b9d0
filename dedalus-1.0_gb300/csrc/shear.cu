// Shearing-box Fourier representation (the reference's
// FourierShearRepresentation, dedalus/data_objects/representations.py:558-740)
// and the small field operations its right-hand sides are built from.
//
// Transforms (FP64): the x transform and its 2/3 cut are static, so they reuse
// the pruned x pass; between the x and y passes the x-transformed rows are
// multiplied by exp(+i S kx y t) (forward) or exp(-i S kx y t) (backward),
// representations.py:681-704.  The y transform runs over every ky index
// (which ky indices survive depends on time), and the 2/3 rule is evaluated
// against the sheared, wrapped k_y(t) of each (ky, kx) column, read from a
// table the host keeps (representations.py:627-643): entries with
// k_y >= cut or k_y <= -cut are zero (dealias_cy_3d.pyx:39-45,
// dealias_cy_2d.pyx:36-40).  The z cut stays static.
//
// Tables (device, float64): kys = the component's k['y'] array, [ky][kx]
// (Ny x Nh) in 3D and [kx][ky] (Nh x Ny) in 2D; pr = the phase rate S * kx * y
// of the x-transformed rows, [y][kx] (Ny x Nh) in both.
#include "fft_impl.cuh"

namespace dd {

DD_FFT_INSTANTIATE(extern, double)

// v * exp(+-i th) as numpy's complex product with (cos th, +-sin th), each
// product and sum rounded separately (no contraction).
__device__ __forceinline__ C<double> shear_rot(C<double> v, double th, bool inv) {
    double s, c;
    sincos(th, &s, &c);
    if (inv) s = -s;
    return mk<double>(__dsub_rn(__dmul_rn(v.x, c), __dmul_rn(v.y, s)), __dadd_rn(__dmul_rn(v.x, s), __dmul_rn(v.y, c)));
}

__device__ __forceinline__ bool shear_cut(double k, double cut) { return k >= cut || k <= -cut; }

// ------------------------------------------------------------ 3D passes
// Forward along y: W2[z][y][kxc] * exp(+i pr t) -> WS[ky][z][kxc], every ky.
struct OpYFwd3S {
    using V = double2;
    static constexpr const char* name = "y_fwd_shear";
    static constexpr int lmin = 8, lmax = 512;
    Geo3 g; CPtrs in; Ptrs out; const V* tw; const double* pr; double t;
    __device__ int npencil() const { return g.Kx; }
    __device__ int nstore() const { return g.Ny; }
    __device__ C<double> load(int fld, int z, int e, int kx) const {
        const C<double> v = ldc<double>((const V*)in.p[fld] + ((int64_t)z * g.Ny + e) * g.Kx + kx);
        return shear_rot(v, pr[(int64_t)e * g.Nh + kx] * t, false);
    }
    __device__ void store(int fld, int z, int e, int kx, const C<double>* col, int PS) const {
        stc<double>((V*)out.p[fld] + ((int64_t)e * g.Nz + z) * g.Kx + kx, col[e * PS]);
    }
};

// Forward along z: WS[ky][z][kxc] -> K[ky][kz][kx], zero where cut.
struct OpZFwd3S {
    using V = double2;
    static constexpr const char* name = "z_fwd_shear";
    static constexpr int lmin = 8, lmax = 512;
    Geo3 g; CPtrs in; Ptrs out; const V* tw; const double* kys; double cut;
    __device__ int npencil() const { return g.Kx; }
    __device__ int nstore() const { return g.Nz; }
    __device__ C<double> load(int fld, int ky, int e, int kx) const {
        return ldc<double>((const V*)in.p[fld] + ((int64_t)ky * g.Nz + e) * g.Kx + kx);
    }
    __device__ void store(int fld, int ky, int e, int kx, const C<double>* col, int PS) const {
        const bool keep = kept_full(e, g.Nz, g.Mz) && !shear_cut(kys[(int64_t)ky * g.Nh + kx], cut);
        const C<double> c = keep ? col[e * PS] : mk<double>(0., 0.);
        ((V*)out.p[fld])[((int64_t)ky * g.Nz + e) * g.Nh + kx] = make_double2(c.x, c.y);
    }
};

// Inverse along z: K[ky][kz][kx] (zero where cut) -> WS[ky][z][kxc].
struct OpZInv3S {
    using V = double2;
    static constexpr const char* name = "z_inv_shear";
    static constexpr int lmin = 8, lmax = 512;
    Geo3 g; CPtrs in; Ptrs out; const V* tw; const double* kys; double cut;
    __device__ int npencil() const { return g.Kx; }
    __device__ int nstore() const { return g.Nz; }
    __device__ C<double> load(int fld, int ky, int e, int kx) const {
        if (!kept_full(e, g.Nz, g.Mz) || shear_cut(kys[(int64_t)ky * g.Nh + kx], cut)) return mk<double>(0., 0.);
        return ldc<double>((const V*)in.p[fld] + ((int64_t)ky * g.Nz + e) * g.Nh + kx);
    }
    __device__ void store(int fld, int ky, int e, int kx, const C<double>* col, int PS) const {
        stc<double>((V*)out.p[fld] + ((int64_t)ky * g.Nz + e) * g.Kx + kx, col[e * PS]);
    }
};

// Inverse along y: WS[ky][z][kxc] -> W2[z][y][kxc] * exp(-i pr t).
struct OpYInv3S {
    using V = double2;
    static constexpr const char* name = "y_inv_shear";
    static constexpr int lmin = 8, lmax = 512;
    Geo3 g; CPtrs in; Ptrs out; const V* tw; const double* pr; double t;
    __device__ int npencil() const { return g.Kx; }
    __device__ int nstore() const { return g.Ny; }
    __device__ C<double> load(int fld, int z, int e, int kx) const {
        return ldc<double>((const V*)in.p[fld] + ((int64_t)e * g.Nz + z) * g.Kx + kx);
    }
    __device__ void store(int fld, int z, int e, int kx, const C<double>* col, int PS) const {
        stc<double>((V*)out.p[fld] + ((int64_t)z * g.Ny + e) * g.Kx + kx,
                    shear_rot(col[e * PS], pr[(int64_t)e * g.Nh + kx] * t, true));
    }
};

// ------------------------------------------------------------ 2D passes
// Forward along y: W[y][kxc] * exp(+i pr t) -> K[kx][ky], zero where cut.
struct OpYFwd2S {
    using V = double2;
    static constexpr const char* name = "y_fwd2d_shear";
    static constexpr int lmin = 8, lmax = 512;
    Geo2 g; CPtrs in; Ptrs out; const V* tw; const double* pr; double t; const double* kys; double cut;
    __device__ int npencil() const { return g.Kx; }
    __device__ int nstore() const { return g.Ny; }
    __device__ C<double> load(int fld, int, int e, int kx) const {
        const C<double> v = ldc<double>((const V*)in.p[fld] + (int64_t)e * g.Kx + kx);
        return shear_rot(v, pr[(int64_t)e * g.Nh + kx] * t, false);
    }
    __device__ void store(int fld, int, int e, int kx, const C<double>* col, int PS) const {
        const bool keep = !shear_cut(kys[(int64_t)kx * g.Ny + e], cut);
        const C<double> c = keep ? col[e * PS] : mk<double>(0., 0.);
        ((V*)out.p[fld])[(int64_t)kx * g.Ny + e] = make_double2(c.x, c.y);
    }
};

// Inverse along y: K[kx][ky] (zero where cut) -> W[y][kxc] * exp(-i pr t).
struct OpYInv2S {
    using V = double2;
    static constexpr const char* name = "y_inv2d_shear";
    static constexpr int lmin = 8, lmax = 512;
    Geo2 g; CPtrs in; Ptrs out; const V* tw; const double* pr; double t; const double* kys; double cut;
    __device__ int npencil() const { return g.Kx; }
    __device__ int nstore() const { return g.Ny; }
    __device__ C<double> load(int fld, int, int e, int kx) const {
        if (shear_cut(kys[(int64_t)kx * g.Ny + e], cut)) return mk<double>(0., 0.);
        return ldc<double>((const V*)in.p[fld] + (int64_t)kx * g.Ny + e);
    }
    __device__ void store(int fld, int, int e, int kx, const C<double>* col, int PS) const {
        stc<double>((V*)out.p[fld] + (int64_t)e * g.Kx + kx,
                    shear_rot(col[e * PS], pr[(int64_t)e * g.Nh + kx] * t, true));
    }
};

// ------------------------------------------------------ elementwise ops
static inline unsigned sh_grid(int64_t n) {
    int64_t b = (n + 255) / 256;
    if (b > 152 * 16) b = 152 * 16;
    return (unsigned)(b < 1 ? 1 : b);
}

// Columns kx >= Kx of a 3D k array (beyond the static x cut) set to zero.
__global__ void k_shear_zero_cols3(Geo3 g, Ptrs k) {
    double2* K = (double2*)k.p[blockIdx.y];
    const int64_t n = g.kcount();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if ((int)(i % g.Nh) >= g.Kx) K[i] = make_double2(0., 0.);
}

// In-place 2/3 rule with the sheared k_y (dealias_cy_{2d,3d}.pyx, sheared branch).
__global__ void k_shear_dealias(int ndim, Geo3 g3, Geo2 g2, const double* kys, double cut, Ptrs k) {
    double2* K = (double2*)k.p[blockIdx.y];
    const int64_t n = ndim == 3 ? g3.kcount() : g2.kcount();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        bool zero;
        if (ndim == 3) {
            const int kx = (int)(i % g3.Nh);
            const int64_t r = i / g3.Nh;
            const int kz = (int)(r % g3.Nz), ky = (int)(r / g3.Nz);
            zero = kx > g3.Mx || !kept_full(kz, g3.Nz, g3.Mz) || shear_cut(kys[(int64_t)ky * g3.Nh + kx], cut);
        } else {
            const int kx = (int)(i / g2.Ny);
            zero = kx > g2.Mx || shear_cut(kys[i], cut);
        }
        if (zero) K[i] = make_double2(0., 0.);
    }
}

// out = in * (1j * k) with k the sheared k_y table (broadcast over kz in 3D):
// numpy's complex product ((-b k), a k), as the static dd_deriv.
__global__ void k_shear_deriv_y(int ndim, Geo3 g3, Geo2 g2, const double* kys, const double2* in, double2* out) {
    const int64_t n = ndim == 3 ? g3.kcount() : g2.kcount();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double k;
        if (ndim == 3) {
            const int kx = (int)(i % g3.Nh);
            const int ky = (int)(i / ((int64_t)g3.Nh * g3.Nz));
            k = kys[(int64_t)ky * g3.Nh + kx];
        } else {
            k = kys[i];
        }
        const double2 a = in[i];
        out[i] = make_double2(-(a.y * k), a.x * k);
    }
}

// k-space: out = (in / r) * w (mode 0) or (in * r) * w (mode 1), r a real array
// of the same shape; (accumulate) out + that.  The division is numpy's
// complex-by-real one: a product with the rounded reciprocal 1 / r.  Every
// operation is rounded separately, as numpy's elementwise expressions are.
__global__ void k_kreal(int64_t n, const double2* in, const double* r, double w, int mode, int accumulate,
                        double2* out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 a = in[i];
        const double f = mode == 0 ? __ddiv_rn(1.0, r[i]) : r[i];
        double2 v = make_double2(__dmul_rn(a.x, f), __dmul_rn(a.y, f));
        if (w != 1.) v = make_double2(__dmul_rn(v.x, w), __dmul_rn(v.y, w));
        if (accumulate) { const double2 b = out[i]; v = make_double2(__dadd_rn(b.x, v.x), __dadd_rn(b.y, v.y)); }
        out[i] = v;
    }
}

// Grid points: out = (accumulate ? out : 0) + (a * b) * w (b == NULL: a * w),
// each operation rounded separately.
__global__ void k_xfma(int64_t n, const double* a, const double* b, double w, int accumulate, double* out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double v = b ? __dmul_rn(a[i], b[i]) : a[i];
        if (w != 1.) v = __dmul_rn(v, w);
        out[i] = accumulate ? __dadd_rn(out[i], v) : v;
    }
}

static int shear_check(const dd_plan* p, const double* kys, double cut) {
    DD_CHECK_ARG(p && kys, "shear transforms: null plan or k_y table");
    DD_CHECK_ARG(cut > 0., "shear transforms: the k_y cut must be positive");
    return DD_OK;
}

static size_t shear_ws_bytes(const dd_plan* p, int nf) {
    if (p->ndim == 3) return (size_t)nf * 2 * (size_t)p->g3.w2count() * sizeof(double2);
    return (size_t)nf * (size_t)p->g2.wcount() * sizeof(double2);
}

}  // namespace dd

using namespace dd;

extern "C" {

int dd_shear_workspace_size(const dd_plan* p, int nfield, size_t* bytes) {
    DD_CHECK_ARG(p && bytes, "dd_shear_workspace_size: null pointer");
    DD_CHECK_ARG(nfield >= 1 && nfield <= 8, "nfield must be in [1, 8]");
    *bytes = shear_ws_bytes(p, nfield);
    return DD_OK;
}

int dd_shear_r2c(const dd_plan* p, int nfield, const double* const* x, void* const* k, const double* kys, double cut,
                 const double* pr, double t, void* work, size_t wb, void* stream) {
    DD_TRY(shear_check(p, kys, cut));
    DD_CHECK_ARG(x && k && pr && work, "dd_shear_r2c: null pointer");
    DD_CHECK_ARG(nfield >= 1 && nfield <= 8, "nfield must be in [1, 8]");
    DD_CHECK_ARG(wb >= shear_ws_bytes(p, nfield), "workspace too small: %zu < %zu", wb, shear_ws_bytes(p, nfield));
    cudaStream_t st = (cudaStream_t)stream;
    CPtrs xin{};
    Ptrs ko{};
    for (int f = 0; f < nfield; f++) {
        DD_CHECK_ARG(x[f] && k[f], "dd_shear_r2c: null field pointer %d", f);
        xin.p[f] = x[f];
        ko.p[f] = k[f];
    }
    const double s = p->inv_n;
    if (p->ndim == 3) {
        const Geo3& g = p->g3;
        double2* W2 = (double2*)work;
        double2* WS = W2 + (size_t)nfield * g.w2count();
        Ptrs w2{}, ws{};
        CPtrs w2c{}, wsc{};
        for (int f = 0; f < nfield; f++) {
            w2.p[f] = W2 + f * g.w2count(); w2c.p[f] = w2.p[f];
            ws.p[f] = WS + f * g.w2count(); wsc.p[f] = ws.p[f];
        }
        const int nrows = g.Nz * g.Ny;
        OpXr2c3<double, double> a{nrows, g.Nx, g.Kx, s, xin, w2, TwSel<double>::x(p)};
        DD_TRY((launch_pass_len<double, false, true, true>(g.Nx, a, (nrows + 1) / 2, 1, nfield, st)));
        OpYFwd3S b{g, w2c, ws, TwSel<double>::y(p), pr, t};
        DD_TRY((launch_pass_len<double, false, false, false>(g.Ny, b, g.Kx, g.Nz, nfield, st)));
        OpZFwd3S c{g, wsc, ko, TwSel<double>::z(p), kys, cut};
        DD_TRY((launch_pass_len<double, false, false, false>(g.Nz, c, g.Kx, g.Ny, nfield, st)));
        if (g.Kx < g.Nh) {
            DD_KT("shear_zero_cols3", st,
                  k_shear_zero_cols3<<<dim3(sh_grid(g.kcount()), nfield), 256, 0, st>>>(g, ko));
            DD_LAUNCH_CHECK();
        }
    } else {
        const Geo2& g = p->g2;
        double2* W = (double2*)work;
        Ptrs w{};
        CPtrs wc{};
        for (int f = 0; f < nfield; f++) { w.p[f] = W + f * g.wcount(); wc.p[f] = w.p[f]; }
        OpXr2c3<double, double> a{g.Ny, g.Nx, g.Kx, s, xin, w, TwSel<double>::x(p)};
        DD_TRY((launch_pass_len<double, false, true, true>(g.Nx, a, (g.Ny + 1) / 2, 1, nfield, st)));
        OpYFwd2S b{g, wc, ko, TwSel<double>::y(p), pr, t, kys, cut};
        DD_TRY((launch_pass_len<double, false, false, true>(g.Ny, b, g.Kx, 1, nfield, st)));
        const int64_t nz = g.kcount() - (int64_t)g.Kx * g.Ny;
        if (nz > 0) {
            DD_KT("zero_nonkept2", st, k_zero_nonkept2<double><<<dim3(sh_grid(nz), nfield), 256, 0, st>>>(g, ko));
            DD_LAUNCH_CHECK();
        }
    }
    return DD_OK;
}

int dd_shear_c2r(const dd_plan* p, int nfield, const void* const* k, double* const* x, const double* kys, double cut,
                 const double* pr, double t, void* work, size_t wb, void* stream) {
    DD_TRY(shear_check(p, kys, cut));
    DD_CHECK_ARG(x && k && pr && work, "dd_shear_c2r: null pointer");
    DD_CHECK_ARG(nfield >= 1 && nfield <= 8, "nfield must be in [1, 8]");
    DD_CHECK_ARG(wb >= shear_ws_bytes(p, nfield), "workspace too small: %zu < %zu", wb, shear_ws_bytes(p, nfield));
    cudaStream_t st = (cudaStream_t)stream;
    CPtrs kin{};
    Ptrs xo{};
    for (int f = 0; f < nfield; f++) {
        DD_CHECK_ARG(x[f] && k[f], "dd_shear_c2r: null field pointer %d", f);
        kin.p[f] = k[f];
        xo.p[f] = x[f];
    }
    if (p->ndim == 3) {
        const Geo3& g = p->g3;
        double2* W2 = (double2*)work;
        double2* WS = W2 + (size_t)nfield * g.w2count();
        Ptrs w2{}, ws{};
        CPtrs w2c{}, wsc{};
        for (int f = 0; f < nfield; f++) {
            w2.p[f] = W2 + f * g.w2count(); w2c.p[f] = w2.p[f];
            ws.p[f] = WS + f * g.w2count(); wsc.p[f] = ws.p[f];
        }
        OpZInv3S a{g, kin, ws, TwSel<double>::z(p), kys, cut};
        DD_TRY((launch_pass_len<double, true, false, false>(g.Nz, a, g.Kx, g.Ny, nfield, st)));
        OpYInv3S b{g, wsc, w2, TwSel<double>::y(p), pr, t};
        DD_TRY((launch_pass_len<double, true, false, false>(g.Ny, b, g.Kx, g.Nz, nfield, st)));
        const int nrows = g.Nz * g.Ny;
        OpXc2r3<double, double> c{nrows, g.Nx, g.Kx, w2c, xo, TwSel<double>::x(p)};
        DD_TRY((launch_pass_len<double, true, true, true>(g.Nx, c, (nrows + 1) / 2, 1, nfield, st)));
    } else {
        const Geo2& g = p->g2;
        double2* W = (double2*)work;
        Ptrs w{};
        CPtrs wc{};
        for (int f = 0; f < nfield; f++) { w.p[f] = W + f * g.wcount(); wc.p[f] = w.p[f]; }
        OpYInv2S a{g, kin, w, TwSel<double>::y(p), pr, t, kys, cut};
        DD_TRY((launch_pass_len<double, true, true, false>(g.Ny, a, g.Kx, 1, nfield, st)));
        OpXc2r3<double, double> c{g.Ny, g.Nx, g.Kx, wc, xo, TwSel<double>::x(p)};
        DD_TRY((launch_pass_len<double, true, true, true>(g.Nx, c, (g.Ny + 1) / 2, 1, nfield, st)));
    }
    return DD_OK;
}

int dd_shear_dealias(const dd_plan* p, int nfield, void* const* k, const double* kys, double cut, void* stream) {
    DD_TRY(shear_check(p, kys, cut));
    DD_CHECK_ARG(k && nfield >= 1 && nfield <= DD_MAXF, "dd_shear_dealias: bad arguments");
    Ptrs kp{};
    for (int f = 0; f < nfield; f++) { DD_CHECK_ARG(k[f], "null field %d", f); kp.p[f] = k[f]; }
    const int64_t n = p->ndim == 3 ? p->g3.kcount() : p->g2.kcount();
    cudaStream_t st = (cudaStream_t)stream;
    DD_KT("shear_dealias", st,
          k_shear_dealias<<<dim3(sh_grid(n), nfield), 256, 0, st>>>(p->ndim, p->g3, p->g2, kys, cut, kp));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

int dd_shear_deriv_y(const dd_plan* p, const double* kys, const void* k_in, void* k_out, void* stream) {
    DD_CHECK_ARG(p && kys && k_in && k_out, "dd_shear_deriv_y: null pointer");
    const int64_t n = p->ndim == 3 ? p->g3.kcount() : p->g2.kcount();
    cudaStream_t st = (cudaStream_t)stream;
    DD_KT("shear_deriv_y", st,
          k_shear_deriv_y<<<sh_grid(n), 256, 0, st>>>(p->ndim, p->g3, p->g2, kys, (const double2*)k_in,
                                                       (double2*)k_out));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

int dd_kspace_real(int64_t n, const void* in, const double* r, double w, int mode, int accumulate, void* out,
                   void* stream) {
    DD_CHECK_ARG(in && r && out && n >= 0, "dd_kspace_real: bad arguments");
    DD_CHECK_ARG(mode == 0 || mode == 1, "dd_kspace_real: mode must be 0 (divide) or 1 (multiply)");
    if (n == 0) return DD_OK;
    cudaStream_t st = (cudaStream_t)stream;
    DD_KT("kspace_real", st,
          k_kreal<<<sh_grid(n), 256, 0, st>>>(n, (const double2*)in, r, w, mode, accumulate, (double2*)out));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

int dd_xspace_fma(int64_t n, const double* a, const double* b, double w, int accumulate, double* out, void* stream) {
    DD_CHECK_ARG(a && out && n >= 0, "dd_xspace_fma: bad arguments");
    if (n == 0) return DD_OK;
    cudaStream_t st = (cudaStream_t)stream;
    DD_KT("xspace_fma", st, k_xfma<<<sh_grid(n), 256, 0, st>>>(n, a, b, w, accumulate, out));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

}  // extern "C"
