// Pruned 2D/3D real transforms as templates over the arithmetic type;
// instantiated per precision in fft_<precision>.cu.
#pragma once
#include "launch_len.cuh"

namespace dd {

// -------------------------------------------------------- zero / dealias
template <typename KT>
__global__ void k_zero_nonkept3(Geo3 g, Ptrs k) {
    using KV = typename Vec2<KT>::type;
    KV* K = (KV*)pick_ptr<DD_MAXF>(k.p, (int)blockIdx.y);
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
    KV* K = (KV*)pick_ptr<DD_MAXF>(k.p, (int)blockIdx.y);
    const int64_t n0 = (int64_t)g.Kx * g.Ny, n = g.kcount();
    for (int64_t i = n0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        KV z; z.x = 0; z.y = 0; K[i] = z;
    }
}

static __global__ void k_dealias3(Geo3 g, double2* K) {
    const int64_t n = g.kcount();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int kx = (int)(i % g.Nh);
        const int64_t r = i / g.Nh;
        const int kz = (int)(r % g.Nz), ky = (int)(r / g.Nz);
        if (kx > g.Mx || !kept_full(ky, g.Ny, g.My) || !kept_full(kz, g.Nz, g.Mz)) K[i] = make_double2(0., 0.);
    }
}

static __global__ void k_dealias2(Geo2 g, double2* K) {
    const int64_t n = g.kcount();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int ky = (int)(i % g.Ny), kx = (int)(i / g.Ny);
        if (kx > g.Mx || !kept_full(ky, g.Ny, g.My)) K[i] = make_double2(0., 0.);
    }
}

static inline unsigned ew_grid(int64_t n) {
    int64_t b = (n + 255) / 256;
    if (b > 152 * 16) b = 152 * 16;
    return (unsigned)(b < 1 ? 1 : b);
}

// -------------------------------------------------------- transforms
template <typename T>
inline size_t ws_bytes(const dd_plan* pl, int nf) {
    if (pl->ndim == 3) return (size_t)nf * (pl->g3.w1count() + pl->g3.w2count()) * sizeof(C<T>);
    return (size_t)nf * pl->g2.wcount() * sizeof(C<T>);
}

// XT is the type of the grid-point values (double, or float beside float
// arithmetic: the values are the same, at half the bytes).
template <typename T, typename XT = double>
int fft_c2r(const dd_plan* pl, int nf, const void* const* k, XT* const* x, void* work, size_t wb,
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
        OpXc2r3<T, XT> c{nrows, g.Nx, g.Kx, w2c, xo, TwSel<T>::x(pl)};
        DD_TRY((launch_pass_len<T, true, true, true>(g.Nx, c, (nrows + 1) / 2, 1, nf, st)));
    } else {
        const Geo2& g = pl->g2;
        C<T>* W = (C<T>*)work;
        Ptrs w{}; CPtrs wc{};
        for (int f = 0; f < nf; f++) { w.p[f] = W + f * g.wcount(); wc.p[f] = w.p[f]; }
        OpYInv2<T, double> a{g, kin, w, TwSel<T>::y(pl)};
        DD_TRY((launch_pass_len<T, true, true, false>(g.Ny, a, g.Kx, 1, nf, st)));
        OpXc2r3<T, XT> c{g.Ny, g.Nx, g.Kx, wc, xo, TwSel<T>::x(pl)};
        DD_TRY((launch_pass_len<T, true, true, true>(g.Nx, c, (g.Ny + 1) / 2, 1, nf, st)));
    }
    return DD_OK;
}

// zero_nonkept = false leaves the entries outside the kept set unwritten (for
// internal callers that read kept modes only).
template <typename T, typename XT = double>
int fft_r2c(const dd_plan* pl, int nf, const XT* const* x, void* const* k, void* work, size_t wb,
            cudaStream_t st, bool zero_nonkept = true) {
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
        OpXr2c3<T, XT> a{nrows, g.Nx, g.Kx, s, xin, w2, TwSel<T>::x(pl)};
        DD_TRY((launch_pass_len<T, false, true, true>(g.Nx, a, (nrows + 1) / 2, 1, nf, st)));
        OpYFwd3<T> b{g, w2c, w1, TwSel<T>::y(pl)};
        DD_TRY((launch_pass_len<T, false, false, false>(g.Ny, b, g.Kx, g.Nz, nf, st)));
        OpZFwd3<T, double> c{g, w1c, ko, TwSel<T>::z(pl)};
        DD_TRY((launch_pass_len<T, false, false, false>(g.Nz, c, g.Kx, g.Ky, nf, st)));
        if (zero_nonkept) {
            DD_KT("zero_nonkept3", st, k_zero_nonkept3<double><<<dim3(ew_grid(g.kcount()), nf), 256, 0, st>>>(g, ko));
            DD_LAUNCH_CHECK();
        }
    } else {
        const Geo2& g = pl->g2;
        C<T>* W = (C<T>*)work;
        Ptrs w{}; CPtrs wc{};
        for (int f = 0; f < nf; f++) { w.p[f] = W + f * g.wcount(); wc.p[f] = w.p[f]; }
        OpXr2c3<T, XT> a{g.Ny, g.Nx, g.Kx, s, xin, w, TwSel<T>::x(pl)};
        DD_TRY((launch_pass_len<T, false, true, true>(g.Nx, a, (g.Ny + 1) / 2, 1, nf, st)));
        OpYFwd2<T, double> b{g, wc, ko, TwSel<T>::y(pl)};
        DD_TRY((launch_pass_len<T, false, false, true>(g.Ny, b, g.Kx, 1, nf, st)));
        const int64_t nz = g.kcount() - (int64_t)g.Kx * g.Ny;
        if (nz > 0 && zero_nonkept) {
            DD_KT("zero_nonkept2", st, k_zero_nonkept2<double><<<dim3(ew_grid(nz), nf), 256, 0, st>>>(g, ko));
            DD_LAUNCH_CHECK();
        }
    }
    return DD_OK;
}

#define DD_FFT_INSTANTIATE(EXT, T)                                                                       \
    EXT template int fft_c2r<T>(const dd_plan*, int, const void* const*, double* const*, void*, size_t, cudaStream_t); \
    EXT template int fft_r2c<T>(const dd_plan*, int, const double* const*, void* const*, void*, size_t, cudaStream_t, \
                                bool);
#define DD_FFT_INSTANTIATE_X(EXT, T, XT)                                                                 \
    EXT template int fft_c2r<T, XT>(const dd_plan*, int, const void* const*, XT* const*, void*, size_t,        \
                                    cudaStream_t);                                                          \
    EXT template int fft_r2c<T, XT>(const dd_plan*, int, const XT* const*, void* const*, void*, size_t,        \
                                    cudaStream_t, bool);

}  // namespace dd
