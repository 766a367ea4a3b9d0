#pragma once
// Fused 2D right-hand sides and RK2mid step for incompressible hydro and
// Boussinesq flows, batched over independent runs of one grid size.
//
//   hydro:       RHS(u) = P[u x w z]^, w = d_x u_y - d_y u_x          (physics.py:527-599)
//   Boussinesq:  RHS(u) = P[u x w z + g alpha T e_dir]^,
//                RHS(T) = -(u.grad T)^ - beta u_dir                      (physics.py:664-712)
// The rotational form of the momentum term equals the reference's advective
// form on the kept modes to roundoff (the difference is a gradient removed by
// the projection).  u.grad T is formed in x-space as u_x dT/dx + u_y dT/dy, the
// reference's XgradY order (physics.py:221-225).
//
// Passes (k-layout [kx][ky], x-layout [y][x]; run b of a batch is offset by a
// per-run stride):
//   1  Y^-1 per kx row (kept ky), with w (and grad T) formed while loading
//   2  X c2r -> pointwise products -> X r2c, scaled by 1/N   (k_x_prod)
//   3  Y forward, kept ky, into a compact [kxc][kyc] buffer
//   4  projection + buoyancy / stratification terms + RK2mid stage
#include "launch_len.cuh"
#include "xprod.cuh"
#include "etd.cuh"

namespace dd {

__device__ __forceinline__ double2 ideriv2(double2 a, double k) { return make_double2(-(a.y * k), a.x * k); }

enum { PHYS_HYDRO = 0, PHYS_BOUSS = 1 };

template <int PHYS> struct Phys2;
template <> struct Phys2<PHYS_HYDRO> { static constexpr int NF = 2, NI = 3, NO = 2; };
template <> struct Phys2<PHYS_BOUSS> { static constexpr int NF = 3, NI = 5, NO = 3; };
static_assert(Phys2<PHYS_BOUSS>::NI <= DD_MAXF, "too many transform fields for Ptrs");

// ------------------------------------------------------------------ pass 1
template <typename T, bool COMPACT, int PHYS>
struct OpYInvPhys2 {
    using V = typename Vec2<T>::type;
    static constexpr const char* name = PHYS == PHYS_HYDRO ? "y_inv_hydro2d" : "y_inv_bouss2d";
    static constexpr int lmin = 32, lmax = 512;
    Geo2 g; CPtrs st; int64_t st_rs; Ptrs out; int64_t w_rs; const V* tw;
    const double* kx; const double* ky;
    __device__ int npencil() const { return g.Kx; }
    __device__ int nstore() const { return g.Ny; }
    __device__ double2 get(int c, int run, int ix, int e) const {
        const double2* S = (const double2*)st.p[c] + run * st_rs;
        if (COMPACT) return S[(int64_t)ix * g.Ky + full_to_compact(e, g.Ny, g.Ky)];
        return S[(int64_t)ix * g.Ny + e];
    }
    __device__ C<T> load(int fld, int run, int e, int ix) const {
        if (!kept_full(e, g.Ny, g.My)) return zero<T>();
        double2 r;
        if (fld < 2) r = get(fld, run, ix, e);
        else if (fld == 2) {  // curlX, N == 2: X[1].deriv(x) - X[0].deriv(y)  (physics.py:400)
            const double2 a = ideriv2(get(1, run, ix, e), kx[ix]), b = ideriv2(get(0, run, ix, e), ky[e]);
            r = make_double2(a.x - b.x, a.y - b.y);
        } else if (fld == 3) r = ideriv2(get(2, run, ix, e), kx[ix]);
        else r = ideriv2(get(2, run, ix, e), ky[e]);
        return mk<T>((T)r.x, (T)r.y);
    }
    __device__ void store(int fld, int run, int e, int ix, const C<T>* col, int PS) const {
        stc<T>((V*)out.p[fld] + run * w_rs + (int64_t)e * g.Kx + ix, col[e * PS]);
    }
};

// ------------------------------------------------------------------ pass 2
template <typename T>
struct ProdHydro2 {
    static constexpr int NI = 3, NO = 2;
    static constexpr int lmin = 32, lmax = 512;
    __device__ void operator()(const T* in, T* out, int) const {
        out[0] = in[1] * in[2];       // u_y w
        out[1] = -(in[0] * in[2]);    // -u_x w
    }
};
template <typename T>
struct ProdBouss2 {
    static constexpr int NI = 5, NO = 3;
    static constexpr int lmin = 32, lmax = 512;
    __device__ void operator()(const T* in, T* out, int) const {
        out[0] = in[1] * in[2];
        out[1] = -(in[0] * in[2]);
        out[2] = in[0] * in[3] + in[1] * in[4];   // u_x dT/dx + u_y dT/dy
    }
};

// ------------------------------------------------------------------ pass 3
template <typename T>
struct OpYFwdCompact2 {
    using V = typename Vec2<T>::type;
    static constexpr const char* name = "y_fwd_compact2d";
    static constexpr int lmin = 32, lmax = 512;
    Geo2 g; CPtrs in; int64_t w_rs; Ptrs out; int64_t nc_rs; const V* tw;
    __device__ int npencil() const { return g.Kx; }
    __device__ int nstore() const { return g.Ny; }
    __device__ C<T> load(int fld, int run, int e, int ix) const {
        return ldc<T>((const V*)in.p[fld] + run * w_rs + (int64_t)e * g.Kx + ix);
    }
    __device__ void store(int fld, int run, int e, int ix, const C<T>* col, int PS) const {
        if (!kept_full(e, g.Ny, g.My)) return;
        const C<T> c = col[e * PS];
        ((double2*)out.p[fld])[run * nc_rs + (int64_t)ix * g.Ky + full_to_compact(e, g.Ny, g.Ky)] =
            make_double2((double)c.x, (double)c.y);
    }
};

// ------------------------------------------------------------ driver
struct Work2 {
    size_t w, kc;  // complex entries per (field, run): W = Ny*Kx, compact = Kx*Ky
    int nrun;
    char* base;
    template <typename T> C<T>* W(int f) const { return (C<T>*)base + (size_t)f * nrun * w; }
    static size_t up256(size_t b) { return (b + 255) & ~(size_t)255; }
    template <typename T> double2* NC(int f) const {
        return (double2*)((char*)base + up256(sizeof(C<T>) * 5 * nrun * w)) + (size_t)f * nrun * kc;
    }
    template <typename T> double2* K1(int f) const { return NC<T>(3) + (size_t)f * nrun * kc; }
    template <typename T> double2* YS(int f) const { return NC<T>(6) + (size_t)f * nrun * kc; }
    template <typename T> static size_t bytes(const Geo2& g, int nrun) {
        return up256(sizeof(C<T>) * 5 * (size_t)nrun * g.wcount()) + sizeof(double2) * 9 * (size_t)nrun * g.Kx * g.Ky;
    }
};

template <typename T, bool COMPACT, int PHYS>
int nonlinear2(const dd_plan* pl, const Work2& w, const void* const* st, int64_t st_rs, cudaStream_t s) {
    const Geo2& g = pl->g2;
    using PH = Phys2<PHYS>;
    CPtrs sin{}; Ptrs wo{}; CPtrs wi{}; Ptrs nc{};
    for (int c = 0; c < PH::NF; c++) sin.p[c] = st[c];
    for (int f = 0; f < PH::NI; f++) { wo.p[f] = w.W<T>(f); wi.p[f] = wo.p[f]; }
    for (int f = 0; f < PH::NO; f++) nc.p[f] = w.NC<T>(f);
    OpYInvPhys2<T, COMPACT, PHYS> a{g, sin, st_rs, wo, (int64_t)w.w, TwSel<T>::y(pl), pl->kx, pl->ky};
    DD_TRY((launch_pass_len<T, true, true, false>(g.Ny, a, g.Kx, w.nrun, PH::NI, s)));
    if (PHYS == PHYS_HYDRO) {
        DD_TRY((launch_x_prod_len<T>("x_prod_hydro2d", g.Nx, g.Ny, g.Kx, wi, wo, w.nrun, (int64_t)w.w, (int64_t)w.w,
                                     TwSel<T>::x(pl), (T)pl->inv_n, ProdHydro2<T>{}, s)));
    } else {
        DD_TRY((launch_x_prod_len<T>("x_prod_bouss2d", g.Nx, g.Ny, g.Kx, wi, wo, w.nrun, (int64_t)w.w, (int64_t)w.w,
                                     TwSel<T>::x(pl), (T)pl->inv_n, ProdBouss2<T>{}, s)));
    }
    OpYFwdCompact2<T> c{g, wi, (int64_t)w.w, nc, (int64_t)w.kc, TwSel<T>::y(pl)};
    DD_TRY((launch_pass_len<T, false, false, true>(g.Ny, c, g.Kx, w.nrun, PH::NO, s)));
    return DD_OK;
}

#define DD_RHS2D_INSTANTIATE(EXT, T)                                                                     \
    EXT template int nonlinear2<T, false, PHYS_HYDRO>(const dd_plan*, const Work2&, const void* const*, int64_t, \
                                                      cudaStream_t);                                         \
    EXT template int nonlinear2<T, true, PHYS_HYDRO>(const dd_plan*, const Work2&, const void* const*, int64_t,  \
                                                     cudaStream_t);                                          \
    EXT template int nonlinear2<T, false, PHYS_BOUSS>(const dd_plan*, const Work2&, const void* const*, int64_t, \
                                                      cudaStream_t);                                         \
    EXT template int nonlinear2<T, true, PHYS_BOUSS>(const dd_plan*, const Work2&, const void* const*, int64_t,  \
                                                     cudaStream_t);

}  // namespace dd
