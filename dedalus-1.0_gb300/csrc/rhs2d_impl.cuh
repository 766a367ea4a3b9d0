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

// PHYS_*_DIV: the same physics with the nonlinear terms in divergence form,
// valid for a solenoidal u: -(u.grad)u = -d_j (u_i u_j) and u.grad T =
// div(u T).  Basdevant's trick leaves two momentum products (u_x^2 - u_y^2,
// u_x u_y; the dropped u_y^2 I is a gradient the projection removes) and two
// temperature fluxes (u_x T, u_y T): 2 or 3 inverse transforms (u, T) and 2 or
// 4 forward ones per RHS instead of 3 + 2 (hydro) and 5 + 3 (Boussinesq).
enum { PHYS_HYDRO = 0, PHYS_BOUSS = 1, PHYS_HYDRO_DIV = 2, PHYS_BOUSS_DIV = 3 };
__host__ __device__ constexpr bool p2_div(int ph) { return ph == PHYS_HYDRO_DIV || ph == PHYS_BOUSS_DIV; }
__host__ __device__ constexpr bool p2_bouss(int ph) { return ph == PHYS_BOUSS || ph == PHYS_BOUSS_DIV; }

template <int PHYS> struct Phys2;
template <> struct Phys2<PHYS_HYDRO> { static constexpr int NF = 2, NI = 3, NO = 2; };
template <> struct Phys2<PHYS_BOUSS> { static constexpr int NF = 3, NI = 5, NO = 3; };
template <> struct Phys2<PHYS_HYDRO_DIV> { static constexpr int NF = 2, NI = 2, NO = 2; };
template <> struct Phys2<PHYS_BOUSS_DIV> { static constexpr int NF = 3, NI = 3, NO = 4; };
static_assert(Phys2<PHYS_BOUSS>::NI <= DD_MAXF, "too many transform fields for Ptrs");

// ------------------------------------------------------------------ pass 1
// SST: the type of a compact input state (stage states of the low-storage
// FP32 step are complex64); full-layout inputs are complex128.
template <typename T, bool COMPACT, int PHYS, typename SST = double>
struct OpYInvPhys2 {
    using V = typename Vec2<T>::type;
    static constexpr const char* name = PHYS == PHYS_HYDRO ? "y_inv_hydro2d" : PHYS == PHYS_BOUSS ? "y_inv_bouss2d"
                                        : PHYS == PHYS_HYDRO_DIV ? "y_inv_hydro2d_div" : "y_inv_bouss2d_div";
    static constexpr int lmin = 32, lmax = 512;
    Geo2 g; CPtrs st; int64_t st_rs; Ptrs out; int64_t w_rs; const V* tw;
    const double* kx; const double* ky;
    __device__ int kept() const { return g.My; }
    __device__ int npencil() const { return g.Kx; }
    __device__ int nstore() const { return g.Ny; }
    __device__ double2 get(int c, int run, int ix, int e) const {
        const double2* S = (const double2*)st.p[c] + run * st_rs;
        if (COMPACT) return S[(int64_t)ix * g.Ky + full_to_compact(e, g.Ny, g.Ky)];
        return S[(int64_t)ix * g.Ny + e];
    }
    __device__ C<T> load(int fld, int run, int e, int ix) const {
        if (!kept_full(e, g.Ny, g.My)) return zero<T>();
        if constexpr (COMPACT && std::is_same<SST, float>::value) {
            static_assert(p2_div(PHYS), "complex64 stage states are for the divergence forms");
            const float2* S = (const float2*)st.p[fld] + run * st_rs;
            const float2 v = S[(int64_t)ix * g.Ky + full_to_compact(e, g.Ny, g.Ky)];
            return mk<T>((T)v.x, (T)v.y);
        }
        double2 r;
        if (p2_div(PHYS) || fld < 2) r = get(fld, run, ix, e);   // divergence forms: the state itself
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

template <typename T>
struct ProdHydroDiv2 {
    static constexpr int NI = 2, NO = 2;
    static constexpr int lmin = 32, lmax = 512;
    __device__ void operator()(const T* in, T* out, int) const {
        out[0] = in[0] * in[0] - in[1] * in[1];   // u_x^2 - u_y^2
        out[1] = in[0] * in[1];                   // u_x u_y
    }
};
template <typename T>
struct ProdBoussDiv2 {
    static constexpr int NI = 3, NO = 4;
    static constexpr int lmin = 32, lmax = 512;
    __device__ void operator()(const T* in, T* out, int) const {
        out[0] = in[0] * in[0] - in[1] * in[1];
        out[1] = in[0] * in[1];
        out[2] = in[0] * in[2];                   // u_x T
        out[3] = in[1] * in[2];                   // u_y T
    }
};

// ------------------------------------------------------------------ pass 3
// ST: the type of the compact products (complex128, or complex64 on the
// low-storage FP32 step).
template <typename T, typename ST = double>
struct OpYFwdCompact2 {
    using V = typename Vec2<T>::type;
    static constexpr const char* name = "y_fwd_compact2d";
    static constexpr int lmin = 32, lmax = 512;
    Geo2 g; CPtrs in; int64_t w_rs; Ptrs out; int64_t nc_rs; const V* tw;
    __device__ int kept() const { return g.My; }
    __device__ int npencil() const { return g.Kx; }
    __device__ int nstore() const { return g.Ny; }
    __device__ C<T> load(int fld, int run, int e, int ix) const {
        return ldc<T>((const V*)in.p[fld] + run * w_rs + (int64_t)e * g.Kx + ix);
    }
    __device__ void store(int fld, int run, int e, int ix, const C<T>* col, int PS) const {
        if (!kept_full(e, g.Ny, g.My)) return;
        const C<T> c = col[e * PS];
        const int64_t o = run * nc_rs + (int64_t)ix * g.Ky + full_to_compact(e, g.Ny, g.Ky);
        if constexpr (std::is_same<ST, float>::value) ((float2*)out.p[fld])[o] = make_float2((float)c.x, (float)c.y);
        else ((double2*)out.p[fld])[o] = make_double2((double)c.x, (double)c.y);
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
    // compact regions: products NC (up to 4), then K1 (3) and YS (3)
    template <typename T> double2* K1(int f) const { return NC<T>(4) + (size_t)f * nrun * kc; }
    template <typename T> double2* YS(int f) const { return NC<T>(7) + (size_t)f * nrun * kc; }
    // the same ten compact regions as complex64 (low-storage FP32 step), in the
    // first half of the complex128 space
    float2* NCf(int f) const { return (float2*)NC<float>(0) + (size_t)f * nrun * kc; }
    float2* K1f(int f) const { return NCf(4) + (size_t)f * nrun * kc; }
    float2* YSf(int f) const { return NCf(7) + (size_t)f * nrun * kc; }
    template <typename T> static size_t bytes(const Geo2& g, int nrun) {
        return up256(sizeof(C<T>) * 5 * (size_t)nrun * g.wcount()) + sizeof(double2) * 10 * (size_t)nrun * g.Kx * g.Ky;
    }
};

// ST = float (FP32 transforms, divergence forms): complex64 products out of
// pass 3 and, with COMPACT, complex64 stage states into pass 1.
template <typename T, bool COMPACT, int PHYS, typename ST = double>
int nonlinear2(const dd_plan* pl, const Work2& w, const void* const* st, int64_t st_rs, cudaStream_t s) {
    const Geo2& g = pl->g2;
    using PH = Phys2<PHYS>;
    CPtrs sin{}; Ptrs wo{}; CPtrs wi{}; Ptrs nc{};
    for (int c = 0; c < PH::NF; c++) sin.p[c] = st[c];
    // W buffers: the inverse-transformed fields, then (in place, row by row) the
    // products; the divergence form has more products (4) than inputs (3)
    constexpr int NW = PH::NI > PH::NO ? PH::NI : PH::NO;
    static_assert(NW <= 5, "Work2 holds 5 transform buffers");
    for (int f = 0; f < NW; f++) { wo.p[f] = w.W<T>(f); wi.p[f] = wo.p[f]; }
    for (int f = 0; f < PH::NO; f++) {
        if constexpr (std::is_same<ST, float>::value) nc.p[f] = w.NCf(f);
        else nc.p[f] = w.NC<T>(f);
    }
    // one run of a 64- or 128-point grid: small tiles, so that the y passes
    // have enough blocks (the default 32-pencil tiles give 2 per field)
    // (a tuned tile variant, set on the plan, takes precedence)
    const int yv = pl->sched_y2d;
    const bool small = yv == 0 && w.nrun == 1 && (g.Ny == 64 || g.Ny == 128);
    OpYInvPhys2<T, COMPACT, PHYS, ST> a{g, sin, st_rs, wo, (int64_t)w.w, TwSel<T>::y(pl), pl->kx, pl->ky};
    int rc = 1;
    if (yv) rc = launch_pass_variant<T, true, true, false>(g.Ny, yv, a, g.Kx, w.nrun, PH::NI, s);
    if (rc == 1 && small) rc = launch_pass_small<T, true, true, false>(g.Ny, a, g.Kx, w.nrun, PH::NI, s);
    if (rc == 1) rc = launch_pass_len<T, true, true, false>(g.Ny, a, g.Kx, w.nrun, PH::NI, s);
    DD_TRY(rc);
    if constexpr (PHYS == PHYS_HYDRO_DIV) {
        DD_TRY((launch_x_prod_len<T>("x_div_hydro2d", g.Nx, g.Ny, g.Kx, wi, wo, w.nrun, (int64_t)w.w, (int64_t)w.w,
                                     TwSel<T>::x(pl), (T)pl->inv_n, ProdHydroDiv2<T>{}, s)));
    } else if constexpr (PHYS == PHYS_BOUSS_DIV) {
        DD_TRY((launch_x_prod_len<T>("x_div_bouss2d", g.Nx, g.Ny, g.Kx, wi, wo, w.nrun, (int64_t)w.w, (int64_t)w.w,
                                     TwSel<T>::x(pl), (T)pl->inv_n, ProdBoussDiv2<T>{}, s)));
    } else if constexpr (PHYS == PHYS_HYDRO) {
        DD_TRY((launch_x_prod_len<T>("x_prod_hydro2d", g.Nx, g.Ny, g.Kx, wi, wo, w.nrun, (int64_t)w.w, (int64_t)w.w,
                                     TwSel<T>::x(pl), (T)pl->inv_n, ProdHydro2<T>{}, s)));
    } else {
        DD_TRY((launch_x_prod_len<T>("x_prod_bouss2d", g.Nx, g.Ny, g.Kx, wi, wo, w.nrun, (int64_t)w.w, (int64_t)w.w,
                                     TwSel<T>::x(pl), (T)pl->inv_n, ProdBouss2<T>{}, s)));
    }
    OpYFwdCompact2<T, ST> c{g, wi, (int64_t)w.w, nc, (int64_t)w.kc, TwSel<T>::y(pl)};
    rc = 1;
    if (yv) rc = launch_pass_variant<T, false, false, true>(g.Ny, yv, c, g.Kx, w.nrun, PH::NO, s);
    if (rc == 1 && small) rc = launch_pass_small<T, false, false, true>(g.Ny, c, g.Kx, w.nrun, PH::NO, s);
    if (rc == 1) rc = launch_pass_len<T, false, false, true>(g.Ny, c, g.Kx, w.nrun, PH::NO, s);
    DD_TRY(rc);
    return DD_OK;
}

#define DD_RHS2D_INSTANTIATE_PH(EXT, T, PH)                                                            \
    EXT template int nonlinear2<T, false, PH>(const dd_plan*, const Work2&, const void* const*, int64_t,    \
                                              cudaStream_t);                                            \
    EXT template int nonlinear2<T, true, PH>(const dd_plan*, const Work2&, const void* const*, int64_t,     \
                                             cudaStream_t);
// hydro forms and Boussinesq forms, each compiled in its own translation unit
#define DD_RHS2D_INSTANTIATE_A(EXT, T) DD_RHS2D_INSTANTIATE_PH(EXT, T, PHYS_HYDRO) \
    DD_RHS2D_INSTANTIATE_PH(EXT, T, PHYS_HYDRO_DIV)
#define DD_RHS2D_INSTANTIATE_B(EXT, T) DD_RHS2D_INSTANTIATE_PH(EXT, T, PHYS_BOUSS) \
    DD_RHS2D_INSTANTIATE_PH(EXT, T, PHYS_BOUSS_DIV)
#define DD_RHS2D_INSTANTIATE(EXT, T) DD_RHS2D_INSTANTIATE_A(EXT, T) DD_RHS2D_INSTANTIATE_B(EXT, T)
// the low-storage FP32 step (divergence forms, complex64 products and stage states)
#define DD_RHS2D_INSTANTIATE_LO(EXT, PH)                                                                \
    EXT template int nonlinear2<float, false, PH, float>(const dd_plan*, const Work2&, const void* const*,  \
                                                         int64_t, cudaStream_t);                        \
    EXT template int nonlinear2<float, true, PH, float>(const dd_plan*, const Work2&, const void* const*,   \
                                                        int64_t, cudaStream_t);

}  // namespace dd
