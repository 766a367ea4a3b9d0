#pragma once
// Fused 3D right-hand sides and RK4 step for incompressible hydro and MHD.
//
//   hydro: RHS(u) = P[u x w]^, w = curl u                  (physics.py:527-599)
//          or, for a solenoidal state, P[-i k_j T_ij] (ProdDiv3 below)
//   MHD:   RHS(u) = P[u x w + (J x B) / (4 pi rho0)]^, J = curl B,
//          RHS(B) = curl (u x B)^                            (physics.py:770-819)
//          or, for solenoidal u and B, RHS(u) = P[-i k_j M_ij] (ProdMHDDiv3)
// The rotational form u x w equals the reference's -(u.grad)u on the kept
// modes to roundoff: the difference is a gradient, which the projection
// removes, and products of dealiased fields alias only onto non-kept modes.
// The Lorentz term is added in x-space before the forward transform (one
// transform per component instead of two; equal by linearity).
//
// Passes (all pruned to the kept modes; T = FP64 or FP32 arithmetic):
//   1  Z^-1 of each vector field and its curl (formed while loading); the
//      divergence forms load the state fields only
//   2  Y^-1
//   3  X c2r -> pointwise products -> X r2c, scaled by 1/N   (k_x_prod)
//   4  Y forward, kept ky only
//   5  Z forward, kept kz only, into a compact [kyc][kzc][kx] buffer
//   6  (divergence forms: -i k_j T_ij from the product spectra) projection
//      (physics.py:588-599, laplace_solve 407-416) and, for B, the spectral
//      curl (physics.py:394-396), fused with the RK4 stage.
#include "launch_len.cuh"
#include "xprod.cuh"
#include "etd.cuh"

namespace dd {

// P3_HYDRO_DIV: hydro with the nonlinear term in divergence form, valid for a
// solenoidal state (below).  NI = transform buffers, NINV = inverse-transformed
// fields, NO = forward-transformed products.
enum { P3_HYDRO = 0, P3_MHD = 1, P3_HYDRO_DIV = 2, P3_MHD_DIV = 3 };
template <int PH> struct Phys3;
template <> struct Phys3<P3_HYDRO>     { static constexpr int NG = 1, NF = 3, NI = 6, NINV = 6, NO = 3; };
template <> struct Phys3<P3_MHD>       { static constexpr int NG = 2, NF = 6, NI = 12, NINV = 12, NO = 6; };
template <> struct Phys3<P3_HYDRO_DIV> { static constexpr int NG = 1, NF = 3, NI = 5, NINV = 3, NO = 5; };
template <> struct Phys3<P3_MHD_DIV>   { static constexpr int NG = 2, NF = 6, NI = 8, NINV = 6, NO = 8; };
__host__ __device__ constexpr bool p3_curl_inputs(int ph) { return ph == P3_HYDRO || ph == P3_MHD; }
__host__ __device__ constexpr bool p3_mhd(int ph) { return ph == P3_MHD || ph == P3_MHD_DIV; }
static_assert(Phys3<P3_MHD>::NI <= DD_MAXF, "too many transform fields for Ptrs");

// a * (1j * k) as numpy computes it (representations.py:423)
__device__ __forceinline__ double2 ideriv(double2 a, double k) { return make_double2(-(a.y * k), a.x * k); }

// ------------------------------------------------------------------ pass 1
// Field f: group g = f / 6 (vector field g of the state), j = f % 6:
// j < 3 -> component j; j >= 3 -> component j - 3 of its curl (curlX,
// physics.py:394-396: (d_y X_z - d_z X_y, d_z X_x - d_x X_z, d_x X_y - d_y X_x)).
// The state is read from the full reference layout [ky][kz][kx] or from the
// compact kept layout [kyc][kzc][kx] used for RK stage states.
// ST: element type of a compact state (double; float for the FP32 step's
// stage states).  The full-layout state is always complex128.
template <typename T, bool COMPACT, int NG, bool CURL = true, typename ST = double>
struct OpZInvCurl3 {
    using V = typename Vec2<T>::type;
    static constexpr const char* name = NG == 1 ? "z_inv_curl" : (CURL ? "z_inv_curl_mhd" : "z_inv_mhd");
    static constexpr int lmin = 16, lmax = 512;
    Geo3 g; CPtrs u; Ptrs out; const V* tw;
    const double* kx; const double* ky; const double* kz;
    __device__ int kept() const { return g.Mz; }
    __device__ int npencil() const { return g.Kx; }
    __device__ int nstore() const { return g.Nz; }
    __device__ double2 get(int c, int kyc, int ky_i, int e, int ix) const {
        if (COMPACT) {
            using SV = typename Vec2<ST>::type;
            const SV v = ((const SV*)u.p[c])[((int64_t)kyc * g.Kz + full_to_compact(e, g.Nz, g.Kz)) * g.Kx + ix];
            return make_double2((double)v.x, (double)v.y);
        }
        return ((const double2*)u.p[c])[((int64_t)ky_i * g.Nz + e) * g.Nh + ix];
    }
    __device__ C<T> load(int fld, int kyc, int e, int ix) const {
        if (!kept_full(e, g.Nz, g.Mz)) return zero<T>();
        const int ky_i = compact_to_full(kyc, g.Ny, g.Ky);
        if constexpr (!CURL) {     // state components only (fld = component)
            const double2 v = get(fld, kyc, ky_i, e, ix);
            return mk<T>((T)v.x, (T)v.y);
        }
        const int grp = fld / 6, j = fld % 6, c0 = 3 * grp;
        double2 r;
        if (j < 3) {
            r = get(c0 + j, kyc, ky_i, e, ix);
        } else {
            const double kxv = kx[ix], kyv = ky[ky_i], kzv = kz[e];
            double2 a, b;
            if (j == 3) { a = ideriv(get(c0 + 2, kyc, ky_i, e, ix), kyv); b = ideriv(get(c0 + 1, kyc, ky_i, e, ix), kzv); }
            else if (j == 4) { a = ideriv(get(c0 + 0, kyc, ky_i, e, ix), kzv); b = ideriv(get(c0 + 2, kyc, ky_i, e, ix), kxv); }
            else { a = ideriv(get(c0 + 1, kyc, ky_i, e, ix), kxv); b = ideriv(get(c0 + 0, kyc, ky_i, e, ix), kyv); }
            r = make_double2(a.x - b.x, a.y - b.y);
        }
        return mk<T>((T)r.x, (T)r.y);
    }
    __device__ void store(int fld, int kyc, int e, int ix, const C<T>* col, int PS) const {
        stc<T>((V*)out.p[fld] + ((int64_t)kyc * g.Nz + e) * g.Kx + ix, col[e * PS]);
    }
};

// ------------------------------------------------------------------ pass 3
template <typename T>
struct ProdHydro3 {
    static constexpr int NI = 6, NO = 3;
    static constexpr int lmin = 16, lmax = 512;
    __device__ void operator()(const T* in, T* out, int) const {
        const T ux = in[0], uy = in[1], uz = in[2], wx = in[3], wy = in[4], wz = in[5];
        out[0] = uy * wz - uz * wy;
        out[1] = uz * wx - ux * wz;
        out[2] = ux * wy - uy * wx;
    }
};

// in: u, w, B, J;  out: u x w + (J x B) / (4 pi rho0), u x B  (physics.py:795-815)
template <typename T>
struct ProdMHD3 {
    static constexpr int NI = 12, NO = 6;
    static constexpr int lmin = 16, lmax = 512;
    T inv_fpr;
    __device__ void operator()(const T* in, T* out, int) const {
        const T ux = in[0], uy = in[1], uz = in[2], wx = in[3], wy = in[4], wz = in[5];
        const T bx = in[6], by = in[7], bz = in[8], jx = in[9], jy = in[10], jz = in[11];
        out[0] = (uy * wz - uz * wy) + (jy * bz - jz * by) * inv_fpr;
        out[1] = (uz * wx - ux * wz) + (jz * bx - jx * bz) * inv_fpr;
        out[2] = (ux * wy - uy * wx) + (jx * by - jy * bx) * inv_fpr;
        out[3] = uy * bz - uz * by;
        out[4] = uz * bx - ux * bz;
        out[5] = ux * by - uy * bx;
    }
};

// Divergence form (Basdevant's five products): for a solenoidal u,
// -(u.grad)u = -d_j (u_i u_j) = -d_j T_ij - grad(u_z u_z) with T = u u^T - u_z^2 I,
// whose diagonal (xx - zz, yy - zz, 0) leaves five independent entries.  The
// gradient is removed by the projection, so P[-i k_j T_ij] is the reference's
// RHS whenever div u = 0: 3 inverse and 5 forward transforms per RHS instead of
// 6 + 3.  out: xx - zz, yy - zz, xy, xz, yz.
template <typename T>
struct ProdDiv3 {
    static constexpr int NI = 3, NO = 5;
    static constexpr int lmin = 16, lmax = 512;
    __device__ void operator()(const T* in, T* out, int) const {
        const T ux = in[0], uy = in[1], uz = in[2];
        const T zz = uz * uz;
        out[0] = ux * ux - zz;
        out[1] = uy * uy - zz;
        out[2] = ux * uy;
        out[3] = ux * uz;
        out[4] = uy * uz;
    }
};

// MHD in divergence form, for solenoidal u and B: the momentum products
// M = u u^T - B B^T / (4 pi rho0) (J x B = (B.grad)B - grad(B^2/2) and
// (B.grad)B = d_j(B_i B_j) when div B = 0) in Basdevant's five entries, and the
// induction products u x B (its curl needs no divergence assumption).
// in: u, B;  out: Mxx - Mzz, Myy - Mzz, Mxy, Mxz, Myz, (u x B)_x, _y, _z.
template <typename T>
struct ProdMHDDiv3 {
    static constexpr int NI = 6, NO = 8;
    static constexpr int lmin = 16, lmax = 512;
    T inv_fpr;
    __device__ void operator()(const T* in, T* out, int) const {
        const T ux = in[0], uy = in[1], uz = in[2], bx = in[3], by = in[4], bz = in[5];
        const T mzz = uz * uz - bz * bz * inv_fpr;
        out[0] = (ux * ux - bx * bx * inv_fpr) - mzz;
        out[1] = (uy * uy - by * by * inv_fpr) - mzz;
        out[2] = ux * uy - bx * by * inv_fpr;
        out[3] = ux * uz - bx * bz * inv_fpr;
        out[4] = uy * uz - by * bz * inv_fpr;
        out[5] = uy * bz - uz * by;
        out[6] = uz * bx - ux * bz;
        out[7] = ux * by - uy * bx;
    }
};

// ------------------------------------------------------------------ pass 5
// ST: element type of the compact products (double; float for the FP32 step).
template <typename T, typename ST = double>
struct OpZFwdCompact3 {
    using V = typename Vec2<T>::type;
    using SV = typename Vec2<ST>::type;
    static constexpr const char* name = "z_fwd_compact";
    static constexpr int lmin = 16, lmax = 512;
    Geo3 g; CPtrs in; Ptrs out; const V* tw;
    __device__ int kept() const { return g.Mz; }
    __device__ int npencil() const { return g.Kx; }
    __device__ int nstore() const { return g.Nz; }
    __device__ C<T> load(int fld, int kyc, int e, int kx) const {
        return ldc<T>((const V*)in.p[fld] + ((int64_t)kyc * g.Nz + e) * g.Kx + kx);
    }
    __device__ void store(int fld, int kyc, int e, int kx, const C<T>* col, int PS) const {
        if (!kept_full(e, g.Nz, g.Mz)) return;
        const C<T> c = col[e * PS];
        SV v; v.x = (ST)c.x; v.y = (ST)c.y;
        ((SV*)out.p[fld])[((int64_t)kyc * g.Kz + full_to_compact(e, g.Nz, g.Kz)) * g.Kx + kx] = v;
    }
};

// ------------------------------------------------------------ drivers
// workspace: W1 (NI fields), W2 (NI), NC (NO, complex128), then for the RK4
// step tot (NF) and the stage state (NF), both compact complex128.
struct Work3 {
    size_t w1, w2, kc;
    int ni, no, nf;
    char* base;
    template <typename T> C<T>* W1(int f) const { return (C<T>*)base + f * w1; }
    template <typename T> C<T>* W2(int f) const { return (C<T>*)base + ni * w1 + f * w2; }
    // transform intermediates first, then the complex128 regions from a
    // 256-byte boundary
    static size_t up256(size_t b) { return (b + 255) & ~(size_t)255; }
    template <typename T> double2* NC(int f) const {
        return (double2*)((char*)base + up256(sizeof(C<T>) * ni * (w1 + w2))) + f * kc;
    }
    template <typename T> double2* TOT(int f) const { return NC<T>(no) + f * kc; }
    template <typename T> double2* YS(int f) const { return NC<T>(no + nf) + f * kc; }
    template <typename T> static size_t bytes(const Geo3& g, int ni, int no, int nf, bool step) {
        const size_t kc = (size_t)g.Ky * g.Kz * g.Kx;
        return up256(sizeof(C<T>) * ni * (size_t)(g.w1count() + g.w2count())) +
               sizeof(double2) * kc * (no + (step ? 2 * nf : 0));
    }
};

template <int PH>
static Work3 make_work(const Geo3& g, void* base) {
    using P = Phys3<PH>;
    return Work3{(size_t)g.w1count(), (size_t)g.w2count(), (size_t)g.Ky * g.Kz * g.Kx, P::NI, P::NO, P::NF,
                 (char*)base};
}

// ST = float (FP32 transforms only): compact stage states are read and the
// compact products written as complex64 (the FP32 step's low-storage stages).
template <typename T, bool COMPACT, int PH, typename ST = double>
int nonlinear3(const dd_plan* pl, const void* const* u, double inv_fpr, const Work3& w, cudaStream_t st) {
    using P = Phys3<PH>;
    const Geo3& g = pl->g3;
    CPtrs uin{}; Ptrs w1{}, w2{}, nc{}; CPtrs w1c{}, w2c{};
    static_assert(P::NI >= P::NO && P::NI >= P::NINV, "transform buffers must hold inputs and products");
    for (int c = 0; c < P::NF; c++) uin.p[c] = u[c];
    for (int c = 0; c < P::NO; c++) nc.p[c] = w.NC<T>(c);
    for (int f = 0; f < P::NI; f++) {
        w1.p[f] = w.W1<T>(f); w1c.p[f] = w1.p[f];
        w2.p[f] = w.W2<T>(f); w2c.p[f] = w2.p[f];
    }
    OpZInvCurl3<T, COMPACT, P::NG, p3_curl_inputs(PH), ST> a{g, uin, w1, TwSel<T>::z(pl), pl->kx, pl->ky, pl->kz};
    DD_TRY((launch_pass_len<T, true, false, false>(g.Nz, a, g.Kx, g.Ky, P::NINV, st)));
    OpYInv3<T> b{g, w1c, w2, TwSel<T>::y(pl)};
    DD_TRY((launch_pass_len<T, true, false, false>(g.Ny, b, g.Kx, g.Nz, P::NINV, st)));
    // products overwrite fields 0..NO-1 of W2 row by row (each block reads its rows first)
    if constexpr (PH == P3_HYDRO_DIV) {
        DD_TRY((launch_x_prod_len<T>("x_div", g.Nx, g.Nz * g.Ny, g.Kx, w2c, w2, 1, 0, 0, TwSel<T>::x(pl),
                                     (T)pl->inv_n, ProdDiv3<T>{}, st)));
    } else if constexpr (PH == P3_MHD_DIV) {
        DD_TRY((launch_x_prod_len<T>("x_div_mhd", g.Nx, g.Nz * g.Ny, g.Kx, w2c, w2, 1, 0, 0, TwSel<T>::x(pl),
                                     (T)pl->inv_n, ProdMHDDiv3<T>{(T)inv_fpr}, st)));
    } else if constexpr (PH == P3_HYDRO) {
        DD_TRY((launch_x_prod_len<T>("x_cross", g.Nx, g.Nz * g.Ny, g.Kx, w2c, w2, 1, 0, 0, TwSel<T>::x(pl),
                                     (T)pl->inv_n, ProdHydro3<T>{}, st)));
    } else {
        DD_TRY((launch_x_prod_len<T>("x_cross_mhd", g.Nx, g.Nz * g.Ny, g.Kx, w2c, w2, 1, 0, 0, TwSel<T>::x(pl),
                                     (T)pl->inv_n, ProdMHD3<T>{(T)inv_fpr}, st)));
    }
    OpYFwd3<T> d{g, w2c, w1, TwSel<T>::y(pl)};
    DD_TRY((launch_pass_len<T, false, false, false>(g.Ny, d, g.Kx, g.Nz, P::NO, st)));
    OpZFwdCompact3<T, ST> e{g, w1c, nc, TwSel<T>::z(pl)};
    DD_TRY((launch_pass_len<T, false, false, false>(g.Nz, e, g.Kx, g.Ky, P::NO, st)));
    return DD_OK;
}

// Explicit instantiations live in rhs3d_<precision>.cu, one translation unit
// per arithmetic type, so the heavy transform kernels compile in parallel.
#define DD_RHS3D_INSTANTIATE_PH(EXT, T, PH)                                                            \
    EXT template int nonlinear3<T, false, PH>(const dd_plan*, const void* const*, double, const Work3&,     \
                                              cudaStream_t);                                            \
    EXT template int nonlinear3<T, true, PH>(const dd_plan*, const void* const*, double, const Work3&,      \
                                             cudaStream_t);
#define DD_RHS3D_INSTANTIATE_LO(EXT, PH)                                                                \
    EXT template int nonlinear3<float, false, PH, float>(const dd_plan*, const void* const*, double,         \
                                                         const Work3&, cudaStream_t);                        \
    EXT template int nonlinear3<float, true, PH, float>(const dd_plan*, const void* const*, double,          \
                                                        const Work3&, cudaStream_t);
// hydro forms and MHD forms, each compiled in its own translation unit; FP32
// adds the low-storage stage variants of the divergence forms
#define DD_RHS3D_INSTANTIATE_A(EXT, T) DD_RHS3D_INSTANTIATE_PH(EXT, T, P3_HYDRO) \
    DD_RHS3D_INSTANTIATE_PH(EXT, T, P3_HYDRO_DIV)
#define DD_RHS3D_INSTANTIATE_B(EXT, T) DD_RHS3D_INSTANTIATE_PH(EXT, T, P3_MHD) \
    DD_RHS3D_INSTANTIATE_PH(EXT, T, P3_MHD_DIV)
#define DD_RHS3D_INSTANTIATE(EXT, T) DD_RHS3D_INSTANTIATE_A(EXT, T) DD_RHS3D_INSTANTIATE_B(EXT, T)

}  // namespace dd
