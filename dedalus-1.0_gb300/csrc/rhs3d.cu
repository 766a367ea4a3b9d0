// Fused 3D incompressible-hydro right-hand side and RK4 step.
//
// RHS(u) = P[u x w]^ (2/3 dealiased), w = curl u: the rotational form of the
// reference's P[-(u.grad)u]^ (physics.py:527-599).  The two agree on the kept
// modes to roundoff: their difference is a gradient, which the projection
// removes, and products of dealiased fields alias only onto non-kept modes.
//
// Passes (all pruned to the kept modes, FP64 or FP32 arithmetic T):
//   1  Z^-1 of u and w = i k x u (curl formed while loading)      6 fields
//   2  Y^-1                                                         6 fields
//   3  X c2r of (ux,uy),(uz,wx),(wy,wz) packed rows -> u x w in
//      shared memory -> X r2c of the 3 products, scaled by 1/N      3 fields
//   4  Y forward, kept ky only                                      3 fields
//   5  Z forward, kept kz only, into a compact [kyc][kzc][kx] buffer
//   6  solenoidal projection (physics.py:588-599, laplace_solve
//      407-416) fused with the RK stage update (etd1 with phi tables).
#include "launch_len.cuh"
#include "xprod.cuh"
#include "etd.cuh"

namespace dd {

// ------------------------------------------------------------------ pass 1
// Fields 0..2 = u_x,u_y,u_z ; 3..5 = w_x,w_y,w_z (physics.py:394-396 curlX).
// The state is read either from the full reference layout [ky][kz][kx] or
// from the compact kept layout [kyc][kzc][kx] used for RK stage states.
__device__ __forceinline__ double2 ideriv(double2 a, double k) {
    // a * (1j * k) as numpy computes it (representations.py:423)
    return make_double2(-(a.y * k), a.x * k);
}

template <typename T, bool COMPACT>
struct OpZInvCurl3 {
    using V = typename Vec2<T>::type;
    static constexpr const char* name = "z_inv_curl";
    Geo3 g; CPtrs u; Ptrs out; const V* tw;
    const double* kx; const double* ky; const double* kz;
    __device__ int npencil() const { return g.Kx; }
    __device__ int nstore() const { return g.Nz; }
    __device__ double2 get(int c, int kyc, int ky, int e, int ix) const {
        const double2* U = (const double2*)u.p[c];
        if (COMPACT) return U[((int64_t)kyc * g.Kz + full_to_compact(e, g.Nz, g.Kz)) * g.Kx + ix];
        return U[((int64_t)ky * g.Nz + e) * g.Nh + ix];
    }
    __device__ C<T> load(int fld, int kyc, int e, int ix) const {
        if (!kept_full(e, g.Nz, g.Mz)) return zero<T>();
        const int ky_i = compact_to_full(kyc, g.Ny, g.Ky);
        double2 r;
        if (fld < 3) {
            r = get(fld, kyc, ky_i, e, ix);
        } else {
            const double kxv = kx[ix], kyv = ky[ky_i], kzv = kz[e];
            double2 a, b;
            if (fld == 3) { a = ideriv(get(2, kyc, ky_i, e, ix), kyv); b = ideriv(get(1, kyc, ky_i, e, ix), kzv); }
            else if (fld == 4) { a = ideriv(get(0, kyc, ky_i, e, ix), kzv); b = ideriv(get(2, kyc, ky_i, e, ix), kxv); }
            else { a = ideriv(get(1, kyc, ky_i, e, ix), kxv); b = ideriv(get(0, kyc, ky_i, e, ix), kyv); }
            r = make_double2(a.x - b.x, a.y - b.y);
        }
        return mk<T>((T)r.x, (T)r.y);
    }
    __device__ void store(int fld, int kyc, int e, int ix, const C<T>* col, int PS) const {
        stc<T>((V*)out.p[fld] + ((int64_t)kyc * g.Nz + e) * g.Kx + ix, col[e * PS]);
    }
};

// ------------------------------------------------------------------ pass 3
// X c2r of u and w (fields 0..5) -> u x w -> X r2c (k_x_prod, xprod.cuh).
template <typename T>
struct ProdHydro3 {
    static constexpr int NI = 6, NO = 3;
    __device__ void operator()(const T* in, T* out, int) const {
        const T ux = in[0], uy = in[1], uz = in[2], wx = in[3], wy = in[4], wz = in[5];
        out[0] = uy * wz - uz * wy;
        out[1] = uz * wx - ux * wz;
        out[2] = ux * wy - uy * wx;
    }
};

// ------------------------------------------------------------------ pass 5
// Forward along z into the compact kept buffer NC[kyc][kzc][kx].
template <typename T>
struct OpZFwdCompact3 {
    using V = typename Vec2<T>::type;
    static constexpr const char* name = "z_fwd_compact";
    Geo3 g; CPtrs in; Ptrs out; const V* tw;
    __device__ int npencil() const { return g.Kx; }
    __device__ int nstore() const { return g.Nz; }
    __device__ C<T> load(int fld, int kyc, int e, int kx) const {
        return ldc<T>((const V*)in.p[fld] + ((int64_t)kyc * g.Nz + e) * g.Kx + kx);
    }
    __device__ void store(int fld, int kyc, int e, int kx, const C<T>* col, int PS) const {
        if (!kept_full(e, g.Nz, g.Mz)) return;
        const C<T> c = col[e * PS];
        ((double2*)out.p[fld])[((int64_t)kyc * g.Kz + full_to_compact(e, g.Nz, g.Kz)) * g.Kx + kx] =
            make_double2((double)c.x, (double)c.y);
    }
};

// ------------------------------------------------------------------ pass 6
struct ProjArgs {
    Geo3 g;
    const double* kx; const double* ky; const double* kz;
    const double* inv_k2;   // 1/k2 per integer q (q = 0 -> 1), or null
    int intk;               // wavenumbers are integers (q tables valid)
};

__device__ __forceinline__ void kept_index(const Geo3& g, int64_t i, int& kyc, int& kzc, int& ix) {
    ix = (int)(i % g.Kx);
    const int64_t r = i / g.Kx;
    kzc = (int)(r % g.Kz);
    kyc = (int)(r / g.Kz);
}

// Solenoidal projection with the reference's operation order:
// div = ((i kx Nx) + i ky Ny) + i kz Nz; phi = -(div * (1/k2)); N_i -= i k_i phi.
__device__ __forceinline__ void project(double2& nx, double2& ny, double2& nz, double kxv, double kyv,
                                        double kzv, double s) {
    double2 dx = ideriv(nx, kxv), dy = ideriv(ny, kyv), dz = ideriv(nz, kzv);
    double2 dv = make_double2(radd(radd(dx.x, dy.x), dz.x), radd(radd(dx.y, dy.y), dz.y));
    double2 ph = make_double2(-rmul(dv.x, s), -rmul(dv.y, s));
    double2 gx = ideriv(ph, kxv), gy = ideriv(ph, kyv), gz = ideriv(ph, kzv);
    nx = make_double2(rsub(nx.x, gx.x), rsub(nx.y, gx.y));
    ny = make_double2(rsub(ny.x, gy.x), rsub(ny.y, gy.y));
    nz = make_double2(rsub(nz.x, gz.x), rsub(nz.y, gz.y));
}

__device__ __forceinline__ double inv_k2_of(const ProjArgs& a, int ix, int ky_i, int kz_i, int& q) {
    const double kxv = a.kx[ix], kyv = a.ky[ky_i], kzv = a.kz[kz_i];
    // k2 = ((0 + ky^2) + kz^2) + kx^2 (representations.py:434-436, k dict order y, z, x)
    double k2 = radd(radd(rmul(kyv, kyv), rmul(kzv, kzv)), rmul(kxv, kxv));
    q = a.intk ? (int)k2 : 0;
    if (a.intk && a.inv_k2) return a.inv_k2[q];
    if (k2 == 0.) k2 = 1.;
    return rdiv(1., k2);
}

// Projection only, into the full-layout derivative arrays (kept entries).
__global__ void k_project_to_deriv3(ProjArgs a, CPtrs nc, Ptrs deriv) {
    const Geo3& g = a.g;
    const int64_t n = (int64_t)g.Ky * g.Kz * g.Kx;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int kyc, kzc, ix, q;
        kept_index(g, i, kyc, kzc, ix);
        const int ky_i = compact_to_full(kyc, g.Ny, g.Ky), kz_i = compact_to_full(kzc, g.Nz, g.Kz);
        const double s = inv_k2_of(a, ix, ky_i, kz_i, q);
        double2 nx = ((const double2*)nc.p[0])[i], ny = ((const double2*)nc.p[1])[i], nz = ((const double2*)nc.p[2])[i];
        project(nx, ny, nz, a.kx[ix], a.ky[ky_i], a.kz[kz_i], s);
        const int64_t o = ((int64_t)ky_i * g.Nz + kz_i) * g.Nh + ix;
        ((double2*)deriv.p[0])[o] = nx;
        ((double2*)deriv.p[1])[o] = ny;
        ((double2*)deriv.p[2])[o] = nz;
    }
}

// One RK4 stage (time_step.py:426-483 as restated by the project; see the
// oracle): k = P[N];
//   stage 1: tot = k*(1/6);  y1 = etd1(y, k, dt/2)
//   stage 2: tot += k*(1/3); y2 = etd1(y, k, dt/2)
//   stage 3: tot += k*(1/3); y3 = etd1(y, k, dt)
//   stage 4: tot += k*(1/6); y  = etd1(y, tot, dt)
// y (state) is full layout; stage states and tot are compact.
struct RK4Args {
    ProjArgs pa;
    CPtrs nc;          // unprojected RHS, compact
    Ptrs y;            // state, full layout (read; written at stage 4)
    Ptrs ys;           // next stage state, compact (stages 1-3)
    Ptrs tot;          // accumulated increment, compact
    const double4* tab;  // phi table for this stage's step (q-indexed), or null
    double h;            // this stage's step (dt/2 or dt)
    double nu; int vo;   // used when tab is null (non-integer wavenumbers)
    double w;            // increment weight: 1/6 or 1/3
    int stage;
};

template <int NDIM>
__device__ __forceinline__ void phis_for(const RK4Args& a, int q, double k2, double& Z, double& f0, double& f1) {
    if (a.tab) {
        const double4 t = a.tab[q];
        Z = t.x; f0 = t.y; f1 = t.z;
    } else {
        const double k2v = a.vo == 1 ? k2 : (a.vo == 2 ? rmul(k2, k2) : pow(k2, (double)a.vo));
        Z = rmul(-rmul(a.nu, k2v), a.h);
        double f2;
        f0 = 1.; f1 = 1.;
        if (Z != 0.) etd_phis<NDIM>(Z, f0, f1, f2);
    }
}

__global__ void k_rk4_stage3(RK4Args a) {
    const Geo3& g = a.pa.g;
    const int64_t n = (int64_t)g.Ky * g.Kz * g.Kx;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int kyc, kzc, ix, q;
        kept_index(g, i, kyc, kzc, ix);
        const int ky_i = compact_to_full(kyc, g.Ny, g.Ky), kz_i = compact_to_full(kzc, g.Nz, g.Kz);
        const double kxv = a.pa.kx[ix], kyv = a.pa.ky[ky_i], kzv = a.pa.kz[kz_i];
        const double s = inv_k2_of(a.pa, ix, ky_i, kz_i, q);
        double2 k[3] = {((const double2*)a.nc.p[0])[i], ((const double2*)a.nc.p[1])[i], ((const double2*)a.nc.p[2])[i]};
        project(k[0], k[1], k[2], kxv, kyv, kzv, s);
        const double k2 = radd(radd(rmul(kyv, kyv), rmul(kzv, kzv)), rmul(kxv, kxv));
        double Z, f0, f1;
        phis_for<3>(a, q, k2, Z, f0, f1);
        const int64_t o = ((int64_t)ky_i * g.Nz + kz_i) * g.Nh + ix;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const double2 kw = make_double2(rmul(k[c].x, a.w), rmul(k[c].y, a.w));
            double2 t;
            if (a.stage == 1) t = kw;
            else { t = ((const double2*)a.tot.p[c])[i]; t = make_double2(radd(t.x, kw.x), radd(t.y, kw.y)); }
            const double2 y0 = ((const double2*)a.y.p[c])[o];
            if (a.stage < 4) {
                ((double2*)a.tot.p[c])[i] = t;
                ((double2*)a.ys.p[c])[i] = etd1_entry(y0, k[c], Z, f0, f1, a.h);
            } else {
                ((double2*)a.y.p[c])[o] = etd1_entry(y0, t, Z, f0, f1, a.h);
            }
        }
    }
}

// Non-kept modes of the state see no nonlinear forcing: y <- etd1(y, 0, dt).
__global__ void k_decay_nonkept3(Geo3 g, Ptrs y, const double* kx, const double* ky, const double* kz,
                                 const double4* tab, double nu, int vo, double dt) {
    const int64_t n = g.kcount();
    const int c = blockIdx.y;
    double2* Y = (double2*)y.p[c];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int ix = (int)(i % g.Nh);
        const int64_t r = i / g.Nh;
        const int kz_i = (int)(r % g.Nz), ky_i = (int)(r / g.Nz);
        if (ix <= g.Mx && kept_full(ky_i, g.Ny, g.My) && kept_full(kz_i, g.Nz, g.Mz)) continue;
        const double2 y0 = Y[i];
        if (y0.x == 0. && y0.y == 0.) continue;
        const double k2 = radd(radd(rmul(ky[ky_i], ky[ky_i]), rmul(kz[kz_i], kz[kz_i])), rmul(kx[ix], kx[ix]));
        double Z, f0 = 1., f1 = 1., f2;
        if (tab) { const double4 t = tab[(int)k2]; Z = t.x; f0 = t.y; f1 = t.z; }
        else {
            const double k2v = vo == 1 ? k2 : (vo == 2 ? rmul(k2, k2) : pow(k2, (double)vo));
            Z = rmul(-rmul(nu, k2v), dt);
            if (Z != 0.) etd_phis<3>(Z, f0, f1, f2);
        }
        Y[i] = etd1_entry(y0, make_double2(0., 0.), Z, f0, f1, dt);
    }
}

// Any non-zero entry outside the kept set? (flag[0] |= 1)
__global__ void k_any_nonkept3(Geo3 g, CPtrs y, int ncomp, int* flag) {
    const int64_t n = g.kcount();
    int found = 0;
    for (int c = 0; c < ncomp; c++) {
        const double2* Y = (const double2*)y.p[c];
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
            const int ix = (int)(i % g.Nh);
            const int64_t r = i / g.Nh;
            const int kz_i = (int)(r % g.Nz), ky_i = (int)(r / g.Nz);
            if (ix <= g.Mx && kept_full(ky_i, g.Ny, g.My) && kept_full(kz_i, g.Nz, g.Mz)) continue;
            const double2 v = Y[i];
            if (v.x != 0. || v.y != 0.) found = 1;
        }
    }
    if (__syncthreads_or(found) && threadIdx.x == 0) atomicOr(flag, 1);
}

// Zero every non-kept entry of ncomp full-layout arrays (grid.y = component).
__global__ void k_dealias3_all(Geo3 g, Ptrs k) {
    double2* K = (double2*)k.p[blockIdx.y];
    const int64_t n = g.kcount();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int ix = (int)(i % g.Nh);
        const int64_t r = i / g.Nh;
        const int kz_i = (int)(r % g.Nz), ky_i = (int)(r / g.Nz);
        if (ix > g.Mx || !kept_full(ky_i, g.Ny, g.My) || !kept_full(kz_i, g.Nz, g.Mz)) K[i] = make_double2(0., 0.);
    }
}

static unsigned ew_grid(int64_t n) {
    int64_t b = (n + 255) / 256;
    if (b > 152 * 16) b = 152 * 16;
    return (unsigned)(b < 1 ? 1 : b);
}

// ------------------------------------------------------------ RHS driver
struct Hydro3Work {
    size_t w1, w2, kc;   // complex entries per field
    char* base;
    template <typename T> C<T>* W1(int f) const { return (C<T>*)base + f * w1; }
    template <typename T> C<T>* W2(int f) const { return (C<T>*)base + 6 * w1 + f * w2; }
    template <typename T> double2* NC(int f) const {
        return (double2*)((char*)base + sizeof(C<T>) * (6 * w1 + 6 * w2)) + f * kc;
    }
    template <typename T> static size_t bytes(const Geo3& g) {
        return sizeof(C<T>) * (6 * g.w1count() + 6 * g.w2count()) + sizeof(double2) * 3 * (size_t)g.Ky * g.Kz * g.Kx;
    }
};

// Passes 1-5: state u (3 comps; full layout, or compact when COMPACT) ->
// unprojected dealiased RHS in NC (compact).
template <typename T, bool COMPACT>
static int hydro3_nonlinear(const dd_plan* pl, const void* const* u, const Hydro3Work& w, cudaStream_t st) {
    const Geo3& g = pl->g3;
    CPtrs uin{}; Ptrs w1{}, w2{}, nc{}; CPtrs w1c{}, w2c{};
    for (int c = 0; c < 3; c++) { uin.p[c] = u[c]; nc.p[c] = w.NC<T>(c); }
    for (int f = 0; f < 6; f++) {
        w1.p[f] = w.W1<T>(f); w1c.p[f] = w1.p[f];
        w2.p[f] = w.W2<T>(f); w2c.p[f] = w2.p[f];
    }
    OpZInvCurl3<T, COMPACT> a{g, uin, w1, TwSel<T>::z(pl), pl->kx, pl->ky, pl->kz};
    DD_TRY((launch_pass_len<T, true, false, false>(g.Nz, a, g.Kx, g.Ky, 6, st)));
    OpYInv3<T> b{g, w1c, w2, TwSel<T>::y(pl)};
    DD_TRY((launch_pass_len<T, true, false, false>(g.Ny, b, g.Kx, g.Nz, 6, st)));
    // products overwrite fields 0..2 of W2 row by row (each block reads its rows first)
    DD_TRY((launch_x_prod_len<T>("x_cross", g.Nx, g.Nz * g.Ny, g.Kx, w2c, w2, 1, 0, 0, TwSel<T>::x(pl), (T)pl->inv_n,
                                 ProdHydro3<T>{}, st)));
    OpYFwd3<T> d{g, w2c, w1, TwSel<T>::y(pl)};
    DD_TRY((launch_pass_len<T, false, false, false>(g.Ny, d, g.Kx, g.Nz, 3, st)));
    OpZFwdCompact3<T> e{g, w1c, nc, TwSel<T>::z(pl)};
    DD_TRY((launch_pass_len<T, false, false, false>(g.Nz, e, g.Kx, g.Ky, 3, st)));
    return DD_OK;
}

}  // namespace dd

using namespace dd;

static int check_hydro3(const dd_plan* p, const void* const* a, const void* const* b) {
    DD_CHECK_ARG(p, "null plan");
    DD_CHECK_ARG(p->ndim == 3, "plan is not 3D");
    DD_CHECK_ARG(a && a[0] && a[1] && a[2], "null field pointer");
    if (b) DD_CHECK_ARG(b[0] && b[1] && b[2], "null field pointer");
    return DD_OK;
}

extern "C" {

int dd_hydro3d_workspace_size(const dd_plan* p, int precision, size_t* bytes) {
    DD_CHECK_ARG(p && bytes && p->ndim == 3, "dd_hydro3d_workspace_size: bad arguments");
    const Geo3& g = p->g3;
    const size_t stage = sizeof(double2) * 3 * (size_t)g.Ky * g.Kz * g.Kx * 2;  // tot + stage state
    *bytes = (precision == DD_FP32 ? Hydro3Work::bytes<float>(g) : Hydro3Work::bytes<double>(g)) + stage;
    return DD_OK;
}

int dd_hydro3d_rhs(const dd_plan* p, const void* const* u, void* const* deriv, const double* inv_k2,
                   int precision, int zero_nonkept, void* work, size_t work_bytes, void* stream) {
    DD_TRY(check_hydro3(p, (const void* const*)u, (const void* const*)deriv));
    DD_CHECK_ARG(work, "null workspace");
    DD_CHECK_ARG(precision == DD_FP64 || precision == DD_FP32, "bad precision");
    const Geo3& g = p->g3;
    cudaStream_t st = (cudaStream_t)stream;
    Hydro3Work w{(size_t)g.w1count(), (size_t)g.w2count(), (size_t)g.Ky * g.Kz * g.Kx, (char*)work};
    const size_t need = precision == DD_FP32 ? Hydro3Work::bytes<float>(g) : Hydro3Work::bytes<double>(g);
    DD_CHECK_ARG(work_bytes >= need, "workspace too small: %zu < %zu", work_bytes, need);
    if (precision == DD_FP64) DD_TRY((hydro3_nonlinear<double, false>(p, u, w, st)));
    else DD_TRY((hydro3_nonlinear<float, false>(p, u, w, st)));
    ProjArgs pa{g, p->kx, p->ky, p->kz, inv_k2, inv_k2 != nullptr};
    CPtrs nc{}; Ptrs d{};
    for (int c = 0; c < 3; c++) {
        nc.p[c] = precision == DD_FP64 ? (void*)w.NC<double>(c) : (void*)w.NC<float>(c);
        d.p[c] = deriv[c];
    }
    if (zero_nonkept) {
        DD_KT("zero_nonkept3", st, k_dealias3_all<<<dim3(ew_grid(g.kcount()), 3), 256, 0, st>>>(g, d));
        DD_LAUNCH_CHECK();
    }
    DD_KT("project3", st, k_project_to_deriv3<<<ew_grid((int64_t)g.Ky * g.Kz * g.Kx), 256, 0, st>>>(pa, nc, d));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

int dd_hydro3d_rk4_step(const dd_plan* p, void* const* u, const double* inv_k2, const void* tab_half,
                        const void* tab_full, double nu, int viscosity_order, double dt, int precision,
                        int* nonkept_flag, void* work, size_t work_bytes, void* stream) {
    DD_TRY(check_hydro3(p, (const void* const*)u, nullptr));
    DD_CHECK_ARG(work, "null workspace");
    DD_CHECK_ARG(precision == DD_FP64 || precision == DD_FP32, "bad precision");
    DD_CHECK_ARG(viscosity_order >= 1, "viscosity_order must be >= 1");
    const Geo3& g = p->g3;
    cudaStream_t st = (cudaStream_t)stream;
    Hydro3Work w{(size_t)g.w1count(), (size_t)g.w2count(), (size_t)g.Ky * g.Kz * g.Kx, (char*)work};
    const size_t base = precision == DD_FP32 ? Hydro3Work::bytes<float>(g) : Hydro3Work::bytes<double>(g);
    const size_t kc = (size_t)g.Ky * g.Kz * g.Kx;
    DD_CHECK_ARG(work_bytes >= base + sizeof(double2) * 6 * kc, "workspace too small");
    double2* tot = (double2*)((char*)work + base);
    double2* ys = tot + 3 * kc;
    const bool intk = inv_k2 != nullptr;
    DD_CHECK_ARG(!intk || (tab_half && tab_full), "phi tables required with integer wavenumbers");
    ProjArgs pa{g, p->kx, p->ky, p->kz, inv_k2, intk};
    RK4Args a{};
    a.pa = pa;
    a.nu = nu; a.vo = viscosity_order;
    for (int c = 0; c < 3; c++) {
        a.nc.p[c] = precision == DD_FP64 ? (void*)w.NC<double>(c) : (void*)w.NC<float>(c);
        a.y.p[c] = u[c];
        a.ys.p[c] = ys + c * kc;
        a.tot.p[c] = tot + c * kc;
    }
    const void* ysc[3] = {ys, ys + kc, ys + 2 * kc};
    const double hs[4] = {dt / 2., dt / 2., dt, dt};
    const double ws[4] = {1. / 6., 1. / 3., 1. / 3., 1. / 6.};
    const void* tabs[4] = {tab_half, tab_half, tab_full, tab_full};
    for (int s = 1; s <= 4; s++) {
        if (s == 1) {
            if (precision == DD_FP64) DD_TRY((hydro3_nonlinear<double, false>(p, (const void* const*)u, w, st)));
            else DD_TRY((hydro3_nonlinear<float, false>(p, (const void* const*)u, w, st)));
        } else {
            if (precision == DD_FP64) DD_TRY((hydro3_nonlinear<double, true>(p, ysc, w, st)));
            else DD_TRY((hydro3_nonlinear<float, true>(p, ysc, w, st)));
        }
        a.stage = s; a.h = hs[s - 1]; a.w = ws[s - 1]; a.tab = (const double4*)tabs[s - 1];
        DD_KT("rk4_stage3", st, k_rk4_stage3<<<ew_grid((int64_t)kc), 256, 0, st>>>(a));
        DD_LAUNCH_CHECK();
    }
    if (nonkept_flag && *nonkept_flag) {
        DD_KT("decay_nonkept3", st,
              k_decay_nonkept3<<<dim3(ew_grid(g.kcount()), 3), 256, 0, st>>>(g, a.y, p->kx, p->ky, p->kz,
                                                                           (const double4*)tab_full, nu, viscosity_order, dt));
        DD_LAUNCH_CHECK();
    }
    return DD_OK;
}

int dd_any_nonkept(const dd_plan* p, int ncomp, const void* const* k, int* dflag, void* stream) {
    DD_CHECK_ARG(p && k && dflag && ncomp >= 1 && ncomp <= 8, "dd_any_nonkept: bad arguments");
    DD_CHECK_ARG(p->ndim == 3, "dd_any_nonkept: 3D plans only");
    CPtrs y{};
    for (int c = 0; c < ncomp; c++) y.p[c] = k[c];
    DD_KT("any_nonkept3", (cudaStream_t)stream,
          k_any_nonkept3<<<ew_grid(p->g3.kcount()), 256, 0, (cudaStream_t)stream>>>(p->g3, y, ncomp, dflag));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

}  // extern "C"
