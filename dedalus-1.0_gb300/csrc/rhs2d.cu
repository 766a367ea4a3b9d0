// Fused 2D right-hand sides and RK2mid step: projection/stage kernels, drivers
// and the C ABI.  Transform passes are in rhs2d_impl.cuh / rhs2d_<precision>.cu.
#include "rhs2d_impl.cuh"

namespace dd {

DD_RHS2D_INSTANTIATE(extern, double)
DD_RHS2D_INSTANTIATE(extern, float)
DD_RHS2D_INSTANTIATE_LO(extern, PHYS_HYDRO_DIV)
DD_RHS2D_INSTANTIATE_LO(extern, PHYS_BOUSS_DIV)

// ------------------------------------------------------------------ pass 4
struct Phys2Params {
    double g, alpha_t, beta;
    int dir;   // component receiving buoyancy (0 = x, 1 = y)
};

struct Stage2Args {
    Geo2 g;
    const double* kx; const double* ky; const double* inv_k2; int intk;
    const float* kxf; const float* kyf;   // the wavenumber tables rounded to float
    int phys; Phys2Params pp;
    int nrun;
    CPtrs nc; int64_t nc_rs;          // unprojected products (compact)
    CPtrs rin; int64_t rin_rs; int rin_compact;   // state the RHS was evaluated on
    Ptrs y; int64_t y_rs;             // state (full layout)
    Ptrs ys; Ptrs k1; int64_t c_rs;   // stage state / first derivative (compact)
    Ptrs deriv; int64_t d_rs;         // RHS output (full layout), mode 0
    const double4* tab[3];            // phi tables per state field for this stage (q-indexed) or null
    double nu[3]; int vo; double h;
    int mode;                         // 0 = write deriv, 1 = RK2mid stage 1, 2 = RK2mid stage 2
};

__device__ __forceinline__ void project2(double2& nx, double2& ny, double kxv, double kyv, double s) {
    const double2 dx = ideriv2(nx, kxv), dy = ideriv2(ny, kyv);
    const double2 dv = make_double2(radd(dx.x, dy.x), radd(dx.y, dy.y));
    const double2 ph = make_double2(-rmul(dv.x, s), -rmul(dv.y, s));
    const double2 gx = ideriv2(ph, kxv), gy = ideriv2(ph, kyv);
    nx = make_double2(rsub(nx.x, gx.x), rsub(nx.y, gx.y));
    ny = make_double2(rsub(ny.x, gy.x), rsub(ny.y, gy.y));
}

// The projection with fused multiply-adds (N -= k (k . N) / k^2), for the
// fused RK2mid stages.
__device__ __forceinline__ void project2_fma(double2& nx, double2& ny, double kxv, double kyv, double s) {
    const double cr = fma(kyv, ny.x, kxv * nx.x) * s;
    const double ci = fma(kyv, ny.y, kxv * nx.y) * s;
    nx = make_double2(fma(-kxv, cr, nx.x), fma(-kxv, ci, nx.y));
    ny = make_double2(fma(-kyv, cr, ny.x), fma(-kyv, ci, ny.y));
}

__device__ __forceinline__ void phis2(const Stage2Args& a, int c, int q, double k2, double& Z, double& f0,
                                      double& f1, double& f2) {
    if (a.tab[c]) {
        const double4 t = a.tab[c][q];
        Z = t.x; f0 = t.y; f1 = t.z; f2 = t.w;
    } else {
        const double k2v = a.vo == 1 ? k2 : (a.vo == 2 ? rmul(k2, k2) : pow(k2, (double)a.vo));
        Z = rmul(-rmul(a.nu[c], k2v), a.h);
        f0 = 1.; f1 = 1.; f2 = 0.5;
        if (Z != 0.) etd_phis<2>(Z, f0, f1, f2);
    }
}

// One thread per kept entry of every run.  NF (2 hydro, 3 Boussinesq) and
// MODE (0 = write deriv, 1 = RK2mid stage 1, 2 = stage 2) are template
// parameters so that the per-field loop unrolls with static indices.
template <int NF, int MODE, bool DIV>
__global__ void k_stage2(Stage2Args a) {
    const Geo2& g = a.g;
    const int per = g.Kx * g.Ky;
    const int64_t n = (int64_t)per * a.nrun;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int run = (int)(i / per);
        const int j = (int)(i - (int64_t)run * per);
        const int kyc = j % g.Ky, ix = j / g.Ky;
        const int ky_i = compact_to_full(kyc, g.Ny, g.Ky);
        const double kxv = a.kx[ix], kyv = a.ky[ky_i];
        // k2 = (0 + kx^2) + ky^2 (2D k dict order x, y)
        const double k2 = radd(rmul(kxv, kxv), rmul(kyv, kyv));
        const int q = a.intk ? (int)k2 : 0;
        double s;
        if (a.intk && a.inv_k2) s = a.inv_k2[q];
        else s = rdiv(1., k2 == 0. ? 1. : k2);
        double2 N[NF];
        const int64_t ni = run * a.nc_rs + j;
        if constexpr (DIV) {
            // N = -i k_j T_ij with T_xx = u_x^2 - u_y^2, T_xy = u_x u_y, T_yy = 0; -i s = (s.y, -s.x)
            const double2 p0 = ((const double2*)a.nc.p[0])[ni], p1 = ((const double2*)a.nc.p[1])[ni];
            const double sxr = fma(kyv, p1.x, kxv * p0.x), sxi = fma(kyv, p1.y, kxv * p0.y);
            N[0] = make_double2(sxi, -sxr);
            N[1] = make_double2(kxv * p1.y, -(kxv * p1.x));
        } else {
            N[0] = ((const double2*)a.nc.p[0])[ni];
            N[1] = ((const double2*)a.nc.p[1])[ni];
        }
        if constexpr (NF == 3) {
            const int64_t ri = a.rin_compact ? run * a.rin_rs + j : run * a.rin_rs + (int64_t)ix * g.Ny + ky_i;
            const double2 T = ((const double2*)a.rin.p[2])[ri];
            const double2 ud = ((const double2*)(a.pp.dir == 0 ? a.rin.p[0] : a.rin.p[1]))[ri];
            // buoyancy: ((T * g) * alpha_t) added to u_dir (physics.py:691-694)
            const double2 b = make_double2(rmul(rmul(T.x, a.pp.g), a.pp.alpha_t), rmul(rmul(T.y, a.pp.g), a.pp.alpha_t));
            if (a.pp.dir == 0) N[0] = make_double2(radd(N[0].x, b.x), radd(N[0].y, b.y));
            else N[1] = make_double2(radd(N[1].x, b.x), radd(N[1].y, b.y));
            // temperature: (-(u.grad T)) - (u_dir * beta) (physics.py:702-708); in divergence
            // form u.grad T = i k . (u T)^, i s = (-s.y, s.x)
            double2 adv;
            if constexpr (DIV) {
                const double2 fx = ((const double2*)a.nc.p[2])[ni], fy = ((const double2*)a.nc.p[3])[ni];
                const double sr = fma(kyv, fy.x, kxv * fx.x), si = fma(kyv, fy.y, kxv * fx.y);
                adv = make_double2(-si, sr);
            } else {
                adv = ((const double2*)a.nc.p[2])[ni];
            }
            N[2] = make_double2(rsub(-adv.x, rmul(ud.x, a.pp.beta)), rsub(-adv.y, rmul(ud.y, a.pp.beta)));
        }
        if constexpr (MODE == 0) project2(N[0], N[1], kxv, kyv, s);
        else project2_fma(N[0], N[1], kxv, kyv, s);
        const int64_t full = run * a.y_rs + (int64_t)ix * g.Ny + ky_i;
#pragma unroll
        for (int c = 0; c < NF; c++) {
            if constexpr (MODE == 0) {
                ((double2*)a.deriv.p[c])[run * a.d_rs + (int64_t)ix * g.Ny + ky_i] = N[c];
            } else {
                double Z, f0, f1, f2;
                phis2(a, c, q, k2, Z, f0, f1, f2);
                const double2 y0 = ((const double2*)a.y.p[c])[full];
                const int64_t ci = run * a.c_rs + j;
                if constexpr (MODE == 1) {
                    ((double2*)a.k1.p[c])[ci] = N[c];
                    ((double2*)a.ys.p[c])[ci] = etd1_fma(y0, N[c], f0, f1 * a.h);
                } else {
                    const double2 d1 = ((const double2*)a.k1.p[c])[ci];
                    ((double2*)a.y.p[c])[full] = etd2rk2_fma(y0, d1, N[c], f0, f1 * a.h, 2. * f2 * a.h);
                }
            }
        }
    }
}

// The RK2mid stages of the low-storage FP32 step (divergence forms): complex64
// products, stage derivative k1 and stage state; N, the projection and the
// buoyancy / stratification terms in float from float wavenumbers (k^2 exact
// for integer wavenumbers); stage 1 forms the float stage state in float;
// stage 2 forms the increment h phi1 k1 + 2 h phi2 (k2 - k1) in float and adds
// it to f0 y in FP64 (the state stays FP64).
template <int NF, int MODE>
__global__ void k_stage2_lo(Stage2Args a) {
    static_assert(MODE == 1 || MODE == 2, "RK2mid stages only");
    const Geo2& g = a.g;
    const int per = g.Kx * g.Ky;
    const int64_t n = (int64_t)per * a.nrun;
    bool tabs = a.intk && a.inv_k2;
#pragma unroll
    for (int c = 0; c < NF; c++) tabs = tabs && a.tab[c];
    const float hf = (float)a.h;
    const float pg = (float)a.pp.g, pat = (float)a.pp.alpha_t, pbeta = (float)a.pp.beta;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int run = (int)(i / per);
        const int j = (int)(i - (int64_t)run * per);
        const int kyc = j % g.Ky, ix = j / g.Ky;
        const int ky_i = compact_to_full(kyc, g.Ny, g.Ky);
        const float kx = a.kxf[ix], ky = a.kyf[ky_i];
        int q = 0;
        double k2 = 0.;
        float s;
        if (tabs) {
            q = (int)(kx * kx + ky * ky);
            s = (float)a.inv_k2[q];
        } else {
            const double kxv = a.kx[ix], kyv = a.ky[ky_i];
            k2 = radd(rmul(kxv, kxv), rmul(kyv, kyv));
            q = a.intk ? (int)k2 : 0;
            s = (float)((a.intk && a.inv_k2) ? a.inv_k2[q] : rdiv(1., k2 == 0. ? 1. : k2));
        }
        const int64_t ni = run * a.nc_rs + j;
        // N = -i k_j T_ij with T_xx = u_x^2 - u_y^2, T_xy = u_x u_y; -i s = (s.y, -s.x)
        const float2 p0 = ((const float2*)a.nc.p[0])[ni], p1 = ((const float2*)a.nc.p[1])[ni];
        float2 N[NF];
        N[0] = make_float2(fmaf(ky, p1.y, kx * p0.y), -fmaf(ky, p1.x, kx * p0.x));
        N[1] = make_float2(kx * p1.y, -(kx * p1.x));
        if constexpr (NF == 3) {
            // T and u_dir of the state the RHS was evaluated on: the FP64 state
            // in stage 1, the complex64 stage state in stage 2
            float2 T, ud;
            const void* up = a.pp.dir == 0 ? a.rin.p[0] : a.rin.p[1];
            if constexpr (MODE == 1) {
                const int64_t ri = run * a.rin_rs + (int64_t)ix * g.Ny + ky_i;
                const double2 Td = ((const double2*)a.rin.p[2])[ri], udd = ((const double2*)up)[ri];
                T = make_float2((float)Td.x, (float)Td.y);
                ud = make_float2((float)udd.x, (float)udd.y);
            } else {
                const int64_t ri = run * a.rin_rs + j;
                T = ((const float2*)a.rin.p[2])[ri];
                ud = ((const float2*)up)[ri];
            }
            const float2 b = make_float2(T.x * pg * pat, T.y * pg * pat);   // (T g) alpha_t
            if (a.pp.dir == 0) N[0] = make_float2(N[0].x + b.x, N[0].y + b.y);
            else N[1] = make_float2(N[1].x + b.x, N[1].y + b.y);
            // -div(u T) - beta u_dir; i s = (-s.y, s.x)
            const float2 fx = ((const float2*)a.nc.p[2])[ni], fy = ((const float2*)a.nc.p[3])[ni];
            const float sr = fmaf(ky, fy.x, kx * fx.x), si = fmaf(ky, fy.y, kx * fx.y);
            N[2] = make_float2(si - ud.x * pbeta, -sr - ud.y * pbeta);
        }
        // projection: N -= k (k . N) / k^2
        const float cr = fmaf(ky, N[1].x, kx * N[0].x) * s, ci = fmaf(ky, N[1].y, kx * N[0].y) * s;
        N[0] = make_float2(fmaf(-kx, cr, N[0].x), fmaf(-kx, ci, N[0].y));
        N[1] = make_float2(fmaf(-ky, cr, N[1].x), fmaf(-ky, ci, N[1].y));
        const int64_t full = run * a.y_rs + (int64_t)ix * g.Ny + ky_i;
        const int64_t ci2 = run * a.c_rs + j;
#pragma unroll
        for (int c = 0; c < NF; c++) {
            double f0, f1, f2;
            if (tabs) {
                const double* t = reinterpret_cast<const double*>(a.tab[c] + q);
                f0 = t[1]; f1 = t[2]; f2 = t[3];
            } else {
                double Z;
                phis2(a, c, q, k2, Z, f0, f1, f2);
            }
            const double2 y0 = ((const double2*)a.y.p[c])[full];
            if constexpr (MODE == 1) {
                ((float2*)a.k1.p[c])[ci2] = N[c];
                const float f0f = (float)f0, f1hf = (float)f1 * hf;
                ((float2*)a.ys.p[c])[ci2] = make_float2(fmaf(f1hf, N[c].x, (float)y0.x * f0f),
                                                        fmaf(f1hf, N[c].y, (float)y0.y * f0f));
            } else {
                // the increment h phi1 k1 + 2 h phi2 (k2 - k1), float like k1 and k2,
                // added to f0 y in FP64
                const float2 d1 = ((const float2*)a.k1.p[c])[ci2];
                const float f1hf = (float)f1 * hf, f2hf = 2.f * (float)f2 * hf;
                const float ir = fmaf(f1hf, d1.x, f2hf * (N[c].x - d1.x));
                const float ii = fmaf(f1hf, d1.y, f2hf * (N[c].y - d1.y));
                ((double2*)a.y.p[c])[full] = make_double2(fma(f0, y0.x, (double)ir), fma(f0, y0.y, (double)ii));
            }
        }
    }
}

template <int MODE>
static int launch_stage2_lo(const Stage2Args& a, unsigned nb, cudaStream_t st) {
    if (a.phys == PHYS_HYDRO_DIV) DD_KT("rk2mid_stage2d_lo", st, k_stage2_lo<2, MODE><<<nb, 256, 0, st>>>(a));
    else DD_KT("rk2mid_stage2d_lo", st, k_stage2_lo<3, MODE><<<nb, 256, 0, st>>>(a));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

template <int MODE>
static int launch_stage2(const Stage2Args& a, unsigned nb, const char* label, cudaStream_t st) {
    if (a.phys == PHYS_HYDRO) DD_KT(label, st, k_stage2<2, MODE, false><<<nb, 256, 0, st>>>(a));
    else if (a.phys == PHYS_BOUSS) DD_KT(label, st, k_stage2<3, MODE, false><<<nb, 256, 0, st>>>(a));
    else if (a.phys == PHYS_HYDRO_DIV) DD_KT(label, st, k_stage2<2, MODE, true><<<nb, 256, 0, st>>>(a));
    else DD_KT(label, st, k_stage2<3, MODE, true><<<nb, 256, 0, st>>>(a));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

// Non-kept modes see no forcing: RK2mid gives y <- etd2rk2(y, 0, 0, dt) = f0 y.
__global__ void k_decay_nonkept2(Geo2 g, Ptrs y, int64_t y_rs, int nf, int nrun, const double* kx,
                                 const double* ky, Stage2Args a) {
    const int64_t per = g.kcount(), n = per * nrun;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int run = (int)(i / per);
        const int64_t j = i - run * per;
        const int ky_i = (int)(j % g.Ny), ix = (int)(j / g.Ny);
        if (ix <= g.Mx && kept_full(ky_i, g.Ny, g.My)) continue;
        const double k2 = radd(rmul(kx[ix], kx[ix]), rmul(ky[ky_i], ky[ky_i]));
        const int q = a.intk ? (int)k2 : 0;
        for (int c = 0; c < nf; c++) {
            double2* Y = (double2*)pick_ptr<DD_MAXF>(y.p, c) + run * y_rs;
            const double2 y0 = Y[j];
            if (y0.x == 0. && y0.y == 0.) continue;
            double Z, f0, f1, f2;
            phis2(a, c, q, k2, Z, f0, f1, f2);
            const double2 z = make_double2(0., 0.);
            Y[j] = etd2rk2_entry(y0, z, z, Z, f0, f1, f2, a.h);
        }
    }
}

__global__ void k_zero_nonkept2_all(Geo2 g, Ptrs k, int64_t rs, int nrun) {
    double2* K = (double2*)pick_ptr<DD_MAXF>(k.p, (int)blockIdx.y);
    const int64_t per = g.kcount(), n = per * nrun;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int run = (int)(i / per);
        const int64_t j = i - run * per;
        const int ky_i = (int)(j % g.Ny), ix = (int)(j / g.Ny);
        if (ix > g.Mx || !kept_full(ky_i, g.Ny, g.My)) K[run * rs + j] = make_double2(0., 0.);
    }
}

// Sums over the kept modes of nrun 2D velocities (run r at offset r * rs):
// out[0] += |k . u|^2, out[1] += |k|^2 |u|^2 (block partials, one atomic per block).
__global__ void __launch_bounds__(256) k_div_sums2(Geo2 g, const double* kx, const double* ky, const double2* ux,
                                                    const double2* uy, int64_t rs, int nrun, double* out) {
    __shared__ double r0[256], r1[256];
    const int per = g.Kx * g.Ky;
    const int64_t n = (int64_t)per * nrun;
    double s0 = 0., s1 = 0.;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int run = (int)(i / per);
        const int j = (int)(i - (int64_t)run * per);
        const int kyc = j % g.Ky, ix = j / g.Ky;
        const int ky_i = compact_to_full(kyc, g.Ny, g.Ky);
        const int64_t o = run * rs + (int64_t)ix * g.Ny + ky_i;
        const double a = kx[ix], b = ky[ky_i];
        const double2 u = ux[o], v = uy[o];
        const double dr = a * u.x + b * v.x, di = a * u.y + b * v.y;
        s0 += dr * dr + di * di;
        s1 += (a * a + b * b) * (u.x * u.x + u.y * u.y + v.x * v.x + v.y * v.y);
    }
    r0[threadIdx.x] = s0;
    r1[threadIdx.x] = s1;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if (threadIdx.x < h) { r0[threadIdx.x] += r0[threadIdx.x + h]; r1[threadIdx.x] += r1[threadIdx.x + h]; }
        __syncthreads();
    }
    if (threadIdx.x == 0) { atomicAdd(out, r0[0]); atomicAdd(out + 1, r1[0]); }
}

static unsigned ew_grid2(int64_t n) {
    int64_t b = (n + 255) / 256;
    if (b > 152 * 16) b = 152 * 16;
    return (unsigned)(b < 1 ? 1 : b);
}

template <int PHYS>
static int nonlinear2_any(const dd_plan* pl, int prec, bool compact, const Work2& w, const void* const* st,
                          int64_t st_rs, cudaStream_t s) {
    if (prec == DD_FP64) return compact ? nonlinear2<double, true, PHYS>(pl, w, st, st_rs, s)
                                        : nonlinear2<double, false, PHYS>(pl, w, st, st_rs, s);
    if (prec == DD_FP32) return compact ? nonlinear2<float, true, PHYS>(pl, w, st, st_rs, s)
                                        : nonlinear2<float, false, PHYS>(pl, w, st, st_rs, s);
    set_error("2D fused physics supports FP64 and FP32 arithmetic");
    return DD_ERR_UNSUPPORTED;
}

// the passes of the low-storage FP32 step: complex64 products out and, with
// compact, complex64 stage states in
static int nonlinear2_lo(int phys, const dd_plan* pl, bool compact, const Work2& w, const void* const* st,
                         int64_t st_rs, cudaStream_t s) {
    if (phys == PHYS_HYDRO_DIV)
        return compact ? nonlinear2<float, true, PHYS_HYDRO_DIV, float>(pl, w, st, st_rs, s)
                       : nonlinear2<float, false, PHYS_HYDRO_DIV, float>(pl, w, st, st_rs, s);
    return compact ? nonlinear2<float, true, PHYS_BOUSS_DIV, float>(pl, w, st, st_rs, s)
                   : nonlinear2<float, false, PHYS_BOUSS_DIV, float>(pl, w, st, st_rs, s);
}

static size_t work2_bytes(int prec, const Geo2& g, int nrun) {
    size_t b = 0;
    DD_PREC_DISPATCH(prec, T, b = Work2::bytes<T>(g, nrun));
    return b;
}

static int nonlinear2_phys(int phys, const dd_plan* pl, int prec, bool compact, const Work2& w,
                           const void* const* st, int64_t st_rs, cudaStream_t s) {
    if (phys == PHYS_HYDRO) return nonlinear2_any<PHYS_HYDRO>(pl, prec, compact, w, st, st_rs, s);
    if (phys == PHYS_HYDRO_DIV) return nonlinear2_any<PHYS_HYDRO_DIV>(pl, prec, compact, w, st, st_rs, s);
    if (phys == PHYS_BOUSS_DIV) return nonlinear2_any<PHYS_BOUSS_DIV>(pl, prec, compact, w, st, st_rs, s);
    return nonlinear2_any<PHYS_BOUSS>(pl, prec, compact, w, st, st_rs, s);
}

static void fill_common(Stage2Args& a, const dd_plan* p, int phys, const double* pp, const double* inv_k2,
                        int nrun, const Work2& w, int prec) {
    a.g = p->g2; a.kx = p->kx; a.ky = p->ky; a.inv_k2 = inv_k2; a.intk = inv_k2 != nullptr;
    a.kxf = p->kxf; a.kyf = p->kyf;
    a.phys = phys; a.nrun = nrun;
    if (pp) { a.pp.g = pp[0]; a.pp.alpha_t = pp[1]; a.pp.beta = pp[2]; a.pp.dir = (int)pp[3]; }
    const int no = phys == PHYS_HYDRO || phys == PHYS_HYDRO_DIV ? 2 : (phys == PHYS_BOUSS ? 3 : 4);
    for (int f = 0; f < no; f++)
        DD_PREC_DISPATCH(prec, T, a.nc.p[f] = (void*)w.NC<T>(f));
    a.nc_rs = (int64_t)w.kc; a.c_rs = (int64_t)w.kc;
}

static int check2(const dd_plan* p, int phys, int nrun, const double* pp) {
    DD_CHECK_ARG(p && p->ndim == 2, "plan must be 2D");
    DD_CHECK_ARG(phys >= PHYS_HYDRO && phys <= PHYS_BOUSS_DIV,
                 "physics must be 0 (hydro), 1 (Boussinesq), 2 or 3 (the same in divergence form)");
    DD_CHECK_ARG(nrun >= 1 && nrun <= 65535, "nrun must be in [1, 65535]");
    if (p2_bouss(phys)) {
        DD_CHECK_ARG(pp, "Boussinesq parameters required");
        DD_CHECK_ARG(pp[3] == 0. || pp[3] == 1., "boussinesq direction must be 0 (x) or 1 (y) in 2D");
    }
    return DD_OK;
}

}  // namespace dd

using namespace dd;

extern "C" {

int dd_rhs2d_workspace_size(const dd_plan* p, int nrun, int precision, size_t* bytes) {
    DD_CHECK_ARG(p && bytes && p->ndim == 2 && nrun >= 1, "dd_rhs2d_workspace_size: bad arguments");
    DD_CHECK_ARG(precision >= DD_FP64 && precision <= DD_DF64, "bad precision");
    *bytes = work2_bytes(precision, p->g2, nrun);
    return DD_OK;
}

int dd_rhs2d(const dd_plan* p, int phys, const double* params, int nrun, const void* const* state, int64_t state_rs,
             void* const* deriv, int64_t deriv_rs, const double* inv_k2, int precision, int zero_nonkept, void* work,
             size_t work_bytes, void* stream) {
    DD_TRY(check2(p, phys, nrun, params));
    DD_CHECK_ARG(state && deriv && work, "dd_rhs2d: null pointer");
    const int nf = p2_bouss(phys) ? 3 : 2;
    for (int c = 0; c < nf; c++) DD_CHECK_ARG(state[c] && deriv[c], "dd_rhs2d: null field pointer %d", c);
    DD_CHECK_ARG(precision >= DD_FP64 && precision <= DD_DF64, "bad precision");
    const size_t need = work2_bytes(precision, p->g2, nrun);
    DD_CHECK_ARG(work_bytes >= need, "workspace too small: %zu < %zu", work_bytes, need);
    cudaStream_t st = (cudaStream_t)stream;
    Work2 w{(size_t)p->g2.wcount(), (size_t)p->g2.Kx * p->g2.Ky, nrun, (char*)work};
    DD_TRY(nonlinear2_phys(phys, p, precision, false, w, state, state_rs, st));
    Stage2Args a{};
    fill_common(a, p, phys, params, inv_k2, nrun, w, precision);
    for (int c = 0; c < nf; c++) { a.rin.p[c] = state[c]; a.deriv.p[c] = deriv[c]; }
    a.rin_rs = state_rs; a.rin_compact = 0; a.d_rs = deriv_rs; a.mode = 0; a.y_rs = 0;
    if (zero_nonkept) {
        Ptrs d{};
        for (int c = 0; c < nf; c++) d.p[c] = deriv[c];
        DD_KT("zero_nonkept2", st, k_zero_nonkept2_all<<<dim3(ew_grid2(p->g2.kcount() * nrun), nf), 256, 0, st>>>(
                                       p->g2, d, deriv_rs, nrun));
        DD_LAUNCH_CHECK();
    }
    return launch_stage2<0>(a, ew_grid2((int64_t)p->g2.Kx * p->g2.Ky * nrun), "stage2d", st);
}

int dd_rk2mid_step2d(const dd_plan* p, int phys, const double* params, int nrun, void* const* state,
                     int64_t state_rs, const double* inv_k2, const void* const* tab_half,
                     const void* const* tab_full, const double* nu, int viscosity_order, double dt,
                     int precision, const int* nonkept_flag, void* work, size_t work_bytes, void* stream) {
    DD_TRY(check2(p, phys, nrun, params));
    DD_CHECK_ARG(state && work && nu, "dd_rk2mid_step2d: null pointer");
    DD_CHECK_ARG(viscosity_order >= 1, "viscosity_order must be >= 1");
    const int nf = p2_bouss(phys) ? 3 : 2;
    for (int c = 0; c < nf; c++) DD_CHECK_ARG(state[c], "dd_rk2mid_step2d: null field pointer %d", c);
    DD_CHECK_ARG(precision >= DD_FP64 && precision <= DD_DF64, "bad precision");
    const bool intk = inv_k2 != nullptr;
    DD_CHECK_ARG(!intk || (tab_half && tab_full), "phi tables required with integer wavenumbers");
    const size_t need = work2_bytes(precision, p->g2, nrun);
    DD_CHECK_ARG(work_bytes >= need, "workspace too small: %zu < %zu", work_bytes, need);
    cudaStream_t st = (cudaStream_t)stream;
    Work2 w{(size_t)p->g2.wcount(), (size_t)p->g2.Kx * p->g2.Ky, nrun, (char*)work};
    Stage2Args a{};
    fill_common(a, p, phys, params, inv_k2, nrun, w, precision);
    a.vo = viscosity_order;
    // FP32 transforms in divergence form: the low-storage step (complex64
    // products, stage derivative and stage state; FP64 state)
    const bool lo = p2_div(phys) && precision == DD_FP32;
    if (lo)
        for (int f = 0; f < 4; f++) a.nc.p[f] = w.NCf(f);
    for (int c = 0; c < nf; c++) {
        a.y.p[c] = state[c];
        a.nu[c] = nu[c];
        if (lo) { a.ys.p[c] = w.YSf(c); a.k1.p[c] = w.K1f(c); }
        else DD_PREC_DISPATCH(precision, T, a.ys.p[c] = (void*)w.YS<T>(c); a.k1.p[c] = (void*)w.K1<T>(c));
    }
    a.y_rs = state_rs;
    const unsigned nb = ew_grid2((int64_t)p->g2.Kx * p->g2.Ky * nrun);
    // stage 1: k1 = N(y); y2 = etd1(y, k1, dt/2)            (time_step.py:286-294)
    if (lo) DD_TRY(nonlinear2_lo(phys, p, false, w, (const void* const*)state, state_rs, st));
    else DD_TRY(nonlinear2_phys(phys, p, precision, false, w, (const void* const*)state, state_rs, st));
    for (int c = 0; c < nf; c++) { a.rin.p[c] = state[c]; a.tab[c] = intk ? (const double4*)tab_half[c] : nullptr; }
    a.rin_rs = state_rs; a.rin_compact = 0; a.h = dt / 2.; a.mode = 1;
    if (lo) DD_TRY(launch_stage2_lo<1>(a, nb, st));
    else DD_TRY(launch_stage2<1>(a, nb, "rk2mid_stage2d", st));
    // stage 2: k2 = N(y2); y = etd2rk2(y, k1, k2, dt)       (time_step.py:297-305)
    const void* ysp[3] = {a.ys.p[0], a.ys.p[1], a.ys.p[2]};
    if (lo) DD_TRY(nonlinear2_lo(phys, p, true, w, ysp, (int64_t)w.kc, st));
    else DD_TRY(nonlinear2_phys(phys, p, precision, true, w, ysp, (int64_t)w.kc, st));
    for (int c = 0; c < nf; c++) { a.rin.p[c] = ysp[c]; a.tab[c] = intk ? (const double4*)tab_full[c] : nullptr; }
    a.rin_rs = (int64_t)w.kc; a.rin_compact = 1; a.h = dt; a.mode = 2;
    if (lo) DD_TRY(launch_stage2_lo<2>(a, nb, st));
    else DD_TRY(launch_stage2<2>(a, nb, "rk2mid_stage2d", st));
    if (!nonkept_flag || *nonkept_flag) {
        DD_KT("decay_nonkept2", st, k_decay_nonkept2<<<ew_grid2(p->g2.kcount() * nrun), 256, 0, st>>>(
                                        p->g2, a.y, state_rs, nf, nrun, p->kx, p->ky, a));
        DD_LAUNCH_CHECK();
    }
    return DD_OK;
}

int dd_divergence_sums2d(const dd_plan* p, int nrun, const void* ux, const void* uy, int64_t run_stride, double* out,
                         void* stream) {
    DD_CHECK_ARG(p && p->ndim == 2, "dd_divergence_sums2d: plan must be 2D");
    DD_CHECK_ARG(ux && uy && out && nrun >= 1, "dd_divergence_sums2d: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    DD_CUDA(cudaMemsetAsync(out, 0, 2 * sizeof(double), st));
    const Geo2& g = p->g2;
    const int64_t n = (int64_t)g.Kx * g.Ky * nrun;
    const unsigned nb = (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 4);
    DD_KT("div_sums2", st, k_div_sums2<<<nb, 256, 0, st>>>(g, p->kx, p->ky, (const double2*)ux, (const double2*)uy,
                                                          run_stride, nrun, out));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

}  // extern "C"
