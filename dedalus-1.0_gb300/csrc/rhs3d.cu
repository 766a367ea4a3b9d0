// Fused 3D right-hand sides and RK4 step: projection/stage kernels, drivers and
// the C ABI.  The transform passes and their instantiations are in
// rhs3d_impl.cuh / rhs3d_<precision>.cu.
#include "rhs3d_impl.cuh"
#include "les.cuh"

namespace dd {

DD_RHS3D_INSTANTIATE(extern, double)
DD_RHS3D_INSTANTIATE(extern, float)
DD_RHS3D_INSTANTIATE_LO(extern, P3_HYDRO_DIV)
DD_RHS3D_INSTANTIATE_LO(extern, P3_MHD_DIV)
DD_RHS3D_INSTANTIATE_PH(extern, df64, P3_HYDRO)

// ------------------------------------------------------------------ pass 6
struct ProjArgs {
    Geo3 g;
    const double* kx; const double* ky; const double* kz;
    const double* inv_k2;   // 1/k2 per integer q (q = 0 -> 1), or null
    int intk;               // wavenumbers are integers (q tables valid)
    const float* kxf = nullptr; const float* kyf = nullptr; const float* kzf = nullptr;   // float copies
};

__device__ __forceinline__ void kept_index(const Geo3& g, int64_t i, int& kyc, int& kzc, int& ix) {
    ix = (int)(i % g.Kx);
    const int64_t r = i / g.Kx;
    kzc = (int)(r % g.Kz);
    kyc = (int)(r / g.Kz);
}

// div = ((i kx Nx) + i ky Ny) + i kz Nz; phi = -(div * (1/k2)); N_i -= i k_i phi
__device__ __forceinline__ void project(double2& nx, double2& ny, double2& nz, double kxv, double kyv,
                                        double kzv, double s) {
    const double2 dx = ideriv(nx, kxv), dy = ideriv(ny, kyv), dz = ideriv(nz, kzv);
    const double2 dv = make_double2(radd(radd(dx.x, dy.x), dz.x), radd(radd(dx.y, dy.y), dz.y));
    const double2 ph = make_double2(-rmul(dv.x, s), -rmul(dv.y, s));
    const double2 gx = ideriv(ph, kxv), gy = ideriv(ph, kyv), gz = ideriv(ph, kzv);
    nx = make_double2(rsub(nx.x, gx.x), rsub(nx.y, gx.y));
    ny = make_double2(rsub(ny.x, gy.x), rsub(ny.y, gy.y));
    nz = make_double2(rsub(nz.x, gz.x), rsub(nz.y, gz.y));
}

// The same projection with fused multiply-adds: c = (k . N) / k^2, N -= k c
// (i k_i (-(i k . N) / k^2) = k_i (k . N) / k^2).  Used inside the fused step.
__device__ __forceinline__ void project_fma(double2& nx, double2& ny, double2& nz, double kxv, double kyv,
                                            double kzv, double s) {
    const double cr = fma(kzv, nz.x, fma(kyv, ny.x, kxv * nx.x)) * s;
    const double ci = fma(kzv, nz.y, fma(kyv, ny.y, kxv * nx.y)) * s;
    nx = make_double2(fma(-kxv, cr, nx.x), fma(-kxv, ci, nx.y));
    ny = make_double2(fma(-kyv, cr, ny.x), fma(-kyv, ci, ny.y));
    nz = make_double2(fma(-kzv, cr, nz.x), fma(-kzv, ci, nz.y));
}

// curlX of a k-space vector (physics.py:394-396), in place.
__device__ __forceinline__ void curl_k(double2& vx, double2& vy, double2& vz, double kxv, double kyv, double kzv) {
    const double2 a0 = ideriv(vz, kyv), b0 = ideriv(vy, kzv);
    const double2 a1 = ideriv(vx, kzv), b1 = ideriv(vz, kxv);
    const double2 a2 = ideriv(vy, kxv), b2 = ideriv(vx, kyv);
    vx = make_double2(a0.x - b0.x, a0.y - b0.y);
    vy = make_double2(a1.x - b1.x, a1.y - b1.y);
    vz = make_double2(a2.x - b2.x, a2.y - b2.y);
}

__device__ __forceinline__ double k2_of(const ProjArgs& a, int ix, int ky_i, int kz_i) {
    const double kxv = a.kx[ix], kyv = a.ky[ky_i], kzv = a.kz[kz_i];
    // ((0 + ky^2) + kz^2) + kx^2 (representations.py:434-436, k dict order y, z, x)
    return radd(radd(rmul(kyv, kyv), rmul(kzv, kzv)), rmul(kxv, kxv));
}

__device__ __forceinline__ double inv_k2_of(const ProjArgs& a, double k2, int& q) {
    q = a.intk ? (int)k2 : 0;
    if (a.intk && a.inv_k2) return a.inv_k2[q];
    return rdiv(1., k2 == 0. ? 1. : k2);
}

// N_i = -i k_j T_ij from the five divergence-form products at entry i (order
// xx - zz, yy - zz, xy, xz, yz; T_zz = 0).  -i s = (s.y, -s.x).
__device__ __forceinline__ void div_form(const CPtrs& nc, int64_t i, double kxv, double kyv, double kzv, double2* k) {
    const double2 a = ((const double2*)nc.p[0])[i], b = ((const double2*)nc.p[1])[i];
    const double2 c = ((const double2*)nc.p[2])[i], d = ((const double2*)nc.p[3])[i];
    const double2 e = ((const double2*)nc.p[4])[i];
    const double sxr = fma(kzv, d.x, fma(kyv, c.x, kxv * a.x)), sxi = fma(kzv, d.y, fma(kyv, c.y, kxv * a.y));
    const double syr = fma(kzv, e.x, fma(kyv, b.x, kxv * c.x)), syi = fma(kzv, e.y, fma(kyv, b.y, kxv * c.y));
    const double szr = fma(kyv, e.x, kxv * d.x), szi = fma(kyv, e.y, kxv * d.y);
    k[0] = make_double2(sxi, -sxr);
    k[1] = make_double2(syi, -syr);
    k[2] = make_double2(szi, -szr);
}

// Unprojected nonlinear term of every state component at kept entry i.
template <int PH>
__device__ __forceinline__ void load_nc(const CPtrs& nc, int64_t i, double kxv, double kyv, double kzv, double2* k) {
    if constexpr (PH == P3_HYDRO_DIV) {
        div_form(nc, i, kxv, kyv, kzv, k);
    } else if constexpr (PH == P3_MHD_DIV) {
        div_form(nc, i, kxv, kyv, kzv, k);      // momentum from products 0..4
#pragma unroll
        for (int c = 3; c < 6; c++) k[c] = ((const double2*)nc.p[c + 2])[i];   // u x B
    } else {
#pragma unroll
        for (int c = 0; c < Phys3<PH>::NO; c++) k[c] = ((const double2*)nc.p[c])[i];
    }
}

// RHS of every state component at one kept entry from the compact products.
template <int PH>
__device__ __forceinline__ void rhs_at(const CPtrs& nc, int64_t i, double kxv, double kyv, double kzv, double s,
                                       double2* k) {
    load_nc<PH>(nc, i, kxv, kyv, kzv, k);
    project(k[0], k[1], k[2], kxv, kyv, kzv, s);
    if constexpr (p3_mhd(PH)) curl_k(k[3], k[4], k[5], kxv, kyv, kzv);
}

template <int PH>
__global__ void k_project_to_deriv3(ProjArgs a, CPtrs nc, Ptrs deriv) {
    const Geo3& g = a.g;
    const int64_t n = (int64_t)g.Ky * g.Kz * g.Kx;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int kyc, kzc, ix, q;
        kept_index(g, i, kyc, kzc, ix);
        const int ky_i = compact_to_full(kyc, g.Ny, g.Ky), kz_i = compact_to_full(kzc, g.Nz, g.Kz);
        const double s = inv_k2_of(a, k2_of(a, ix, ky_i, kz_i), q);
        double2 k[6];
        rhs_at<PH>(nc, i, a.kx[ix], a.ky[ky_i], a.kz[kz_i], s, k);
        const int64_t o = ((int64_t)ky_i * g.Nz + kz_i) * g.Nh + ix;
#pragma unroll
        for (int c = 0; c < Phys3<PH>::NF; c++) ((double2*)deriv.p[c])[o] = k[c];
    }
}

// One RK4 stage (time_step.py:426-483 as restated; see the oracle):
//   stage 1: tot = k*(1/6);  y1 = etd1(y, k, dt/2)
//   stage 2: tot += k*(1/3); y2 = etd1(y, k, dt/2)
//   stage 3: tot += k*(1/3); y3 = etd1(y, k, dt)
//   stage 4: tot += k*(1/6); y  = etd1(y, tot, dt)
// y (state) is full layout; stage states and tot are compact.
struct RK4Args {
    ProjArgs pa;
    CPtrs nc;            // unprojected products, compact
    Ptrs y;              // state, full layout (written at stage 4)
    Ptrs ys;             // next stage state, compact (stages 1-3)
    Ptrs tot;            // accumulated increment, compact
    const double4* tab[2];  // phi table per vector group for this stage's step, or null
    double coeff[2];     // diffusivity per group (nu, eta), used when tab is null
    double h; int vo;
    double w;            // increment weight: 1/6 or 1/3
    int stage;
};

__device__ __forceinline__ void phis_for(const RK4Args& a, int grp, int q, double k2, double& Z, double& f0,
                                         double& f1) {
    if (a.tab[grp]) {
        const double4 t = a.tab[grp][q];
        Z = t.x; f0 = t.y; f1 = t.z;
    } else {
        const double k2v = a.vo == 1 ? k2 : (a.vo == 2 ? rmul(k2, k2) : pow(k2, (double)a.vo));
        Z = rmul(-rmul(a.coeff[grp], k2v), a.h);
        double f2;
        f0 = 1.; f1 = 1.;
        if (Z != 0.) etd_phis<3>(Z, f0, f1, f2);
    }
}

template <int PH>
__global__ void k_rk4_stage3(RK4Args a) {
    const Geo3& g = a.pa.g;
    constexpr int NF = Phys3<PH>::NF, NG = Phys3<PH>::NG;
    const int n = g.Ky * g.Kz * g.Kx;      // < 2^31 for every supported grid
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int ix = i % g.Kx, r = i / g.Kx;
        const int kzc = r % g.Kz, kyc = r / g.Kz;
        const int ky_i = compact_to_full(kyc, g.Ny, g.Ky), kz_i = compact_to_full(kzc, g.Nz, g.Kz);
        const double kxv = a.pa.kx[ix], kyv = a.pa.ky[ky_i], kzv = a.pa.kz[kz_i];
        const double k2 = k2_of(a.pa, ix, ky_i, kz_i);
        int q;
        const double s = inv_k2_of(a.pa, k2, q);
        double2 k[6];
        load_nc<PH>(a.nc, i, kxv, kyv, kzv, k);
        project_fma(k[0], k[1], k[2], kxv, kyv, kzv, s);
        if constexpr (p3_mhd(PH)) curl_k(k[3], k[4], k[5], kxv, kyv, kzv);
        double f0[NG], f1h[NG];
#pragma unroll
        for (int grp = 0; grp < NG; grp++) {
            double Z, f1;
            phis_for(a, grp, q, k2, Z, f0[grp], f1);
            f1h[grp] = f1 * a.h;
        }
        const int64_t o = ((int64_t)ky_i * g.Nz + kz_i) * g.Nh + ix;
#pragma unroll
        for (int c = 0; c < NF; c++) {
            const int grp = c / 3;
            double2 t;
            if (a.stage == 1) t = make_double2(k[c].x * a.w, k[c].y * a.w);
            else {
                t = ((const double2*)a.tot.p[c])[i];
                t = make_double2(fma(k[c].x, a.w, t.x), fma(k[c].y, a.w, t.y));
            }
            const double2 y0 = ((const double2*)a.y.p[c])[o];
            if (a.stage < 4) {
                ((double2*)a.tot.p[c])[i] = t;
                ((double2*)a.ys.p[c])[i] = etd1_fma(y0, k[c], f0[grp], f1h[grp]);
            } else {
                ((double2*)a.y.p[c])[o] = etd1_fma(y0, t, f0[grp], f1h[grp]);
            }
        }
    }
}

// The same stage for the FP32 step in divergence form, with low-storage
// intermediates: the compact products, the stage states and the increment are
// complex64, and N = -i k_j T_ij, its projection (and, for MHD, the curl of
// u x B) are formed in FP32, the precision the FP32 transforms give them; the
// ETD update of the complex128 state -- phi functions, y phi0 + h phi1 N --
// stays FP64.  Same stage definitions as k_rk4_stage3.
__device__ __forceinline__ float2 fderiv(float2 a, float k) { return make_float2(-(a.y * k), a.x * k); }

template <int PH>
__global__ void k_rk4_stage3_lo(RK4Args a) {
    static_assert(PH == P3_HYDRO_DIV || PH == P3_MHD_DIV, "low-storage stages are for the divergence forms");
    const Geo3& g = a.pa.g;
    constexpr int NF = Phys3<PH>::NF, NG = Phys3<PH>::NG;
    const int n = g.Ky * g.Kz * g.Kx;      // < 2^31 for every supported grid
    // integer wavenumbers with their q tables: k^2 is an integer below 2^24,
    // exact in float, and the phi values come from the tables
    const bool tabs = a.pa.intk && a.pa.inv_k2 && a.tab[0] && (NG == 1 || a.tab[1]);
    const float w = (float)a.w, hf = (float)a.h;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int ix = i % g.Kx, r = i / g.Kx;
        const int kzc = r % g.Kz, kyc = r / g.Kz;
        const int ky_i = compact_to_full(kyc, g.Ny, g.Ky), kz_i = compact_to_full(kzc, g.Nz, g.Kz);
        const float kx = a.pa.kxf[ix], ky = a.pa.kyf[ky_i], kz = a.pa.kzf[kz_i];
        int q = 0;
        double k2 = 0.;
        float s;
        if (tabs) {
            q = (int)((ky * ky + kz * kz) + kx * kx);
            s = (float)a.pa.inv_k2[q];
        } else {
            k2 = k2_of(a.pa, ix, ky_i, kz_i);
            s = (float)inv_k2_of(a.pa, k2, q);
        }
        const float2* P[8];
#pragma unroll
        for (int c = 0; c < Phys3<PH>::NO; c++) P[c] = (const float2*)a.nc.p[c];
        // N = -i k_j T_ij from xx - zz, yy - zz, xy, xz, yz; -i s = (s.y, -s.x)
        const float2 A = P[0][i], B = P[1][i], Cc = P[2][i], D = P[3][i], E = P[4][i];
        const float sxr = fmaf(kz, D.x, fmaf(ky, Cc.x, kx * A.x)), sxi = fmaf(kz, D.y, fmaf(ky, Cc.y, kx * A.y));
        const float syr = fmaf(kz, E.x, fmaf(ky, B.x, kx * Cc.x)), syi = fmaf(kz, E.y, fmaf(ky, B.y, kx * Cc.y));
        const float szr = fmaf(ky, E.x, kx * D.x), szi = fmaf(ky, E.y, kx * D.y);
        float2 k[6];
        k[0] = make_float2(sxi, -sxr); k[1] = make_float2(syi, -syr); k[2] = make_float2(szi, -szr);
        // projection: N -= k (k . N) / k^2
        const float cr = fmaf(kz, k[2].x, fmaf(ky, k[1].x, kx * k[0].x)) * s;
        const float ci = fmaf(kz, k[2].y, fmaf(ky, k[1].y, kx * k[0].y)) * s;
        k[0] = make_float2(fmaf(-kx, cr, k[0].x), fmaf(-kx, ci, k[0].y));
        k[1] = make_float2(fmaf(-ky, cr, k[1].x), fmaf(-ky, ci, k[1].y));
        k[2] = make_float2(fmaf(-kz, cr, k[2].x), fmaf(-kz, ci, k[2].y));
        if constexpr (p3_mhd(PH)) {   // curl (u x B)
            const float2 vx = P[5][i], vy = P[6][i], vz = P[7][i];
            const float2 a0 = fderiv(vz, ky), b0 = fderiv(vy, kz), a1 = fderiv(vx, kz), b1 = fderiv(vz, kx);
            const float2 a2 = fderiv(vy, kx), b2 = fderiv(vx, ky);
            k[3] = make_float2(a0.x - b0.x, a0.y - b0.y);
            k[4] = make_float2(a1.x - b1.x, a1.y - b1.y);
            k[5] = make_float2(a2.x - b2.x, a2.y - b2.y);
        }
        double f0[NG], f1[NG];
#pragma unroll
        for (int grp = 0; grp < NG; grp++) {
            if (tabs) {
                const double* t = reinterpret_cast<const double*>(a.tab[grp] + q);
                f0[grp] = t[1];
                f1[grp] = t[2];
            } else {
                double Z;
                phis_for(a, grp, q, k2, Z, f0[grp], f1[grp]);
            }
        }
        const int64_t o = ((int64_t)ky_i * g.Nz + kz_i) * g.Nh + ix;
        if (a.stage < 4) {
            // stages 1-3: the accumulated increment and the next stage state,
            // both float, in float arithmetic: ys = f0 y + h phi1 N
            float f0f[NG], f1hf[NG];
#pragma unroll
            for (int grp = 0; grp < NG; grp++) { f0f[grp] = (float)f0[grp]; f1hf[grp] = (float)f1[grp] * hf; }
#pragma unroll
            for (int c = 0; c < NF; c++) {
                const int grp = c / 3;
                float2 t;
                if (a.stage == 1) t = make_float2(k[c].x * w, k[c].y * w);
                else {
                    t = ((const float2*)a.tot.p[c])[i];
                    t = make_float2(fmaf(k[c].x, w, t.x), fmaf(k[c].y, w, t.y));
                }
                ((float2*)a.tot.p[c])[i] = t;
                const double2 y0 = ((const double2*)a.y.p[c])[o];
                const float yr = (float)y0.x, yi = (float)y0.y;
                ((float2*)a.ys.p[c])[i] =
                    make_float2(fmaf(f1hf[grp], k[c].x, yr * f0f[grp]), fmaf(f1hf[grp], k[c].y, yi * f0f[grp]));
            }
        } else {
            // stage 4: the FP64 state update y = f0 y + h phi1 (sum of the weighted N)
#pragma unroll
            for (int c = 0; c < NF; c++) {
                const int grp = c / 3;
                float2 t = ((const float2*)a.tot.p[c])[i];
                t = make_float2(fmaf(k[c].x, w, t.x), fmaf(k[c].y, w, t.y));
                const double2 y0 = ((const double2*)a.y.p[c])[o];
                ((double2*)a.y.p[c])[o] =
                    etd1_fma(y0, make_double2((double)t.x, (double)t.y), f0[grp], f1[grp] * a.h);
            }
        }
    }
}

// Non-kept modes of the state see no nonlinear forcing: y <- etd1(y, 0, dt).
__global__ void k_decay_nonkept3(RK4Args a, int ncomp) {
    const Geo3& g = a.pa.g;
    const int64_t n = g.kcount();
    const int c = blockIdx.y;
    if (c >= ncomp) return;
    const int grp = c / 3;
    double2* Y = (double2*)a.y.p[c];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int ix = (int)(i % g.Nh);
        const int64_t r = i / g.Nh;
        const int kz_i = (int)(r % g.Nz), ky_i = (int)(r / g.Nz);
        if (ix <= g.Mx && kept_full(ky_i, g.Ny, g.My) && kept_full(kz_i, g.Nz, g.Mz)) continue;
        const double2 y0 = Y[i];
        if (y0.x == 0. && y0.y == 0.) continue;
        const double k2 = k2_of(a.pa, ix, ky_i, kz_i);
        const int q = a.pa.intk ? (int)k2 : 0;
        double Z, f0, f1;
        phis_for(a, grp, q, k2, Z, f0, f1);
        Y[i] = etd1_entry(y0, make_double2(0., 0.), Z, f0, f1, a.h);
    }
}

// Any non-zero entry outside the kept set? (flag[0] |= 1)
__global__ void k_any_nonkept3(Geo3 g, CPtrs y, int ncomp, int* flag) {
    const int64_t n = g.kcount();
    int found = 0;
#pragma unroll
    for (int c = 0; c < DD_MAXF; c++) {   // constant indices keep y in the parameter space
        if (c >= ncomp) break;
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

// Zero every non-kept entry of full-layout arrays (grid.y = component).
__global__ void k_dealias3_all(Geo3 g, Ptrs k) {
    double2* K = (double2*)pick_ptr<DD_MAXF>(k.p, (int)blockIdx.y);
    const int64_t n = g.kcount();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int ix = (int)(i % g.Nh);
        const int64_t r = i / g.Nh;
        const int kz_i = (int)(r % g.Nz), ky_i = (int)(r / g.Nz);
        if (ix > g.Mx || !kept_full(ky_i, g.Ny, g.My) || !kept_full(kz_i, g.Nz, g.Mz)) K[i] = make_double2(0., 0.);
    }
}

// Sums over the kept modes of a full-layout velocity: out[0] += |k . u|^2,
// out[1] += |k|^2 |u|^2 (block partials, then one atomic add per block).
__global__ void __launch_bounds__(256) k_div_sums3(Geo3 g, const double* kx, const double* ky, const double* kz,
                                                    CPtrs u, double* out) {
    __shared__ double r0[256], r1[256];
    const int n = g.Ky * g.Kz * g.Kx;      // < 2^31 for every supported grid
    double s0 = 0., s1 = 0.;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int ix = i % g.Kx, r = i / g.Kx;
        const int kzc = r % g.Kz, kyc = r / g.Kz;
        const int ky_i = compact_to_full(kyc, g.Ny, g.Ky), kz_i = compact_to_full(kzc, g.Nz, g.Kz);
        const int64_t o = ((int64_t)ky_i * g.Nz + kz_i) * g.Nh + ix;
        const double kv[3] = {kx[ix], ky[ky_i], kz[kz_i]};
        double dr = 0., di = 0., uu = 0.;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const double2 v = ((const double2*)u.p[a])[o];
            dr += kv[a] * v.x;
            di += kv[a] * v.y;
            uu += v.x * v.x + v.y * v.y;
        }
        s0 += dr * dr + di * di;
        s1 += (kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2]) * uu;
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

static unsigned ew_grid(int64_t n) {
    int64_t b = (n + 255) / 256;
    if (b > 152 * 16) b = 152 * 16;
    return (unsigned)(b < 1 ? 1 : b);
}

template <int PH>
static int nonlinear3_any(const dd_plan* pl, int prec, bool compact, const void* const* u, double inv_fpr,
                          const Work3& w, cudaStream_t st) {
    if (prec == DD_FP64) return compact ? nonlinear3<double, true, PH>(pl, u, inv_fpr, w, st)
                                        : nonlinear3<double, false, PH>(pl, u, inv_fpr, w, st);
    if (prec == DD_FP32) return compact ? nonlinear3<float, true, PH>(pl, u, inv_fpr, w, st)
                                        : nonlinear3<float, false, PH>(pl, u, inv_fpr, w, st);
    if constexpr (PH == P3_HYDRO) {
        return compact ? nonlinear3<df64, true, PH>(pl, u, inv_fpr, w, st)
                       : nonlinear3<df64, false, PH>(pl, u, inv_fpr, w, st);
    }
    set_error("double-float arithmetic is implemented for 3D hydro in rotational form only");
    return DD_ERR_UNSUPPORTED;
}

// Workspace bytes and compact-region pointers for precision code prec.
static size_t work3_bytes(int prec, const Geo3& g, int ni, int no, int nf, bool step) {
    size_t b = 0;
    DD_PREC_DISPATCH(prec, T, b = Work3::bytes<T>(g, ni, no, nf, step));
    return b;
}
static void* work3_nc(int prec, const Work3& w, int f) {
    void* p = nullptr;
    DD_PREC_DISPATCH(prec, T, p = (void*)w.NC<T>(f));
    return p;
}
static void* work3_tot(int prec, const Work3& w, int f) {
    void* p = nullptr;
    DD_PREC_DISPATCH(prec, T, p = (void*)w.TOT<T>(f));
    return p;
}
static void* work3_ys(int prec, const Work3& w, int f) {
    void* p = nullptr;
    DD_PREC_DISPATCH(prec, T, p = (void*)w.YS<T>(f));
    return p;
}

// 1 / (4 pi rho0): fpr = 4 * np.pi * rho0 (physics.py:791); numpy divides a
// complex array by a float by multiplying with the reciprocal.
static double inv_fpr_of(const double* params) { return 1.0 / ((4.0 * M_PI) * params[0]); }

template <int PH>
static int rhs3(const dd_plan* p, const double* params, const void* const* u, void* const* deriv,
                const double* inv_k2, int prec, int zero_nonkept, void* work, size_t wb, cudaStream_t st,
                const LesHook* les = nullptr) {
    using P = Phys3<PH>;
    const Geo3& g = p->g3;
    const size_t need = work3_bytes(prec, g, P::NI, P::NO, P::NF, false);
    DD_CHECK_ARG(wb >= need, "workspace too small: %zu < %zu", wb, need);
    const double inv_fpr = p3_mhd(PH) ? inv_fpr_of(params) : 0.;
    Work3 w = make_work<PH>(g, work);
    DD_TRY(nonlinear3_any<PH>(p, prec, false, u, inv_fpr, w, st));
    ProjArgs pa{g, p->kx, p->ky, p->kz, inv_k2, inv_k2 != nullptr};
    CPtrs nc{}; Ptrs d{};
    for (int c = 0; c < P::NO; c++) nc.p[c] = work3_nc(prec, w, c);
    for (int c = 0; c < P::NF; c++) d.p[c] = deriv[c];
    if (les) {
        void* ncp[3] = {(void*)nc.p[0], (void*)nc.p[1], (void*)nc.p[2]};
        DD_TRY(les_closure_add(p, *les, prec, false, u, ncp, st));
    }
    if (zero_nonkept) {
        DD_KT("zero_nonkept3", st, k_dealias3_all<<<dim3(ew_grid(g.kcount()), P::NF), 256, 0, st>>>(g, d));
        DD_LAUNCH_CHECK();
    }
    DD_KT("project3", st, k_project_to_deriv3<PH><<<ew_grid((int64_t)g.Ky * g.Kz * g.Kx), 256, 0, st>>>(pa, nc, d));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

template <int PH>
static int rk4_3(const dd_plan* p, const double* params, void* const* u, const double* inv_k2,
                 const void* const* tab_half, const void* const* tab_full, const double* coeff, int vo, double dt,
                 int prec, const int* nonkept_flag, void* work, size_t wb, cudaStream_t st,
                 const LesHook* les = nullptr) {
    using P = Phys3<PH>;
    const Geo3& g = p->g3;
    const size_t need = work3_bytes(prec, g, P::NI, P::NO, P::NF, true);
    DD_CHECK_ARG(wb >= need, "workspace too small: %zu < %zu", wb, need);
    const bool intk = inv_k2 != nullptr;
    DD_CHECK_ARG(!intk || (tab_half && tab_full), "phi tables required with integer wavenumbers");
    const double inv_fpr = p3_mhd(PH) ? inv_fpr_of(params) : 0.;
    Work3 w = make_work<PH>(g, work);
    RK4Args a{};
    a.pa = ProjArgs{g, p->kx, p->ky, p->kz, inv_k2, intk, p->kxf, p->kyf, p->kzf};
    a.vo = vo;
    for (int grp = 0; grp < P::NG; grp++) a.coeff[grp] = coeff[grp];
    const void* ysc[6] = {};
    for (int c = 0; c < P::NO; c++) a.nc.p[c] = work3_nc(prec, w, c);
    for (int c = 0; c < P::NF; c++) {
        a.y.p[c] = u[c];
        a.ys.p[c] = work3_ys(prec, w, c);
        a.tot.p[c] = work3_tot(prec, w, c);
        ysc[c] = a.ys.p[c];
    }
    const double hs[4] = {dt / 2., dt / 2., dt, dt};
    const double ws[4] = {1. / 6., 1. / 3., 1. / 3., 1. / 6.};
    const unsigned nb = ew_grid((int64_t)w.kc);
    // FP32 transforms in divergence form without a closure: low-storage stages
    constexpr bool lo_ok = PH == P3_HYDRO_DIV || PH == P3_MHD_DIV;
    const bool lo = lo_ok && prec == DD_FP32 && les == nullptr;
    for (int s = 1; s <= 4; s++) {
        if constexpr (lo_ok) {
            if (lo) {
                if (s == 1) DD_TRY((nonlinear3<float, false, PH, float>(p, (const void* const*)u, inv_fpr, w, st)));
                else DD_TRY((nonlinear3<float, true, PH, float>(p, ysc, inv_fpr, w, st)));
                a.stage = s; a.h = hs[s - 1]; a.w = ws[s - 1];
                for (int grp = 0; grp < P::NG; grp++)
                    a.tab[grp] = intk ? (const double4*)(s <= 2 ? tab_half[grp] : tab_full[grp]) : nullptr;
                DD_KT("rk4_stage3_lo", st, k_rk4_stage3_lo<PH><<<nb, 256, 0, st>>>(a));
                DD_LAUNCH_CHECK();
                continue;
            }
        }
        DD_TRY(nonlinear3_any<PH>(p, prec, s > 1, s == 1 ? (const void* const*)u : ysc, inv_fpr, w, st));
        if (les) {
            void* ncp[3] = {(void*)a.nc.p[0], (void*)a.nc.p[1], (void*)a.nc.p[2]};
            DD_TRY(les_closure_add(p, *les, prec, s > 1, s == 1 ? (const void* const*)u : ysc, ncp, st));
        }
        a.stage = s; a.h = hs[s - 1]; a.w = ws[s - 1];
        for (int grp = 0; grp < P::NG; grp++)
            a.tab[grp] = intk ? (const double4*)(s <= 2 ? tab_half[grp] : tab_full[grp]) : nullptr;
        DD_KT("rk4_stage3", st, k_rk4_stage3<PH><<<nb, 256, 0, st>>>(a));
        DD_LAUNCH_CHECK();
    }
    if (!nonkept_flag || *nonkept_flag) {
        DD_KT("decay_nonkept3", st, k_decay_nonkept3<<<dim3(ew_grid(g.kcount()), P::NF), 256, 0, st>>>(a, P::NF));
        DD_LAUNCH_CHECK();
    }
    return DD_OK;
}

}  // namespace dd

using namespace dd;

static int check3(const dd_plan* p, int phys, const double* params, const void* const* a, const void* const* b) {
    DD_CHECK_ARG(p, "null plan");
    DD_CHECK_ARG(p->ndim == 3, "plan is not 3D");
    DD_CHECK_ARG(phys >= P3_HYDRO && phys <= P3_MHD_DIV,
                 "physics must be 0 (hydro), 1 (MHD), 2 (hydro, divergence form) or 3 (MHD, divergence form)");
    DD_CHECK_ARG(!p3_mhd(phys) || (params && params[0] > 0.), "MHD needs params = {rho0 > 0}");
    const int nf = p3_mhd(phys) ? 6 : 3;
    DD_CHECK_ARG(a, "null field array");
    for (int c = 0; c < nf; c++) {
        DD_CHECK_ARG(a[c], "null field pointer %d", c);
        if (b) DD_CHECK_ARG(b[c], "null output field pointer %d", c);
    }
    return DD_OK;
}

extern "C" {

int dd_rhs3d_workspace_size(const dd_plan* p, int physics, int precision, size_t* bytes) {
    DD_CHECK_ARG(p && bytes && p->ndim == 3, "dd_rhs3d_workspace_size: bad arguments");
    DD_CHECK_ARG(physics >= P3_HYDRO && physics <= P3_MHD_DIV,
                 "physics must be 0 (hydro), 1 (MHD), 2 (hydro, divergence form) or 3 (MHD, divergence form)");
    DD_CHECK_ARG(precision >= DD_FP64 && precision <= DD_DF64, "bad precision");
    if (physics == P3_HYDRO) *bytes = work3_bytes(precision, p->g3, 6, 3, 3, true);
    else if (physics == P3_MHD) *bytes = work3_bytes(precision, p->g3, 12, 6, 6, true);
    else if (physics == P3_HYDRO_DIV) *bytes = work3_bytes(precision, p->g3, 5, 5, 3, true);
    else *bytes = work3_bytes(precision, p->g3, 8, 8, 6, true);
    return DD_OK;
}

int dd_rhs3d(const dd_plan* p, int physics, const double* params, const void* const* state, void* const* deriv,
             const double* inv_k2, int precision, int zero_nonkept, void* work, size_t work_bytes, void* stream) {
    DD_TRY(check3(p, physics, params, state, (const void* const*)deriv));
    DD_CHECK_ARG(work, "null workspace");
    DD_CHECK_ARG(precision >= DD_FP64 && precision <= DD_DF64, "bad precision");
    cudaStream_t st = (cudaStream_t)stream;
    if (physics == P3_HYDRO)
        return rhs3<P3_HYDRO>(p, params, state, deriv, inv_k2, precision, zero_nonkept, work, work_bytes, st);
    if (physics == P3_HYDRO_DIV)
        return rhs3<P3_HYDRO_DIV>(p, params, state, deriv, inv_k2, precision, zero_nonkept, work, work_bytes, st);
    if (physics == P3_MHD_DIV)
        return rhs3<P3_MHD_DIV>(p, params, state, deriv, inv_k2, precision, zero_nonkept, work, work_bytes, st);
    return rhs3<P3_MHD>(p, params, state, deriv, inv_k2, precision, zero_nonkept, work, work_bytes, st);
}

int dd_rk4_step3d(const dd_plan* p, int physics, const double* params, void* const* state, const double* inv_k2,
                  const void* const* tab_half, const void* const* tab_full, const double* coeff,
                  int viscosity_order, double dt, int precision, const int* nonkept_flag, void* work,
                  size_t work_bytes, void* stream) {
    DD_TRY(check3(p, physics, params, (const void* const*)state, nullptr));
    DD_CHECK_ARG(work && coeff, "null workspace or coefficients");
    DD_CHECK_ARG(precision >= DD_FP64 && precision <= DD_DF64, "bad precision");
    DD_CHECK_ARG(viscosity_order >= 1, "viscosity_order must be >= 1");
    cudaStream_t st = (cudaStream_t)stream;
    if (physics == P3_HYDRO)
        return rk4_3<P3_HYDRO>(p, params, state, inv_k2, tab_half, tab_full, coeff, viscosity_order, dt, precision,
                               nonkept_flag, work, work_bytes, st);
    if (physics == P3_HYDRO_DIV)
        return rk4_3<P3_HYDRO_DIV>(p, params, state, inv_k2, tab_half, tab_full, coeff, viscosity_order, dt,
                                   precision, nonkept_flag, work, work_bytes, st);
    if (physics == P3_MHD_DIV)
        return rk4_3<P3_MHD_DIV>(p, params, state, inv_k2, tab_half, tab_full, coeff, viscosity_order, dt,
                                 precision, nonkept_flag, work, work_bytes, st);
    return rk4_3<P3_MHD>(p, params, state, inv_k2, tab_half, tab_full, coeff, viscosity_order, dt, precision,
                         nonkept_flag, work, work_bytes, st);
}

// Closed LES (hydro with the learned closure term in every RHS evaluation).
static size_t les_total_bytes(const dd_plan* p, int prec) {
    return Work3::up256(work3_bytes(prec, p->g3, 6, 3, 3, true)) + les_work_bytes(p);
}

static LesHook les_hook(const dd_plan* p, int prec, const dd_closure* cl, void* work, size_t wb) {
    const size_t off = Work3::up256(work3_bytes(prec, p->g3, 6, 3, 3, true));
    return LesHook{cl, (char*)work + off, wb > off ? wb - off : 0};
}

static int les_check(const dd_plan* p, const dd_closure* cl, int precision, void* work, size_t wb) {
    DD_CHECK_ARG(p && p->ndim == 3, "the closed LES needs a 3D plan");
    DD_CHECK_ARG(cl && cl->wbf16 && cl->params && cl->norm, "closure weights, parameters and norm are required");
    DD_CHECK_ARG(precision == DD_FP64 || precision == DD_FP32, "precision must be DD_FP64 or DD_FP32");
    DD_CHECK_ARG(work, "null workspace");
    DD_CHECK_ARG(wb >= les_total_bytes(p, precision), "workspace too small: %zu < %zu", wb,
                 les_total_bytes(p, precision));
    return DD_OK;
}

int dd_les_workspace_size(const dd_plan* p, int precision, size_t* bytes) {
    DD_CHECK_ARG(p && bytes && p->ndim == 3, "dd_les_workspace_size: bad arguments");
    DD_CHECK_ARG(precision == DD_FP64 || precision == DD_FP32, "precision must be DD_FP64 or DD_FP32");
    *bytes = les_total_bytes(p, precision);
    return DD_OK;
}

int dd_les_rhs3d(const dd_plan* p, const void* const* state, void* const* deriv, const double* inv_k2, int precision,
                 int zero_nonkept, const dd_closure* cl, void* work, size_t work_bytes, void* stream) {
    DD_TRY(check3(p, P3_HYDRO, nullptr, state, (const void* const*)deriv));
    DD_TRY(les_check(p, cl, precision, work, work_bytes));
    const LesHook h = les_hook(p, precision, cl, work, work_bytes);
    return rhs3<P3_HYDRO>(p, nullptr, state, deriv, inv_k2, precision, zero_nonkept, work, work_bytes,
                          (cudaStream_t)stream, &h);
}

int dd_les_rk4_step3d(const dd_plan* p, void* const* state, const double* inv_k2, const void* const* tab_half,
                      const void* const* tab_full, const double* coeff, int viscosity_order, double dt, int precision,
                      const int* nonkept_flag, const dd_closure* cl, void* work, size_t work_bytes, void* stream) {
    DD_TRY(check3(p, P3_HYDRO, nullptr, (const void* const*)state, nullptr));
    DD_TRY(les_check(p, cl, precision, work, work_bytes));
    DD_CHECK_ARG(coeff, "null coefficients");
    DD_CHECK_ARG(viscosity_order >= 1, "viscosity_order must be >= 1");
    const LesHook h = les_hook(p, precision, cl, work, work_bytes);
    return rk4_3<P3_HYDRO>(p, nullptr, state, inv_k2, tab_half, tab_full, coeff, viscosity_order, dt, precision,
                           nonkept_flag, work, work_bytes, (cudaStream_t)stream, &h);
}

// Hydro-only forms of the first interface.
int dd_hydro3d_workspace_size(const dd_plan* p, int precision, size_t* bytes) {
    return dd_rhs3d_workspace_size(p, P3_HYDRO, precision, bytes);
}

int dd_hydro3d_rhs(const dd_plan* p, const void* const* u, void* const* deriv, const double* inv_k2,
                   int precision, int zero_nonkept, void* work, size_t work_bytes, void* stream) {
    return dd_rhs3d(p, P3_HYDRO, nullptr, u, deriv, inv_k2, precision, zero_nonkept, work, work_bytes, stream);
}

int dd_hydro3d_rk4_step(const dd_plan* p, void* const* u, const double* inv_k2, const void* tab_half,
                        const void* tab_full, double nu, int viscosity_order, double dt, int precision,
                        int* nonkept_flag, void* work, size_t work_bytes, void* stream) {
    const void* th[1] = {tab_half};
    const void* tf[1] = {tab_full};
    const double c[1] = {nu};
    return dd_rk4_step3d(p, P3_HYDRO, nullptr, u, inv_k2, th, tf, c, viscosity_order, dt, precision, nonkept_flag,
                         work, work_bytes, stream);
}

int dd_divergence_sums(const dd_plan* p, const void* const* u, double* out, void* stream) {
    DD_CHECK_ARG(p && u && out, "dd_divergence_sums: null pointer");
    DD_CHECK_ARG(p->ndim == 3, "dd_divergence_sums: 3D plans only");
    CPtrs uc{};
    for (int a = 0; a < 3; a++) { DD_CHECK_ARG(u[a], "null velocity %d", a); uc.p[a] = u[a]; }
    cudaStream_t st = (cudaStream_t)stream;
    DD_CUDA(cudaMemsetAsync(out, 0, 2 * sizeof(double), st));
    const Geo3& g = p->g3;
    const int64_t nk = (int64_t)g.Ky * g.Kz * g.Kx;
    const unsigned nb = (unsigned)std::min<int64_t>((nk + 255) / 256, 152 * 4);
    DD_KT("div_sums3", st, k_div_sums3<<<nb, 256, 0, st>>>(g, p->kx, p->ky, p->kz, uc, out));
    DD_LAUNCH_CHECK();
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
