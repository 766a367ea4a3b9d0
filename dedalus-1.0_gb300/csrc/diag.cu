// Diagnostics on the device: the reference's volume averages in k-space
// (dedalus/analysis/volume_average.py:71-118, 254-300) and the binned power
// spectrum (dedalus/analysis/analysis_set.py:778-815).
//
// Sums are accumulated in FP64 with a compensated (Neumaier) running sum per
// thread, merged with error-free two-sums through the warp and the block, and
// the per-block partials are reduced in a fixed order by a second kernel, so
// the result is deterministic and its error is independent of the number of
// entries to first order.
#include "dd_common.cuh"
#include "geometry.cuh"
#include "plan.cuh"

namespace dd {

enum {
    DIAG_ENERGY = 0,       // 1/2 sum_c |u_c|^2                  (ekin, emag, volume_average.py:109-118)
    DIAG_DISSIPATION = 1,  // 1/2 |curl u|^2 (times 2 nu by the caller; 254-265)
    DIAG_ENSTROPHY2D = 2,  // 1/2 |d_x u_y - d_y u_x|^2        (191-200)
    DIAG_HELICITY = 3,     // Re(u . conj(curl u))
    DIAG_DIV_L2 = 4,       // |sum_i i k_i u_i|^2
    DIAG_DIV_ABS_SUM = 5,  // |sum_i i k_i u_i|, unweighted     (divergence_sum, 288-295)
    DIAG_SQUARE = 6,       // |u_c|^2 of one component          (ux2, temp2, ...)
};

struct KSum {
    double s, c;  // value = s + c
};

__device__ __forceinline__ void ksum_add(KSum& a, double x) {
    const double t = a.s + x;
    if (fabs(a.s) >= fabs(x)) a.c += (a.s - t) + x;
    else a.c += (x - t) + a.s;
    a.s = t;
}

__device__ __forceinline__ KSum ksum_merge(KSum a, KSum b) {
    const double t = a.s + b.s;
    const double bb = t - a.s;
    const double e = (a.s - (t - bb)) + (b.s - bb);
    return KSum{t, e + a.c + b.c};
}

__device__ __forceinline__ double2 ik(double2 a, double k) { return make_double2(-(a.y * k), a.x * k); }

// Per-entry quantity for one k index.
struct DiagArgs {
    int ndim, kind, ncomp;
    Geo3 g3; Geo2 g2;
    const double* kx; const double* ky; const double* kz;
    CPtrs f;  // components (x, y[, z]) or the single component for DIAG_SQUARE / ENERGY of a scalar
};

__device__ __forceinline__ double entry_value(const DiagArgs& a, int64_t i, int ix, int iy, int iz, double& w) {
    double2 u[3];
    for (int c = 0; c < a.ncomp; c++) u[c] = ((const double2*)a.f.p[c])[i];
    w = (ix > 0) ? 2.0 : 1.0;   // Hermitian weight (kx > 0 entries stand for two modes)
    const double kxv = a.kx[ix], kyv = a.ky[iy], kzv = a.ndim == 3 ? a.kz[iz] : 0.0;
    switch (a.kind) {
        case DIAG_ENERGY: {
            double s = 0.;
            for (int c = 0; c < a.ncomp; c++) s += 0.5 * (u[c].x * u[c].x + u[c].y * u[c].y);
            return s;
        }
        case DIAG_SQUARE:
            return u[0].x * u[0].x + u[0].y * u[0].y;
        case DIAG_DISSIPATION:
        case DIAG_HELICITY: {
            // curl: (d_y u_z - d_z u_y, d_z u_x - d_x u_z, d_x u_y - d_y u_x)
            const double2 a0 = ik(u[2], kyv), b0 = ik(u[1], kzv), a1 = ik(u[0], kzv), b1 = ik(u[2], kxv);
            const double2 a2 = ik(u[1], kxv), b2 = ik(u[0], kyv);
            const double2 w0 = make_double2(a0.x - b0.x, a0.y - b0.y), w1 = make_double2(a1.x - b1.x, a1.y - b1.y);
            const double2 w2 = make_double2(a2.x - b2.x, a2.y - b2.y);
            if (a.kind == DIAG_DISSIPATION)
                return 0.5 * ((w0.x * w0.x + w0.y * w0.y) + (w1.x * w1.x + w1.y * w1.y) + (w2.x * w2.x + w2.y * w2.y));
            return (u[0].x * w0.x + u[0].y * w0.y) + (u[1].x * w1.x + u[1].y * w1.y) + (u[2].x * w2.x + u[2].y * w2.y);
        }
        case DIAG_ENSTROPHY2D: {
            const double2 a0 = ik(u[1], kxv), b0 = ik(u[0], kyv);
            const double2 wz = make_double2(a0.x - b0.x, a0.y - b0.y);
            return 0.5 * (wz.x * wz.x + wz.y * wz.y);
        }
        case DIAG_DIV_L2:
        case DIAG_DIV_ABS_SUM: {
            double2 d = ik(u[0], kxv);
            const double2 dy = ik(u[1], kyv);
            d = make_double2(d.x + dy.x, d.y + dy.y);
            if (a.ncomp == 3) { const double2 dz = ik(u[2], kzv); d = make_double2(d.x + dz.x, d.y + dz.y); }
            if (a.kind == DIAG_DIV_ABS_SUM) { w = 1.0; return sqrt(d.x * d.x + d.y * d.y); }
            return d.x * d.x + d.y * d.y;
        }
    }
    return 0.;
}

__device__ __forceinline__ void unravel(const DiagArgs& a, int64_t i, int& ix, int& iy, int& iz) {
    if (a.ndim == 3) {  // [ky][kz][kx]
        ix = (int)(i % a.g3.Nh);
        const int64_t r = i / a.g3.Nh;
        iz = (int)(r % a.g3.Nz);
        iy = (int)(r / a.g3.Nz);
    } else {            // [kx][ky]
        iy = (int)(i % a.g2.Ny);
        ix = (int)(i / a.g2.Ny);
        iz = 0;
    }
}

__device__ KSum block_merge(KSum v) {
    for (int o = 16; o > 0; o >>= 1) {
        KSum u{__shfl_down_sync(0xffffffffu, v.s, o), __shfl_down_sync(0xffffffffu, v.c, o)};
        v = ksum_merge(v, u);
    }
    __shared__ KSum sh[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    KSum r{0., 0.};
    if (threadIdx.x == 0)
        for (int j = 0; j < (int)(blockDim.x + 31) / 32; j++) r = ksum_merge(r, sh[j]);
    return r;
}

__global__ void k_diag_partial(DiagArgs a, int64_t n, KSum* part) {
    KSum acc{0., 0.};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int ix, iy, iz;
        unravel(a, i, ix, iy, iz);
        double w;
        const double v = entry_value(a, i, ix, iy, iz, w);
        ksum_add(acc, w * v);
    }
    const KSum r = block_merge(acc);
    if (threadIdx.x == 0) part[blockIdx.x] = r;
}

__global__ void k_diag_final(const KSum* part, int nb, double* out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    KSum r{0., 0.};
    for (int j = 0; j < nb; j++) r = ksum_merge(r, part[j]);
    out[0] = r.s + r.c;
}

// Spectrum: power = sum_c |u_c|^2; p1d = norm * power * 4 pi k^2 (3D) or 2 pi k (2D);
// entry goes to bin i when kbottom[i] <= |k| < ktop[i] and p1d != 0.
__global__ void k_spectrum_partial(DiagArgs a, int64_t n, double norm, int nbins, const double* kb, const double* kt,
                                   double dk, double* psum, double* pcnt) {
    extern __shared__ double sbin[];   // [nbins] sums, [nbins] counts
    for (int j = threadIdx.x; j < 2 * nbins; j += blockDim.x) sbin[j] = 0.;
    __syncthreads();
    const double geo = a.ndim == 3 ? 4. * M_PI : 2. * M_PI;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int ix, iy, iz;
        unravel(a, i, ix, iy, iz);
        double power = 0.;
        for (int c = 0; c < a.ncomp; c++) {
            const double2 u = ((const double2*)a.f.p[c])[i];
            power += u.x * u.x + u.y * u.y;
        }
        const double kxv = a.kx[ix], kyv = a.ky[iy];
        double k2;   // k dict order: (y, z, x) in 3D, (x, y) in 2D (representations.py:434-436)
        if (a.ndim == 3) {
            const double kzv = a.kz[iz];
            k2 = __dadd_rn(__dadd_rn(__dmul_rn(kyv, kyv), __dmul_rn(kzv, kzv)), __dmul_rn(kxv, kxv));
        } else {
            k2 = __dadd_rn(__dmul_rn(kxv, kxv), __dmul_rn(kyv, kyv));
        }
        const double kmag = sqrt(k2);
        const double p1d = a.ndim == 3 ? __dmul_rn(__dmul_rn(norm * power, geo), __dmul_rn(kmag, kmag))
                                       : __dmul_rn(__dmul_rn(norm * power, geo), kmag);
        if (p1d == 0.) continue;
        const int i0 = (int)floor(kmag / dk);
        for (int b = i0 - 1; b <= i0 + 1; b++) {
            if (b < 0 || b >= nbins) continue;
            if (kmag >= kb[b] && kmag < kt[b]) {
                atomicAdd(&sbin[b], p1d);
                atomicAdd(&sbin[nbins + b], 1.0);
            }
        }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < nbins; j += blockDim.x) {
        psum[(int64_t)blockIdx.x * nbins + j] = sbin[j];
        pcnt[(int64_t)blockIdx.x * nbins + j] = sbin[nbins + j];
    }
}

__global__ void k_spectrum_final(const double* psum, const double* pcnt, int nb, int nbins, double* out_sum,
                                 double* out_cnt) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nbins) return;
    double s = 0., c = 0., cnt = 0.;
    for (int b = 0; b < nb; b++) {
        const double x = psum[(int64_t)b * nbins + j];
        const double t = s + x;
        c += (fabs(s) >= fabs(x)) ? (s - t) + x : (x - t) + s;
        s = t;
        cnt += pcnt[(int64_t)b * nbins + j];
    }
    out_sum[j] = s + c;
    out_cnt[j] = cnt;
}

static const int kDiagBlocks = 152 * 4;

static void fill_args(DiagArgs& a, const dd_plan* p, int kind, int ncomp, const void* const* comps) {
    a.ndim = p->ndim; a.kind = kind; a.ncomp = ncomp;
    a.g3 = p->g3; a.g2 = p->g2;
    a.kx = p->kx; a.ky = p->ky; a.kz = p->kz;
    for (int c = 0; c < ncomp; c++) a.f.p[c] = comps[c];
}

}  // namespace dd

using namespace dd;

extern "C" {

int dd_diag_workspace_size(const dd_plan* p, int nbins, size_t* bytes) {
    DD_CHECK_ARG(p && bytes && nbins >= 0, "dd_diag_workspace_size: bad arguments");
    *bytes = sizeof(KSum) * kDiagBlocks + 2 * sizeof(double) * (size_t)kDiagBlocks * (nbins > 0 ? nbins : 1);
    return DD_OK;
}

int dd_volume_average(const dd_plan* p, int kind, int ncomp, const void* const* comps, double* out, void* work,
                      size_t work_bytes, void* stream) {
    DD_CHECK_ARG(p && comps && out && work, "dd_volume_average: null pointer");
    DD_CHECK_ARG(kind >= DIAG_ENERGY && kind <= DIAG_SQUARE, "dd_volume_average: unknown kind %d", kind);
    DD_CHECK_ARG(ncomp >= 1 && ncomp <= 3, "dd_volume_average: ncomp must be 1..3");
    const int need = (kind == DIAG_DISSIPATION || kind == DIAG_HELICITY) ? 3
                   : (kind == DIAG_ENSTROPHY2D) ? 2
                   : (kind == DIAG_DIV_L2 || kind == DIAG_DIV_ABS_SUM) ? p->ndim : 1;
    DD_CHECK_ARG(ncomp >= need, "dd_volume_average: kind %d needs %d components", kind, need);
    DD_CHECK_ARG(!(kind == DIAG_DISSIPATION || kind == DIAG_HELICITY) || p->ndim == 3, "kind %d is 3D only", kind);
    DD_CHECK_ARG(kind != DIAG_ENSTROPHY2D || p->ndim == 2, "enstrophy is 2D only");
    for (int c = 0; c < ncomp; c++) DD_CHECK_ARG(comps[c], "null component %d", c);
    DD_CHECK_ARG(work_bytes >= sizeof(KSum) * kDiagBlocks, "workspace too small");
    DiagArgs a{};
    fill_args(a, p, kind, ncomp, comps);
    const int64_t n = p->ndim == 3 ? p->g3.kcount() : p->g2.kcount();
    cudaStream_t st = (cudaStream_t)stream;
    DD_KT("diag_partial", st, k_diag_partial<<<kDiagBlocks, 256, 0, st>>>(a, n, (KSum*)work));
    DD_LAUNCH_CHECK();
    DD_KT("diag_final", st, k_diag_final<<<1, 32, 0, st>>>((const KSum*)work, kDiagBlocks, out));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

int dd_spectrum(const dd_plan* p, int ncomp, const void* const* comps, double norm, int nbins, const double* kbottom,
                const double* ktop, double dk, double* out_sum, double* out_count, void* work, size_t work_bytes,
                void* stream) {
    DD_CHECK_ARG(p && comps && kbottom && ktop && out_sum && out_count && work, "dd_spectrum: null pointer");
    DD_CHECK_ARG(ncomp >= 1 && ncomp <= 3, "dd_spectrum: ncomp must be 1..3");
    DD_CHECK_ARG(nbins >= 2 && nbins <= 4096, "dd_spectrum: nbins must be in [2, 4096]");
    const size_t need = 2 * sizeof(double) * (size_t)kDiagBlocks * nbins;
    DD_CHECK_ARG(work_bytes >= need, "workspace too small: %zu < %zu", work_bytes, need);
    for (int c = 0; c < ncomp; c++) DD_CHECK_ARG(comps[c], "null component %d", c);
    DiagArgs a{};
    fill_args(a, p, DIAG_ENERGY, ncomp, comps);
    const int64_t n = p->ndim == 3 ? p->g3.kcount() : p->g2.kcount();
    cudaStream_t st = (cudaStream_t)stream;
    double* psum = (double*)work;
    double* pcnt = psum + (size_t)kDiagBlocks * nbins;
    DD_CHECK_ARG(dk > 0., "dd_spectrum: bin width must be positive");
    const size_t smem = 2 * sizeof(double) * nbins;
    DD_KT("spectrum_partial", st,
          k_spectrum_partial<<<kDiagBlocks, 256, smem, st>>>(a, n, norm, nbins, kbottom, ktop, dk, psum, pcnt));
    DD_LAUNCH_CHECK();
    DD_KT("spectrum_final", st,
          k_spectrum_final<<<(nbins + 127) / 128, 128, 0, st>>>(psum, pcnt, kDiagBlocks, nbins, out_sum, out_count));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

}  // extern "C"
