// Learned subgrid closure of the 3D LES (les.cuh): velocity gradients at the
// grid points, the fused normalise -> MLP -> stress kernel, the closure term
// added to the unprojected nonlinear products, and the kernels that make the
// training data from a DNS (products, sharp spectral truncation, samples).
#include "fft_impl.cuh"
#include "les.cuh"
#include "mlp.cuh"

namespace dd {

DD_FFT_INSTANTIATE(extern, double)
DD_FFT_INSTANTIATE(extern, float)
DD_FFT_INSTANTIATE_X(extern, float, float)

static inline size_t up256(size_t b) { return (b + 255) & ~(size_t)255; }

static inline unsigned les_grid(int64_t n, int per = 256) {
    int64_t b = (n + per - 1) / per;
    if (b > 152 * 16) b = 152 * 16;
    return (unsigned)(b < 1 ? 1 : b);
}

// kept entry i of the compact order [kyc][kzc][kx] -> full-layout indices
__device__ __forceinline__ void les_kept(const Geo3& g, int64_t i, int& ky_i, int& kz_i, int& ix, int64_t& o) {
    ix = (int)(i % g.Kx);
    const int64_t r = i / g.Kx;
    const int kzc = (int)(r % g.Kz), kyc = (int)(r / g.Kz);
    ky_i = compact_to_full(kyc, g.Ny, g.Ky);
    kz_i = compact_to_full(kzc, g.Nz, g.Kz);
    o = ((int64_t)ky_i * g.Nz + kz_i) * g.Nh + ix;
}

// (i k) a
__device__ __forceinline__ double2 les_ik(double2 a, double k) { return make_double2(-(k * a.y), k * a.x); }

// gk[3 a + j] = i k_j y_a on the kept modes (full layout out).
template <bool COMPACT>
__global__ void k_les_grad9(Geo3 g, const double* kx, const double* ky, const double* kz, CPtrs y, Ptrs gk) {
    const int64_t n = (int64_t)g.Ky * g.Kz * g.Kx;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int ky_i, kz_i, ix;
        int64_t o;
        les_kept(g, i, ky_i, kz_i, ix, o);
        const double kv[3] = {kx[ix], ky[ky_i], kz[kz_i]};
        const int64_t src = COMPACT ? i : o;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const double2 u = ((const double2*)y.p[a])[src];
#pragma unroll
            for (int j = 0; j < 3; j++) ((double2*)gk.p[3 * a + j])[o] = les_ik(u, kv[j]);
        }
    }
}

// Closure network at the grid points, one warp per tile of 16 points, with no
// shared memory but the weights.  A lane loads its own entries of the first
// product's A fragment straight from the gradient fields (lane 4 g + t holds
// points g and g + 8 of the tile, inputs 2t, 2t + 1, 2t + 8, 2t + 9; input 8
// is the ninth gradient and input 9 the width, so only t = 0 has the upper
// pair), and the accumulator fragments of two adjacent 8-column tiles of a
// layer are, rounded to BF16, the A fragment of one 16-column k tile of the
// next layer: the activations never leave registers.  The products, their
// order and the rounding points are those of mlp_forward16.  The next tile's
// gradients are loaded while the current tile computes.  tau may alias
// gx[0..5]: a warp has all inputs of a tile in registers before it writes that
// tile's outputs, and tiles are disjoint.
constexpr int LES_WARPS = 4;

struct LesMlpSmem {
    bf16 w1[MLP_H * LDI];
    bf16 w2[MLP_H * LDH];
    bf16 w3[8 * LDH];         // the 8 output rows in use
    float b1[MLP_H], b2[MLP_H], b3[MLP_OUT];
};

// B fragments from a row-major [out][in] BF16 weight matrix in shared memory
// by ldmatrix (lane 4 g + t receives row g, columns 2t, 2t + 1 of each 8 x 8
// matrix; lane 8 i + r gives the address of row r of matrix i).  Row strides
// are multiples of 16 bytes.
__device__ __forceinline__ void les_ldsm(uint32_t r[4], const bf16* q) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(q);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}
// rows [n0, n0 + 8), k tiles [k0, k0 + 16) and [k0 + 16, k0 + 32): r[0..1]
// and r[2..3] are the B fragments of the two k tiles
__device__ __forceinline__ void les_ldb_k32(uint32_t r[4], const bf16* w, int ld, int n0, int k0) {
    const int lane = threadIdx.x & 31;
    les_ldsm(r, w + (n0 + (lane & 7)) * ld + k0 + 8 * (lane >> 3));
}
// rows [n0, n0 + 8) and [n0 + 8, n0 + 16), k tile [k0, k0 + 16): r[0..1] and
// r[2..3] are the B fragments of the two n tiles
__device__ __forceinline__ void les_ldb_n16(uint32_t r[4], const bf16* w, int ld, int n0, int k0) {
    const int lane = threadIdx.x & 31;
    les_ldsm(r, w + (n0 + 8 * (lane >> 4) + (lane & 7)) * ld + k0 + 8 * ((lane >> 3) & 1));
}

__device__ __forceinline__ void les_mma(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
    const uint32_t b[2] = {b0, b1};
    mma_bf16_16816(c, a, b);
}

// Hidden activations of an accumulator tile (rows g, g + 8; columns n + 2t,
// n + 2t + 1 with bias + n the bias pair): lo/hi = the A-fragment registers of
// rows g and g + 8 in the next layer.
__device__ __forceinline__ void les_act(const float c[4], const float* bias, uint32_t& lo, uint32_t& hi) {
    const float2 bb = *reinterpret_cast<const float2*>(bias);
    lo = pack2(__float2bfloat16_rn(tanhf(c[0] + bb.x)), __float2bfloat16_rn(tanhf(c[1] + bb.y)));
    hi = pack2(__float2bfloat16_rn(tanhf(c[2] + bb.x)), __float2bfloat16_rn(tanhf(c[3] + bb.y)));
}

template <typename GT, typename TT>
__global__ void __launch_bounds__(32 * LES_WARPS) k_les_mlp(CPtrs gx, Ptrs tau, int64_t npts, const bf16* wb,
                                                            const float* p, const float* norm, double delta) {
    __shared__ __align__(16) LesMlpSmem s;
    for (int i = threadIdx.x; i < MLP_H * MLP_IN; i += blockDim.x)
        s.w1[(i / MLP_IN) * LDI + i % MLP_IN] = wb[BOFF_W1 + i];
    for (int i = threadIdx.x; i < MLP_H * MLP_H; i += blockDim.x)
        s.w2[(i / MLP_H) * LDH + i % MLP_H] = wb[BOFF_W2 + i];
    for (int i = threadIdx.x; i < 8 * MLP_H; i += blockDim.x)
        s.w3[(i / MLP_H) * LDH + i % MLP_H] = wb[BOFF_W3 + i];
    for (int i = threadIdx.x; i < MLP_H; i += blockDim.x) {
        s.b1[i] = p[OFF_B1 + i];
        s.b2[i] = p[OFF_B2 + i];
    }
    if (threadIdx.x < MLP_OUT) s.b3[threadIdx.x] = p[OFF_B3 + threadIdx.x];
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const bool lead = t == 0;
    // this lane's inputs 2t, 2t + 1 (and 8 for t = 0), their normalisation
    const GT* src0 = (const GT*)pick_ptr<8>(gx.p, 2 * t);
    const GT* src1 = (const GT*)pick_ptr<8>(gx.p, 2 * t + 1);
    const GT* src8 = (const GT*)gx.p[8];
    const float m0 = norm[NORM_IN_MEAN + 2 * t], s0 = norm[NORM_IN_SCALE + 2 * t];
    const float m1 = norm[NORM_IN_MEAN + 2 * t + 1], s1 = norm[NORM_IN_SCALE + 2 * t + 1];
    const float m8 = norm[NORM_IN_MEAN + 8], s8 = norm[NORM_IN_SCALE + 8];
    const bf16 xd = __float2bfloat16_rn(((float)delta - norm[NORM_IN_MEAN + 9]) * norm[NORM_IN_SCALE + 9]);
    // this lane's outputs 2t, 2t + 1 (stresses 0..5: t < 3)
    const bool out = t < 3;
    TT* dst0 = (TT*)pick_ptr<MLP_NOUT>(tau.p, out ? 2 * t : 0);
    TT* dst1 = (TT*)pick_ptr<MLP_NOUT>(tau.p, out ? 2 * t + 1 : 0);
    const float om0 = norm[NORM_OUT_MEAN + 2 * t], os0 = norm[NORM_OUT_SCALE + 2 * t];
    const float om1 = norm[NORM_OUT_MEAN + 2 * t + 1], os1 = norm[NORM_OUT_SCALE + 2 * t + 1];
    const float b30 = s.b3[2 * t], b31 = s.b3[2 * t + 1];
    // the output layer's B fragments (8 x 64) stay in registers
    uint32_t w3[8];
    les_ldb_k32(w3, s.w3, LDH, 0, 0);
    les_ldb_k32(w3 + 4, s.w3, LDH, 0, 32);

    const int64_t ntiles = (npts + 15) / 16;
    const int64_t stride = (int64_t)gridDim.x * LES_WARPS;
    float f[6];
    auto fetch = [&](int64_t tile) {
        const int64_t pa = tile * 16 + g, pb = pa + 8;
        const bool oka = tile < ntiles && pa < npts, okb = tile < ntiles && pb < npts;
        f[0] = oka ? (float)src0[pa] : 0.f;
        f[1] = oka ? (float)src1[pa] : 0.f;
        f[2] = okb ? (float)src0[pb] : 0.f;
        f[3] = okb ? (float)src1[pb] : 0.f;
        f[4] = (lead && oka) ? (float)src8[pa] : 0.f;
        f[5] = (lead && okb) ? (float)src8[pb] : 0.f;
    };
    auto nrm = [](float v, float m, float sc) { return __float2bfloat16_rn((v - m) * sc); };
    int64_t tile = (int64_t)blockIdx.x * LES_WARPS + warp;
    fetch(tile);
    for (; tile < ntiles; tile += stride) {
        uint32_t x[1][4];
        x[0][0] = pack2(nrm(f[0], m0, s0), nrm(f[1], m1, s1));
        x[0][1] = pack2(nrm(f[2], m0, s0), nrm(f[3], m1, s1));
        x[0][2] = lead ? pack2(nrm(f[4], m8, s8), xd) : 0u;   // inputs 10..15 are zero
        x[0][3] = lead ? pack2(nrm(f[5], m8, s8), xd) : 0u;
        fetch(tile + stride);
        // first hidden layer, n tiles in pairs
        uint32_t h1[4][4];
#pragma unroll
        for (int np = 0; np < 4; np++) {
            uint32_t b[4];
            les_ldb_n16(b, s.w1, LDI, 16 * np, 0);
            float c0[4] = {0.f, 0.f, 0.f, 0.f}, c1[4] = {0.f, 0.f, 0.f, 0.f};
            les_mma(c0, x[0], b[0], b[1]);
            les_mma(c1, x[0], b[2], b[3]);
            les_act(c0, s.b1 + 16 * np + 2 * t, h1[np][0], h1[np][1]);
            les_act(c1, s.b1 + 16 * np + 8 + 2 * t, h1[np][2], h1[np][3]);
        }
        // second hidden layer; its n tiles 2 kt, 2 kt + 1 form k tile kt of the
        // output layer, which accumulates as soon as they are done
        float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int kt = 0; kt < 4; kt++) {
            uint32_t h2[4];
#pragma unroll
            for (int hf = 0; hf < 2; hf++) {
                const int nt = 2 * kt + hf;
                float c2[4] = {0.f, 0.f, 0.f, 0.f};
                uint32_t b[4];
                les_ldb_k32(b, s.w2, LDH, 8 * nt, 0);
                les_mma(c2, h1[0], b[0], b[1]);
                les_mma(c2, h1[1], b[2], b[3]);
                les_ldb_k32(b, s.w2, LDH, 8 * nt, 32);
                les_mma(c2, h1[2], b[0], b[1]);
                les_mma(c2, h1[3], b[2], b[3]);
                les_act(c2, s.b2 + 8 * nt + 2 * t, h2[2 * hf], h2[2 * hf + 1]);
            }
            les_mma(c, h2, w3[2 * kt], w3[2 * kt + 1]);
        }
        if (out) {
            const int64_t pa = tile * 16 + g, pb = pa + 8;
            const float y0 = c[0] + b30, y1 = c[1] + b31, y2 = c[2] + b30, y3 = c[3] + b31;
            if (pa < npts) {
                dst0[pa] = (TT)(y0 * os0 + om0);
                dst1[pa] = (TT)(y1 * os1 + om1);
            }
            if (pb < npts) {
                dst0[pb] = (TT)(y2 * os0 + om0);
                dst1[pb] = (TT)(y3 * os1 + om1);
            }
        }
    }
}

// Closure-term weight at |k| = kk: the shell table sw[0..nsw) linearly
// interpolated (entry i at |k| = i, the last entry beyond the table) when sw
// is given, else the band ramp: 0 at |k| <= lo, 1 at |k| >= hi, linear between
// (1 everywhere when hi <= 0).
__device__ __forceinline__ double les_weight(double kk, const double* sw, int nsw, double lo, double hi) {
    if (sw) {
        const int i = (int)kk;
        if (i >= nsw - 1) return sw[nsw - 1];
        const double f = kk - (double)i;
        return sw[i] + f * (sw[i + 1] - sw[i]);
    }
    if (hi > 0.) return kk <= lo ? 0. : (kk >= hi ? 1. : (kk - lo) / (hi - lo));
    return 1.;
}

// nc_i -= w(|k|) i k_j tau_ij on the kept modes; tau spectra in full layout,
// order xx, yy, zz, xy, xz, yz; nc compact complex128; w from les_weight.
__global__ void k_les_add(Geo3 g, const double* kx, const double* ky, const double* kz, CPtrs tk, Ptrs nc,
                          double lo, double hi, const double* sw, int nsw) {
    const int64_t n = (int64_t)g.Ky * g.Kz * g.Kx;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int ky_i, kz_i, ix;
        int64_t o;
        les_kept(g, i, ky_i, kz_i, ix, o);
        const double k0 = kx[ix], k1 = ky[ky_i], k2 = kz[kz_i];
        double w = 1.;
        if (sw || hi > 0.) w = les_weight(sqrt(k0 * k0 + k1 * k1 + k2 * k2), sw, nsw, lo, hi);
        if (w == 0.) continue;
        double2 t[6];
#pragma unroll
        for (int c = 0; c < 6; c++) t[c] = ((const double2*)tk.p[c])[o];
        // rows of tau: (xx, xy, xz), (xy, yy, yz), (xz, yz, zz)
        const int row[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const double2 d0 = les_ik(t[row[a][0]], k0), d1 = les_ik(t[row[a][1]], k1), d2 = les_ik(t[row[a][2]], k2);
            double2* N = (double2*)nc.p[a];
            const double2 v = N[i];
            N[i] = make_double2(v.x - w * ((d0.x + d1.x) + d2.x), v.y - w * ((d0.y + d1.y) + d2.y));
        }
    }
}

__global__ void k_les_products(int64_t npts, CPtrs u, Ptrs out) {
    const int pa[6] = {0, 1, 2, 0, 0, 1}, pb[6] = {0, 1, 2, 1, 2, 2};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npts; i += (int64_t)gridDim.x * blockDim.x) {
        double v[3];
#pragma unroll
        for (int a = 0; a < 3; a++) v[a] = ((const double*)u.p[a])[i];
#pragma unroll
        for (int c = 0; c < 6; c++) ((double*)out.p[c])[i] = v[pa[c]] * v[pb[c]];
    }
}

// Signed wavenumber index m of full index i on an axis of length N, and back.
__device__ __forceinline__ int les_signed(int i, int N) { return i <= N / 2 ? i : i - N; }
__device__ __forceinline__ int les_index(int m, int N) { return m >= 0 ? m : m + N; }

__global__ void k_les_truncate3(Geo3 gs, Geo3 gd, CPtrs s, Ptrs d) {
    const double2* S = (const double2*)s.p[blockIdx.y];
    double2* D = (double2*)d.p[blockIdx.y];
    const int64_t n = gd.kcount();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int ix = (int)(i % gd.Nh);
        const int64_t r = i / gd.Nh;
        const int kz_i = (int)(r % gd.Nz), ky_i = (int)(r / gd.Nz);
        double2 v = make_double2(0., 0.);
        if (ix <= gd.Mx && kept_full(ky_i, gd.Ny, gd.My) && kept_full(kz_i, gd.Nz, gd.Mz)) {
            const int sy = les_index(les_signed(ky_i, gd.Ny), gs.Ny), sz = les_index(les_signed(kz_i, gd.Nz), gs.Nz);
            v = S[((int64_t)sy * gs.Nz + sz) * gs.Nh + ix];
        }
        D[i] = v;
    }
}

__global__ void k_les_band(Geo3 g, const double* kx, const double* ky, const double* kz, Ptrs k, double lo,
                           double hi) {
    double2* K = (double2*)k.p[blockIdx.y];
    const int64_t n = g.kcount();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int ix = (int)(i % g.Nh);
        const int64_t r = i / g.Nh;
        const int kz_i = (int)(r % g.Nz), ky_i = (int)(r / g.Nz);
        double w = 0.;
        if (ix <= g.Mx && kept_full(ky_i, g.Ny, g.My) && kept_full(kz_i, g.Nz, g.Mz)) {
            w = 1.;
            if (hi > 0.) {
                const double kk = sqrt(kx[ix] * kx[ix] + ky[ky_i] * ky[ky_i] + kz[kz_i] * kz[kz_i]);
                w = kk <= lo ? 0. : (kk >= hi ? 1. : (kk - lo) / (hi - lo));
            }
        }
        const double2 v = K[i];
        K[i] = make_double2(v.x * w, v.y * w);
    }
}

__global__ void k_les_samples(int64_t npts, CPtrs gx, CPtrs f, CPtrs fr, double delta, float* raw) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npts; i += (int64_t)gridDim.x * blockDim.x) {
        __align__(16) float r[16];
#pragma unroll
        for (int a = 0; a < 9; a++) r[a] = (float)((const double*)gx.p[a])[i];
        r[9] = (float)delta;
#pragma unroll
        for (int c = 0; c < 6; c++) r[10 + c] = (float)(((const double*)f.p[c])[i] - ((const double*)fr.p[c])[i]);
        float4* dst = reinterpret_cast<float4*>(raw + i * 16);
#pragma unroll
        for (int q = 0; q < 4; q++) dst[q] = reinterpret_cast<const float4*>(r)[q];
    }
}

// Subgrid transfer per kept mode: c[i] = m Re(conj(u_a) (-i k_j tau_ij)_a), m = 2
// for 0 < kx < Nx/2 (the mode and its conjugate), else 1; bin[i] =
// round(|k|) (as a double), -1 beyond the last bin.
__global__ void k_les_transfer_modes(Geo3 g, const double* kx, const double* ky, const double* kz, CPtrs u, CPtrs tk,
                                     int nbins, double* c, double* bin) {
    const int64_t n = (int64_t)g.Ky * g.Kz * g.Kx;
    const int rows[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int ky_i, kz_i, ix;
        int64_t o;
        les_kept(g, i, ky_i, kz_i, ix, o);
        const double kv[3] = {kx[ix], ky[ky_i], kz[kz_i]};
        double t = 0.;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            double fx = 0., fy = 0.;          // F_a = -i k_j tau_aj
#pragma unroll
            for (int j = 0; j < 3; j++) {
                const double2 tv = ((const double2*)tk.p[rows[a][j]])[o];
                fx += kv[j] * tv.y;
                fy -= kv[j] * tv.x;
            }
            const double2 ua = ((const double2*)u.p[a])[o];
            t += ua.x * fx + ua.y * fy;
        }
        const double m = (ix > 0 && 2 * ix < g.Nx) ? 2. : 1.;
        const double kk = sqrt(kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2]);
        const double b = floor(kk + 0.5);
        c[i] = m * t;
        bin[i] = b < (double)nbins ? b : -1.;
    }
}

// out[b] = sum of c[i] over bin[i] == b, one block per bin, fixed order.
__global__ void __launch_bounds__(256) k_les_transfer_bins(int64_t n, const double* c, const double* bin,
                                                           double* out) {
    __shared__ double red[256];
    const double b = (double)blockIdx.x;
    double s = 0.;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x)
        if (bin[i] == b) s += c[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = red[0];
}

// ------------------------------------------------------------- drivers
struct LesWork {
    double2* gk[9];   // gradient spectra, later the stress spectra (0..5)
    double* gx[9];    // gradients at the grid points, later the stresses (0..5)
    float* gxf[9];    // the same region as float fields (FP32 path)
    void* fw;
    size_t fwb;
};

size_t les_work_bytes(const dd_plan* p) {
    const Geo3& g = p->g3;
    return up256(9 * (size_t)g.kcount() * sizeof(double2)) + up256(9 * (size_t)g.xcount() * sizeof(double)) +
           up256(ws_bytes<double>(p, 9));
}

static LesWork les_carve(const dd_plan* p, void* work) {
    const Geo3& g = p->g3;
    LesWork w;
    char* b = (char*)work;
    for (int f = 0; f < 9; f++) w.gk[f] = (double2*)b + f * g.kcount();
    b += up256(9 * (size_t)g.kcount() * sizeof(double2));
    for (int f = 0; f < 9; f++) {
        w.gx[f] = (double*)b + f * g.xcount();
        w.gxf[f] = (float*)b + f * g.xcount();
    }
    b += up256(9 * (size_t)g.xcount() * sizeof(double));
    w.fw = b;
    w.fwb = up256(ws_bytes<double>(p, 9));
    return w;
}

// Gradients at the grid points: into w.gxf as float when xf32 (FP32
// transforms only), else into w.gx as double.
static int les_grads(const dd_plan* p, int prec, bool compact, const void* const* y, const LesWork& w,
                     bool xf32, cudaStream_t st) {
    const Geo3& g = p->g3;
    CPtrs yc{};
    Ptrs gk{};
    for (int a = 0; a < 3; a++) yc.p[a] = y[a];
    for (int f = 0; f < 9; f++) gk.p[f] = w.gk[f];
    const unsigned nb = les_grid((int64_t)g.Ky * g.Kz * g.Kx);
    if (compact) DD_KT("les_grad9", st, k_les_grad9<true><<<nb, 256, 0, st>>>(g, p->kx, p->ky, p->kz, yc, gk));
    else DD_KT("les_grad9", st, k_les_grad9<false><<<nb, 256, 0, st>>>(g, p->kx, p->ky, p->kz, yc, gk));
    DD_LAUNCH_CHECK();
    const void* kin[9];
    for (int f = 0; f < 9; f++) kin[f] = w.gk[f];
    if (prec == DD_FP32 && xf32) return fft_c2r<float, float>(p, 9, kin, w.gxf, w.fw, w.fwb, st);
    if (prec == DD_FP32) return fft_c2r<float>(p, 9, kin, w.gx, w.fw, w.fwb, st);
    return fft_c2r<double>(p, 9, kin, w.gx, w.fw, w.fwb, st);
}

template <typename GT, typename TT>
static int les_mlp(const dd_plan* p, const dd_closure* cl, const GT* const* gxi, TT* const* tau, cudaStream_t st) {
    const int64_t npts = p->g3.xcount();
    CPtrs gx{};
    Ptrs t{};
    for (int f = 0; f < 9; f++) gx.p[f] = gxi[f];
    for (int c = 0; c < 6; c++) t.p[c] = tau[c];
    // one resident wave of blocks, each warp looping over its tiles
    static std::atomic<int> resident{0};
    int nres = resident.load();
    if (nres == 0) {
        int dev = 0, sms = 0, occ = 0;
        DD_CUDA(cudaGetDevice(&dev));
        DD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        DD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_les_mlp<GT, TT>, 32 * LES_WARPS, 0));
        nres = sms * (occ > 0 ? occ : 1);
        resident.store(nres);
    }
    const int64_t need = (npts + 16 * LES_WARPS - 1) / (16 * LES_WARPS);
    const unsigned nb = (unsigned)(need < nres ? (need < 1 ? 1 : need) : nres);
    DD_KT("les_mlp", st,
          (k_les_mlp<GT, TT><<<nb, 32 * LES_WARPS, 0, st>>>(gx, t, npts, (const bf16*)cl->wbf16, cl->params, cl->norm,
                                                            cl->delta)));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

int les_closure_add(const dd_plan* p, const LesHook& h, int prec, bool compact, const void* const* y,
                    void* const* nc, cudaStream_t st) {
    DD_CHECK_ARG(h.wb >= les_work_bytes(p), "closure workspace too small");
    const LesWork w = les_carve(p, h.work);
    const bool f32 = prec == DD_FP32;
    DD_TRY(les_grads(p, prec, compact, y, w, f32, st));
    // the stresses overwrite gradients 0..5; k_les_add reads the kept modes
    // only, so the forward transform leaves the rest unwritten
    void* kout[6];
    for (int c = 0; c < 6; c++) kout[c] = w.gk[c];
    if (f32) {
        DD_TRY((les_mlp<float, float>(p, h.cl, w.gxf, w.gxf, st)));
        DD_TRY((fft_r2c<float, float>(p, 6, w.gxf, kout, w.fw, w.fwb, st, false)));
    } else {
        DD_TRY((les_mlp<double, double>(p, h.cl, w.gx, w.gx, st)));
        DD_TRY(fft_r2c<double>(p, 6, w.gx, kout, w.fw, w.fwb, st, false));
    }
    const Geo3& g = p->g3;
    CPtrs tk{};
    Ptrs n{};
    for (int c = 0; c < 6; c++) tk.p[c] = w.gk[c];
    for (int a = 0; a < 3; a++) n.p[a] = nc[a];
    DD_KT("les_add", st,
          k_les_add<<<les_grid((int64_t)g.Ky * g.Kz * g.Kx), 256, 0, st>>>(g, p->kx, p->ky, p->kz, tk, n,
                                                                          h.cl->band_lo, h.cl->band_hi,
                                                                          h.cl->shell_w, h.cl->n_shell));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

}  // namespace dd

using namespace dd;

static int les_check_plan(const dd_plan* p) {
    DD_CHECK_ARG(p, "null plan");
    DD_CHECK_ARG(p->ndim == 3, "the closure is implemented for 3D grids");
    return DD_OK;
}

static int les_check_closure(const dd_closure* cl) {
    DD_CHECK_ARG(cl && cl->wbf16 && cl->params && cl->norm, "closure weights, parameters and norm are required");
    return DD_OK;
}

extern "C" {

int dd_les_products(int64_t npts, const double* const* u, double* const* out, void* stream) {
    DD_CHECK_ARG(u && out && npts >= 0, "dd_les_products: bad arguments");
    CPtrs uc{};
    Ptrs o{};
    for (int a = 0; a < 3; a++) { DD_CHECK_ARG(u[a], "null velocity %d", a); uc.p[a] = u[a]; }
    for (int c = 0; c < 6; c++) { DD_CHECK_ARG(out[c], "null product %d", c); o.p[c] = out[c]; }
    if (npts == 0) return DD_OK;
    cudaStream_t st = (cudaStream_t)stream;
    DD_KT("les_products", st, k_les_products<<<les_grid(npts), 256, 0, st>>>(npts, uc, o));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

int dd_les_truncate3(const dd_plan* src, const dd_plan* dst, int nfield, const void* const* s, void* const* d,
                     void* stream) {
    DD_TRY(les_check_plan(src));
    DD_TRY(les_check_plan(dst));
    DD_CHECK_ARG(s && d && nfield >= 1 && nfield <= DD_MAXF, "dd_les_truncate3: bad arguments");
    const Geo3 &gs = src->g3, &gd = dst->g3;
    DD_CHECK_ARG(gd.Mx <= gs.Mx && gd.My <= gs.My && gd.Mz <= gs.Mz,
                 "the kept modes of the target grid must be kept modes of the source grid");
    CPtrs sc{};
    Ptrs dc{};
    for (int f = 0; f < nfield; f++) {
        DD_CHECK_ARG(s[f] && d[f], "null field %d", f);
        sc.p[f] = s[f];
        dc.p[f] = d[f];
    }
    cudaStream_t st = (cudaStream_t)stream;
    DD_KT("les_truncate3", st, k_les_truncate3<<<dim3(les_grid(gd.kcount()), nfield), 256, 0, st>>>(gs, gd, sc, dc));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

int dd_les_samples(int64_t npts, const double* const* g, const double* const* f, const double* const* fr,
                   double delta, float* raw, void* stream) {
    DD_CHECK_ARG(g && f && fr && raw && npts >= 0, "dd_les_samples: bad arguments");
    CPtrs gc{}, fc{}, rc{};
    for (int a = 0; a < 9; a++) { DD_CHECK_ARG(g[a], "null gradient %d", a); gc.p[a] = g[a]; }
    for (int c = 0; c < 6; c++) { DD_CHECK_ARG(f[c], "null product %d", c); fc.p[c] = f[c]; }
    for (int c = 0; c < 6; c++) { DD_CHECK_ARG(fr[c], "null resolved product %d", c); rc.p[c] = fr[c]; }
    if (npts == 0) return DD_OK;
    cudaStream_t st = (cudaStream_t)stream;
    DD_KT("les_samples", st, k_les_samples<<<les_grid(npts), 256, 0, st>>>(npts, gc, fc, rc, delta, raw));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

int dd_les_gradients(const dd_plan* p, const void* const* u, double* const* gx, int precision, void* work,
                     size_t work_bytes, void* stream) {
    DD_TRY(les_check_plan(p));
    DD_CHECK_ARG(u && gx && work, "dd_les_gradients: null pointer");
    DD_CHECK_ARG(precision == DD_FP64 || precision == DD_FP32, "precision must be DD_FP64 or DD_FP32");
    DD_CHECK_ARG(work_bytes >= les_work_bytes(p), "workspace too small: %zu < %zu", work_bytes, les_work_bytes(p));
    for (int a = 0; a < 3; a++) DD_CHECK_ARG(u[a], "null velocity %d", a);
    for (int f = 0; f < 9; f++) DD_CHECK_ARG(gx[f], "null gradient %d", f);
    cudaStream_t st = (cudaStream_t)stream;
    const LesWork w = les_carve(p, work);
    DD_TRY(les_grads(p, precision, false, u, w, false, st));
    const int64_t xb = p->g3.xcount() * (int64_t)sizeof(double);
    for (int f = 0; f < 9; f++) DD_CUDA(cudaMemcpyAsync(gx[f], w.gx[f], xb, cudaMemcpyDeviceToDevice, st));
    return DD_OK;
}

int dd_les_band(const dd_plan* p, int nfield, void* const* k, double lo, double hi, void* stream) {
    DD_TRY(les_check_plan(p));
    DD_CHECK_ARG(k && nfield >= 1 && nfield <= DD_MAXF, "dd_les_band: bad arguments");
    Ptrs kp{};
    for (int f = 0; f < nfield; f++) { DD_CHECK_ARG(k[f], "null field %d", f); kp.p[f] = k[f]; }
    const Geo3& g = p->g3;
    cudaStream_t st = (cudaStream_t)stream;
    DD_KT("les_band", st,
          k_les_band<<<dim3(les_grid(g.kcount()), nfield), 256, 0, st>>>(g, p->kx, p->ky, p->kz, kp, lo, hi));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

int dd_les_stress(const dd_plan* p, const void* const* u, double* const* tau, const dd_closure* cl, int precision,
                  void* work, size_t work_bytes, void* stream) {
    DD_TRY(les_check_plan(p));
    DD_TRY(les_check_closure(cl));
    DD_CHECK_ARG(u && tau && work, "dd_les_stress: null pointer");
    DD_CHECK_ARG(precision == DD_FP64 || precision == DD_FP32, "precision must be DD_FP64 or DD_FP32");
    DD_CHECK_ARG(work_bytes >= les_work_bytes(p), "workspace too small: %zu < %zu", work_bytes, les_work_bytes(p));
    for (int c = 0; c < 6; c++) DD_CHECK_ARG(tau[c], "null stress %d", c);
    cudaStream_t st = (cudaStream_t)stream;
    const LesWork w = les_carve(p, work);
    const bool f32 = precision == DD_FP32;
    DD_TRY(les_grads(p, precision, false, u, w, f32, st));
    if (f32) return les_mlp<float, double>(p, cl, w.gxf, tau, st);
    return les_mlp<double, double>(p, cl, w.gx, tau, st);
}

int dd_les_transfer(const dd_plan* p, const void* const* u, const double* const* tau, int nbins, double* out,
                    void* work, size_t work_bytes, void* stream) {
    DD_TRY(les_check_plan(p));
    DD_CHECK_ARG(u && tau && out && work, "dd_les_transfer: null pointer");
    DD_CHECK_ARG(nbins >= 1 && nbins <= 4096, "nbins must be in [1, 4096]");
    DD_CHECK_ARG(work_bytes >= les_work_bytes(p), "workspace too small: %zu < %zu", work_bytes, les_work_bytes(p));
    for (int a = 0; a < 3; a++) DD_CHECK_ARG(u[a], "null velocity %d", a);
    for (int c = 0; c < 6; c++) DD_CHECK_ARG(tau[c], "null stress %d", c);
    cudaStream_t st = (cudaStream_t)stream;
    const LesWork w = les_carve(p, work);
    const Geo3& g = p->g3;
    const double* xin[6];
    void* kout[6];
    for (int c = 0; c < 6; c++) { xin[c] = tau[c]; kout[c] = w.gk[c]; }
    DD_TRY(fft_r2c<double>(p, 6, xin, kout, w.fw, w.fwb, st, false));
    // per-mode terms and bins in two grid-point buffers (kept count <= grid points)
    const int64_t n = (int64_t)g.Ky * g.Kz * g.Kx;
    CPtrs uc{}, tk{};
    for (int a = 0; a < 3; a++) uc.p[a] = u[a];
    for (int c = 0; c < 6; c++) tk.p[c] = w.gk[c];
    DD_KT("les_transfer_modes", st,
          k_les_transfer_modes<<<les_grid(n), 256, 0, st>>>(g, p->kx, p->ky, p->kz, uc, tk, nbins, w.gx[6], w.gx[7]));
    DD_LAUNCH_CHECK();
    DD_KT("les_transfer_bins", st, k_les_transfer_bins<<<nbins, 256, 0, st>>>(n, w.gx[6], w.gx[7], out));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

}  // extern "C"
