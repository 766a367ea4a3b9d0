// Batched shared-memory FFT engine.
//
// A thread block holds P pencils of length L in a shared-memory tile laid out
// [element][pencil] (pencil fastest; row stride PS >= P, by default odd, so
// that for tiles of 16 or more pencils both pencil-contiguous and
// element-contiguous accesses are bank-conflict free for 8- and 16-byte
// complex entries; narrower tiles may use a skewed row layout, see Sched).  The transform is a mixed-radix
// Stockham autosort (decimation in time): each pass reads R inputs at stride
// L/R, twiddles by W_{Ns R}^{r k}, does an in-register radix-R DFT and writes
// the outputs at ((j-k) R + k) + r Ns.  Radices are 2, 3, 4, 8 and 16 (a radix
// 3 only as the last pass, so that every Ns before it is a power of two); in-register
// twiddles are exact constants (multiples of pi/8, and sqrt(3)/2), the inter-pass twiddles
// come from a per-length table W_L^m = exp(-2 pi i m / L) staged in shared
// memory (conjugated for the inverse transform).
//
// FP64 and FP32 butterflies are written for fused multiply-add hardware
// (Linzer and Feig, "Implementation of efficient FFT algorithms on fused
// multiply-add architectures", IEEE Trans. Signal Processing 41(1), 1993):
// a twiddle is stored as (g, t) with W = g (1 + i t), t = Im W / Re W, so
// that a twiddled radix-2 step a +/- W b costs six FMAs (b (1 + i t), then
// a +/- g (...)) instead of a complex product plus two complex additions.
// A radix-R butterfly with inter-pass twiddles w^r is split 4 x 4 (R = 16),
// 4 x 2 (R = 8) or 2 x 2 (R = 4) so that every twiddle it applies is a power
// of one factor per sub-DFT: the first sub-DFTs take w^(R/4) (and its square),
// the second ones w W_R^k1 (and its square), which folds the leftover w^n2
// of the first stage into the second (24 FMAs per twiddled radix-4, 192
// operations per twiddled radix 16 instead of 220).  A twiddle with Re W = 0
// is stored with g = 2^-60 and t = Im W * 2^60: the product is exact and the
// extra 2^-60 |b| is far below the rounding of the result.  The double-float
// type keeps the plain butterflies on (cos, sin) tables.
//
// Forward transforms use exp(-i...), inverse exp(+i...); neither is scaled.
#pragma once
#include "dd_common.cuh"
#include "df64.cuh"

namespace dd {

// --------------------------------------------------- in-register DFTs
// cos/sin of pi/8 and pi/4, correctly rounded decimal expansions.
#define DD_C8 0.92387953251128675613
#define DD_S8 0.38268343236508977173
#define DD_R2 0.70710678118654752440
#define DD_S3 0.86602540378443864676

// v * W_R^m (forward) or v * conj(W_R^m) (inverse), m a compile-time constant
// with R in {8, 16}; trivial multiples are exact.
template <int M, int R, bool INV, typename T>
__device__ __forceinline__ C<T> tw_const(C<T> v) {
    constexpr int m16 = ((M % R) * (16 / R)) % 16;  // angle in units of 2 pi / 16
    if constexpr (m16 == 0) {
        return v;
    } else if constexpr (m16 == 4) {
        return mul_mi<INV>(v);
    } else if constexpr (m16 == 8) {
        return mk<T>(-v.x, -v.y);
    } else if constexpr (m16 == 12) {
        return mul_mi<!INV>(v);
    } else {
        // forward twiddle exp(-2 pi i m16/16) = (c, -s)
        constexpr double ang_c[16] = {1, DD_C8, DD_R2, DD_S8, 0, -DD_S8, -DD_R2, -DD_C8,
                                      -1, -DD_C8, -DD_R2, -DD_S8, 0, DD_S8, DD_R2, DD_C8};
        constexpr double ang_s[16] = {0, DD_S8, DD_R2, DD_C8, 1, DD_C8, DD_R2, DD_S8,
                                      0, -DD_S8, -DD_R2, -DD_C8, -1, -DD_C8, -DD_R2, -DD_S8};
        constexpr T c = T(ang_c[m16]);
        constexpr T s = INV ? T(ang_s[m16]) : T(-ang_s[m16]);
        return mk<T>(v.x * c - v.y * s, v.x * s + v.y * c);
    }
}

template <bool INV, typename T>
__device__ __forceinline__ void dft2(C<T>& a, C<T>& b) {
    C<T> t = a;
    a = t + b;
    b = t - b;
}

template <bool INV, typename T>
__device__ __forceinline__ void dft4(C<T>& a0, C<T>& a1, C<T>& a2, C<T>& a3) {
    C<T> t0 = a0 + a2, t1 = a0 - a2, t2 = a1 + a3, t3 = mul_mi<INV>(a1 - a3);
    a0 = t0 + t2;
    a2 = t0 - t2;
    a1 = t1 + t3;
    a3 = t1 - t3;
}

// In-place DFT of R values v[0..R-1], natural order in and out.
template <int R, bool INV, typename T>
__device__ __forceinline__ void dft(C<T>* v) {
    if constexpr (R == 2) {
        dft2<INV>(v[0], v[1]);
    } else if constexpr (R == 4) {
        dft4<INV>(v[0], v[1], v[2], v[3]);
    } else if constexpr (R == 8) {
        // even/odd split: E = DFT4(v0,v2,v4,v6), O = DFT4(v1,v3,v5,v7)
        C<T> e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
        C<T> o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
        dft4<INV>(e0, e1, e2, e3);
        dft4<INV>(o0, o1, o2, o3);
        o1 = tw_const<1, 8, INV>(o1);
        o2 = tw_const<2, 8, INV>(o2);
        o3 = tw_const<3, 8, INV>(o3);
        v[0] = e0 + o0; v[4] = e0 - o0;
        v[1] = e1 + o1; v[5] = e1 - o1;
        v[2] = e2 + o2; v[6] = e2 - o2;
        v[3] = e3 + o3; v[7] = e3 - o3;
    } else if constexpr (R == 16) {
        // 4 x 4: n = 4 n1 + n2; Y[n2][k1] = DFT4_n1 v[4 n1 + n2]; twiddle
        // W16^(n2 k1); X[k1 + 4 k2] = DFT4_n2 Y[n2][k1].
        C<T> y[4][4];
#pragma unroll
        for (int n2 = 0; n2 < 4; n2++) {
            y[n2][0] = v[n2]; y[n2][1] = v[4 + n2]; y[n2][2] = v[8 + n2]; y[n2][3] = v[12 + n2];
            dft4<INV>(y[n2][0], y[n2][1], y[n2][2], y[n2][3]);
        }
        y[1][1] = tw_const<1, 16, INV>(y[1][1]);
        y[1][2] = tw_const<2, 16, INV>(y[1][2]);
        y[1][3] = tw_const<3, 16, INV>(y[1][3]);
        y[2][1] = tw_const<2, 16, INV>(y[2][1]);
        y[2][2] = tw_const<4, 16, INV>(y[2][2]);
        y[2][3] = tw_const<6, 16, INV>(y[2][3]);
        y[3][1] = tw_const<3, 16, INV>(y[3][1]);
        y[3][2] = tw_const<6, 16, INV>(y[3][2]);
        y[3][3] = tw_const<9, 16, INV>(y[3][3]);
#pragma unroll
        for (int k1 = 0; k1 < 4; k1++) {
            C<T> a0 = y[0][k1], a1 = y[1][k1], a2 = y[2][k1], a3 = y[3][k1];
            dft4<INV>(a0, a1, a2, a3);
            v[k1] = a0; v[k1 + 4] = a1; v[k1 + 8] = a2; v[k1 + 12] = a3;
        }
    } else if constexpr (R == 3) {
        // X1,2 = v0 - (v1 + v2)/2 -/+ i sqrt(3)/2 (v1 - v2) (forward; conjugate for inverse)
        const C<T> t1 = v[1] + v[2], t2 = v[1] - v[2];
        const C<T> m1 = mk<T>(v[0].x - t1.x * T(0.5), v[0].y - t1.y * T(0.5));
        const C<T> r = mul_mi<INV>(t2);
        const C<T> m2 = mk<T>(r.x * T(DD_S3), r.y * T(DD_S3));
        v[0] = v[0] + t1;
        v[1] = m1 + m2;
        v[2] = m1 - m2;
    } else {
        static_assert(R == 2 || R == 3 || R == 4 || R == 8 || R == 16, "unsupported radix");
    }
}

// --------------------------------------------------- FMA (Linzer-Feig) butterflies
template <typename T> struct IsLF { static constexpr bool value = false; };
template <> struct IsLF<double> { static constexpr bool value = true; };
template <> struct IsLF<float> { static constexpr bool value = true; };

__device__ __forceinline__ double fmx(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fmx(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// tan(pi/8) and tan(3 pi/8) = sqrt(2) -+ 1 (correctly rounded decimal expansions)
#define DD_T8 0.41421356237309504880
#define DD_T38 2.41421356237309504880

// b (1 + i t) for the forward sign, b (1 - i t) for the inverse (the
// conjugate twiddle): two FMAs.
template <bool INV, typename T>
__device__ __forceinline__ C<T> lf_rot(C<T> b, T t) {
    const T tt = INV ? -t : t;
    return mk<T>(fmx(-tt, b.y, b.x), fmx(tt, b.x, b.y));
}

// s = a + g u, d = a - g u: four FMAs.
template <typename T>
__device__ __forceinline__ void lf_pm(C<T> a, C<T> u, T g, C<T>& s, C<T>& d) {
    s = mk<T>(fmx(g, u.x, a.x), fmx(g, u.y, a.y));
    d = mk<T>(fmx(-g, u.x, a.x), fmx(-g, u.y, a.y));
}

// In place X_m = sum_n x_n z^n W4^(nm) with z = g1 (1 + i t1) and
// z^2 = g2 (1 + i t2) (conjugated for INV): 24 FMAs.
template <bool INV, typename T>
__device__ __forceinline__ void dft4_lf(C<T>& x0, C<T>& x1, C<T>& x2, C<T>& x3, T g1, T t1, T g2, T t2) {
    C<T> A, B, Cp, Dp;
    lf_pm(x0, lf_rot<INV>(x2, t2), g2, A, B);
    lf_pm(x1, lf_rot<INV>(x3, t2), g2, Cp, Dp);
    lf_pm(A, lf_rot<INV>(Cp, t1), g1, x0, x2);
    lf_pm(B, mul_mi<INV>(lf_rot<INV>(Dp, t1)), g1, x1, x3);
}

// The same with z^2 = W4 (-i forward, +i inverse), i.e. z = W8: 20 operations.
template <bool INV, typename T>
__device__ __forceinline__ void dft4_lf_zsq_w4(C<T>& x0, C<T>& x1, C<T>& x2, C<T>& x3, T g1, T t1) {
    const C<T> a2 = mul_mi<INV>(x2), a3 = mul_mi<INV>(x3);
    const C<T> A = x0 + a2, B = x0 - a2, Cp = x1 + a3, Dp = x1 - a3;
    lf_pm(A, lf_rot<INV>(Cp, t1), g1, x0, x2);
    lf_pm(B, mul_mi<INV>(lf_rot<INV>(Dp, t1)), g1, x1, x3);
}

// --------------------------------------------------- 2/3-band pruning
// Under the 2/3 rule an L-point axis keeps |mode index| <= kept23(L); the
// band kept23(L) < i < L - kept23(L) is zero on the way in (inverse
// transforms) and discarded on the way out (forward transforms).
__host__ __device__ constexpr int kept23(int L) { return (L + 2) / 3 - 1; }

// Bit r set: in a radix-R pass of L points whose butterfly j touches the
// elements j + r (L/R) (first pass: inputs; last pass: outputs), all L/R of
// them lie in the 2/3 band.  Only radices 8 and 16 use it.
template <int L, int R>
constexpr unsigned band_mask() {
    if (R != 8 && R != 16) return 0u;
    unsigned m = 0u;
    const int NB = L / R, K = kept23(L);
    for (int r = 0; r < R; r++)
        if (r * NB > K && (r + 1) * NB - 1 < L - K) m |= 1u << r;
    return m;
}

// dft4 of (a0, a1, a2, a3) with the inputs flagged Zi known to be zero (at
// most one per pair (a0, a2), (a1, a3)): the additions with a zero vanish.
template <bool INV, bool Z0, bool Z1, bool Z2, bool Z3, typename T>
__device__ __forceinline__ void dft4_zin(C<T>& a0, C<T>& a1, C<T>& a2, C<T>& a3) {
    static_assert(!(Z0 && Z2) && !(Z1 && Z3), "at most one zero input per pair");
    C<T> t0, t1, t2, t3;
    if constexpr (Z2) { t0 = a0; t1 = a0; }
    else if constexpr (Z0) { t0 = a2; t1 = mk<T>(-a2.x, -a2.y); }
    else { t0 = a0 + a2; t1 = a0 - a2; }
    if constexpr (Z3) { t2 = a1; t3 = mul_mi<INV>(a1); }
    else if constexpr (Z1) { t2 = a3; t3 = mul_mi<INV>(mk<T>(-a3.x, -a3.y)); }
    else { t2 = a1 + a3; t3 = mul_mi<INV>(a1 - a3); }
    a0 = t0 + t2; a2 = t0 - t2; a1 = t1 + t3; a3 = t1 - t3;
}

// dft4_lf computing only the outputs not flagged Di (the others keep
// whatever they held).
template <bool INV, bool D0, bool D1, bool D2, bool D3, typename T>
__device__ __forceinline__ void dft4_lf_out(C<T>& x0, C<T>& x1, C<T>& x2, C<T>& x3, T g1, T t1, T g2, T t2) {
    C<T> A, B, Cp, Dp;
    lf_pm(x0, lf_rot<INV>(x2, t2), g2, A, B);
    lf_pm(x1, lf_rot<INV>(x3, t2), g2, Cp, Dp);
    if constexpr (!(D0 && D2)) {
        const C<T> p = lf_rot<INV>(Cp, t1);
        if constexpr (!D0) x0 = mk<T>(fmx(g1, p.x, A.x), fmx(g1, p.y, A.y));
        if constexpr (!D2) x2 = mk<T>(fmx(-g1, p.x, A.x), fmx(-g1, p.y, A.y));
    }
    if constexpr (!(D1 && D3)) {
        const C<T> q = mul_mi<INV>(lf_rot<INV>(Dp, t1));
        if constexpr (!D1) x1 = mk<T>(fmx(g1, q.x, B.x), fmx(g1, q.y, B.y));
        if constexpr (!D3) x3 = mk<T>(fmx(-g1, q.x, B.x), fmx(-g1, q.y, B.y));
    }
}

template <unsigned M, int B>
constexpr bool bit() { return (M >> B) & 1u; }

// Radix-R butterfly of Stockham pass NS on v[0..R-1] (natural order in and
// out), with the inter-pass twiddles w^r, w = W_(NS R)^k, taken from the
// staged (g, t) table lf (W_L^m at index m).  ZIN (first pass only): inputs
// v[r] known zero; ZOUT (a pass with NS > 1 only): outputs v[r] not needed.
template <int R, int NS, int L, bool INV, unsigned ZIN = 0u, unsigned ZOUT = 0u, typename T>
__device__ __forceinline__ void bfly_lf(C<T>* v, const C<T>* lf, int k) {
    static_assert(ZIN == 0u || NS == 1, "zero inputs only in a first pass");
    static_assert(ZOUT == 0u || NS > 1, "discarded outputs only in a later pass");
    constexpr int STEP = L / (NS * R);
    if constexpr (R == 16) {
        if constexpr (NS > 1) {
            const C<T> a4 = lf[(4 * k) * STEP], a8 = lf[(8 * k) * STEP];
#pragma unroll
            for (int n2 = 0; n2 < 4; n2++) dft4_lf<INV>(v[n2], v[4 + n2], v[8 + n2], v[12 + n2], a4.x, a4.y, a8.x, a8.y);
        } else {
            dft4_zin<INV, bit<ZIN, 0>(), bit<ZIN, 4>(), bit<ZIN, 8>(), bit<ZIN, 12>()>(v[0], v[4], v[8], v[12]);
            dft4_zin<INV, bit<ZIN, 1>(), bit<ZIN, 5>(), bit<ZIN, 9>(), bit<ZIN, 13>()>(v[1], v[5], v[9], v[13]);
            dft4_zin<INV, bit<ZIN, 2>(), bit<ZIN, 6>(), bit<ZIN, 10>(), bit<ZIN, 14>()>(v[2], v[6], v[10], v[14]);
            dft4_zin<INV, bit<ZIN, 3>(), bit<ZIN, 7>(), bit<ZIN, 11>(), bit<ZIN, 15>()>(v[3], v[7], v[11], v[15]);
        }
        // now v[4 k1 + n2] = Y'[n2][k1]; second sub-DFTs over n2 with z = w W16^k1,
        // whose outputs are X[k1 + 4 k2]
        C<T> y[4][4];
#pragma unroll
        for (int k1 = 0; k1 < 4; k1++) {
#pragma unroll
            for (int n2 = 0; n2 < 4; n2++) y[k1][n2] = v[4 * k1 + n2];
            if constexpr (NS > 1) {
                const int e = k + k1 * NS;
                const C<T> z = lf[e * STEP], z2 = lf[(2 * e) * STEP];
                if (k1 == 0)
                    dft4_lf_out<INV, bit<ZOUT, 0>(), bit<ZOUT, 4>(), bit<ZOUT, 8>(), bit<ZOUT, 12>()>(
                        y[0][0], y[0][1], y[0][2], y[0][3], z.x, z.y, z2.x, z2.y);
                else if (k1 == 1)
                    dft4_lf_out<INV, bit<ZOUT, 1>(), bit<ZOUT, 5>(), bit<ZOUT, 9>(), bit<ZOUT, 13>()>(
                        y[1][0], y[1][1], y[1][2], y[1][3], z.x, z.y, z2.x, z2.y);
                else if (k1 == 2)
                    dft4_lf_out<INV, bit<ZOUT, 2>(), bit<ZOUT, 6>(), bit<ZOUT, 10>(), bit<ZOUT, 14>()>(
                        y[2][0], y[2][1], y[2][2], y[2][3], z.x, z.y, z2.x, z2.y);
                else
                    dft4_lf_out<INV, bit<ZOUT, 3>(), bit<ZOUT, 7>(), bit<ZOUT, 11>(), bit<ZOUT, 15>()>(
                        y[3][0], y[3][1], y[3][2], y[3][3], z.x, z.y, z2.x, z2.y);
            } else if (k1 == 0) {
                dft4<INV>(y[0][0], y[0][1], y[0][2], y[0][3]);
            } else if (k1 == 1) {   // z = W16, z^2 = W8
                dft4_lf<INV>(y[1][0], y[1][1], y[1][2], y[1][3], T(DD_C8), T(-DD_T8), T(DD_R2), T(-1));
            } else if (k1 == 2) {   // z = W8, z^2 = W4
                dft4_lf_zsq_w4<INV>(y[2][0], y[2][1], y[2][2], y[2][3], T(DD_R2), T(-1));
            } else {                // z = W16^3, z^2 = W16^6
                dft4_lf<INV>(y[3][0], y[3][1], y[3][2], y[3][3], T(DD_S8), T(-DD_T38), T(-DD_R2), T(1));
            }
        }
#pragma unroll
        for (int k1 = 0; k1 < 4; k1++) {
#pragma unroll
            for (int k2 = 0; k2 < 4; k2++) v[k1 + 4 * k2] = y[k1][k2];
        }
    } else if constexpr (R == 8) {
        if constexpr (NS > 1) {
            const C<T> a2 = lf[(2 * k) * STEP], a4 = lf[(4 * k) * STEP];
#pragma unroll
            for (int n2 = 0; n2 < 2; n2++) dft4_lf<INV>(v[n2], v[2 + n2], v[4 + n2], v[6 + n2], a2.x, a2.y, a4.x, a4.y);
        } else {
            dft4_zin<INV, bit<ZIN, 0>(), bit<ZIN, 2>(), bit<ZIN, 4>(), bit<ZIN, 6>()>(v[0], v[2], v[4], v[6]);
            dft4_zin<INV, bit<ZIN, 1>(), bit<ZIN, 3>(), bit<ZIN, 5>(), bit<ZIN, 7>()>(v[1], v[3], v[5], v[7]);
        }
        // v[2 k1 + n2] = Y'[n2][k1]; radix-2 steps with z = w W8^k1
        C<T> X[8];
#pragma unroll
        for (int k1 = 0; k1 < 4; k1++) {
            const C<T> y0 = v[2 * k1], y1 = v[2 * k1 + 1];
            if constexpr (NS > 1) {
                const C<T> z = lf[(k + k1 * NS) * STEP];
                if (((ZOUT >> k1) & 1u) && ((ZOUT >> (k1 + 4)) & 1u)) continue;
                const C<T> u = lf_rot<INV>(y1, z.y);
                if (!((ZOUT >> k1) & 1u)) X[k1] = mk<T>(fmx(z.x, u.x, y0.x), fmx(z.x, u.y, y0.y));
                if (!((ZOUT >> (k1 + 4)) & 1u)) X[k1 + 4] = mk<T>(fmx(-z.x, u.x, y0.x), fmx(-z.x, u.y, y0.y));
            } else if (k1 == 0) {
                X[0] = y0 + y1; X[4] = y0 - y1;
            } else if (k1 == 1) {
                lf_pm(y0, lf_rot<INV>(y1, T(-1)), T(DD_R2), X[1], X[5]);
            } else if (k1 == 2) {
                const C<T> a = mul_mi<INV>(y1);
                X[2] = y0 + a; X[6] = y0 - a;
            } else {
                lf_pm(y0, lf_rot<INV>(y1, T(1)), T(-DD_R2), X[3], X[7]);
            }
        }
#pragma unroll
        for (int r = 0; r < 8; r++) v[r] = X[r];
    } else if constexpr (R == 4) {
        if constexpr (NS > 1) {
            const C<T> z = lf[k * STEP], z2 = lf[(2 * k) * STEP];
            dft4_lf<INV>(v[0], v[1], v[2], v[3], z.x, z.y, z2.x, z2.y);
        } else {
            dft4<INV>(v[0], v[1], v[2], v[3]);
        }
    } else if constexpr (R == 2) {
        if constexpr (NS > 1) {
            const C<T> z = lf[k * STEP];
            C<T> a, b;
            lf_pm(v[0], lf_rot<INV>(v[1], z.y), z.x, a, b);
            v[0] = a; v[1] = b;
        } else {
            dft2<INV>(v[0], v[1]);
        }
    } else {
        static_assert(R == 3, "unsupported radix");
        if constexpr (NS > 1) {
#pragma unroll
            for (int r = 1; r < 3; r++) {
                const C<T> z = lf[(r * k) * STEP];
                const C<T> u = lf_rot<INV>(v[r], z.y);
                v[r] = mk<T>(u.x * z.x, u.y * z.x);
            }
        }
        dft<3, INV>(v);
    }
}

// --------------------------------------------------- pencil configuration
// Per length: pencils per block (P), threads per block (NT) and radix
// schedule (R1, R2, R3; 1 = unused).  Threads per pencil TPP = NT / P and every
// pass has (L / R) / TPP butterflies per thread, an integer >= 1.
template <int L> struct FFTCfg;
template <> struct FFTCfg<8>    { static constexpr int P = 64, NT = 64,  R1 = 8,  R2 = 1,  R3 = 1; };
template <> struct FFTCfg<24>   { static constexpr int P = 64, NT = 64,  R1 = 8,  R2 = 3,  R3 = 1; };
template <> struct FFTCfg<48>   { static constexpr int P = 64, NT = 256, R1 = 4,  R2 = 4,  R3 = 3; };
template <> struct FFTCfg<96>   { static constexpr int P = 64, NT = 256, R1 = 8,  R2 = 4,  R3 = 3; };
template <> struct FFTCfg<192>  { static constexpr int P = 32, NT = 256, R1 = 8,  R2 = 8,  R3 = 3; };
template <> struct FFTCfg<16>   { static constexpr int P = 64, NT = 256, R1 = 4,  R2 = 4,  R3 = 1; };
template <> struct FFTCfg<32>   { static constexpr int P = 64, NT = 256, R1 = 8,  R2 = 4,  R3 = 1; };
template <> struct FFTCfg<64>   { static constexpr int P = 32, NT = 256, R1 = 8,  R2 = 8,  R3 = 1; };
template <> struct FFTCfg<128>  { static constexpr int P = 32, NT = 256, R1 = 16, R2 = 8,  R3 = 1; };
template <> struct FFTCfg<256>  { static constexpr int P = 16, NT = 256, R1 = 16, R2 = 16, R3 = 1; };
template <> struct FFTCfg<512>  { static constexpr int P = 8,  NT = 256, R1 = 8,  R2 = 8,  R3 = 8; };
template <> struct FFTCfg<1024> { static constexpr int P = 4,  NT = 256, R1 = 16, R2 = 16, R3 = 4; };

// A schedule: length L, P pencils per tile, NT threads (TPP = NT / P per
// pencil) and the radix sequence R1 R2 R3 (1 = unused).  Row e of the tile
// starts at entry off(e) = e PS + (e / 8) SKD.  The default is PS = P | 1 and
// no skew.  A schedule with few pencils (6, 10) may take PS = P and a skew of
// SKD entries every 8 rows instead.  That keeps the pencil-contiguous Stockham
// accesses (a half-warp spanning 2-3 rows) and the element-contiguous ones
// (16 consecutive rows of one pencil) largely free of bank conflicts for 8-byte
// entries, which no odd stride does for both.
template <int L_, int P_, int NT_, int R1_, int R2_, int R3_, int PS_ = (P_ | 1), int SKD_ = 0>
struct Sched {
    static constexpr int L = L_, P = P_, NT = NT_, R1 = R1_, R2 = R2_, R3 = R3_;
    static constexpr int PS = PS_, SKD = SKD_;
    static constexpr int TPP = NT / P;
    static_assert(PS >= P, "row stride below the pencil count");
    static_assert(NT % P == 0, "threads must split evenly over pencils");
    static_assert(R1 * R2 * R3 == L, "radix schedule does not multiply to L");
    __host__ __device__ static constexpr int off(int e) { return e * PS + (e >> 3) * SKD; }
    // tile entries (the twiddle table follows them)
    static constexpr int span = SKD == 0 ? L * PS : off(L - 1) + P;
    template <typename T>
    static constexpr size_t smem_bytes() { return sizeof(C<T>) * ((size_t)span + L); }
};

template <int L>
using DefSched = Sched<L, FFTCfg<L>::P, FFTCfg<L>::NT, FFTCfg<L>::R1, FFTCfg<L>::R2, FFTCfg<L>::R3>;

template <int L>
struct Pencil {
    static constexpr int P = FFTCfg<L>::P;
    static constexpr int NT = FFTCfg<L>::NT;
    static constexpr int PS = DefSched<L>::PS;
    static constexpr int TPP = NT / P;
    template <typename T>
    static constexpr size_t smem_bytes() { return DefSched<L>::template smem_bytes<T>(); }
};

// One Stockham pass of radix R with current sub-transform length NS.  tw is
// the staged twiddle table: (g, t) pairs for FP64 / FP32, (cos, sin) for
// double-float.
template <typename T, class S, int R, int NS, bool INV, unsigned ZIN = 0u, unsigned ZOUT = 0u>
__device__ __forceinline__ void stockham_pass(C<T>* tile, const C<T>* tw, int p, int jt) {
    constexpr int L = S::L, TPP = S::TPP;
    constexpr int NB = L / R;          // butterflies per pencil
    constexpr int BPT = NB / TPP;      // butterflies per thread
    static_assert(BPT >= 1 && NB % TPP == 0, "bad radix schedule");
    C<T> v[BPT][R];
#pragma unroll
    for (int b = 0; b < BPT; b++) {
        const int j = jt + TPP * b;
#pragma unroll
        for (int r = 0; r < R; r++) {
            // off() is additive over multiples of 8 rows: with such a stride the
            // row offsets are compile-time constants from the thread's base row
            const int o = (S::SKD == 0 || NB % 8 == 0) ? S::off(j) + S::off(r * NB) : S::off(j + r * NB);
            v[b][r] = ((ZIN >> r) & 1u) ? zero<T>() : tile[o + p];
        }
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < BPT; b++) {
        const int j = jt + TPP * b;
        const int k = j & (NS - 1);
        if constexpr (IsLF<T>::value) {
            bfly_lf<R, NS, L, INV, ZIN, ZOUT>(v[b], tw, k);
        } else {
            if constexpr (NS > 1) {
                constexpr int STEP = L / (NS * R);
#pragma unroll
                for (int r = 1; r < R; r++) {
                    const C<T> w = tw[(r * k) * STEP];
                    v[b][r] = INV ? cmulc(v[b][r], w) : cmul(v[b][r], w);
                }
            }
            dft<R, INV>(v[b]);
        }
        const int d = (j - k) * R + k;
        // the same for the outputs: a stride of 8 rows, or d a multiple of 8 (the
        // first pass, d = j R, with R a multiple of 8)
        constexpr bool lin = S::SKD == 0 || NS % 8 == 0 || (NS == 1 && R % 8 == 0);
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int o = lin ? S::off(d) + S::off(r * NS) : S::off(d + r * NS);
            if (!((ZOUT >> r) & 1u)) tile[o + p] = v[b][r];
        }
    }
    __syncthreads();
}

// Transform the S::P pencils of the tile in place.  Called by the first S::NT
// threads of the block (all of them must reach the barriers: threads beyond
// S::NT call with active = false).  The caller synchronises before (tile
// filled); this returns synchronised with the result in natural order.
// PRUNE (FP64 / FP32 only, with at least two passes): the pencils follow the
// 2/3 rule, so an inverse transform's first pass skips the inputs in the
// removed band (they are zero) and a forward transform's last pass skips the
// outputs in it (the caller never reads them; those tile entries are left
// stale).
template <typename T, class S, bool INV, bool PRUNE = false>
__device__ __forceinline__ void pencil_fft_s(C<T>* tile, const C<T>* tw, bool active = true) {
    const int p = active ? threadIdx.x % S::P : 0;
    const int jt = active ? threadIdx.x / S::P : 0;
    constexpr bool PR = PRUNE && IsLF<T>::value && S::R2 > 1;
    constexpr int RL = S::R3 > 1 ? S::R3 : S::R2;
    constexpr unsigned ZI = (PR && INV) ? band_mask<S::L, S::R1>() : 0u;
    constexpr unsigned ZO = (PR && !INV) ? band_mask<S::L, RL>() : 0u;
    if (active) {
        if constexpr (S::R3 > 1) {
            stockham_pass<T, S, S::R1, 1, INV, ZI>(tile, tw, p, jt);
            stockham_pass<T, S, S::R2, S::R1, INV>(tile, tw, p, jt);
            stockham_pass<T, S, S::R3, S::R1 * S::R2, INV, 0u, ZO>(tile, tw, p, jt);
        } else if constexpr (S::R2 > 1) {
            stockham_pass<T, S, S::R1, 1, INV, ZI>(tile, tw, p, jt);
            stockham_pass<T, S, S::R2, S::R1, INV, 0u, ZO>(tile, tw, p, jt);
        } else {
            stockham_pass<T, S, S::R1, 1, INV>(tile, tw, p, jt);
        }
    } else {
        __syncthreads(); __syncthreads();
        if constexpr (S::R2 > 1) { __syncthreads(); __syncthreads(); }
        if constexpr (S::R3 > 1) { __syncthreads(); __syncthreads(); }
    }
}

template <typename T, int L, bool INV>
__device__ __forceinline__ void pencil_fft(C<T>* tile, const C<T>* tw) {
    pencil_fft_s<T, DefSched<L>, INV>(tile, tw);
}

// Stage the length-L twiddle table (global, L entries) into shared memory.
template <typename T, int L>
__device__ __forceinline__ void load_twiddles(C<T>* s_tw, const typename Vec2<T>::type* g_tw) {
    for (int i = threadIdx.x; i < L; i += blockDim.x) s_tw[i] = ldc<T>(g_tw + i);
}

}  // namespace dd
