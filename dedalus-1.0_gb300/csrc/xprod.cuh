// Fused x-direction pass: NI half-spectrum fields -> c2r -> pointwise
// nonlinear products in shared memory -> r2c of NO fields, for Q rows per block.
//
// Real rows are paired into complex pencils in row-major (row, field) order:
// real row t = r*NI + f lives in pencil t/2, real part if t is even, imaginary
// part if odd.  The forward side pairs its outputs the same way with NO.  The
// inverse and forward transforms use their own schedules (SI, SF) so the
// pencil slots of the block can be filled on both sides.
//
// Op provides: static NI, NO; __device__ void operator()(const T* in, T* out,
// int run) on the NI grid values of one point, producing NO values.  Blocks
// are (row block, run): run b's fields start at win.p[f] + b * in_rs and
// wout.p[g] + b * out_rs (complex entries).
#pragma once
#include "launch_len.cuh"

namespace dd {

template <int L, int NI, int NO>
struct ProdCfg {
    using SI = DefSched<L>;
    using SF = DefSched<L>;
    static constexpr int q_of(int n) { return ((2 * SI::P) / n) & ~1; }
    static constexpr int Q = (q_of(NI) < q_of(NO) ? q_of(NI) : q_of(NO));
    static constexpr int NT = SI::NT;
};
// Hydro (6 -> 3) and MHD (12 -> 6): forward pencils are half the inverse
// ones, so SF doubles the threads per pencil and both sides are full.
template <> struct ProdCfg<64, 6, 3> {
    using SI = Sched<64, 24, 192, 8, 8, 1>;  using SF = Sched<64, 12, 192, 4, 4, 4>;
    static constexpr int Q = 8, NT = 192;
};
template <> struct ProdCfg<128, 6, 3> {
    using SI = Sched<128, 24, 192, 16, 8, 1>;  using SF = Sched<128, 12, 192, 8, 4, 4>;
    static constexpr int Q = 8, NT = 192;
};
template <> struct ProdCfg<256, 6, 3> {
    using SI = Sched<256, 12, 192, 16, 16, 1>;  using SF = Sched<256, 6, 192, 8, 8, 4>;
    static constexpr int Q = 4, NT = 192;
};
template <> struct ProdCfg<512, 6, 3> {
    using SI = Sched<512, 6, 192, 8, 8, 8>;  using SF = Sched<512, 3, 192, 8, 8, 8>;
    static constexpr int Q = 2, NT = 192;
};
// Hydro in divergence form (3 -> 5): the forward side has 5/3 of the inverse
// pencils; 4 rows per block fill 6 inverse pencils (32 threads each) and 10
// forward pencils (16 threads each).
template <> struct ProdCfg<256, 3, 5> {
    using SI = Sched<256, 6, 192, 8, 8, 4>;  using SF = Sched<256, 10, 160, 16, 16, 1>;
    static constexpr int Q = 4, NT = 192;
};
// 2D hydro (3 -> 2) on 64- and 128-point rows: 2 rows per block (3 inverse
// and 2 forward pencils of 16 threads), so that one 128^2 run has 64 blocks.
template <> struct ProdCfg<64, 3, 2> {
    using SI = Sched<64, 3, 48, 4, 4, 4>;  using SF = Sched<64, 2, 32, 4, 4, 4>;
    static constexpr int Q = 2, NT = 48;
};
template <> struct ProdCfg<128, 3, 2> {
    using SI = Sched<128, 3, 48, 8, 4, 4>;  using SF = Sched<128, 2, 32, 8, 4, 4>;
    static constexpr int Q = 2, NT = 48;
};
template <> struct ProdCfg<64, 12, 6> {
    using SI = Sched<64, 24, 192, 8, 8, 1>;  using SF = Sched<64, 12, 192, 4, 4, 4>;
    static constexpr int Q = 4, NT = 192;
};
template <> struct ProdCfg<128, 12, 6> {
    using SI = Sched<128, 24, 192, 16, 8, 1>;  using SF = Sched<128, 12, 192, 8, 4, 4>;
    static constexpr int Q = 4, NT = 192;
};
template <> struct ProdCfg<256, 12, 6> {
    using SI = Sched<256, 12, 192, 16, 16, 1>;  using SF = Sched<256, 6, 192, 8, 8, 4>;
    static constexpr int Q = 2, NT = 192;
};
template <> struct ProdCfg<512, 12, 6> {
    using SI = Sched<512, 12, 384, 8, 8, 8>;  using SF = Sched<512, 6, 384, 8, 8, 8>;
    static constexpr int Q = 2, NT = 384;
};

// The schedule a precision runs (ProdCfg unless specialised).  per_point:
// the tile fill, the product phase and the output unpacking are organised by
// grid point, with the pencils, rows and fields of a point in compile-time
// loops.  A thread fills and multiplies whole tile rows (complex entries, not
// their halves), and the field pointers are fixed per loop step instead of
// selected at run time.  Otherwise each thread takes one tile entry or one
// point of one row at a time.
template <typename T, int L, int NI, int NO>
struct ProdCfgT : ProdCfg<L, NI, NO> {
    static constexpr bool per_point = false;
    static constexpr int min_blocks = std::is_same<T, df64>::value ? 5 : 1;   // __launch_bounds__
};
// FP32 hydro in divergence form on 256-point rows: 6 inverse and 10 forward
// pencils in tiles with unpadded rows and a skew every 8 rows (P / 2 entries),
// and the per-point product phase.  With the odd strides 7 and 11, 41% of the
// shared-memory wavefronts of a launch were bank conflicts (23.3 M of 57.2 M);
// a model of every access of the kernel puts this layout at 37% fewer
// wavefronts.  (Tiles 16 pencils wide, 9 inverse and 15 forward pencils per
// 6 rows, cut the conflicts to 4% but ran slower: their idle pencil slots cost
// more than the conflicts.)
template <>
struct ProdCfgT<float, 256, 3, 5> {
    using SI = Sched<256, 6, 192, 8, 8, 4, 6, 3>;
    using SF = Sched<256, 10, 160, 16, 16, 1, 10, 5>;
    static constexpr int Q = 4, NT = 192;
    static constexpr bool per_point = true;
    static constexpr int min_blocks = 6;   // 56 registers: 6 blocks per SM (72 and 4 blocks without the bound)
};

// FP32 MHD in divergence form (6 -> 8) on 256-point rows: the default 16-pencil
// tiles (12 inverse, 16 forward pencils for 4 rows), point-major phases.
template <>
struct ProdCfgT<float, 256, 6, 8> : ProdCfg<256, 6, 8> {
    static constexpr bool per_point = true;
    static constexpr int min_blocks = 4;   // 64 registers (90 unbounded: 2 blocks per SM, 565 vs 348 us)
};

// FP32 2D Boussinesq in divergence form (3 -> 4) on 256- and 512-point rows:
// the default tiles (16 pencils, 8 rows per block; 8 pencils, 4 rows),
// point-major phases.
template <>
struct ProdCfgT<float, 256, 3, 4> : ProdCfg<256, 3, 4> {
    static constexpr bool per_point = true;
    static constexpr int min_blocks = 4;   // 64 registers (72 unbounded, 3 blocks per SM)
};
template <>
struct ProdCfgT<float, 512, 3, 4> : ProdCfg<512, 3, 4> {
    static constexpr bool per_point = true;
    static constexpr int min_blocks = 1;
};

template <typename T, int L, int NI, int NO>
constexpr size_t prod_smem(size_t csize) {
    using CC = ProdCfgT<T, L, NI, NO>;
    const size_t a = (size_t)CC::SI::span, b = (size_t)CC::SF::span;
    return csize * ((a > b ? a : b) + L);
}

template <typename T, int L, class Op>
__global__ void __launch_bounds__(ProdCfgT<T, L, Op::NI, Op::NO>::NT, ProdCfgT<T, L, Op::NI, Op::NO>::min_blocks)
k_x_prod(int nrows, int Kx, CPtrs win, Ptrs wout, int64_t in_rs, int64_t out_rs,
         const typename Vec2<T>::type* gtw, T scale, const Op op) {
    using V = typename Vec2<T>::type;
    constexpr int NI = Op::NI, NO = Op::NO;
    static_assert(NI <= DD_MAXF && NO <= DD_MAXF, "too many fields for Ptrs");
    using CC = ProdCfgT<T, L, NI, NO>;
    using SI = typename CC::SI;
    using SF = typename CC::SF;
    extern __shared__ __align__(16) unsigned char dd_smem[];
    constexpr int NT = CC::NT, Q = CC::Q;
    static_assert(Q >= 2 && Q % 2 == 0, "need an even number of rows per block");
    static_assert((NI * Q + 1) / 2 <= SI::P && (NO * Q + 1) / 2 <= SF::P, "schedule too small for Q rows");
    static_assert(SI::NT == NT && SF::NT <= NT, "schedules must fit the block");
    C<T>* tile = reinterpret_cast<C<T>*>(dd_smem);
    constexpr size_t TA = (size_t)SI::span, TB = (size_t)SF::span;
    C<T>* tw = tile + (TA > TB ? TA : TB);
    load_twiddles<T, L>(tw, gtw);
    const int row0 = blockIdx.x * Q;
    const int nr = min(Q, nrows - row0);
    const int64_t ib = blockIdx.y * in_rs, ob = blockIdx.y * out_rs;  // run (batch) offsets
    constexpr int NPI = (NI * Q + 1) / 2;  // inverse pencils in use
    if constexpr (CC::per_point) {
        // tile row e = grid point e of the block's rows: all NPI pencils of a
        // row, the loads of a thread's rows in flight together
        constexpr int NE = (L + NT - 1) / NT;
        C<T> zv[NE][NPI];
#pragma unroll
        for (int i = 0; i < NE; i++) {
            const int e = threadIdx.x + i * NT;
#pragma unroll
            for (int pj = 0; pj < NPI; pj++) {
                const int ta = 2 * pj, tb = 2 * pj + 1;
                const int ra = ta / NI, fa = ta % NI, rb = tb / NI, fb = tb % NI;
                const bool va = ra < nr, vb = tb < NI * Q && rb < nr;
                C<T> z = zero<T>();
                if ((NE * NT == L || e < L) && (va || vb)) {
                    const V* pa = (const V*)win.p[fa] + ib + (int64_t)(row0 + ra) * Kx;
                    const V* pb = (const V*)win.p[tb < NI * Q ? fb : fa] + ib + (int64_t)(row0 + rb) * Kx;
                    z = pack_rows<T>(va ? pa : pb, vb ? pb : pa, e, L, Kx);
                    if (!va) z.x = T(0);
                    if (!vb) z.y = T(0);
                }
                zv[i][pj] = z;
            }
        }
#pragma unroll
        for (int i = 0; i < NE; i++) {
            const int e = threadIdx.x + i * NT;
            if (NE * NT == L || e < L) {
#pragma unroll
                for (int pj = 0; pj < NPI; pj++) tile[SI::off(e) + pj] = zv[i][pj];
#pragma unroll
                for (int pj = NPI; pj < SI::P; pj++) tile[SI::off(e) + pj] = zero<T>();
            }
        }
    } else {
        // the loads of a group of GX entries are in flight together (see load_tile)
        constexpr int NLD = L * SI::P, NPL = (NLD + NT - 1) / NT;
        constexpr int GX0 = (int)(128 / sizeof(C<T>)), GX = NPL < GX0 ? NPL : GX0;
#pragma unroll
        for (int i0 = 0; i0 < NPL; i0 += GX) {
            C<T> zv[GX];
#pragma unroll
            for (int i = 0; i < GX; i++) {
                const int idx = threadIdx.x + (i0 + i) * NT;
                const int e = idx % L, pj = idx / L;
                C<T> z = zero<T>();
                if (i0 + i < NPL && idx < NLD && pj < NPI) {
                    const int ta = 2 * pj, tb = 2 * pj + 1;
                    const int ra = ta / NI, fa = ta % NI, rb = tb / NI, fb = tb % NI;
                    const bool va = ra < nr, vb = tb < NI * Q && rb < nr;
                    if (va || vb) {
                        const V* pa = (const V*)pick_ptr<NI>(win.p, fa) + ib + (int64_t)(row0 + (va ? ra : rb)) * Kx;
                        const V* pb =
                            (const V*)pick_ptr<NI>(win.p, vb ? fb : fa) + ib + (int64_t)(row0 + (vb ? rb : ra)) * Kx;
                        z = pack_rows<T>(pa, pb, e, L, Kx);
                        if (!va) z.x = T(0);
                        if (!vb) z.y = T(0);
                    }
                }
                zv[i] = z;
            }
#pragma unroll
            for (int i = 0; i < GX; i++) {
                const int idx = threadIdx.x + (i0 + i) * NT;
                if (i0 + i < NPL && idx < NLD) tile[SI::off(idx % L) + idx / L] = zv[i];
            }
        }
    }
    __syncthreads();
    // kept kx <= Kx - 1: under the 2/3 rule the packed pencils are zero in the
    // removed band and the unpacking never reads it
    // (double-float has no pruned butterflies: one copy of its transform)
    const bool prune = IsLF<T>::value && Kx - 1 == kept23(L);
    if constexpr (IsLF<T>::value) {
        if (prune) pencil_fft_s<T, SI, true, true>(tile, tw);
        else pencil_fft_s<T, SI, true>(tile, tw);
    } else {
        pencil_fft_s<T, SI, true>(tile, tw);
    }
    if constexpr (CC::per_point) {
        // one grid point of all Q rows per thread: the NPI inverse pencils of a
        // row of the tile in, the NPF forward pencils out (the last one's
        // imaginary half zero when NO Q is odd)
        constexpr int NPP = (L + NT - 1) / NT, NPF = (NO * Q + 1) / 2;
        T outv[NPP][NO * Q];
#pragma unroll
        for (int i = 0; i < NPP; i++) {
            const int e = threadIdx.x + i * NT;
            if (e < L) {
                C<T> pin[NPI];
#pragma unroll
                for (int pj = 0; pj < NPI; pj++) pin[pj] = tile[SI::off(e) + pj];
#pragma unroll
                for (int r = 0; r < Q; r++) {
                    T in[NI];
#pragma unroll
                    for (int f = 0; f < NI; f++) {
                        const int t = r * NI + f;
                        in[f] = (t & 1) ? pin[t / 2].y : pin[t / 2].x;
                    }
                    op(in, &outv[i][r * NO], blockIdx.y);
                }
            }
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < NPP; i++) {
            const int e = threadIdx.x + i * NT;
            if (e < L) {
#pragma unroll
                for (int pj = 0; pj < NPF; pj++)
                    tile[SF::off(e) + pj] = mk<T>(outv[i][2 * pj], 2 * pj + 1 < NO * Q ? outv[i][2 * pj + 1] : T(0));
            }
        }
    } else {
        constexpr int NPT = (L * Q + NT - 1) / NT;
        T outv[NPT][NO];
#pragma unroll
        for (int i = 0; i < NPT; i++) {
            const int idx = threadIdx.x + i * NT;
            if (idx < L * Q) {
                const int e = idx % L, r = idx / L;
                T in[NI];
#pragma unroll
                for (int f = 0; f < NI; f++) {
                    const int t = r * NI + f;
                    const C<T> c = tile[SI::off(e) + t / 2];
                    in[f] = (t & 1) ? c.y : c.x;
                }
                op(in, outv[i], blockIdx.y);
            }
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < NPT; i++) {
            const int idx = threadIdx.x + i * NT;
            if (idx < L * Q) {
                const int e = idx % L, r = idx / L;
#pragma unroll
                for (int g = 0; g < NO; g++) {
                    const int t = r * NO + g;
                    if (t & 1) tile[SF::off(e) + t / 2].y = outv[i][g];
                    else tile[SF::off(e) + t / 2].x = outv[i][g];
                }
            }
        }
        if constexpr ((NO * Q) & 1) {  // the last pencil's imaginary half is unused
            for (int e = threadIdx.x; e < L; e += NT) tile[SF::off(e) + (NO * Q) / 2].y = T(0);
        }
    }
    __syncthreads();
    if constexpr (IsLF<T>::value) {
        if (prune) pencil_fft_s<T, SF, false, true>(tile, tw, threadIdx.x < SF::NT);
        else pencil_fft_s<T, SF, false>(tile, tw, threadIdx.x < SF::NT);
    } else {
        pencil_fft_s<T, SF, false>(tile, tw, threadIdx.x < SF::NT);
    }
    if constexpr (CC::per_point) {
        // two halves of the block take the rows r < Q/2 and r >= Q/2; within a
        // half consecutive threads take consecutive kx of one output row
        constexpr int KG = NT / 2;
        const int half = threadIdx.x / KG;
        for (int k = threadIdx.x % KG; k < Kx; k += KG) {
            const C<T>* zr = tile + SF::off(k);
            const C<T>* znr = tile + SF::off(k == 0 ? 0 : L - k);
#pragma unroll
            for (int r2 = 0; r2 < Q / 2; r2++) {
                const int r = half * (Q / 2) + r2;
                if (r >= nr) continue;
#pragma unroll
                for (int g = 0; g < NO; g++) {
                    const int t = r * NO + g;
                    C<T> A, B;
                    unpack_pair<T>(zr[t / 2], znr[t / 2], scale, A, B);
                    stc<T>((V*)wout.p[g] + ob + (int64_t)(row0 + r) * Kx + k, (t & 1) ? B : A);
                }
            }
        }
    } else {
        // field-major order: consecutive threads write the block's Q consecutive rows
        // of one output field, a contiguous range, so a 32-byte sector shared by two
        // rows (complex64 rows of an odd number of half-sectors) is written whole by
        // one warp instead of in two halves at different times
        for (int idx = threadIdx.x; idx < Kx * Q * NO; idx += NT) {
            const int k = idx % Kx, u = idx / Kx;
            const int g = u / Q, r = u % Q;
            if (r >= nr) continue;
            const int t = r * NO + g;              // its real row in the packed tile
            C<T> A, B;
            unpack_pair<T>(tile[SF::off(k) + t / 2], tile[SF::off(k == 0 ? 0 : L - k) + t / 2], scale, A, B);
            stc<T>((V*)pick_ptr<NO>(wout.p, g) + ob + (int64_t)(row0 + r) * Kx + k, (t & 1) ? B : A);
        }
    }
}

template <typename T, int L, class Op>
int launch_x_prod(const char* name, int nrows, int Kx, const CPtrs& win, const Ptrs& wout, int nrun, int64_t in_rs,
                  int64_t out_rs, const typename Vec2<T>::type* tw, T scale, const Op& op, cudaStream_t st) {
    using CC = ProdCfgT<T, L, Op::NI, Op::NO>;
    const size_t smem = prod_smem<T, L, Op::NI, Op::NO>(sizeof(C<T>));
    static std::atomic<unsigned long long> configured{0};
    DD_TRY(ensure_smem((const void*)k_x_prod<T, L, Op>, smem, configured));
    static const std::string label = std::string(name) + "_" + std::to_string(L) + PrecName<T>::s;
    DD_KT(label.c_str(), st,
          k_x_prod<T, L, Op><<<dim3(cdiv(nrows, CC::Q), nrun), CC::NT, smem, st>>>(nrows, Kx, win, wout, in_rs, out_rs,
                                                                                  tw, scale, op));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

template <typename T, class Op>
int launch_x_prod_len(const char* name, int L, int nrows, int Kx, const CPtrs& win, const Ptrs& wout, int nrun,
                      int64_t in_rs, int64_t out_rs, const typename Vec2<T>::type* tw, T scale, const Op& op,
                      cudaStream_t st) {
    DD_CHECK_SUPPORTED(nrun >= 1 && nrun <= 65535, "run batch of %d not supported", nrun);
#define DD_XP(N) (launch_x_prod<T, N>(name, nrows, Kx, win, wout, nrun, in_rs, out_rs, tw, scale, op, st))
    switch (L) {
        DD_LEN_CASE(8, DD_XP(8))
        DD_LEN_CASE(16, DD_XP(16))
        DD_LEN_CASE(24, DD_XP(24))
        DD_LEN_CASE(48, DD_XP(48))
        DD_LEN_CASE(96, DD_XP(96))
        DD_LEN_CASE(192, DD_XP(192))
        DD_LEN_CASE(32, DD_XP(32))
        DD_LEN_CASE(64, DD_XP(64))
        DD_LEN_CASE(128, DD_XP(128))
        DD_LEN_CASE(256, DD_XP(256))
        DD_LEN_CASE(512, DD_XP(512))
        default: break;
    }
#undef DD_XP
    set_error("x length %d is not supported for %s%s", L, name, PrecName<T>::s);
    return DD_ERR_UNSUPPORTED;
}

}  // namespace dd
