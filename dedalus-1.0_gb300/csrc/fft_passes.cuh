// Transform passes: one kernel template moves a tile of pencils between
// global memory and shared memory around the pencil FFT engine.  The source
// and destination layouts (pruned/dealiased loads, compact intermediates,
// Hermitian packing of real rows, scaling) live in small "Op" structs whose
// load/store members are inlined into the kernel, so every pass is a single
// read and a single write of its data.
//
// Grid: x = (pencil tile) * nfield + field, y = slow index (up to 65535), z =
// slow index / 65535.  The field index varies fastest so that the blocks
// working on the same tile for different fields run together and re-reads of
// a shared input hit L2.
// LD_E / ST_E select whether consecutive threads walk elements (the pencil is
// contiguous in memory) or pencils (pencils are adjacent in memory) when
// moving data to and from the tile, so global accesses stay coalesced.
#pragma once
#include <type_traits>
#include <utility>

#include "fft_engine.cuh"
#include "geometry.cuh"

namespace dd {

// An Op whose pencils follow the 2/3 rule along the transform axis says so
// with kept() (its largest kept |mode index| there): an inverse Op's load then
// returns zero in the removed band and a forward Op's store never reads it,
// and the transform prunes that band when kept() == kept23(L).
template <class Op, class = void> struct HasKept : std::false_type {};
template <class Op>
struct HasKept<Op, std::void_t<decltype(std::declval<const Op&>().kept())>> : std::true_type {};

template <typename T, class S, bool INV, class Op>
__device__ __forceinline__ void pass_fft(const Op& op, C<T>* tile, const C<T>* tw) {
    if constexpr (HasKept<Op>::value && IsLF<T>::value) {   // one copy of the transform for double-float
        if (op.kept() == kept23(S::L)) { pencil_fft_s<T, S, INV, true>(tile, tw); return; }
    }
    pencil_fft_s<T, S, INV, false>(tile, tw);
}

// Global -> tile: the P pencils of L elements starting at pencil f0, pencils
// beyond npen zero.  Each thread loads its elements in groups of G into
// registers before storing any of the group to shared memory, so a group's
// global loads are in flight together (element-by-element load / store keeps
// one load in flight per thread: the shared stores may not move above the
// loads of generic pointers).
template <typename T, int L, int P, int PS, int NT, bool LD_E, class Op>
__device__ __forceinline__ void load_tile(const Op& op, C<T>* tile, int fld, int s, int f0, int npen) {
    constexpr int N = L * P;
    constexpr int NPT = (N + NT - 1) / NT;
    constexpr int GB = (int)(128 / sizeof(C<T>));   // 128 bytes of loads per thread in flight
    constexpr int G = NPT < GB ? NPT : GB;
#pragma unroll
    for (int i0 = 0; i0 < NPT; i0 += G) {
        C<T> v[G];
#pragma unroll
        for (int i = 0; i < G; i++) {
            const int idx = threadIdx.x + (i0 + i) * NT;
            v[i] = zero<T>();
            if (i0 + i < NPT && (N % NT == 0 || idx < N)) {
                const int e = LD_E ? idx % L : idx / P;
                const int p = LD_E ? idx / L : idx % P;
                if (f0 + p < npen) v[i] = op.load(fld, s, e, f0 + p);
            }
        }
#pragma unroll
        for (int i = 0; i < G; i++) {
            const int idx = threadIdx.x + (i0 + i) * NT;
            if (i0 + i < NPT && (N % NT == 0 || idx < N)) {
                const int e = LD_E ? idx % L : idx / P;
                const int p = LD_E ? idx / L : idx % P;
                tile[e * PS + p] = v[i];
            }
        }
    }
}

template <typename T, int L, bool INV, bool LD_E, bool ST_E, class Op>
__global__ void __launch_bounds__(FFTCfg<L>::NT) k_pass(const Op op, int nfield) {
    extern __shared__ __align__(16) unsigned char dd_smem[];
    constexpr int P = Pencil<L>::P, PS = Pencil<L>::PS, NT = Pencil<L>::NT;
    C<T>* tile = reinterpret_cast<C<T>*>(dd_smem);
    C<T>* tw = tile + L * PS;
    load_twiddles<T, L>(tw, op.tw);
    const int fld = blockIdx.x % nfield;
    const int f0 = (blockIdx.x / nfield) * P;
    const int s = blockIdx.y + 65535 * blockIdx.z;
    const int npen = op.npencil();
    load_tile<T, L, P, PS, NT, LD_E>(op, tile, fld, s, f0, npen);
    __syncthreads();
    pass_fft<T, DefSched<L>, INV>(op, tile, tw);
    const int nst = op.nstore();
    for (int idx = threadIdx.x; idx < nst * P; idx += NT) {
        const int e = ST_E ? idx % nst : idx / P;
        const int p = ST_E ? idx / nst : idx % P;
        const int f = f0 + p;
        if (f < npen) op.store(fld, s, e, f, tile + p, PS);
    }
}

template <typename T, int L, bool INV, bool LD_E, bool ST_E, class Op>
int launch_pass(const Op& op, int npencil, int nslow, int nfield, cudaStream_t st) {
    constexpr int P = Pencil<L>::P, NT = Pencil<L>::NT;
    const size_t smem = Pencil<L>::template smem_bytes<T>();
    auto kern = k_pass<T, L, INV, LD_E, ST_E, Op>;
    static std::atomic<unsigned long long> configured{0};  // per instantiation and device
    DD_TRY(ensure_smem((const void*)kern, smem, configured));
    if (npencil <= 0 || nslow <= 0 || nfield <= 0) return DD_OK;
    if (nslow > 65535 && nslow % 65535 != 0) {
        set_error("pass: slow extent %d must be <= 65535 or a multiple of it", nslow);
        return DD_ERR_UNSUPPORTED;
    }
    dim3 grid(cdiv(npencil, P) * nfield, nslow > 65535 ? 65535 : nslow, nslow > 65535 ? nslow / 65535 : 1);
    static const std::string label = std::string(Op::name) + "_" + std::to_string(L) + PrecName<T>::s;
    DD_KT(label.c_str(), st, kern<<<grid, NT, smem, st>>>(op, nfield));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

// The same pass with an explicit schedule S (pencils per tile, threads, radix
// sequence): small tiles give a small single-run grid enough blocks to fill
// the GPU (a 128-point y pass of 43 kx pencils is 2 tiles of the default 32
// pencils, but 11 tiles of 4).
template <typename T, class S, bool INV, bool LD_E, bool ST_E, class Op>
__global__ void __launch_bounds__(S::NT) k_pass_sched(const Op op, int nfield) {
    extern __shared__ __align__(16) unsigned char dd_smem[];
    constexpr int L = S::L, P = S::P, PS = S::PS, NT = S::NT;
    C<T>* tile = reinterpret_cast<C<T>*>(dd_smem);
    C<T>* tw = tile + L * PS;
    load_twiddles<T, L>(tw, op.tw);
    const int fld = blockIdx.x % nfield;
    const int f0 = (blockIdx.x / nfield) * P;
    const int s = blockIdx.y + 65535 * blockIdx.z;
    const int npen = op.npencil();
    load_tile<T, L, P, PS, NT, LD_E>(op, tile, fld, s, f0, npen);
    __syncthreads();
    pass_fft<T, S, INV>(op, tile, tw);
    const int nst = op.nstore();
    for (int idx = threadIdx.x; idx < nst * P; idx += NT) {
        const int e = ST_E ? idx % nst : idx / P;
        const int p = ST_E ? idx / nst : idx % P;
        const int f = f0 + p;
        if (f < npen) op.store(fld, s, e, f, tile + p, PS);
    }
}

template <typename T, class S, bool INV, bool LD_E, bool ST_E, class Op>
int launch_pass_sched(const Op& op, int npencil, int nslow, int nfield, cudaStream_t st) {
    const size_t smem = S::template smem_bytes<T>();
    auto kern = k_pass_sched<T, S, INV, LD_E, ST_E, Op>;
    static std::atomic<unsigned long long> configured{0};
    DD_TRY(ensure_smem((const void*)kern, smem, configured));
    if (npencil <= 0 || nslow <= 0 || nfield <= 0) return DD_OK;
    DD_CHECK_ARG(nslow <= 65535, "pass: slow extent %d must be <= 65535", nslow);
    dim3 grid(cdiv(npencil, S::P) * nfield, nslow, 1);
    static const std::string label = std::string(Op::name) + "_" + std::to_string(S::L) + "s" + PrecName<T>::s;
    DD_KT(label.c_str(), st, kern<<<grid, S::NT, smem, st>>>(op, nfield));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

// Small-tile schedules (4 pencils, 16 threads each) for single-run 2D grids.
template <int L> struct SmallSched;
template <> struct SmallSched<64> { using S = Sched<64, 4, 64, 4, 4, 4>; };
template <> struct SmallSched<128> { using S = Sched<128, 4, 64, 8, 4, 4>; };

// Launch a pass with the small-tile schedule when one exists for length L;
// returns 1 (not launched) otherwise.
template <typename T, bool INV, bool LD_E, bool ST_E, class Op>
int launch_pass_small(int L, const Op& op, int npencil, int nslow, int nfield, cudaStream_t st) {
    if (L == 64) return launch_pass_sched<T, typename SmallSched<64>::S, INV, LD_E, ST_E>(op, npencil, nslow, nfield, st);
    if (L == 128) return launch_pass_sched<T, typename SmallSched<128>::S, INV, LD_E, ST_E>(op, npencil, nslow, nfield, st);
    return 1;
}

// Tile variants of the default schedule for the 2D y passes of 64..512-point
// grids, chosen per plan by the ensemble autotuner (dd_plan_set_schedule):
// the same radix sequence as the default (so every pencil's arithmetic, and
// its result, is identical) on fewer pencils per block: variant 1 the
// smallest tile (2-4 pencils), variant 2 a middle one (4-8 pencils).
constexpr int kYSchedVariants = 3;
template <int L, int V> struct YVariant;
template <> struct YVariant<64, 1>  { using S = Sched<64, 4, 32, 8, 8, 1>; };
template <> struct YVariant<64, 2>  { using S = Sched<64, 8, 64, 8, 8, 1>; };
template <> struct YVariant<128, 1> { using S = Sched<128, 4, 32, 16, 8, 1>; };
template <> struct YVariant<128, 2> { using S = Sched<128, 8, 64, 16, 8, 1>; };
template <> struct YVariant<256, 1> { using S = Sched<256, 4, 64, 16, 16, 1>; };
template <> struct YVariant<256, 2> { using S = Sched<256, 8, 128, 16, 16, 1>; };
template <> struct YVariant<512, 1> { using S = Sched<512, 2, 64, 8, 8, 8>; };
template <> struct YVariant<512, 2> { using S = Sched<512, 4, 128, 8, 8, 8>; };

// Launch a pass with tile variant v (1 or 2) of length L; returns 1 (not
// launched) when no variant exists.
template <typename T, bool INV, bool LD_E, bool ST_E, class Op>
int launch_pass_variant(int L, int v, const Op& op, int npencil, int nslow, int nfield, cudaStream_t st) {
#define DD_YV(N, VV) \
    if (L == N && v == VV) \
        return launch_pass_sched<T, typename YVariant<N, VV>::S, INV, LD_E, ST_E>(op, npencil, nslow, nfield, st);
    DD_YV(64, 1) DD_YV(64, 2) DD_YV(128, 1) DD_YV(128, 2) DD_YV(256, 1) DD_YV(256, 2) DD_YV(512, 1) DD_YV(512, 2)
#undef DD_YV
    return 1;
}

// ============================================================ 3D operators
// Inverse along kz: K[ky][kz][kx] (kept entries) -> W1[kyc][z][kxc].
template <typename T, typename KT>
struct OpZInv3 {
    using V = typename Vec2<T>::type;
    static constexpr const char* name = "z_inv";
    static constexpr int lmin = 8, lmax = 512;
    using KV = typename Vec2<KT>::type;
    Geo3 g; CPtrs in; Ptrs out; const V* tw;
    __device__ int kept() const { return g.Mz; }
    __device__ int npencil() const { return g.Kx; }
    __device__ int nstore() const { return g.Nz; }
    __device__ C<T> load(int fld, int kyc, int e, int kx) const {
        if (!kept_full(e, g.Nz, g.Mz)) return zero<T>();
        const int ky = compact_to_full(kyc, g.Ny, g.Ky);
        const KV v = ((const KV*)in.p[fld])[((int64_t)ky * g.Nz + e) * g.Nh + kx];
        return mk<T>((T)v.x, (T)v.y);
    }
    __device__ void store(int fld, int kyc, int e, int kx, const C<T>* col, int PS) const {
        stc<T>((V*)out.p[fld] + ((int64_t)kyc * g.Nz + e) * g.Kx + kx, col[e * PS]);
    }
};

// Inverse along ky: W1[kyc][z][kxc] -> W2[z][y][kxc].
template <typename T>
struct OpYInv3 {
    using V = typename Vec2<T>::type;
    static constexpr const char* name = "y_inv";
    static constexpr int lmin = 8, lmax = 512;
    Geo3 g; CPtrs in; Ptrs out; const V* tw;
    __device__ int kept() const { return g.My; }
    __device__ int npencil() const { return g.Kx; }
    __device__ int nstore() const { return g.Ny; }
    __device__ C<T> load(int fld, int z, int e, int kx) const {
        if (!kept_full(e, g.Ny, g.My)) return zero<T>();
        const int kyc = full_to_compact(e, g.Ny, g.Ky);
        return ldc<T>((const V*)in.p[fld] + ((int64_t)kyc * g.Nz + z) * g.Kx + kx);
    }
    __device__ void store(int fld, int z, int e, int kx, const C<T>* col, int PS) const {
        stc<T>((V*)out.p[fld] + ((int64_t)z * g.Ny + e) * g.Kx + kx, col[e * PS]);
    }
};

// Hermitian packing of two half-spectrum rows A, B (kx < Kx) into one full
// complex sequence Z = A + iB whose inverse DFT is a + ib.  The imaginary
// parts at kx = 0 and kx = N/2 are dropped, as a c2r transform does.
template <typename T, typename V>
__device__ __forceinline__ C<T> pack_rows(const V* ra, const V* rb, int e, int N, int K) {
    const int kx = e <= N / 2 ? e : N - e;
    if (kx >= K) return zero<T>();
    C<T> A = ldc<T>(ra + kx), B = ldc<T>(rb + kx);
    if (kx == 0 || 2 * kx == N) { A.y = T(0); B.y = T(0); }
    if (e > N / 2) { A.y = -A.y; B.y = -B.y; }
    return mk<T>(A.x - B.y, A.y + B.x);
}

// Separation of the forward DFT Z of a + ib into the half spectra A (a), B (b)
// at bin k, times s, from z = Z[k] and zn = Z[N - k] (Z[0] at k = 0).
template <typename T>
__device__ __forceinline__ void unpack_pair(C<T> z, C<T> zn, T s, C<T>& A, C<T>& B) {
    const T h = T(0.5) * s;
    A = mk<T>((z.x + zn.x) * h, (z.y - zn.y) * h);
    B = mk<T>((z.y + zn.y) * h, (zn.x - z.x) * h);
}

// The same with Z read from a tile column of row stride PS.
template <typename T>
__device__ __forceinline__ void unpack_rows(const C<T>* col, int PS, int k, int N, T s, C<T>& A, C<T>& B) {
    unpack_pair<T>(col[k * PS], col[(k == 0 ? 0 : N - k) * PS], s, A, B);
}

// c2r along x: W2 rows [r][kxc] (r = z*Ny + y) -> x rows; pencil f = row pair.
template <typename T, typename XT>
struct OpXc2r3 {
    using V = typename Vec2<T>::type;
    static constexpr const char* name = "x_c2r";
    static constexpr int lmin = 8, lmax = 512;
    int nrows, Nx, Kx; CPtrs in; Ptrs out; const V* tw;
    __device__ int kept() const { return Kx - 1; }
    __device__ int npencil() const { return (nrows + 1) / 2; }
    __device__ int nstore() const { return Nx; }
    __device__ C<T> load(int fld, int, int e, int f) const {
        const V* W = (const V*)in.p[fld];
        const int ra = 2 * f, rb = min(2 * f + 1, nrows - 1);
        C<T> z = pack_rows<T>(W + (int64_t)ra * Kx, W + (int64_t)rb * Kx, e, Nx, Kx);
        if (rb == ra) z.y = T(0);
        return z;
    }
    __device__ void store(int fld, int, int e, int f, const C<T>* col, int PS) const {
        XT* x = (XT*)out.p[fld];
        const C<T> v = col[e * PS];
        x[(int64_t)(2 * f) * Nx + e] = (XT)v.x;
        if (2 * f + 1 < nrows) x[(int64_t)(2 * f + 1) * Nx + e] = (XT)v.y;
    }
};

// r2c along x: x rows -> W2 rows [r][kxc], scaled by s (the 1/N of the
// reference's forward transform).
template <typename T, typename XT>
struct OpXr2c3 {
    using V = typename Vec2<T>::type;
    static constexpr const char* name = "x_r2c";
    static constexpr int lmin = 8, lmax = 512;
    int nrows, Nx, Kx; T s; CPtrs in; Ptrs out; const V* tw;
    __device__ int kept() const { return Kx - 1; }
    __device__ int npencil() const { return (nrows + 1) / 2; }
    __device__ int nstore() const { return Kx; }
    __device__ C<T> load(int fld, int, int e, int f) const {
        const XT* x = (const XT*)in.p[fld];
        const T a = (T)x[(int64_t)(2 * f) * Nx + e];
        const T b = (2 * f + 1 < nrows) ? (T)x[(int64_t)(2 * f + 1) * Nx + e] : T(0);
        return mk<T>(a, b);
    }
    __device__ void store(int fld, int, int k, int f, const C<T>* col, int PS) const {
        C<T> A, B;
        unpack_rows<T>(col, PS, k, Nx, s, A, B);
        V* W = (V*)out.p[fld];
        stc<T>(W + (int64_t)(2 * f) * Kx + k, A);
        if (2 * f + 1 < nrows) stc<T>(W + (int64_t)(2 * f + 1) * Kx + k, B);
    }
};

// Forward along y: W2[z][y][kxc] -> W1[kyc][z][kxc] (kept ky only).
template <typename T>
struct OpYFwd3 {
    using V = typename Vec2<T>::type;
    static constexpr const char* name = "y_fwd";
    static constexpr int lmin = 8, lmax = 512;
    Geo3 g; CPtrs in; Ptrs out; const V* tw;
    __device__ int kept() const { return g.My; }
    __device__ int npencil() const { return g.Kx; }
    __device__ int nstore() const { return g.Ny; }
    __device__ C<T> load(int fld, int z, int e, int kx) const {
        return ldc<T>((const V*)in.p[fld] + ((int64_t)z * g.Ny + e) * g.Kx + kx);
    }
    __device__ void store(int fld, int z, int e, int kx, const C<T>* col, int PS) const {
        if (!kept_full(e, g.Ny, g.My)) return;
        const int kyc = full_to_compact(e, g.Ny, g.Ky);
        stc<T>((V*)out.p[fld] + ((int64_t)kyc * g.Nz + z) * g.Kx + kx, col[e * PS]);
    }
};

// Forward along z: W1[kyc][z][kxc] -> K[ky][kz][kx] (kept ky, kx < Kx); the
// non-kept kz entries of those columns are written as zeros.
template <typename T, typename KT>
struct OpZFwd3 {
    using V = typename Vec2<T>::type;
    static constexpr const char* name = "z_fwd";
    static constexpr int lmin = 8, lmax = 512;
    using KV = typename Vec2<KT>::type;
    Geo3 g; CPtrs in; Ptrs out; const V* tw;
    __device__ int kept() const { return g.Mz; }
    __device__ int npencil() const { return g.Kx; }
    __device__ int nstore() const { return g.Nz; }
    __device__ C<T> load(int fld, int kyc, int e, int kx) const {
        return ldc<T>((const V*)in.p[fld] + ((int64_t)kyc * g.Nz + e) * g.Kx + kx);
    }
    __device__ void store(int fld, int kyc, int e, int kx, const C<T>* col, int PS) const {
        const int ky = compact_to_full(kyc, g.Ny, g.Ky);
        KV v;
        if (kept_full(e, g.Nz, g.Mz)) { const C<T> c = col[e * PS]; v.x = (KT)c.x; v.y = (KT)c.y; }
        else { v.x = KT(0); v.y = KT(0); }
        ((KV*)out.p[fld])[((int64_t)ky * g.Nz + e) * g.Nh + kx] = v;
    }
};

// ============================================================ 2D operators
// Inverse along ky: K[kx][ky] (kept) -> W[y][kxc]; pencil = kx row.
template <typename T, typename KT>
struct OpYInv2 {
    using V = typename Vec2<T>::type;
    static constexpr const char* name = "y_inv2d";
    static constexpr int lmin = 8, lmax = 512;
    using KV = typename Vec2<KT>::type;
    Geo2 g; CPtrs in; Ptrs out; const V* tw;
    __device__ int kept() const { return g.My; }
    __device__ int npencil() const { return g.Kx; }
    __device__ int nstore() const { return g.Ny; }
    __device__ C<T> load(int fld, int, int e, int kx) const {
        if (!kept_full(e, g.Ny, g.My)) return zero<T>();
        const KV v = ((const KV*)in.p[fld])[(int64_t)kx * g.Ny + e];
        return mk<T>((T)v.x, (T)v.y);
    }
    __device__ void store(int fld, int, int e, int kx, const C<T>* col, int PS) const {
        stc<T>((V*)out.p[fld] + (int64_t)e * g.Kx + kx, col[e * PS]);
    }
};

// Forward along y: W[y][kxc] -> K[kx][ky] (all ky; zeros where not kept).
template <typename T, typename KT>
struct OpYFwd2 {
    using V = typename Vec2<T>::type;
    static constexpr const char* name = "y_fwd2d";
    static constexpr int lmin = 8, lmax = 512;
    using KV = typename Vec2<KT>::type;
    Geo2 g; CPtrs in; Ptrs out; const V* tw;
    __device__ int kept() const { return g.My; }
    __device__ int npencil() const { return g.Kx; }
    __device__ int nstore() const { return g.Ny; }
    __device__ C<T> load(int fld, int, int e, int kx) const {
        return ldc<T>((const V*)in.p[fld] + (int64_t)e * g.Kx + kx);
    }
    __device__ void store(int fld, int, int e, int kx, const C<T>* col, int PS) const {
        KV v;
        if (kept_full(e, g.Ny, g.My)) { const C<T> c = col[e * PS]; v.x = (KT)c.x; v.y = (KT)c.y; }
        else { v.x = KT(0); v.y = KT(0); }
        ((KV*)out.p[fld])[(int64_t)kx * g.Ny + e] = v;
    }
};

}  // namespace dd
