// Training and inference kernels of the closure MLP (layout, rounding points
// and tiling in mlp.cuh): forward, forward + backward with per-block FP32
// gradient partials reduced in a fixed order (bitwise reproducible), Adam, the
// FP32 -> BF16 weight copy, and the sample normalisation.
#include "dd_common.cuh"
#include "mlp.cuh"

namespace dd {

constexpr int MLP_GRAD_MAX_BLOCKS = 152 * 3;
constexpr int MLP_PSTRIDE = MLP_NPARAM + 1;   // per-block partial: gradients, then the squared-error sum

static inline int grad_blocks(int64_t n) {
    const int64_t tiles = (n + 63) / 64;
    int64_t b = (tiles + 1) / 2;
    if (b > MLP_GRAD_MAX_BLOCKS) b = MLP_GRAD_MAX_BLOCKS;
    return (int)(b < 1 ? 1 : b);
}

static inline unsigned ew_blocks(int64_t n, int per) {
    int64_t b = (n + per - 1) / per;
    if (b > 152 * 16) b = 152 * 16;
    return (unsigned)(b < 1 ? 1 : b);
}

// X rows of a tile (optionally gathered through idx) into s.x.
__device__ __forceinline__ void load_x_tile(MlpFwdSmem& s, const bf16* X, const int64_t* idx, int64_t base,
                                            int64_t n) {
    // 64 rows x 16 bf16 = 64 x 2 uint4
    for (int i = threadIdx.x; i < 64 * 2; i += blockDim.x) {
        const int r = i >> 1, h = i & 1;
        const int64_t sidx = base + r;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (sidx < n) {
            const int64_t row = idx ? idx[sidx] : sidx;
            v = reinterpret_cast<const uint4*>(X + row * MLP_IN)[h];
        }
        const bf16* e = reinterpret_cast<const bf16*>(&v);
#pragma unroll
        for (int j = 0; j < 8; j++) s.x[r * LDI + 8 * h + j] = e[j];
    }
}

// Inference: X [n][16] bf16 -> Y [n][8] f32.
__global__ void __launch_bounds__(MLP_THREADS) k_mlp_infer(const bf16* __restrict__ X, float* __restrict__ Y,
                                                           int64_t n, const bf16* wb, const float* p) {
    extern __shared__ __align__(16) unsigned char mlp_smem[];
    MlpFwdSmem& s = *reinterpret_cast<MlpFwdSmem*>(mlp_smem);
    mlp_load_weights(s, wb, p);
    const int r0 = 16 * (threadIdx.x >> 5);
    for (int64_t base = (int64_t)blockIdx.x * 64; base < n; base += (int64_t)gridDim.x * 64) {
        __syncthreads();
        load_x_tile(s, X, nullptr, base, n);
        __syncthreads();
        float y[4];
        mlp_forward_warp(s, r0, y);
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int64_t sidx = base + r0 + frag_row(q);
            if (sidx < n) Y[sidx * MLP_OUT + frag_col(q)] = y[q];
        }
    }
}

// Forward + backward over samples [0, n) (row idx[s] when idx is given) for
// the loss L = sum_s sum_{c<6} (Y - T)^2 / (n_total * 6).  Block b writes its
// gradient sums and squared-error sum to part[b][0 .. NPARAM].
__global__ void __launch_bounds__(MLP_THREADS) k_mlp_grad(const bf16* __restrict__ X, const float* __restrict__ T,
                                                          const int64_t* __restrict__ idx, int64_t n,
                                                          const bf16* wb, const float* p, float scale,
                                                          float* __restrict__ part) {
    extern __shared__ __align__(16) unsigned char mlp_smem[];
    MlpSmem& s = *reinterpret_cast<MlpSmem*>(mlp_smem);
    mlp_load_weights(s, wb, p);
    const int warp = threadIdx.x >> 5, r0 = 16 * warp;
    float gw2[8][4] = {}, gw1[2][4] = {}, gw3[2][4] = {};
    float gb1 = 0.f, gb2 = 0.f, gb3 = 0.f, sse = 0.f;
    for (int64_t base = (int64_t)blockIdx.x * 64; base < n; base += (int64_t)gridDim.x * 64) {
        __syncthreads();
        load_x_tile(s, X, idx, base, n);
        __syncthreads();
        float y[4];
        mlp_forward_warp(s, r0, y);
        // dL/dY (zero for padding samples and the unused outputs 6, 7)
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int r = r0 + frag_row(q), col = frag_col(q);
            const int64_t sidx = base + r;
            float d = 0.f;
            if (sidx < n && col < MLP_NOUT) {
                const int64_t row = idx ? idx[sidx] : sidx;
                const float e = y[q] - T[row * MLP_OUT + col];
                sse += e * e;
                d = scale * e;
            }
            s.dyf[r * MLP_OUT + col] = d;
            s.dy[r * LDI + col] = __float2bfloat16_rn(d);
            s.dy[r * LDI + 8 + col] = __float2bfloat16_rn(0.f);
        }
        __syncwarp();
        {   // dH2 = (dY W3) * (1 - H2^2)
            uint32_t a[4];
            mlp_load_a(a, s.dy + r0 * LDI, LDI, 1);
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                float c[4] = {0.f, 0.f, 0.f, 0.f};
                uint32_t b[2];
                mlp_load_b(b, s.w3 + 8 * nt, LDH, 1);
                mma_bf16_16816(c, a, b);
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int r = r0 + frag_row(q), col = 8 * nt + frag_col(q);
                    const float h = __bfloat162float(s.h2[r * LDH + col]);
                    s.dh2[r * LDH + col] = __float2bfloat16_rn(c[q] * (1.f - h * h));
                }
            }
        }
        __syncwarp();
        {   // dH1 = (dH2 W2) * (1 - H1^2)
            uint32_t a[4][4];
#pragma unroll
            for (int kt = 0; kt < 4; kt++) mlp_load_a(a[kt], s.dh2 + r0 * LDH + 16 * kt, LDH, 1);
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                for (int kt = 0; kt < 4; kt++) {
                    uint32_t b[2];
                    mlp_load_b(b, s.w2 + (16 * kt) * LDH + 8 * nt, LDH, 1);
                    mma_bf16_16816(c, a[kt], b);
                }
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int r = r0 + frag_row(q), col = 8 * nt + frag_col(q);
                    const float h = __bfloat162float(s.h1[r * LDH + col]);
                    s.dh1[r * LDH + col] = __float2bfloat16_rn(c[q] * (1.f - h * h));
                }
            }
        }
        __syncthreads();
        // weight gradients, K = the 64 samples of the tile
        // dW2[o][i] += sum_s dH2[s][o] H1[s][i]: warp w takes o in [16 w, 16 w + 16)
#pragma unroll
        for (int kt = 0; kt < 4; kt++) {
            uint32_t a[4];
            mlp_load_a(a, s.dh2 + (16 * kt) * LDH + 16 * warp, 1, LDH);
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                uint32_t b[2];
                mlp_load_b(b, s.h1 + (16 * kt) * LDH + 8 * nt, LDH, 1);
                mma_bf16_16816(gw2[nt], a, b);
            }
        }
        // dW1[o][i] += sum_s dH1[s][o] X[s][i]
#pragma unroll
        for (int kt = 0; kt < 4; kt++) {
            uint32_t a[4];
            mlp_load_a(a, s.dh1 + (16 * kt) * LDH + 16 * warp, 1, LDH);
#pragma unroll
            for (int nt = 0; nt < 2; nt++) {
                uint32_t b[2];
                mlp_load_b(b, s.x + (16 * kt) * LDI + 8 * nt, LDI, 1);
                mma_bf16_16816(gw1[nt], a, b);
            }
        }
        // dW3[o][i] += sum_s dY[s][o] H2[s][i]: one m-tile (o < 8 used), warp w takes i in [16 w, 16 w + 16)
#pragma unroll
        for (int kt = 0; kt < 4; kt++) {
            uint32_t a[4];
            mlp_load_a(a, s.dy + (16 * kt) * LDI, 1, LDI);
#pragma unroll
            for (int j = 0; j < 2; j++) {
                uint32_t b[2];
                mlp_load_b(b, s.h2 + (16 * kt) * LDH + 8 * (2 * warp + j), LDH, 1);
                mma_bf16_16816(gw3[j], a, b);
            }
        }
        if (threadIdx.x < MLP_H) {
            float a1 = 0.f, a2 = 0.f;
            for (int r = 0; r < 64; r++) {
                a1 += __bfloat162float(s.dh1[r * LDH + threadIdx.x]);
                a2 += __bfloat162float(s.dh2[r * LDH + threadIdx.x]);
            }
            gb1 += a1;
            gb2 += a2;
        }
        if (threadIdx.x < MLP_OUT) {
            float a3 = 0.f;
            for (int r = 0; r < 64; r++) a3 += s.dyf[r * MLP_OUT + threadIdx.x];
            gb3 += a3;
        }
    }
    // every gradient entry has exactly one owner: plain stores
    float* P = part + (int64_t)blockIdx.x * MLP_PSTRIDE;
#pragma unroll
    for (int nt = 0; nt < 8; nt++)
#pragma unroll
        for (int q = 0; q < 4; q++) P[OFF_W2 + (16 * warp + frag_row(q)) * MLP_H + 8 * nt + frag_col(q)] = gw2[nt][q];
#pragma unroll
    for (int nt = 0; nt < 2; nt++)
#pragma unroll
        for (int q = 0; q < 4; q++) P[OFF_W1 + (16 * warp + frag_row(q)) * MLP_IN + 8 * nt + frag_col(q)] = gw1[nt][q];
#pragma unroll
    for (int j = 0; j < 2; j++)
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int o = frag_row(q);
            if (o < MLP_OUT) P[OFF_W3 + o * MLP_H + 8 * (2 * warp + j) + frag_col(q)] = gw3[j][q];
        }
    if (threadIdx.x < MLP_H) {
        P[OFF_B1 + threadIdx.x] = gb1;
        P[OFF_B2 + threadIdx.x] = gb2;
    }
    if (threadIdx.x < MLP_OUT) P[OFF_B3 + threadIdx.x] = gb3;
    for (int o = 16; o > 0; o >>= 1) sse += __shfl_down_sync(0xffffffffu, sse, o);
    if ((threadIdx.x & 31) == 0) s.red[warp] = sse;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int w = 0; w < MLP_THREADS / 32; w++) t += s.red[w];
        P[MLP_NPARAM] = t;
    }
}

// grad[j] = sum_b part[b][j] in block order; loss[0] = sum_b part[b][NPARAM].
__global__ void k_mlp_reduce(const float* __restrict__ part, int nblk, float* grad, float* loss) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j <= MLP_NPARAM; j += gridDim.x * blockDim.x) {
        float t = 0.f;
        for (int b = 0; b < nblk; b++) t += part[(int64_t)b * MLP_PSTRIDE + j];
        if (j < MLP_NPARAM) grad[j] = t;
        else if (loss) loss[0] = t;
    }
}

// FP32 master -> BF16 weight copy (W3 rows 8..15 zero).
__global__ void k_mlp_pack(const float* p, bf16* wb) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < MLP_NBF; i += gridDim.x * blockDim.x) {
        float v;
        if (i < BOFF_W2) v = p[OFF_W1 + i];
        else if (i < BOFF_W3) v = p[OFF_W2 + (i - BOFF_W2)];
        else {
            const int j = i - BOFF_W3;
            v = j < MLP_OUT * MLP_H ? p[OFF_W3 + j] : 0.f;
        }
        wb[i] = __float2bfloat16_rn(v);
    }
}

// Adam (Kingma & Ba, 2015): m = b1 m + (1 - b1) g; v = b2 v + (1 - b2) g^2;
// p -= lr (m / bc1) / (sqrt(v / bc2) + eps) with bc = 1 - beta^step.
__global__ void k_mlp_adam(float* p, const float* g, float* m, float* v, float lr, float b1, float b2, float eps,
                           float bc1, float bc2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < MLP_NPARAM; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    }
}

// raw [n][16] f32 (features 0..9, stresses 10..15) -> X [n][16] bf16 and
// T [n][8] f32 normalised by norm (mlp.cuh).
__global__ void k_mlp_normalize(const float* __restrict__ raw, int64_t n, const float* __restrict__ norm,
                                bf16* __restrict__ X, float* __restrict__ T) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float* r = raw + i * 16;
        __align__(16) bf16 xr[MLP_IN];
#pragma unroll
        for (int a = 0; a < MLP_IN; a++)
            xr[a] = __float2bfloat16_rn(a < MLP_NIN ? (r[a] - norm[NORM_IN_MEAN + a]) * norm[NORM_IN_SCALE + a] : 0.f);
        reinterpret_cast<uint4*>(X + i * MLP_IN)[0] = reinterpret_cast<const uint4*>(xr)[0];
        reinterpret_cast<uint4*>(X + i * MLP_IN)[1] = reinterpret_cast<const uint4*>(xr)[1];
#pragma unroll
        for (int c = 0; c < MLP_OUT; c++)
            T[i * MLP_OUT + c] =
                c < MLP_NOUT ? (r[MLP_NIN + c] - norm[NORM_OUT_MEAN + c]) / norm[NORM_OUT_SCALE + c] : 0.f;
    }
}

}  // namespace dd

using namespace dd;

extern "C" {

int dd_mlp_sizes(int* nparam, int* nbf16, int* nnorm, int* in_dim, int* out_dim) {
    DD_CHECK_ARG(nparam && nbf16 && nnorm && in_dim && out_dim, "dd_mlp_sizes: null pointer");
    *nparam = MLP_NPARAM;
    *nbf16 = MLP_NBF;
    *nnorm = MLP_NNORM;
    *in_dim = MLP_IN;
    *out_dim = MLP_OUT;
    return DD_OK;
}

int dd_mlp_workspace_size(int64_t n, size_t* bytes) {
    DD_CHECK_ARG(bytes && n >= 0, "dd_mlp_workspace_size: bad arguments");
    *bytes = (size_t)grad_blocks(n) * MLP_PSTRIDE * sizeof(float);
    return DD_OK;
}

int dd_mlp_pack(const float* params, void* wbf16, void* stream) {
    DD_CHECK_ARG(params && wbf16, "dd_mlp_pack: null pointer");
    cudaStream_t st = (cudaStream_t)stream;
    DD_KT("mlp_pack", st, k_mlp_pack<<<ew_blocks(MLP_NBF, 256), 256, 0, st>>>(params, (bf16*)wbf16));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

int dd_mlp_infer(const void* X, float* Y, int64_t n, const void* wbf16, const float* params, void* stream) {
    DD_CHECK_ARG(X && Y && wbf16 && params && n >= 0, "dd_mlp_infer: bad arguments");
    if (n == 0) return DD_OK;
    cudaStream_t st = (cudaStream_t)stream;
    static std::atomic<unsigned long long> configured{0};
    DD_TRY(ensure_smem((const void*)k_mlp_infer, sizeof(MlpFwdSmem), configured));
    unsigned nb = ew_blocks(n, 64);
    if (nb > 152 * 4) nb = 152 * 4;
    DD_KT("mlp_infer", st,
          k_mlp_infer<<<nb, MLP_THREADS, sizeof(MlpFwdSmem), st>>>((const bf16*)X, Y, n, (const bf16*)wbf16, params));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

int dd_mlp_grad(const void* X, const float* T, const int64_t* idx, int64_t n, int64_t n_total, const void* wbf16,
                const float* params, float* grad, float* loss, void* work, size_t work_bytes, void* stream) {
    DD_CHECK_ARG(X && T && wbf16 && params && grad && work && n > 0 && n_total >= n, "dd_mlp_grad: bad arguments");
    const int nb = grad_blocks(n);
    DD_CHECK_ARG(work_bytes >= (size_t)nb * MLP_PSTRIDE * sizeof(float), "dd_mlp_grad: workspace too small");
    cudaStream_t st = (cudaStream_t)stream;
    static std::atomic<unsigned long long> configured{0};
    DD_TRY(ensure_smem((const void*)k_mlp_grad, sizeof(MlpSmem), configured));
    const float scale = 2.0f / ((float)n_total * (float)MLP_NOUT);
    float* part = (float*)work;
    DD_KT("mlp_grad", st,
          k_mlp_grad<<<nb, MLP_THREADS, sizeof(MlpSmem), st>>>((const bf16*)X, T, idx, n, (const bf16*)wbf16, params,
                                                                scale, part));
    DD_LAUNCH_CHECK();
    DD_KT("mlp_reduce", st, k_mlp_reduce<<<ew_blocks(MLP_NPARAM + 1, 256), 256, 0, st>>>(part, nb, grad, loss));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

int dd_mlp_adam(float* params, const float* grad, float* m, float* v, int step, float lr, float beta1, float beta2,
                float eps, void* wbf16, void* stream) {
    DD_CHECK_ARG(params && grad && m && v && wbf16 && step >= 1, "dd_mlp_adam: bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    const float bc1 = 1.f - powf(beta1, (float)step), bc2 = 1.f - powf(beta2, (float)step);
    DD_KT("mlp_adam", st,
          k_mlp_adam<<<ew_blocks(MLP_NPARAM, 256), 256, 0, st>>>(params, grad, m, v, lr, beta1, beta2, eps, bc1, bc2));
    DD_LAUNCH_CHECK();
    return dd_mlp_pack(params, wbf16, stream);
}

int dd_mlp_normalize(const float* raw, int64_t n, const float* norm, void* X, float* T, void* stream) {
    DD_CHECK_ARG(raw && norm && X && T && n >= 0, "dd_mlp_normalize: bad arguments");
    if (n == 0) return DD_OK;
    cudaStream_t st = (cudaStream_t)stream;
    DD_KT("mlp_normalize", st, k_mlp_normalize<<<ew_blocks(n, 256), 256, 0, st>>>(raw, n, norm, (bf16*)X, T));
    DD_LAUNCH_CHECK();
    return DD_OK;
}

}  // extern "C"
