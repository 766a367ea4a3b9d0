// Pointwise MLP of the learned subgrid closure: 10 -> 64 -> 64 -> 6 with tanh
// hidden activations (inputs padded to 16 columns, outputs to 8), BF16
// weights and activations on the tensor cores (mma.sync m16n8k16, BF16 x BF16
// -> FP32) with FP32 accumulation, FP32 biases and FP32 master weights.
//
// Rounding points, reproduced by the CPU oracle: the inputs X, the weights,
// the hidden activations H1 and H2 and the backward signals dY, dH2, dH1 are
// BF16; every matrix product accumulates in FP32; biases, outputs, the loss
// and the weight gradients are FP32.  tanh'(z) is taken as 1 - H^2 from the
// BF16 activation H.
//
// A block of 4 warps works on tiles of 64 samples; warp w owns samples
// [16 w, 16 w + 16) of a tile.  Shared-memory rows are padded (24 and 72
// elements) so that the fragment loads of both orientations are free of bank
// conflicts.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace dd {

typedef __nv_bfloat16 bf16;

constexpr int MLP_IN = 16, MLP_H = 64, MLP_OUT = 8;
constexpr int MLP_NIN = 10, MLP_NOUT = 6;   // inputs / outputs in use
// FP32 parameter vector: W1[64][16], b1[64], W2[64][64], b2[64], W3[8][64], b3[8]
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + MLP_H * MLP_IN, OFF_W2 = OFF_B1 + MLP_H;
constexpr int OFF_B2 = OFF_W2 + MLP_H * MLP_H, OFF_W3 = OFF_B2 + MLP_H, OFF_B3 = OFF_W3 + MLP_OUT * MLP_H;
constexpr int MLP_NPARAM = OFF_B3 + MLP_OUT;
// BF16 weight copy: W1[64][16], W2[64][64], W3[16][64] (rows 8..15 zero)
constexpr int BOFF_W1 = 0, BOFF_W2 = BOFF_W1 + MLP_H * MLP_IN, BOFF_W3 = BOFF_W2 + MLP_H * MLP_H;
constexpr int MLP_NBF = BOFF_W3 + 16 * MLP_H;
// normalisation vector: in_mean[16], in_scale[16], out_mean[8], out_scale[8];
// network input = (feature - in_mean) * in_scale, stress = y * out_scale + out_mean
constexpr int NORM_IN_MEAN = 0, NORM_IN_SCALE = 16, NORM_OUT_MEAN = 32, NORM_OUT_SCALE = 40, MLP_NNORM = 48;
// padded shared-memory row strides (elements)
constexpr int LDI = 24, LDH = 72;
constexpr int MLP_THREADS = 128;

struct MlpFwdSmem {
    bf16 w1[MLP_H * LDI];     // [out][in]
    bf16 w2[MLP_H * LDH];     // [out][in]
    bf16 w3[16 * LDH];        // [out][in], rows 8..15 zero
    float b1[MLP_H], b2[MLP_H], b3[MLP_OUT];
    bf16 x[64 * LDI];         // [sample][in]
    bf16 h1[64 * LDH];        // [sample][hidden]
    bf16 h2[64 * LDH];
};

struct MlpSmem : MlpFwdSmem {
    bf16 dy[64 * LDI];        // [sample][out], columns 8..15 zero
    float dyf[64 * MLP_OUT];
    bf16 dh2[64 * LDH];
    bf16 dh1[64 * LDH];
    float red[MLP_THREADS / 32];
};

__device__ __forceinline__ uint32_t pack2(bf16 lo, bf16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

// A fragment (16 x 16, row major): element (r, k) at base[r * rs + k * ks]
__device__ __forceinline__ void mlp_load_a(uint32_t a[4], const bf16* base, int rs, int ks) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    a[0] = pack2(base[g * rs + (2 * t) * ks], base[g * rs + (2 * t + 1) * ks]);
    a[1] = pack2(base[(g + 8) * rs + (2 * t) * ks], base[(g + 8) * rs + (2 * t + 1) * ks]);
    a[2] = pack2(base[g * rs + (2 * t + 8) * ks], base[g * rs + (2 * t + 9) * ks]);
    a[3] = pack2(base[(g + 8) * rs + (2 * t + 8) * ks], base[(g + 8) * rs + (2 * t + 9) * ks]);
}

// B fragment (16 x 8, column major): element (k, n) at base[k * ks + n * ns]
__device__ __forceinline__ void mlp_load_b(uint32_t b[2], const bf16* base, int ks, int ns) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    b[0] = pack2(base[(2 * t) * ks + g * ns], base[(2 * t + 1) * ks + g * ns]);
    b[1] = pack2(base[(2 * t + 8) * ks + g * ns], base[(2 * t + 9) * ks + g * ns]);
}

__device__ __forceinline__ void mma_bf16_16816(float c[4], const uint32_t a[4], const uint32_t b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Position of accumulator element q (0..3) of this lane in a 16 x 8 tile.
__device__ __forceinline__ int frag_row(int q) { return ((threadIdx.x & 31) >> 2) + (q >= 2 ? 8 : 0); }
__device__ __forceinline__ int frag_col(int q) { return 2 * (threadIdx.x & 3) + (q & 1); }

// BF16 weights (global, unpadded) and FP32 biases into shared memory.
__device__ inline void mlp_load_weights(MlpFwdSmem& s, const bf16* wb, const float* p) {
    for (int i = threadIdx.x; i < MLP_H * MLP_IN; i += blockDim.x)
        s.w1[(i / MLP_IN) * LDI + i % MLP_IN] = wb[BOFF_W1 + i];
    for (int i = threadIdx.x; i < MLP_H * MLP_H; i += blockDim.x)
        s.w2[(i / MLP_H) * LDH + i % MLP_H] = wb[BOFF_W2 + i];
    for (int i = threadIdx.x; i < 16 * MLP_H; i += blockDim.x)
        s.w3[(i / MLP_H) * LDH + i % MLP_H] = wb[BOFF_W3 + i];
    for (int i = threadIdx.x; i < MLP_H; i += blockDim.x) {
        s.b1[i] = p[OFF_B1 + i];
        s.b2[i] = p[OFF_B2 + i];
    }
    for (int i = threadIdx.x; i < MLP_OUT; i += blockDim.x) s.b3[i] = p[OFF_B3 + i];
}

// Shared-memory weights of the network (padded rows).
struct MlpW {
    const bf16* w1;
    const bf16* w2;
    const bf16* w3;
    const float* b1;
    const float* b2;
    const float* b3;
};

// Forward pass of 16 samples: x (16 rows, stride LDI) -> BF16 activations h1,
// h2 (16 rows, stride LDH) and the FP32 outputs as the accumulator fragment y
// (16 x 8).  One warp; x must be complete before the call.
__device__ inline void mlp_forward16(const MlpW& W, const bf16* x, bf16* h1, bf16* h2, float y[4]) {
    {   // H1 = tanh(X W1^T + b1)
        uint32_t a[4];
        mlp_load_a(a, x, LDI, 1);
#pragma unroll
        for (int nt = 0; nt < MLP_H / 8; nt++) {
            float c[4] = {0.f, 0.f, 0.f, 0.f};
            uint32_t b[2];
            mlp_load_b(b, W.w1 + (8 * nt) * LDI, 1, LDI);
            mma_bf16_16816(c, a, b);
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int col = 8 * nt + frag_col(q);
                h1[frag_row(q) * LDH + col] = __float2bfloat16_rn(tanhf(c[q] + W.b1[col]));
            }
        }
    }
    __syncwarp();
    {   // H2 = tanh(H1 W2^T + b2)
        uint32_t a[4][4];
#pragma unroll
        for (int kt = 0; kt < 4; kt++) mlp_load_a(a[kt], h1 + 16 * kt, LDH, 1);
#pragma unroll
        for (int nt = 0; nt < MLP_H / 8; nt++) {
            float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int kt = 0; kt < 4; kt++) {
                uint32_t b[2];
                mlp_load_b(b, W.w2 + (8 * nt) * LDH + 16 * kt, 1, LDH);
                mma_bf16_16816(c, a[kt], b);
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int col = 8 * nt + frag_col(q);
                h2[frag_row(q) * LDH + col] = __float2bfloat16_rn(tanhf(c[q] + W.b2[col]));
            }
        }
    }
    __syncwarp();
    {   // Y = H2 W3^T + b3
        float c[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int kt = 0; kt < 4; kt++) {
            uint32_t a[4], b[2];
            mlp_load_a(a, h2 + 16 * kt, LDH, 1);
            mlp_load_b(b, W.w3 + 16 * kt, 1, LDH);
            mma_bf16_16816(c, a, b);
        }
#pragma unroll
        for (int q = 0; q < 4; q++) y[q] = c[q] + W.b3[frag_col(q)];
    }
}

// Forward pass of the 16 samples [r0, r0 + 16) of the tile in s.x.
__device__ inline void mlp_forward_warp(MlpFwdSmem& s, int r0, float y[4]) {
    const MlpW W{s.w1, s.w2, s.w3, s.b1, s.b2, s.b3};
    mlp_forward16(W, s.x + r0 * LDI, s.h1 + r0 * LDH, s.h2 + r0 * LDH, y);
}

}  // namespace dd
