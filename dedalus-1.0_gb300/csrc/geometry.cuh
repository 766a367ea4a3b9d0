// Grid geometry shared by host launchers and kernels.
//
// Layouts follow the reference Fourier representation
// (dedalus/data_objects/representations.py:86-93, 173-176):
//   3D  x-space [z][y][x] float,  k-space [ky][kz][kx] complex, kx in [0, Nx/2]
//   2D  x-space [y][x]    float,  k-space [kx][ky]     complex
// Kept (non-dealiased) modes along each axis are |m| <= M: indices [0, M] and,
// for the full (complex) axes, [N-M, N).  Intermediate transform buffers hold
// kept modes only, in compact order (kept index c -> full index c <= M ? c :
// c + N - K with K = 2M + 1).
#pragma once
#include <stdint.h>

namespace dd {

struct Geo3 {
    int Nz, Ny, Nx, Nh;  // x-space sizes, Nh = Nx/2 + 1
    int Mx, My, Mz;      // largest kept |m| per axis
    int Kx, Ky, Kz;      // kept counts: Kx = Mx+1, Ky = 2My+1, Kz = 2Mz+1
    __host__ __device__ int64_t kcount() const { return (int64_t)Ny * Nz * Nh; }
    __host__ __device__ int64_t xcount() const { return (int64_t)Nz * Ny * Nx; }
    // compact buffers
    __host__ __device__ int64_t w1count() const { return (int64_t)Ky * Nz * Kx; }  // [kyc][z][kxc]
    __host__ __device__ int64_t w2count() const { return (int64_t)Nz * Ny * Kx; }  // [z][y][kxc]
};

struct Geo2 {
    int Ny, Nx, Nh;
    int Mx, My;
    int Kx, Ky;
    __host__ __device__ int64_t kcount() const { return (int64_t)Nh * Ny; }
    __host__ __device__ int64_t xcount() const { return (int64_t)Ny * Nx; }
    __host__ __device__ int64_t wcount() const { return (int64_t)Ny * Kx; }  // [y][kxc]
};

__host__ __device__ __forceinline__ bool kept_full(int i, int N, int M) { return i <= M || i >= N - M; }
__host__ __device__ __forceinline__ int full_to_compact(int i, int N, int K) { return i <= (K - 1) / 2 ? i : i - (N - K); }
__host__ __device__ __forceinline__ int compact_to_full(int c, int N, int K) { return c <= (K - 1) / 2 ? c : c + (N - K); }

// Field pointers passed by value to kernels (MHD uses 12 transform fields).
#define DD_MAXF 16
struct Ptrs {
    void* p[DD_MAXF];
};
struct CPtrs {
    const void* p[DD_MAXF];
};

// p[i] for a runtime i < N from a pointer table passed by value: a chain of
// selects over the compile-time range, so the table stays in the parameter
// space (indexing it directly would copy it to every thread's local memory).
template <int N, typename PT>
__device__ __forceinline__ PT pick_ptr(const PT* p, int i) {
    PT r = p[0];
#pragma unroll
    for (int j = 1; j < N; j++)
        if (i == j) r = p[j];
    return r;
}


}  // namespace dd
