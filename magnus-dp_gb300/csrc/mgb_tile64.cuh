// FP64 tile products for the GPU-wide small-algebra kernels (chunk scans,
// Omega / D / E assembly and their adjoints): one CTA of 256 threads
// (16 x 16) computes a T x T tile (T = 16 or 32) of a sum of d x d products,
// staging T x T operand blocks in shared memory.
#pragma once

#include <cstdint>

namespace mgb {
namespace t64 {

constexpr int SNT = 256;  // 16 x 16 threads

template <int T>
struct ScanTile {
    static constexpr int R = T / 16;  // outputs per thread along each axis
    static constexpr int P = T + 1;   // shared-memory pitch (doubles)
};

// acc[a][b] += sum_k X[r][k] Y[k][c] over all of k, for r = r0 + ty + 16a,
// c = c0 + tx + 16b; X, Y row-major d x d; TRANS_X / TRANS_Y: use the
// transpose of X / Y.
template <int T, bool TRANS_X, bool TRANS_Y = false>
__device__ __forceinline__ void tile_accumulate(double (&acc)[ScanTile<T>::R][ScanTile<T>::R],
                                                const double* __restrict__ X, const double* __restrict__ Y, int d,
                                                int r0, int c0, double* __restrict__ sX, double* __restrict__ sY) {
    constexpr int R = ScanTile<T>::R, P = ScanTile<T>::P;
    const int tid = threadIdx.x, ty = tid / 16, tx = tid % 16;
    for (int k0 = 0; k0 < d; k0 += T) {
        for (int e = tid; e < T * T; e += SNT) {
            if (TRANS_X) {
                const int kk = e / T, i = e % T;
                sX[i * P + kk] = X[(int64_t)(k0 + kk) * d + r0 + i];
            } else {
                const int i = e / T, kk = e % T;
                sX[i * P + kk] = X[(int64_t)(r0 + i) * d + k0 + kk];
            }
            if (TRANS_Y) {
                const int j = e / T, kk = e % T;
                sY[kk * P + j] = Y[(int64_t)(c0 + j) * d + k0 + kk];
            } else {
                const int kk = e / T, j = e % T;
                sY[kk * P + j] = Y[(int64_t)(k0 + kk) * d + c0 + j];
            }
        }
        __syncthreads();
#pragma unroll 8
        for (int kk = 0; kk < T; ++kk) {
            double av[R], bv[R];
#pragma unroll
            for (int a = 0; a < R; ++a) av[a] = sX[(ty + 16 * a) * P + kk];
#pragma unroll
            for (int b = 0; b < R; ++b) bv[b] = sY[kk * P + tx + 16 * b];
#pragma unroll
            for (int a = 0; a < R; ++a)
#pragma unroll
                for (int b = 0; b < R; ++b) acc[a][b] = fma(av[a], bv[b], acc[a][b]);
        }
        __syncthreads();
    }
}

template <int T>
__device__ __forceinline__ void tile_zero(double (&acc)[ScanTile<T>::R][ScanTile<T>::R]) {
#pragma unroll
    for (int a = 0; a < ScanTile<T>::R; ++a)
#pragma unroll
        for (int b = 0; b < ScanTile<T>::R; ++b) acc[a][b] = 0.0;
}

// Element offset inside a d x d matrix of this thread's output (a, b) of
// the tile at (r0, c0).
template <int T>
__device__ __forceinline__ int64_t tile_el(int d, int r0, int c0, int a, int b) {
    const int ty = threadIdx.x / 16, tx = threadIdx.x % 16;
    return (int64_t)(r0 + ty + 16 * a) * d + c0 + tx + 16 * b;
}

}  // namespace t64
}  // namespace mgb
