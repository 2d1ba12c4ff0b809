// Chunk scans for matrix instances with d a multiple of 16, spread over the
// whole GPU.  The scan over chunks is sequential in c,
//     pi^{c+1}_j = pi^c_j + Lambda^c_j + sum_{m<j} Lambda^c_{j-m} pi^c_m,
//     rho^{c-1}_m = rho^c_m + sum_{j>m} (Lambda^c_{j-m})^T rho^c_j,
// (Chen's identity and its adjoint) but each step is n(n-1)/2 independent
// d x d products.  One launch per chunk step covers every instance of a
// segment that still has that step (instances sorted by chunk count, so the
// active ones are a prefix), with one CTA per (instance, level, T x T output
// tile).  FP64 throughout: these carries are where rounding of the mixed form
// would grow.  The one-CTA-per-instance kernels in mgb_generic.cu serialise
// all C steps of an instance on one SM, which at d = 128 made the scans, not
// the chunk kernels, the critical path of a batch.
#include <vector>

#include "mgb_kernels.h"
#include "mgb_tile64.cuh"

namespace mgb {
namespace {

using namespace t64;

// Block -> (instance, level j in 1..nmax, tile); levels beyond the
// instance's order return at once (uniformly for the block).
struct TileIdx {
    int inst, j, r0, c0;
};
template <int T>
__device__ __forceinline__ TileIdx tile_index(int nmax, int tpl, int d) {
    const int per = nmax * tpl;
    TileIdx t;
    t.inst = blockIdx.x / per;
    const int rem = blockIdx.x % per;
    t.j = 1 + rem / tpl;
    const int tt = rem % tpl, tpr = d / T;
    t.r0 = (tt / tpr) * T;
    t.c0 = (tt % tpr) * T;
    return t;
}

// pi^{c+1} from pi^c and Lambda^c; step 0 also writes pi^0 = 0.
template <int T>
__global__ void __launch_bounds__(SNT) k_scan_step(const InstDev* __restrict__ insts, int c, int nmax, int tpl) {
    constexpr int R = ScanTile<T>::R, P = ScanTile<T>::P;
    __shared__ double sX[T * P], sY[T * P];
    const InstDev& I = insts[blockIdx.x / (nmax * tpl)];
    const TileIdx t = tile_index<T>(nmax, tpl, I.d);
    if (t.j > I.n || c >= I.C) return;
    const int d = I.d, m = I.m, j = t.j;
    const int64_t nm = (int64_t)I.n * m;
    const double* pc = I.pi + (int64_t)c * nm;
    const double* lc = I.lam + (int64_t)c * nm;
    double* pn = I.pi + (int64_t)(c + 1) * nm;
    double acc[R][R];
#pragma unroll
    for (int a = 0; a < R; ++a)
#pragma unroll
        for (int b = 0; b < R; ++b) acc[a][b] = 0.0;
    if (c > 0)
        for (int mm = 1; mm < j; ++mm)
            tile_accumulate<T, false>(acc, lc + (int64_t)(j - mm - 1) * m, pc + (int64_t)(mm - 1) * m, d, t.r0, t.c0,
                                      sX, sY);
    const int ty = threadIdx.x / 16, tx = threadIdx.x % 16;
#pragma unroll
    for (int a = 0; a < R; ++a)
#pragma unroll
        for (int b = 0; b < R; ++b) {
            const int64_t idx = (int64_t)(j - 1) * m + (int64_t)(t.r0 + ty + 16 * a) * d + t.c0 + tx + 16 * b;
            if (c == 0) {
                I.pi[idx] = 0.0;
                pn[idx] = lc[idx];
            } else {
                pn[idx] = pc[idx] + lc[idx] + acc[a][b];
            }
        }
}

// rho^{C-1} = tau, and zero the dA rows shared by two chunks (the chunk
// VJP kernels accumulate them with atomics).  PARTS CTAs per instance.
constexpr int PARTS = 8;
__global__ void __launch_bounds__(SNT) k_rscan_init(const InstDev* __restrict__ insts, int f64io) {
    const InstDev& I = insts[blockIdx.x / PARTS];
    const int part = blockIdx.x % PARTS;
    const int64_t nm = (int64_t)I.n * I.m;
    double* last = I.rho + (int64_t)(I.C - 1) * nm;
    for (int64_t idx = part * SNT + threadIdx.x; idx < nm; idx += PARTS * SNT) last[idx] = I.tau[idx];
    const bool f64 = f64io != 0;
    for (int64_t idx = part * SNT + threadIdx.x; idx < (int64_t)(I.C - 1) * I.m; idx += PARTS * SNT) {
        const int c = 1 + (int)(idx / I.m), el = (int)(idx % I.m);
        store_out<double>(I.dA, (int64_t)c * I.K * I.m + el, 0.0, f64);
    }
}

// rho^{c-1} from rho^c and Lambda^c (c >= 1); the block's level is m.
template <int T>
__global__ void __launch_bounds__(SNT) k_rscan_step(const InstDev* __restrict__ insts, int c, int nmax, int tpl) {
    constexpr int R = ScanTile<T>::R, P = ScanTile<T>::P;
    __shared__ double sX[T * P], sY[T * P];
    const InstDev& I = insts[blockIdx.x / (nmax * tpl)];
    const TileIdx t = tile_index<T>(nmax, tpl, I.d);
    if (t.j > I.n || c >= I.C) return;
    const int d = I.d, m = I.m, n = I.n, mm = t.j;
    const int64_t nm = (int64_t)n * m;
    const double* r = I.rho + (int64_t)c * nm;
    const double* lc = I.lam + (int64_t)c * nm;
    double* rn = I.rho + (int64_t)(c - 1) * nm;
    double acc[R][R];
#pragma unroll
    for (int a = 0; a < R; ++a)
#pragma unroll
        for (int b = 0; b < R; ++b) acc[a][b] = 0.0;
    for (int j = mm + 1; j <= n; ++j)
        tile_accumulate<T, true>(acc, lc + (int64_t)(j - mm - 1) * m, r + (int64_t)(j - 1) * m, d, t.r0, t.c0, sX, sY);
    const int ty = threadIdx.x / 16, tx = threadIdx.x % 16;
#pragma unroll
    for (int a = 0; a < R; ++a)
#pragma unroll
        for (int b = 0; b < R; ++b) {
            const int64_t idx = (int64_t)(mm - 1) * m + (int64_t)(t.r0 + ty + 16 * a) * d + t.c0 + tx + 16 * b;
            rn[idx] = r[idx] + acc[a][b];
        }
}

template <int T>
cudaError_t scan_steps(const InstDev* insts, int count, int d, int nmax, const std::vector<int32_t>& active, bool reverse,
                       int f64io, cudaStream_t st) {
    const int tpl = (d / T) * (d / T);
    const int cmax = (int)active.size();
    if (!reverse) {
        for (int c = 0; c < cmax; ++c) {
            const unsigned grid = (unsigned)active[c] * (unsigned)(nmax * tpl);
            k_scan_step<T><<<grid, SNT, 0, st>>>(insts, c, nmax, tpl);
        }
        return cudaGetLastError();
    }
    k_rscan_init<<<(unsigned)count * PARTS, SNT, 0, st>>>(insts, f64io);
    for (int c = cmax - 1; c >= 1; --c) {
        const unsigned grid = (unsigned)active[c] * (unsigned)(nmax * tpl);
        k_rscan_step<T><<<grid, SNT, 0, st>>>(insts, c, nmax, tpl);
    }
    return cudaGetLastError();
}

}  // namespace

bool scan_tiled_ok(int kind, int d) { return kind == KIND_MATRIX && d >= 16 && d % 16 == 0; }

cudaError_t launch_scan_tiled(const InstDev* insts, int count, int d, int nmax, const std::vector<int32_t>& active,
                              bool reverse, int f64io, cudaStream_t st) {
    if (count <= 0 || active.empty()) return cudaSuccess;
    if (d % 32 == 0 && d >= 64) return scan_steps<32>(insts, count, d, nmax, active, reverse, f64io, st);
    return scan_steps<16>(insts, count, d, nmax, active, reverse, f64io, st);
}

}  // namespace mgb
